"""Host-side checks of the launcher for the reference's own traversal kernels
(oracle/ref_gpu.py): the tree walk that guards every launch, and the record
layout it reads. No GPU."""
import json
import os

import numpy as np
import pytest

import gr.scenes as sc
import ref_gpu


def _depth_recursive(nodes, i=0):
    w = nodes.reshape(-1, 8)
    if w[i, 7] & 0xFF:
        return 0
    return 1 + max(_depth_recursive(nodes, i + 1), _depth_recursive(nodes, int(w[i, 6])))


@pytest.mark.parametrize("n", [1, 2, 3, 7, 64, 1000])
def test_tree_depth_matches_recursive_walk(oracle, n):
    v = sc.triangle_soup(n, seed_salt=400 + n)
    nodes = oracle.lbvh(v)["ref_nodes"]
    assert ref_gpu.tree_depth(nodes, n) == _depth_recursive(nodes)


def test_tree_depth_of_identical_triangles(oracle):
    # 64 identical triangles: one Morton code, midpoint splits, depth log2(64)
    v = np.tile(sc.triangle_soup(1, seed_salt=410), (64, 1))
    assert ref_gpu.tree_depth(oracle.lbvh(v)["ref_nodes"], 64) == 6


def test_config2_tree_fits_the_reference_stack(oracle):
    v = sc.triangle_soup(1000000)
    d = ref_gpu.tree_depth(oracle.lbvh(v)["ref_nodes"], 1000000)
    assert d <= ref_gpu.STACK_ENTRIES


@pytest.mark.parametrize("damage", ["child", "leaf_index", "count", "shared_child"])
def test_tree_depth_rejects_indices_out_of_range(oracle, damage):
    n = 100
    nodes = oracle.lbvh(sc.triangle_soup(n, seed_salt=420))["ref_nodes"].copy()
    w = nodes.reshape(-1, 8)
    inner = np.nonzero((w[:, 7] & 0xFF) == 0)[0]
    leaf = np.nonzero(w[:, 7] & 0xFF)[0]
    if damage == "child":
        w[inner[3], 6] = 2 * n + 5
    elif damage == "leaf_index":
        w[leaf[0], 6] = n
    elif damage == "count":
        nodes = nodes[:-8]
    else:
        # the root's right child pointed at a node inside its left subtree
        w[0, 6] = 2
    with pytest.raises(ValueError):
        ref_gpu.tree_depth(nodes, n)


def test_layout_file_when_built():
    if not os.path.exists(ref_gpu.LAYOUT):
        pytest.skip("reference kernels not built here")
    L = ref_gpu.load_layout()
    assert (L["Ray"]["size"], L["Hit"]["size"], L["Hit"]["triangle_id"]) == (32, 16, 4)
    assert L["SceneView"]["m_bvh"] + 8 <= L["SceneView"]["size"]
    assert L["Triangle"]["m_index"] + 4 <= L["Triangle"]["size"]
    assert L["TriangleMeshView"]["m_material"] + L["Material"]["size"] <= L["TriangleMeshView"]["size"]
    assert L["PTContext"]["m_scatter_queue"] + L["RayQueue"]["size"] <= L["PTContext"]["size"]


REF_RECORDS = os.path.join(ref_gpu.REF_DIR, "libref_records.so")
needs_records = pytest.mark.skipif(not (os.path.exists(REF_RECORDS) and os.path.exists(ref_gpu.LAYOUT)),
                                   reason="reference host records not built here")


def _ref_lib():
    import ctypes
    lib = ctypes.CDLL(REF_RECORDS)
    return lib, ctypes


def _floats_close(a, b, rtol=2e-6, atol=1e-6):
    a = np.frombuffer(a.tobytes(), np.float32)
    b = np.frombuffer(b.tobytes(), np.float32)
    np.testing.assert_allclose(a, b, rtol=rtol, atol=atol)


@needs_records
@pytest.mark.parametrize("cam", [
    (sc.cornell_box(256, 256).camera), (sc.cornell_box(64, 48).camera),
    {"to_world": sc.look_at((0.3, 1.2, 4.0), (0.0, 0.4, 0.0), (0, 1, 0)), "fov": 55.0, "width": 1024,
     "height": 768}])
def test_camera_record_matches_reference_setup(cam):
    """Camera() + Camera::setup from the reference's own host code against the
    restatement: integers and flags equal, floats within a few ulp (the
    reference inverts its matrices in float, the restatement in double)."""
    lib, ct = _ref_lib()
    L = ref_gpu.load_layout()
    C = L["Camera"]
    tw = np.ascontiguousarray(np.asarray(cam["to_world"], np.float32).reshape(16))
    want = np.zeros(C["size"], np.uint8)
    rc = lib.ref_camera_record(tw.ctypes.data_as(ct.c_void_p), ct.c_float(cam["fov"]), cam["width"], cam["height"],
                               want.ctypes.data_as(ct.c_void_p), C["size"])
    assert rc == 0
    got = ref_gpu.camera_record(L, np.asarray(cam["to_world"], np.float64).reshape(4, 4), cam["fov"], cam["width"],
                                cam["height"])
    ints = [C["m_resolution_x"], C["m_resolution_y"]]
    for off in ints:
        assert got[off:off + 4].tobytes() == want[off:off + 4].tobytes()
    assert got[C["m_free"]] == want[C["m_free"]] == 0
    for f in ("m_eye", "m_dir", "m_up", "m_yaw", "m_pitch", "m_fov", "m_aspect_ratio"):
        n = {"m_eye": 12, "m_dir": 12, "m_up": 12, "m_fov": 8}.get(f, 4)
        _floats_close(got[C[f]:C[f] + n], want[C[f]:C[f] + n])
    for f in ("m_cameraToWorld", "m_rasterToCamera"):
        g = np.frombuffer(got[C[f]:C[f] + 128].tobytes(), np.float32)
        w = np.frombuffer(want[C[f]:C[f] + 128].tobytes(), np.float32)
        np.testing.assert_allclose(g, w, rtol=1e-5, atol=1e-5 * np.abs(w).max())


@needs_records
@pytest.mark.parametrize("radiance", [None, (0.3, 0.35, 0.45)])
def test_environment_record_matches_reference_setup(radiance):
    lib, ct = _ref_lib()
    L = ref_gpu.load_layout()
    E = L["EnvironmentLightView"]
    center = np.array([0.25, -1.5, 3.0], np.float32)
    rad = np.asarray(radiance or (0, 0, 0), np.float32)
    want = np.zeros(E["size"], np.uint8)
    rc = lib.ref_env_record(1 if radiance else 0, rad.ctypes.data_as(ct.c_void_p), center.ctypes.data_as(ct.c_void_p),
                            want.ctypes.data_as(ct.c_void_p), E["size"])
    assert rc == 0
    got, texels = ref_gpu.env_record(L, radiance, center)
    mask = np.ones(E["size"], bool)
    mask[E["m_buffer"]:E["m_buffer"] + 8] = False  # the pointer (a host address there)
    # bytes the reference leaves unset: padding after the flag
    mask[E["m_has"] + 1:E["m_buffer"]] = False
    np.testing.assert_array_equal(got[mask], want[mask])
    if radiance:
        np.testing.assert_array_equal(texels.reshape(-1), rad)


def test_material_records_follow_the_loader_rules():
    if not os.path.exists(ref_gpu.LAYOUT):
        pytest.skip("reference layout not built here")
    L = ref_gpu.load_layout()
    M, T, E = L["Material"], L["TextureView"], L["enums"]
    mats = [{"type": 2, "color": (0.9, 0.8, 0.7), "alpha": 0.25},
            {"type": 0, "color": (0.5, 0.4, 0.3), "emission": (4.0, 5.0, 6.0)},
            {"type": 1, "color": (1.0, 1.0, 1.0), "ior": 1.33}]
    recs = ref_gpu.material_records(L, mats)

    def typ(b):
        return int(np.frombuffer(b[M["m_type"]:M["m_type"] + 4].tobytes(), np.int32)[0])

    def emission(b):
        return np.frombuffer(b[M["m_emission"]:M["m_emission"] + 12].tobytes(), np.float32)

    (c, ct), (d, dt), (g, gt) = recs
    assert [typ(c), typ(d), typ(g)] == [E["MATERIAL_ROUGH_CONDUCTOR"], E["MATERIAL_DIFFUSE"], E["MATERIAL_SPECULAR"]]
    np.testing.assert_array_equal(emission(d), np.float32([4, 5, 6]))
    np.testing.assert_array_equal(emission(c), np.zeros(3, np.float32))
    # conductor: the loader's default eta / k, etaI 1, alpha as a float texture on both axes
    np.testing.assert_allclose(ct[M["m_etaT"]], ref_gpu.CONDUCTOR_ETA, rtol=1e-6)
    np.testing.assert_allclose(ct[M["m_k"]], ref_gpu.CONDUCTOR_K, rtol=1e-6)
    np.testing.assert_array_equal(ct[M["m_etaI"]], np.ones(3, np.float32))
    np.testing.assert_allclose(ct[M["m_alpha_x"]], [0.25] * 3)
    np.testing.assert_allclose(ct[M["m_alpha_y"]], [0.25] * 3)
    ax = M["m_alpha_x"] + T["m_type"]
    assert int(np.frombuffer(c[ax:ax + 4].tobytes(), np.int32)[0]) == E["TEXTURE_FLOAT"]
    # diffuse after the conductor: its colour replaced, the conductor's textures carried over
    np.testing.assert_allclose(dt[M["m_color"]], [0.5, 0.4, 0.3])
    np.testing.assert_allclose(dt[M["m_k"]], ref_gpu.CONDUCTOR_K, rtol=1e-6)
    # dielectric: ior as a float texture
    np.testing.assert_allclose(gt[M["m_ior"]], [1.33] * 3, rtol=1e-6)
    for b in (c, d, g):
        for f in ("m_color", "m_etaI", "m_etaT", "m_k", "m_ior", "m_alpha_x", "m_alpha_y"):
            o = M[f]
            w, h = np.frombuffer(b[o + T["m_width"]:o + T["m_width"] + 8].tobytes(), np.uint32)
            assert (w, h) == (1, 1)
