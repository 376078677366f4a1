"""The library's Mitsuba-XML / OBJ loader pinned against the reference's own
loader (CPU).

The reference flattens its meshes into Scene::m_cpu_triangles in mesh order
(src/renderer/scene.cpp:4-14), and that order is what every hit's primitive id
refers to, so the loader must produce the same triangles in the same order,
with the same floats: positions, shading normals, texture coordinates, the
mesh of each triangle, the materials, the camera and the environment.

The expected values come from the reference's loader itself (compiled from its
sources by oracle/ref/build_ref.sh, recorded by tests/golden/make_golden_loader.py
into tests/golden/loader_ref.npz):
  - loader_shapes.xml, this project's fixture with every shape type (cube,
    rectangle, sphere, OBJ with texture coordinates and normals), transform
    kind (scale, rotate, translate, matrix, lookat), named and referenced
    materials, twosided, textures and both emitter kinds: compared array by
    array, bit for bit;
  - the reference's own scene/CBox fixtures, where its tree is present:
    compared by SHA-256 digest of each array, and materials / camera /
    environment in full.
"""
import hashlib
import os
import sys

import numpy as np
import pytest

import gr

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
import refloader  # noqa: E402
import refsrc  # noqa: E402

GOLDEN = np.load(os.path.join(HERE, "golden", "loader_ref.npz"))
FIXTURE = os.path.join(HERE, "golden", "loader_shapes.xml")


def same_bits(a, b):
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(
        a[~np.isnan(a)].view(np.uint32), b[~np.isnan(b)].view(np.uint32))


def ours(path):
    p = gr.ParsedScene(path)
    verts, mesh, mats = p.triangles()
    normals, uvs = p.triangle_attributes()
    return p, verts, normals, uvs, mesh, mats


def check_small(p, mats, ref_materials, ref_camera, ref_env):
    assert len(mats) == ref_materials.shape[0]
    for i, m in enumerate(mats):
        want = refloader.material_fields(ref_materials[i])
        got = refloader.gr_material_fields(m)
        assert sorted(got) == sorted(want), (i, sorted(got), sorted(want))
        for k in want:
            assert same_bits(got[k], want[k]), (i, k, got[k], want[k])
    # camera: cameraToWorld word for word; the reference keeps the field of
    # view in radians (degToRad of the parsed degrees)
    assert same_bits(np.asarray(p.camera["to_world"], np.float32).reshape(-1), ref_camera[:16])
    assert same_bits(refloader.deg_to_rad(p.camera["fov"]), ref_camera[16])
    assert (p.camera["width"], p.camera["height"]) == (int(ref_camera[17]), int(ref_camera[18]))
    if ref_env[0]:
        assert p.env is not None and same_bits(np.array(p.env, np.float32), ref_env[1:4])
    else:
        assert p.env is None


def test_shapes_fixture_matches_reference_loader():
    p, verts, normals, uvs, mesh, mats = ours(FIXTURE)
    assert p.warnings == []
    assert same_bits(verts, GOLDEN["shapes_verts"])
    assert same_bits(normals, GOLDEN["shapes_normals"])
    assert same_bits(uvs, GOLDEN["shapes_uvs"])
    assert np.array_equal(mesh, GOLDEN["shapes_mesh"])
    check_small(p, mats, GOLDEN["shapes_materials"], GOLDEN["shapes_camera"], GOLDEN["shapes_env"])
    p.close()


def test_cube_is_the_references_twelve_triangles():
    # the cube shape in the reference's vertex, triangle and corner order
    # (mitsubaloader.cpp:53-116): the fixture's last cube, scaled by 0.1 and moved
    p, verts, _, uvs, mesh, _ = ours(FIXTURE)
    last = verts[mesh == mesh.max()]
    assert last.shape == (12, 9)
    corners = np.unique(np.round(last.reshape(-1, 3), 5), axis=0)
    assert corners.shape == (8, 3)
    p.close()


@pytest.mark.parametrize("name", ["cbox.xml", "cbox(mesh).xml", "cbox(sphere).xml"])
def test_reference_cbox_matches_reference_loader(name):
    path = refsrc.cbox_scenes().get(name)
    if not path:
        pytest.skip("the reference's scene files are not present here")
    key = name.replace(".xml", "").replace("(", "_").replace(")", "")
    p, verts, normals, uvs, mesh, mats = ours(path)
    n, nmesh = (int(x) for x in GOLDEN[key + "_counts"])
    assert verts.shape[0] == n and len(mats) == nmesh
    for k, a in (("verts", verts), ("normals", normals), ("uvs", uvs), ("mesh", mesh)):
        assert hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest() == str(GOLDEN[key + "_sha_" + k]), k
    check_small(p, mats, GOLDEN[key + "_materials"], GOLDEN[key + "_camera"], GOLDEN[key + "_env"])
    p.close()


def test_golden_is_the_reference_loaders_current_output():
    # where the reference's loader is built, the recorded fixture is what it
    # produces now
    if not refloader.available():
        pytest.skip("the reference loader is not built here")
    r = refloader.load(FIXTURE)
    for k, v in r.items():
        assert same_bits(v, GOLDEN["shapes_" + k]) if v.dtype == np.float32 else np.array_equal(v, GOLDEN["shapes_" + k])
