"""CPU oracle traversal self-consistency: the product traversal restatement is
bit-exact with brute force, the reference restatement agrees on every ray the
FP64 oracle calls unambiguous, and the watertight test closes shared edges."""
import numpy as np
import pytest

import gr.scenes as sc


def _soup(n, salt, scale=1.0):
    v = sc.triangle_soup(n, seed_salt=salt).reshape(n, 3, 3)
    c = v.mean(axis=1, keepdims=True)
    return np.ascontiguousarray(((v - c) * scale + c).reshape(n, 9), np.float32)


@pytest.mark.parametrize("n,scale", [(1, 200.0), (2, 200.0), (64, 60.0), (3000, 10.0)])
def test_trace_equals_brute_force(oracle, n, scale):
    v = _soup(n, 60 + n, scale)
    bvh = oracle.lbvh(v)
    rays = sc.incoherent_rays(20000, seed_salt=61)
    h = oracle.trace(bvh, rays)
    b = oracle.trace_brute(v, rays)
    np.testing.assert_array_equal(h.view(np.uint32), b.view(np.uint32))
    assert (h.view(np.int32)[:, 1] >= 0).mean() > 0.01
    s = sc.shadow_rays(20000, seed_salt=62)
    ha = oracle.trace(bvh, s, any_hit=True)
    ba = oracle.trace_brute(v, s, any_hit=True)
    np.testing.assert_array_equal(ha.view(np.int32)[:, 1] >= 0, ba.view(np.int32)[:, 1] >= 0)


def test_reference_restatement_agrees_on_unambiguous_rays(oracle):
    v = _soup(4000, 70, 8.0)
    bvh = oracle.lbvh(v)
    rays = sc.incoherent_rays(20000, seed_salt=71)
    mine = oracle.trace(bvh, rays)
    ref = oracle.trace_ref(bvh["ref_nodes"], v, rays)
    pm, pr = mine.view(np.int32)[:, 1], ref.view(np.int32)[:, 1]
    t64, amb = oracle.fp64_check(bvh["ref_nodes"], v, rays, pr)
    ok = ~amb
    assert ok.mean() > 0.95
    np.testing.assert_array_equal(pm[ok], pr[ok])
    hit = ok & (pm >= 0)
    rel = np.abs(mine[hit, 0] - t64[hit]) / np.maximum(np.abs(t64[hit]), 1e-3)
    assert rel.max() < 1e-5


def test_watertight_shared_edge(oracle):
    # a unit quad split along its diagonal; rays aimed exactly at the diagonal
    q = np.array([[0, 0, 0, 1, 0, 0, 1, 1, 0],
                  [0, 0, 0, 1, 1, 0, 0, 1, 0]], np.float32)
    bvh = oracle.lbvh(q)
    t = np.linspace(0.001, 0.999, 4001, dtype=np.float32)
    rays = np.zeros((t.size, 8), np.float32)
    rays[:, 0] = t
    rays[:, 1] = t
    rays[:, 2] = 1.0
    rays[:, 5] = -1.0
    rays[:, 7] = 1e34
    h = oracle.trace(bvh, rays)
    assert np.all(h.view(np.int32)[:, 1] >= 0), "a ray through the shared edge slipped between the triangles"
    # the tie at equal t goes to the lower prim id
    assert np.all(h.view(np.int32)[:, 1] == 0)


def test_axis_parallel_and_grazing_rays(oracle):
    v = _soup(500, 80, 30.0)
    bvh = oracle.lbvh(v)
    r = sc.rng(2, 81)
    m = 6000
    rays = np.zeros((m, 8), np.float32)
    rays[:, :3] = r.random((m, 3), dtype=np.float32)
    axis = r.integers(0, 3, m)
    sign = np.where(r.random(m) < 0.5, -1.0, 1.0).astype(np.float32)
    rays[np.arange(m), 3 + axis] = sign
    rays[:, 7] = 1e34
    h = oracle.trace(bvh, rays)
    b = oracle.trace_brute(v, rays)
    np.testing.assert_array_equal(h.view(np.uint32), b.view(np.uint32))


def test_empty_scene(oracle):
    v = np.zeros((0, 9), np.float32)
    bvh = oracle.lbvh(v)
    assert bvh["root"] == 0xFFFFFFFF
    rays = sc.incoherent_rays(100, seed_salt=82)
    h = oracle.trace(bvh, rays)
    assert np.all(h.view(np.int32)[:, 1] == -1)


@pytest.mark.parametrize("n", [1, 2, 3, 9, 777, 20000])
def test_wide_layouts_equal_binary(oracle, n):
    """The 4- and 8-wide restatements find the binary traversal's closest hits
    and the same occlusion; the 8-wide build places every leaf triangle once."""
    v = sc.triangle_soup(n, seed_salt=900 + n % 7)
    bvh = oracle.lbvh(v)
    rays = sc.incoherent_rays(8000, seed_salt=901)
    shadow = sc.shadow_rays(8000, seed_salt=902)
    want = oracle.trace(bvh, rays)
    occ = oracle.trace(bvh, shadow, any_hit=True).view(np.uint32)[:, 1] != 0xFFFFFFFF
    nodes8, tris8 = oracle.bvh8(bvh)
    got = oracle.trace8(bvh, nodes8, tris8, rays)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    a8 = oracle.trace8(bvh, nodes8, tris8, shadow, any_hit=True).view(np.uint32)[:, 1] != 0xFFFFFFFF
    np.testing.assert_array_equal(a8, occ)
    prims = np.sort(tris8.reshape(-1, 12)[:, 3].view(np.uint32))
    if n > 1:
        np.testing.assert_array_equal(prims, np.arange(n, dtype=np.uint32))
    for quant in (False, True):
        n4 = oracle.bvh4(bvh, quant)
        np.testing.assert_array_equal(oracle.trace4(bvh, n4, quant, rays).view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("scene", ["cornell", "glossy"])
def test_surface_rays_equal_brute_force_in_every_layout(oracle, scene):
    """Rays that start on surfaces and graze axis-aligned walls: every layout's
    traversal finds exactly the brute-force closest hit (a plane distance with
    an absolute rounding error used to cull such hits)."""
    d = sc.cornell_box(32, 32) if scene == "cornell" else sc.glossy_scene(32, 24, level=3, glass_level=2)
    v = d.flatten()[0]
    bvh = oracle.lbvh(v)
    rays = sc.surface_rays(v, 200000 if scene == "cornell" else 50000, seed_salt=11)
    want = oracle.trace_brute(v, rays).view(np.uint32)
    np.testing.assert_array_equal(oracle.trace(bvh, rays).view(np.uint32), want)
    for quant in (False, True):
        n4 = oracle.bvh4(bvh, quant)
        np.testing.assert_array_equal(oracle.trace4(bvh, n4, quant, rays).view(np.uint32), want)
    n8, t8 = oracle.bvh8(bvh)
    np.testing.assert_array_equal(oracle.trace8(bvh, n8, t8, rays).view(np.uint32), want)


@pytest.mark.parametrize("scale,offset", [(1e4, 1e5), (1e-3, 0.0), (1.0, 1e4), (3e5, -2e6)])
def test_layouts_agree_at_extreme_scales(oracle, scale, offset):
    """Far from the origin or at tiny and huge scales the 8-wide quantised
    traversal, whose plane distances carry explicit error margins, returns the
    binary traversal's hits bit for bit."""
    v = (sc.triangle_soup(20000, seed_salt=77).astype(np.float64) * scale + offset).astype(np.float32)
    bvh = oracle.lbvh(v)
    n8, t8 = oracle.bvh8(bvh)
    r = sc.incoherent_rays(20000, seed_salt=78).astype(np.float64)
    r[:, :3] = r[:, :3] * scale + offset
    for rays in (r.astype(np.float32), sc.surface_rays(v, 20000, seed_salt=79)):
        np.testing.assert_array_equal(oracle.trace8(bvh, n8, t8, rays).view(np.uint32),
                                      oracle.trace(bvh, rays).view(np.uint32))


def test_reference_restatement_differs_only_on_ambiguous_rays_config2(oracle):
    """1M-triangle workload, every 4th of its 4M incoherent rays: each ray on
    which our traversal and the reference's pick different triangles is
    ambiguous in FP64 (a second hit within 1e-6 relative, or the hit within
    FP32 rounding of an edge)."""
    v = sc.triangle_soup(1000000)
    ob = oracle.lbvh(v)
    rays = sc.incoherent_rays(4194304)[::4].copy()
    pm = oracle.trace(ob, rays).view(np.int32)[:, 1]
    pr = oracle.trace_ref(ob["ref_nodes"], v, rays).view(np.int32)[:, 1]
    d = np.nonzero(pm != pr)[0]
    assert d.size < rays.shape[0] * 1e-4
    _, amb = oracle.fp64_check(ob["ref_nodes"], v, rays[d], pm[d])
    assert amb.all(), "unambiguous rays differ: %s" % d[~amb][:10]
