"""Wide node layouts (4-wide FP32 and 8-bit, 8-wide 8-bit child boxes): the
GPU collapse and quantisation equal the oracle's word for word, traversal
results equal the oracle's bit for bit, closest hits equal the binary
layout's, and renders are identical across layouts."""
import numpy as np
import pytest

import gr
from gr import scenes as sc

pytestmark = pytest.mark.gpu


def _bits(h):
    return np.ascontiguousarray(h).view(np.uint32)


@pytest.mark.parametrize("n,scale", [(1, 100.0), (2, 100.0), (7, 50.0), (5000, 8.0), (1000000, 1.0)])
@pytest.mark.parametrize("layout", [gr.LAYOUT_BVH4, gr.LAYOUT_BVH4_Q8])
def test_layout_build_and_trace_match_oracle(ctx, oracle, n, scale, layout):
    v = sc.triangle_soup(n, seed_salt=400 + n % 13).reshape(n, 3, 3)
    c = v.mean(axis=1, keepdims=True)
    v = np.ascontiguousarray(((v - c) * scale + c).reshape(n, 9), np.float32)
    b = gr.BVH(ctx)
    b.build_host(v)
    ob = oracle.lbvh(v)
    quant = layout == gr.LAYOUT_BVH4_Q8
    want_nodes = oracle.bvh4(ob, quant)
    np.testing.assert_array_equal(b.export_layout(layout), want_nodes)
    b.set_layout(layout)
    m = 131072 if n >= 1000000 else 40000
    rays = sc.incoherent_rays(m, seed_salt=401)
    got = b.trace_host(rays)
    np.testing.assert_array_equal(_bits(got), _bits(oracle.trace4(ob, want_nodes, quant, rays)))
    np.testing.assert_array_equal(_bits(got), _bits(oracle.trace(ob, rays)))  # same closest hits as binary
    s = sc.shadow_rays(m, seed_salt=402)
    ga = b.trace_host(s, any_hit=True)
    np.testing.assert_array_equal(_bits(ga), _bits(oracle.trace4(ob, want_nodes, quant, s, any_hit=True)))


@pytest.mark.parametrize("n,scale", [(1, 100.0), (2, 100.0), (7, 50.0), (5000, 8.0), (1000000, 1.0)])
def test_bvh8_build_and_trace_match_oracle(ctx, oracle, n, scale):
    v = sc.triangle_soup(n, seed_salt=420 + n % 11).reshape(n, 3, 3)
    c = v.mean(axis=1, keepdims=True)
    v = np.ascontiguousarray(((v - c) * scale + c).reshape(n, 9), np.float32)
    b = gr.BVH(ctx)
    b.build_host(v)
    ob = oracle.lbvh(v)
    want_nodes, want_tris = oracle.bvh8(ob)
    np.testing.assert_array_equal(b.export_layout(gr.LAYOUT_BVH8_Q8), want_nodes)
    np.testing.assert_array_equal(_bits(b.export_layout_tris(gr.LAYOUT_BVH8_Q8)), _bits(want_tris))
    b.set_layout(gr.LAYOUT_BVH8_Q8)
    m = 131072 if n >= 1000000 else 40000
    rays = sc.incoherent_rays(m, seed_salt=421)
    got = b.trace_host(rays)
    np.testing.assert_array_equal(_bits(got), _bits(oracle.trace8(ob, want_nodes, want_tris, rays)))
    np.testing.assert_array_equal(_bits(got), _bits(oracle.trace(ob, rays)))  # same closest hits as binary
    s = sc.shadow_rays(m, seed_salt=422)
    ga = b.trace_host(s, any_hit=True)
    np.testing.assert_array_equal(_bits(ga), _bits(oracle.trace8(ob, want_nodes, want_tris, s, any_hit=True)))
    occluded = _bits(oracle.trace(ob, s, any_hit=True))[:, 1] != 0xFFFFFFFF
    np.testing.assert_array_equal(_bits(ga)[:, 1] != 0xFFFFFFFF, occluded)


def _tied_soups():
    # a lattice of equal, axis-aligned triangles (equal areas and equal slot
    # scores everywhere), the same lattice with every triangle repeated, and a
    # mesh with mixed-sign zero coordinates: the collapse's ties and -0 / +0
    g = np.stack(np.meshgrid(np.arange(12), np.arange(12), np.arange(12), indexing="ij"), -1).reshape(-1, 3)
    base = np.array([[0, 0, 0], [0.5, 0, 0], [0, 0.5, 0]], np.float32)
    lattice = (g[:, None, :].astype(np.float32) + base[None]).reshape(-1, 9)
    doubled = np.repeat(lattice, 3, axis=0)
    signed = lattice - 6.0
    signed[signed == 0] = -0.0
    return {"lattice": lattice, "repeated": doubled, "signed_zero": np.ascontiguousarray(signed, np.float32)}


@pytest.mark.parametrize("name", ["lattice", "repeated", "signed_zero"])
def test_bvh8_collapse_ties_match_oracle(ctx, oracle, name):
    v = np.ascontiguousarray(_tied_soups()[name], np.float32)
    b = gr.BVH(ctx)
    b.build_host(v)
    ob = oracle.lbvh(v)
    want_nodes, want_tris = oracle.bvh8(ob)
    np.testing.assert_array_equal(b.export_layout(gr.LAYOUT_BVH8_Q8), want_nodes)
    np.testing.assert_array_equal(_bits(b.export_layout_tris(gr.LAYOUT_BVH8_Q8)), _bits(want_tris))


def test_bvh8_rebuild_keeps_layout_current(ctx, oracle):
    b = gr.BVH(ctx)
    b.set_layout(gr.LAYOUT_BVH8_Q8)
    for salt in (430, 431):
        v = sc.triangle_soup(20000, seed_salt=salt)
        b.build_host(v)
        ob = oracle.lbvh(v)
        rays = sc.incoherent_rays(20000, seed_salt=salt)
        np.testing.assert_array_equal(_bits(b.trace_host(rays)), _bits(oracle.trace(ob, rays)))


def test_quantised_boxes_contain_fp32_boxes(ctx, oracle):
    n = 20000
    v = sc.triangle_soup(n, seed_salt=410)
    b = gr.BVH(ctx)
    b.build_host(v)
    f = b.export_layout(gr.LAYOUT_BVH4).reshape(-1, 32)
    q = b.export_layout(gr.LAYOUT_BVH4_Q8).reshape(-1, 16)
    ff = f.view(np.float32)
    for G in np.nonzero(f[:, 28])[0][:2000]:
        mask = int(f[G, 28])
        org = q[G, :3].view(np.float32)
        meta = int(q[G, 3])
        for k in range(4):
            if not mask & (1 << k):
                continue
            for a in range(3):
                sc_ = np.float32(2.0) ** (((meta >> (8 * a)) & 0xFF) - 127)
                qlo = (int(q[G, 4 + 2 * a]) >> (8 * k)) & 0xFF
                qhi = (int(q[G, 5 + 2 * a]) >> (8 * k)) & 0xFF
                lo = np.float32(np.float32(qlo) * sc_ + org[a])
                hi = np.float32(np.float32(qhi) * sc_ + org[a])
                assert lo <= ff[G, 8 * a + k] and hi >= ff[G, 8 * a + 4 + k]


@pytest.mark.parametrize("layout", [gr.LAYOUT_BVH4, gr.LAYOUT_BVH4_Q8, gr.LAYOUT_BVH8_Q8])
def test_render_identical_across_layouts(ctx, layout):
    d = sc.glossy_scene(64, 48, level=3, glass_level=2)
    a = gr.Scene(ctx, d)
    a.render(4, max_depth=10, seed=5, want_image=False)
    b = gr.Scene(ctx, d)
    b.set_layout(layout)
    b.render(4, max_depth=10, seed=5, want_image=False)
    np.testing.assert_array_equal(a.accumulation()[0], b.accumulation()[0])


@pytest.mark.parametrize("layout", [gr.LAYOUT_BVH2, gr.LAYOUT_BVH4, gr.LAYOUT_BVH4_Q8, gr.LAYOUT_BVH8_Q8])
def test_surface_rays_equal_brute_force(ctx, oracle, layout):
    """Secondary-ray-like queries on the Cornell box (origins on walls, grazing
    directions): every layout returns the brute-force closest hit bit for bit."""
    v = sc.cornell_box(32, 32).flatten()[0]
    b = gr.BVH(ctx)
    b.build_host(v)
    b.set_layout(layout)
    rays = sc.surface_rays(v, 400000, seed_salt=12)
    np.testing.assert_array_equal(_bits(b.trace_host(rays)), _bits(oracle.trace_brute(v, rays)))



def test_bvh8_builds_share_the_context_scratch(ctx, oracle):
    # two BVHs of one context collapse alternately through the context's
    # scratch (grown by the larger, reused by the smaller): each layout stays
    # equal to the oracle's word for word
    big, small = gr.BVH(ctx), gr.BVH(ctx)
    for salt in (440, 441):
        vb = sc.triangle_soup(60000, seed_salt=salt)
        vs = sc.triangle_soup(3000, seed_salt=salt + 10)
        for b, v in ((small, vs), (big, vb), (small, vs[::-1].copy())):
            b.build_host(v)
            b.set_layout(gr.LAYOUT_BVH8_Q8)
            want_nodes, want_tris = oracle.bvh8(oracle.lbvh(v))
            np.testing.assert_array_equal(b.export_layout(gr.LAYOUT_BVH8_Q8), want_nodes)
            np.testing.assert_array_equal(_bits(b.export_layout_tris(gr.LAYOUT_BVH8_Q8)), _bits(want_tris))
