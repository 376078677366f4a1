"""Edge cases of the build, traversal and render paths, each against the oracle
or a stated expectation: degenerate triangles (zero area, collinear,
coincident vertices, all the soup's vertices at one point), ray batches of
size zero, empty ray intervals, rays starting on a triangle, every node layout,
and renders with no light, no geometry or no samples."""
import numpy as np
import pytest

import gr
import gr.scenes as sc

pytestmark = pytest.mark.gpu


def _bits(h):
    return np.ascontiguousarray(h).view(np.uint32)


def _degenerate_soup(n=5000, salt=401):
    v = sc.triangle_soup(n, seed_salt=salt).reshape(n, 3, 3).copy()
    v[0::7, 1] = v[0::7, 0]                                  # two coincident vertices
    v[1::7, 2] = 0.5 * (v[1::7, 0] + v[1::7, 1])             # collinear
    v[2::7, :] = v[2::7, 0:1]                                # all three at one point
    v[3::7, :, 2] = 0.25                                     # flat in z (fine: non-degenerate)
    return np.ascontiguousarray(v.reshape(n, 9), np.float32)


@pytest.mark.parametrize("layout", [gr.LAYOUT_BVH2, gr.LAYOUT_BVH4, gr.LAYOUT_BVH4_Q8, gr.LAYOUT_BVH8_Q8])
def test_degenerate_triangles_match_oracle_and_never_hit(ctx, oracle, layout):
    v = _degenerate_soup()
    b = gr.BVH(ctx)
    b.build_host(v)
    ob = oracle.lbvh(v)
    got = b.export()
    np.testing.assert_array_equal(got["ref_nodes"], ob["ref_nodes"])
    b.set_layout(layout)
    rays = sc.incoherent_rays(100000, seed_salt=402)
    h = b.trace_host(rays)
    np.testing.assert_array_equal(_bits(h), _bits(oracle.trace(ob, rays)))
    prim = h.view(np.int32)[:, 1]
    hit = prim[prim >= 0]
    # a triangle of zero area is never reported (zero determinant)
    assert not np.isin(hit % 7, [0, 1, 2]).any()
    b.close()


def test_all_vertices_at_one_point(ctx, oracle):
    v = np.tile(np.array([0.3, 0.4, 0.5] * 3, np.float32), (64, 1))
    b = gr.BVH(ctx)
    b.build_host(v)
    np.testing.assert_array_equal(b.export()["ref_nodes"], oracle.lbvh(v)["ref_nodes"])
    h = b.trace_host(sc.incoherent_rays(4096, seed_salt=403))
    assert np.all(h.view(np.int32)[:, 1] == -1)
    b.close()


def test_zero_rays_and_empty_intervals(ctx):
    import torch
    b = gr.BVH(ctx)
    b.build_host(sc.triangle_soup(20000, seed_salt=404))
    d_rays = torch.zeros((1, 8), dtype=torch.float32, device="cuda")
    d_hits = torch.full((1, 4), -5.0, dtype=torch.float32, device="cuda")
    b.trace_device(d_rays, 0, d_hits)  # nothing to do, nothing written
    torch.cuda.synchronize()
    assert float(d_hits[0, 0]) == -5.0
    assert b.trace_host(np.zeros((0, 8), np.float32)).shape == (0, 4)
    rays = sc.incoherent_rays(20000, seed_salt=405)
    rays[:, 6] = 2.0   # tmin
    rays[:, 7] = 1.0   # tmax < tmin: an empty interval
    h = b.trace_host(rays)
    assert np.all(h.view(np.int32)[:, 1] == -1)
    assert np.array_equal(h[:, 0], rays[:, 7])  # a miss reports tmax
    b.close()


def test_rays_leaving_a_surface(ctx, oracle):
    """Rays that start on a triangle and leave it (tmin 0): the start triangle
    is hit at t = 0 or not at all, exactly as the oracle decides."""
    v = sc.triangle_soup(30000, seed_salt=406)
    b = gr.BVH(ctx)
    b.build_host(v)
    ob = oracle.lbvh(v)
    tri = v[:4096].reshape(-1, 3, 3)
    o = tri.mean(axis=1)
    rng = np.random.default_rng(407)
    d = rng.normal(size=(4096, 3)).astype(np.float32)
    rays = np.zeros((4096, 8), np.float32)
    rays[:, 0:3] = o
    rays[:, 3:6] = d
    rays[:, 7] = 1e34
    for layout in (gr.LAYOUT_BVH2, gr.LAYOUT_BVH8_Q8):
        b.set_layout(layout)
        np.testing.assert_array_equal(_bits(b.trace_host(rays)), _bits(oracle.trace(ob, rays)))
    b.close()


def test_render_without_light_is_black_and_without_samples_is_unchanged(ctx):
    d = sc.cornell_box(32, 32)
    for m in d.materials:
        m.pop("emission", None)
    s = gr.Scene(ctx, d)
    img, st = s.render(4, max_depth=8, seed=1)
    assert st.device_errors == 0 and np.all(img == 0.0)
    img0, st0 = s.render(0, max_depth=8, seed=1)  # zero samples: the accumulation stays
    assert st0.samples == 0 and np.array_equal(img0, img)
    s.close()


def test_render_of_environment_only(ctx):
    d = sc.SceneDesc([], [{"type": 0, "color": (0.5, 0.5, 0.5)}],
                     dict(sc.cornell_box(24, 16).camera), (0.25, 0.5, 0.75))
    s = gr.Scene(ctx, d)
    img, st = s.render(2, max_depth=4, seed=3)
    assert st.device_errors == 0
    np.testing.assert_array_equal(img, np.broadcast_to(np.float32([0.25, 0.5, 0.75]), img.shape))
    s.close()
