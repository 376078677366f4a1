"""Autotuner: every (layout, block, short stack) configuration traces the same
hits bit for bit, the tuner times all 36 and keeps the fastest, invalid
configurations are refused, and a tuned scene renders the same image."""
import numpy as np
import pytest
import torch

import gr
from gr import scenes as sc

pytestmark = pytest.mark.gpu

LAYOUTS = [gr.LAYOUT_BVH2, gr.LAYOUT_BVH4, gr.LAYOUT_BVH4_Q8, gr.LAYOUT_BVH8_Q8]


def _bits(h):
    return np.ascontiguousarray(h).view(np.uint32)


@pytest.fixture(scope="module")
def soup_case(oracle):
    n = 200000
    v = sc.triangle_soup(n, seed_salt=500)
    return v, oracle.lbvh(v)


@pytest.mark.parametrize("layout", LAYOUTS)
@pytest.mark.parametrize("block", [64, 128, 256])
@pytest.mark.parametrize("short_stack", [8, 12, 16])
def test_every_configuration_matches_oracle(ctx, oracle, soup_case, layout, block, short_stack):
    v, ob = soup_case
    b = gr.BVH(ctx)
    b.build_host(v)
    b.set_layout(layout)
    b.set_tuning(layout, block, short_stack)
    assert b.tuning() == {"layout": gr.LAYOUT_NAMES[layout], "block": block, "short_stack": short_stack}
    rays = sc.incoherent_rays(50000, seed_salt=501)
    np.testing.assert_array_equal(_bits(b.trace_host(rays)), _bits(oracle.trace(ob, rays)))
    s = sc.shadow_rays(50000, seed_salt=502)
    got = b.trace_host(s, any_hit=True)
    # any-hit: occlusion flags equal the oracle's for the same node layout
    quant = layout == gr.LAYOUT_BVH4_Q8
    if layout == gr.LAYOUT_BVH2:
        want = oracle.trace(ob, s, any_hit=True)
    elif layout == gr.LAYOUT_BVH8_Q8:
        want = oracle.trace8(ob, *oracle.bvh8(ob), s, any_hit=True)
    else:
        want = oracle.trace4(ob, oracle.bvh4(ob, quant), quant, s, any_hit=True)
    np.testing.assert_array_equal(_bits(got), _bits(want))


def test_invalid_tuning_is_refused(ctx):
    b = gr.BVH(ctx)
    b.build_host(sc.triangle_soup(100, seed_salt=503))
    before = b.tuning()
    for bad in [(4, 128, 12), (0, 96, 12), (0, 128, 10), (0, 512, 8), (-1, 64, 8)]:
        with pytest.raises(gr.GrError):
            b.set_tuning(*bad)
    assert b.tuning() == before


def test_bvh_autotune_times_all_and_keeps_fastest(ctx, oracle, soup_case):
    v, ob = soup_case
    b = gr.BVH(ctx)
    b.build_host(v)
    rays = sc.incoherent_rays(131072, seed_salt=504)
    dr = torch.from_numpy(rays).cuda()
    dh = torch.zeros((rays.shape[0], 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    table = b.autotune(dr, rays.shape[0], dh)
    assert len(table) == 36
    seen = {(t["layout"], t["block"], t["short_stack"]) for t, _ in table}
    assert len(seen) == 36
    assert all(ms > 0 for _, ms in table)
    best = min(table, key=lambda r: r[1])[0]
    assert b.tuning() == best
    # the tuner's own launches wrote the same hits as every other configuration
    np.testing.assert_array_equal(_bits(dh.cpu().numpy()), _bits(oracle.trace(ob, rays)))
    np.testing.assert_array_equal(_bits(b.trace_host(rays)), _bits(oracle.trace(ob, rays)))


def test_scene_autotune_keeps_image(ctx):
    d = sc.glossy_scene(64, 48, level=3, glass_level=2)
    a = gr.Scene(ctx, d)
    a.render(4, max_depth=10, seed=9, want_image=False)
    ref = a.accumulation()[0]
    b = gr.Scene(ctx, d)
    tune, wave = b.autotune(spp=2, max_depth=6)
    assert tune["layout"] in gr.LAYOUT_NAMES.values()
    assert tune["block"] in (64, 128, 256) and tune["short_stack"] in (8, 12, 16)
    assert wave in (4 << 20, 8 << 20, 16 << 20, 32 << 20, 64 << 20)
    assert b.tuning() == (tune, wave)
    b.render(4, max_depth=10, seed=9, want_image=False)  # autotune cleared the accumulation
    np.testing.assert_array_equal(b.accumulation()[0], ref)


@pytest.mark.parametrize("tuning", [(gr.LAYOUT_BVH2, 64, 8, 4096), (gr.LAYOUT_BVH4, 256, 16, 65536),
                                    (gr.LAYOUT_BVH4_Q8, 128, 12, 0), (gr.LAYOUT_BVH8_Q8, 64, 16, 8192)])
def test_scene_tuning_and_wave_size_keep_image(ctx, tuning):
    d = sc.cornell_box(48, 48)
    a = gr.Scene(ctx, d)
    a.render(3, max_depth=8, seed=2, want_image=False)
    b = gr.Scene(ctx, d)
    b.set_tuning(*tuning)
    b.render(3, max_depth=8, seed=2, want_image=False)
    np.testing.assert_array_equal(a.accumulation()[0], b.accumulation()[0])
