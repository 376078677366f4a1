"""Image parity at the benchmark configurations' own sizes (GPU against the
CPU oracle integrator, same seeds, same paths), and convergence at the plain
render configuration's size.

  - the Cornell box exactly as benchmarked: 256 x 256, 16 spp, max depth 8;
  - the glossy scene's full geometry (four level-8 displaced icospheres,
    5,242,880 triangles, plus the glass sphere, ground and light) at its full
    1024 x 768 resolution, max depth 16, roulette after depth 3, at 1 spp (the
    oracle traces every path on the host);
  - whole jobs of the 64-job batch, one per material mix: Lambert only, GGX
    conductors only, dielectrics only, and all three together, each at its own
    resolution and spp, max depth 8.

Both sides round every shading operation as written; they differ only in the
last bits of sqrt / sin / cos between CUDA and the host's libm, so images agree
within IMAGE_TOL (mean per-pixel relative error), not bit for bit.
"""
import numpy as np
import pytest

import gr
from gr import scenes as sc

pytestmark = pytest.mark.gpu

IMAGE_TOL = 1e-3
# 256 x 256 Cornell box, max depth 8: RMSE of a 16-spp render against a
# 16,384-spp render of the same scene, relative to that render's mean
# radiance (measured 0.22-0.24 on GB300); the bound sits 1.5x above it.
CONVERGED_RMSE_16SPP = 0.35


def mean_rel_err(a, b):
    """Mean per-pixel relative error, with a floor of 1% of the image mean for
    near-black pixels."""
    floor = 0.01 * max(float(np.mean(np.abs(b))), 1e-6)
    return float(np.mean(np.abs(a - b) / np.maximum(np.abs(b), floor)))


def test_config1_cornell_256_16spp_matches_oracle(ctx, oracle):
    d = sc.cornell_box(256, 256)
    s = gr.Scene(ctx, d)
    img, st = s.render(16, max_depth=8, seed=2024)
    ref = oracle.render(d, 16, max_depth=8, seed=2024) / 16.0
    err = mean_rel_err(img, ref)
    assert err < IMAGE_TOL, err
    assert st.device_errors == 0 and st.samples == 256 * 256 * 16
    s.close()


def test_config3_full_geometry_1024x768_matches_oracle(ctx, oracle):
    d = sc.glossy_scene()
    assert d.num_triangles > 5_260_000 and (d.camera["width"], d.camera["height"]) == (1024, 768)
    s = gr.Scene(ctx, d)
    img, st = s.render(1, max_depth=16, seed=77, rr_depth=3)
    ref = oracle.render(d, 1, max_depth=16, seed=77, rr_depth=3)
    err = mean_rel_err(img, ref)
    assert err < IMAGE_TOL, err
    assert st.device_errors == 0
    s.close()


# one job of the 64-job batch per material mix (besides the Lambert ground and
# light): Lambert only, GGX only, dielectric only, all three
@pytest.mark.parametrize("job,mix", [(21, {0}), (27, {2}), (44, {1}), (42, {0, 1, 2})])
def test_config4_job_matches_oracle(ctx, oracle, job, mix):
    d, spp = sc.batch_job(job)
    assert set(m["type"] for m in d.materials[2:]) == mix
    s = gr.Scene(ctx, d)
    img, st = s.render(spp, max_depth=8, seed=job)
    ref = oracle.render(d, spp, max_depth=8, seed=job) / spp
    err = mean_rel_err(img, ref)
    assert err < IMAGE_TOL, (job, err)
    assert st.device_errors == 0
    s.close()


def test_config1_converged_rmse_against_16k_spp(ctx):
    """At the benchmark's size: a 16-spp render lies within the stated RMSE of
    a 16,384-spp render, and the RMSE falls as 1/sqrt(spp)."""
    d = sc.cornell_box(256, 256)
    ref_scene = gr.Scene(ctx, d)
    ref, _ = ref_scene.render(16384, max_depth=8, seed=90000)
    mean = float(ref.mean())
    rmse = {}
    for spp in (16, 64, 256):
        s = gr.Scene(ctx, d)
        img, _ = s.render(spp, max_depth=8, seed=spp)
        rmse[spp] = float(np.sqrt(np.mean((img - ref) ** 2))) / mean
        s.close()
    ref_scene.close()
    assert rmse[16] < CONVERGED_RMSE_16SPP, rmse
    # ideal ratios 2 and 4 (the 16k reference's own noise is 1/32 of the
    # 16-spp noise); measured 1.8-2.3 and 3.9-4.5
    assert 1.5 < rmse[16] / rmse[64] < 2.7, rmse
    assert 3.2 < rmse[16] / rmse[256] < 5.0, rmse
