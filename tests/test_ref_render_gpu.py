"""Our integrator against the reference's own, both on the GPU.

The reference's kernels (compiled from its sources, oracle/ref/build_ref.sh)
render the same scene records its loader would build, frame by frame, through
its own frame loop (oracle/ref_frame.cpp, oracle/ref_gpu.py). The two
renderers draw different random numbers, so the images agree statistically:

* the reference does not copy a path's random seed when it appends it to the
  scatter queue (rayqueue.h:19-47), so on alternate bounces the paths of one
  frame share their random numbers and its image mean varies from frame to
  frame far more than independent paths would; its standard error is measured
  from batches of frames;
* our image in reference-compatible mode (GR_RENDER_REFERENCE_COMPAT, the
  reference's estimator quirks kept) must lie within 6 combined standard
  errors (the reference's from batches of its frames, ours from independent
  renders) of the reference's, per colour channel, over the whole image and
  over each image quadrant (15 comparisons per scene; 16 batches a side).
"""
import os

import numpy as np
import pytest
import torch

import gr
import gr.scenes as sc
import ref_gpu

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_gpu.render_available("stock"),
                                 reason="reference kernels not built (reference sources absent at build time)")]


@pytest.fixture(scope="module")
def stock():
    rk = ref_gpu.RefKernels("stock")
    yield rk
    rk.close()


def _regions(img):
    h, w = img.shape[:2]
    out = [img.reshape(-1, 3).mean(0)]
    for ys in (slice(0, h // 2), slice(h // 2, h)):
        for xs in (slice(0, w // 2), slice(w // 2, w)):
            out.append(img[ys, xs].reshape(-1, 3).mean(0))
    return np.array(out)  # (5, 3): whole image, four quadrants


def _reference_batches(rk, ctx, desc, batches, frames, depth):
    """One continuous reference render (its seeds carry from frame to frame as
    in the reference), cut into batches of frames: the region means of each
    batch's own samples."""
    b = gr.BVH(ctx)
    b.build_host(desc.flatten()[0])
    rr = ref_gpu.RefRender(rk, desc, b.export()["ref_nodes"])
    h, w = rr.height, rr.width
    prev = np.zeros((h, w, 3))
    means = []
    for _ in range(batches):
        rr.render(frames, depth)
        acc = rr.fb.double().cpu().numpy().reshape(h, w, 3)
        img = (acc - prev) / frames
        prev = acc
        assert np.isfinite(img).all()
        means.append(_regions(img))
    assert int(rr.fb_count.min().item()) == int(rr.fb_count.max().item()) == batches * frames
    del rr
    torch.cuda.empty_cache()
    return np.array(means)  # (batches, 5, 3)


def _cbox():
    """The reference's own fixture scene/CBox/cbox.xml (mirror and glass
    spheres with vertex normals, coloured walls, area light), as this
    library's loader parses it, at 160 x 120."""
    if not os.path.exists(ref_gpu.CBOX_SCENE):
        pytest.skip("the reference's fixture scene was not parsed at build time")
    return ref_gpu.load_desc(ref_gpu.CBOX_SCENE, 160, 120)


def _our_batches(ctx, desc, batches, frames, depth):
    """Our render in reference-compatible mode, as `batches` independent
    renders of `frames` samples (different seeds): the region means of each."""
    means = []
    for k in range(batches):
        s = gr.Scene(ctx, desc)
        img, _ = s.render(frames, max_depth=depth, seed=1000 + k, flags=gr.RENDER_REFERENCE_COMPAT)
        s.close()
        means.append(_regions(np.asarray(img, np.float64)))
    return np.array(means)


@pytest.mark.parametrize("name,make,batches,frames,depth", [
    ("cornell", lambda: sc.cornell_box(64, 64), 16, 64, 8),
    ("glossy", lambda: sc.glossy_scene(128, 96, level=4, glass_level=3), 16, 16, 16),
    ("reference_cbox", _cbox, 16, 16, 8),
])
def test_compat_render_matches_reference_kernels(ctx, stock, name, make, batches, frames, depth):
    """Both images' region means agree within 6 combined standard errors plus
    0.2 % of the mean. Each side's standard error comes from 16 batches, so the
    difference over its standard error follows a t distribution with about 15
    degrees of freedom or more: |t| > 6 has a chance near 3e-5, under 1e-3
    over the 15 comparisons of a scene."""
    desc = make()
    ref = _reference_batches(stock, ctx, desc, batches, frames, depth)
    ref_mean = ref.mean(0)
    ref_se = ref.std(0, ddof=1) / np.sqrt(batches)
    mine = _our_batches(ctx, desc, batches, frames, depth)
    ours = mine.mean(0)
    our_se = mine.std(0, ddof=1) / np.sqrt(batches)
    tol = 6.0 * np.sqrt(ref_se ** 2 + our_se ** 2) + 2e-3 * np.abs(ref_mean)
    assert np.all(np.abs(ours - ref_mean) <= tol), (ours, ref_mean, ref_se, our_se)
