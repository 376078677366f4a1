"""The reference's own scene fixture (scene/CBox/cbox.xml) rendered from both
loaders' output: the scene this library's loader parses and the scene the
reference's loader builds (oracle/refloader.py, recorded at build time where
the reference's tree is, since the file is absent on the GPU machine). The CPU
tests (tests/test_loader_ref.py) show the two descriptions hold the same
floats; here the renders of the two must be the same image bit for bit.
"""
import os

import numpy as np
import pytest

import gr
import ref_gpu

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not (os.path.exists(ref_gpu.CBOX_SCENE) and
                                      os.path.exists(ref_gpu.CBOX_REFLOADER_SCENE)),
                                 reason="the CBox scenes are recorded only where the reference's tree is")]


def test_cbox_from_both_loaders_renders_the_same_image(ctx):
    ours = ref_gpu.load_desc(ref_gpu.CBOX_SCENE, 200, 150)
    theirs = ref_gpu.load_desc(ref_gpu.CBOX_REFLOADER_SCENE, 200, 150)
    imgs = []
    for d in (ours, theirs):
        s = gr.Scene(ctx, d)
        img, st = s.render(8, max_depth=8, seed=11)
        assert st.device_errors == 0
        imgs.append(img)
        s.close()
    assert np.isfinite(imgs[0]).all() and imgs[0].mean() > 0
    assert np.array_equal(imgs[0].view(np.uint32), imgs[1].view(np.uint32))
