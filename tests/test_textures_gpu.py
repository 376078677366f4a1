"""Textures, environment maps and rough plastic: a scene with a checkerboard (texcoords), a
bitmap looked up at barycentrics, a textured conductor and a rotated
latitude-longitude environment map renders like the oracle, alone and in a
batch, in both integrator modes."""
import numpy as np
import pytest

import gr
from gr import scenes as sc

pytestmark = pytest.mark.gpu

IMAGE_TOL = 1e-3


def _rel(a, b):
    return float(np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-30))


@pytest.mark.parametrize("flags", [0, gr.RENDER_REFERENCE_COMPAT])
def test_textured_scene_matches_oracle(ctx, oracle, flags):
    d = sc.textured_scene(64, 48)
    s = gr.Scene(ctx, d)
    s.render(4, max_depth=6, seed=11, flags=flags, want_image=False)
    got = s.accumulation()[0]
    want = oracle.render(d, 4, max_depth=6, seed=11, flags=flags)
    assert _rel(got, want) < IMAGE_TOL


def test_textures_change_the_image(ctx):
    d = sc.textured_scene(48, 32)
    plain = sc.SceneDesc(d.meshes, [{k: v for k, v in m.items() if k != "color_map"} for m in d.materials],
                         d.camera, (0.5, 0.5, 0.5))
    a, b = gr.Scene(ctx, d), gr.Scene(ctx, plain)
    ia, _ = a.render(4, max_depth=6, seed=2)
    ib, _ = b.render(4, max_depth=6, seed=2)
    assert np.isfinite(ia).all()
    assert _rel(ia, ib) > 0.05


def test_textured_batch_equals_alone(ctx):
    d1, d2 = sc.textured_scene(40, 30, seed_salt=1), sc.cornell_box(32, 32)
    alone = []
    for d in (d1, d2):
        s = gr.Scene(ctx, d)
        s.render(3, max_depth=6, seed=5, want_image=False)
        alone.append(s.accumulation()[0])
    scenes = [gr.Scene(ctx, d1), gr.Scene(ctx, d2)]
    gr.render_batch(ctx, scenes, [dict(spp=3, max_depth=6, seed=5)] * 2)
    for s, want in zip(scenes, alone):
        np.testing.assert_array_equal(s.accumulation()[0], want)


@pytest.mark.parametrize("flags", [0, gr.RENDER_REFERENCE_COMPAT])
def test_rough_plastic_matches_oracle(ctx, oracle, flags):
    d = sc.plastic_scene(64, 48)
    s = gr.Scene(ctx, d)
    s.render(4, max_depth=6, seed=13, flags=flags, want_image=False)
    assert _rel(s.accumulation()[0], oracle.render(d, 4, max_depth=6, seed=13, flags=flags)) < IMAGE_TOL
