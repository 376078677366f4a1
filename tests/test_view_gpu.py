"""View operations: the 8-bit output step (sRGB curve, rounding, alpha, black
unsampled pixels) and the viewer's camera moves (zoom, translate, rotate,
resize), each of which restarts the accumulation and renders exactly like a
scene created with the moved camera."""
import numpy as np
import pytest
import torch

import gr
from gr import scenes as sc

pytestmark = pytest.mark.gpu


def _srgb8(v):
    v = v.astype(np.float64)
    g = np.where(v <= 0.0031308, 12.92 * v, 1.055 * np.power(np.maximum(v, 0.0), 1.0 / 2.4) - 0.055)
    return np.clip(255.0 * g + 0.5, 0.0, 255.0).astype(np.int64)


def test_rgba8_matches_srgb_of_the_mean(ctx):
    s = gr.Scene(ctx, sc.cornell_box(64, 48))
    black = s.rgba8()
    assert black.shape == (48, 64, 4)
    assert (black[..., :3] == 0).all() and (black[..., 3] == 255).all()
    s.render(8, max_depth=8, seed=4, want_image=False)
    sums, cnt = s.accumulation()
    mean = (sums / cnt[..., None]).astype(np.float32)
    got = s.rgba8()
    assert (got[..., 3] == 255).all()
    diff = np.abs(got[..., :3].astype(np.int64) - _srgb8(mean))
    assert diff.max() <= 1, diff.max()  # powf vs numpy pow: at most one step at a rounding boundary
    assert (diff == 0).mean() > 0.999
    d = torch.zeros(64 * 48, dtype=torch.int32, device="cuda")
    s.rgba8_device(d, stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d.cpu().numpy().view(np.uint8).reshape(48, 64, 4), got)


def _fresh_render(ctx, desc, cam, spp=4, seed=7):
    f = gr.Scene(ctx, sc.SceneDesc(desc.meshes, desc.materials, cam, desc.env))
    f.render(spp, max_depth=8, seed=seed, want_image=False)
    return f.accumulation()[0]


def _axes(cam):
    m = np.asarray(cam["to_world"], np.float64)
    return m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3]


def test_camera_moves_equal_fresh_scenes(ctx):
    desc = sc.cornell_box(48, 40)
    s = gr.Scene(ctx, desc)
    c0 = s.camera()
    assert c0["width"] == 48 and c0["height"] == 40
    x0, y0, z0, e0 = _axes(c0)
    dir0 = z0 / np.linalg.norm(z0)

    s.render(2, max_depth=8, seed=1, want_image=False)
    s.zoom(0.5)
    assert s.accumulation()[1].sum() == 0  # a camera change restarts the accumulation
    c1 = s.camera()
    np.testing.assert_allclose(_axes(c1)[3], e0 + 0.5 * dir0, rtol=0, atol=1e-5)
    s.render(4, max_depth=8, seed=7, want_image=False)
    np.testing.assert_array_equal(s.accumulation()[0], _fresh_render(ctx, desc, c1))

    s.translate(0.2, -0.1)
    c2 = s.camera()
    h = np.cross(dir0, [0.0, 1.0, 0.0])
    h /= np.linalg.norm(h)
    v = np.cross(h, dir0)
    v /= np.linalg.norm(v)
    np.testing.assert_allclose(_axes(c2)[3], _axes(c1)[3] + 0.2 * h - 0.1 * v, rtol=0, atol=1e-5)

    s.rotate(0.3, 0.1)
    c3 = s.camera()
    x3, y3, z3, e3 = _axes(c3)
    np.testing.assert_allclose(e3, _axes(c2)[3], atol=0)  # rotation keeps the eye
    for a, b in ((x0, x3), (y0, y3), (z0, z3)):  # and the lengths of the axes
        assert abs(np.linalg.norm(a) - np.linalg.norm(b)) < 1e-5
    yaw = np.arctan2(z3[0], z3[2]) - np.arctan2(z0[0], z0[2])
    assert abs((yaw + np.pi) % (2 * np.pi) - np.pi - 0.3) < 0.12  # turned by about the yaw
    s.render(4, max_depth=8, seed=7, want_image=False)
    np.testing.assert_array_equal(s.accumulation()[0], _fresh_render(ctx, desc, c3))


def test_resize_renders_like_a_fresh_scene(ctx):
    desc = sc.cornell_box(32, 32)
    s = gr.Scene(ctx, desc)
    s.render(2, max_depth=8, seed=3, want_image=False)
    s.resize(80, 50)
    assert (s.width, s.height) == (80, 50)
    img, _ = s.render(4, max_depth=8, seed=7)
    assert img.shape == (50, 80, 3)
    np.testing.assert_array_equal(s.accumulation()[0], _fresh_render(ctx, desc, s.camera()))
    assert s.rgba8().shape == (50, 80, 4)
    with pytest.raises(gr.GrError):
        s.resize(0, 10)


def test_scene_write_image_is_the_mean_radiance(ctx, tmp_path):
    """gr_scene_write_image (PathTracer::output): the accumulation's mean, as
    gr_image_write would write it."""
    from gr import imageio
    s = gr.Scene(ctx, sc.cornell_box(40, 24))
    s.render(4, max_depth=8, seed=2, want_image=False)
    sums, cnt = s.accumulation()
    mean = (sums / cnt[..., None]).astype(np.float32)
    s.write_image(tmp_path / "a.pfm")
    np.testing.assert_array_equal(imageio.read_pfm(tmp_path / "a.pfm")[::-1], mean)
    s.write_image(tmp_path / "a.png")
    gr.image_write(tmp_path / "b.png", mean)
    assert open(tmp_path / "a.png", "rb").read() == open(tmp_path / "b.png", "rb").read()
    with pytest.raises(gr.GrError):
        s.write_image(tmp_path / "no_such_dir" / "a.png")
    s.close()
