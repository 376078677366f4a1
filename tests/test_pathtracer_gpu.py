"""The reference's PathTracer interface (pathtracer.h:16-46) over gr: a
renderer built from a scene file, progressive render(num), output(png),
reset(), the viewer's camera moves and the display image."""
import struct

import numpy as np
import pytest

import gr
from gr import mitsuba
from gr import scenes as sc

pytestmark = pytest.mark.gpu


def _png_size(path):
    data = open(path, "rb").read(33)
    assert data[:8] == b"\x89PNG\r\n\x1a\n" and data[12:16] == b"IHDR"
    return struct.unpack(">II", data[16:24])


def test_progressive_frames_equal_one_multi_sample_render(ctx, tmp_path):
    """render(1) eight times is render(8) once: the sample sequence continues."""
    d = sc.cornell_box(32, 24)
    a = gr.PathTracer(gr.Scene(ctx, d), max_path_length=8, seed=3)
    for _ in range(8):
        img_a, _ = a.render(1)
    b = gr.PathTracer(gr.Scene(ctx, d), max_path_length=8, seed=3)
    img_b, _ = b.render(8)
    np.testing.assert_array_equal(img_a, img_b)
    assert a.sample_num == 8 and a.get_resolution() == (32, 24)
    a.output(tmp_path / "frame.png")
    assert _png_size(tmp_path / "frame.png") == (32, 24)
    assert a.display().shape == (24, 32, 4)
    a.reset()
    assert a.sample_num == 0 and not a.display()[..., :3].any()


def test_renderer_from_a_scene_file(ctx, tmp_path):
    """PathTracer(filename): the scene written as Mitsuba XML + OBJ and loaded
    back renders the image of the scene built from records."""
    d = sc.cornell_box(24, 20)
    path = mitsuba.write_scene(d, str(tmp_path))
    from_file = gr.PathTracer(gr.load_xml(ctx, path), max_path_length=8, seed=1)
    img_file, _ = from_file.render(4)
    img_rec, _ = gr.PathTracer(gr.Scene(ctx, d), max_path_length=8, seed=1).render(4)
    assert img_file.shape == img_rec.shape == (20, 24, 3)
    np.testing.assert_allclose(img_file, img_rec, rtol=1e-5, atol=1e-6)


def test_camera_moves_restart_the_sequence(ctx):
    d = sc.cornell_box(16, 16)
    pt = gr.PathTracer(gr.Scene(ctx, d), max_path_length=4)
    pt.render(2)
    pt.zoom(0.5)
    assert pt.sample_num == 0 and not pt.display()[..., :3].any()
    pt.render(1)
    pt.resize(20, 10)
    assert pt.get_resolution() == (20, 10)
    img, _ = pt.render(1)
    assert img.shape == (10, 20, 3) and np.isfinite(img).all()
