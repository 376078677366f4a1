"""gr_image_write (the reference's FrameBuffer::output / WriteImage step,
framebuffer.cpp:11-26, imageio.cpp:59-82): host-only, no GPU. PNG pixels are
the reference's GammaCorrect + clamp(255 g + 0.5) of each channel with the rows
flipped; PFM holds the floats bit for bit, bottom row first."""
import struct
import zlib

import numpy as np
import pytest

import gr
from gr import imageio


def _read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, ihdr = 8, b"", None
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        tag, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        crc = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        assert crc == zlib.crc32(tag + body) & 0xFFFFFFFF
        if tag == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    w, h, depth, ctype = ihdr[0], ihdr[1], ihdr[2], ihdr[3]
    assert (depth, ctype) == (8, 2)
    raw = zlib.decompress(idat)  # also checks the Adler-32
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + 3 * w)
    assert np.all(rows[:, 0] == 0)
    return rows[:, 1:].reshape(h, w, 3)


def _image(h, w, seed=0):
    r = np.random.default_rng(seed)
    img = r.exponential(0.5, (h, w, 3)).astype(np.float32)
    img[0, 0] = (0.0, 0.002, 0.0031308)  # the linear segment and its end
    if w > 1:
        img[0, 1] = (1.0, 7.5, -0.25)    # clamped above and below
    return img


@pytest.mark.parametrize("h,w", [(1, 1), (3, 5), (300, 250)])
def test_png_is_the_reference_conversion_flipped(tmp_path, h, w):
    img = _image(h, w)
    p = tmp_path / "out.png"
    gr.image_write(p, img)
    got = _read_png(p)
    want = imageio.to_srgb8(img)[::-1]
    assert got.shape == want.shape
    # host powf against numpy's: at most one step apart, almost always equal
    diff = np.abs(got.astype(int) - want.astype(int))
    assert diff.max() <= 1 and (diff == 0).mean() > 0.999


def test_png_of_a_large_image_spans_several_deflate_blocks(tmp_path):
    img = _image(256, 400, seed=3)  # 256 rows x 1,201 bytes > 65,535 bytes
    p = tmp_path / "big.png"
    gr.image_write(p, img)
    assert _read_png(p).shape == (256, 400, 3)


def test_pfm_holds_the_floats_bottom_row_first(tmp_path):
    img = _image(7, 9, seed=1)
    p = tmp_path / "out.pfm"
    gr.image_write(p, img)
    back = imageio.read_pfm(p)  # rows as stored: bottom first
    np.testing.assert_array_equal(back.view(np.uint32), img[::-1].view(np.uint32))
    assert open(p, "rb").read(3) == b"PF\n"


def test_rejects_bad_arguments(tmp_path):
    with pytest.raises(gr.GrError) as e:
        gr.image_write(tmp_path / "x.bmp", np.zeros((2, 2, 3), np.float32))
    assert e.value.status == 1
    with pytest.raises(gr.GrError) as e:
        gr.image_write(tmp_path / "missing_dir" / "x.png", np.zeros((2, 2, 3), np.float32))
    assert e.value.status == 7
    with pytest.raises(ValueError):
        gr.image_write(tmp_path / "x.png", np.zeros((2, 2), np.float32))
