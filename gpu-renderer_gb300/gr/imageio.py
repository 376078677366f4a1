"""Headless image output: PFM (linear float) and 8-bit sRGB PNG.

The reference writes its accumulation through stb (FrameBuffer::output,
src/renderer/framebuffer.cpp:11-26; WriteImage, imageio.cpp:59-82) flipped
vertically, with the sRGB curve of GammaCorrect (spectrum.h:62-72) and the
8-bit rounding of filter_kernel (pathtracer_kernel.h:804-809). The same
conventions are kept here; row 0 of the image array is the first framebuffer
row.
"""
import struct
import zlib

import numpy as np


def gamma_correct(v):
    v = np.asarray(v, np.float32)
    return np.where(v <= np.float32(0.0031308), np.float32(12.92) * v,
                    np.float32(1.055) * np.power(np.maximum(v, 0), np.float32(1.0 / 2.4)) - np.float32(0.055))


def to_srgb8(img):
    return np.clip(255.0 * gamma_correct(img) + 0.5, 0.0, 255.0).astype(np.uint8)


def write_png(path, img, flip=True):
    rgb = to_srgb8(img)
    if flip:
        rgb = rgb[::-1]
    h, w, _ = rgb.shape
    raw = b"".join(b"\x00" + rgb[y].tobytes() for y in range(h))

    def chunk(tag, data):
        c = struct.pack(">I", len(data)) + tag + data
        return c + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0))
    png += chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(png)


def write_pfm(path, img, flip=True):
    a = np.ascontiguousarray(img, np.float32)
    h, w, _ = a.shape
    # PFM stores rows bottom to top; with flip=True the first framebuffer row ends up at the bottom
    rows = a if flip else a[::-1]
    with open(path, "wb") as f:
        f.write(b"PF\n%d %d\n-1.0\n" % (w, h))
        f.write(rows.astype("<f4").tobytes())


def read_pfm(path):
    with open(path, "rb") as f:
        assert f.readline().strip() == b"PF"
        w, h = map(int, f.readline().split())
        scale = float(f.readline())
        data = np.frombuffer(f.read(), "<f4" if scale < 0 else ">f4").reshape(h, w, 3)
    return data.copy()


def write_image(path, img):
    if path.endswith(".pfm"):
        write_pfm(path, img)
    else:
        write_png(path, img)
