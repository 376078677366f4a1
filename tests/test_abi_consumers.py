"""Compiled consumers of include/gr.h, not ctypes: the header compiles as C and
as C++, the records it declares have the layout the Python binding mirrors,
and (on the GPU) a PathTracer-shaped C++ program linked against libgr.so
renders an XML scene to the same image, bit for bit, as the library's Python
mirror does."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

import gr

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
INC = os.path.join(ROOT, "include")
LIBDIR = os.path.dirname(gr.LIB_PATH)

pytestmark = pytest.mark.skipif(shutil.which("gcc") is None or shutil.which("g++") is None,
                                reason="no host C / C++ compiler")


def _build(tmp_path, src, out, cxx):
    exe = str(tmp_path / out)
    cmd = [("g++" if cxx else "gcc"), ("-std=c++17" if cxx else "-std=c99"), "-Wall", "-Wextra", "-Werror",
           "-I", INC, os.path.join(HERE, "cpp", src), "-o", exe, "-L", LIBDIR, "-lgr", "-Wl,-rpath," + LIBDIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_header_layout_matches_the_python_binding(tmp_path):
    gr.load()
    exe = _build(tmp_path, "abi_layout.c", "abi_layout", cxx=False)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = dict(line.rsplit(" ", 1) for line in r.stdout.splitlines() if not line.startswith(("version", "status")))
    mirror = {"gr_trace_tuning": gr.Tuning, "gr_tuning_result": gr.TuningResult, "gr_opts": gr.Opts,
              "gr_material": gr.Material, "gr_mesh": gr.Mesh, "gr_camera": gr.Camera,
              "gr_environment": gr.Environment, "gr_render_opts": gr.RenderOpts, "gr_render_stats": gr.RenderStats,
              "gr_server_opts": gr.ServerOpts, "gr_job_stats": gr.JobStats, "gr_server_stats": gr.ServerStats}
    assert int(got["gr_ray size"]) == gr.RAY_DTYPE.itemsize == 32
    assert int(got["gr_hit size"]) == gr.HIT_DTYPE.itemsize == 16
    for key, value in got.items():
        name, what = key.split(" ")[0], key.split(" ")[-1]
        if name in ("gr_ray", "gr_hit"):
            continue
        rec, _, field = name.partition(".")
        cls = mirror[rec]
        if what == "size" and not field:
            assert ctypes.sizeof(cls) == int(value), (rec, ctypes.sizeof(cls), value)
        else:
            assert getattr(cls, field).offset == int(value), (rec, field)
    assert "status8 server busy" in r.stdout


def test_pathtracer_shim_compiles_as_cpp(tmp_path):
    gr.load()
    _build(tmp_path, "pathtracer_shim.cpp", "pathtracer_shim", cxx=True)


@pytest.mark.gpu
def test_pathtracer_shim_renders_like_the_python_mirror(ctx, tmp_path):
    from gr import imageio, mitsuba
    from gr import scenes as sc
    exe = _build(tmp_path, "pathtracer_shim.cpp", "pathtracer_shim", cxx=True)
    d = sc.cornell_box(64, 48)
    xml = mitsuba.write_scene(d, str(tmp_path))
    pfm = str(tmp_path / "shim.pfm")
    r = subprocess.run([exe, xml, "16", "8", "5", pfm], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    w, h, samples, rays = (int(x) for x in r.stdout.split())
    assert (w, h, samples) == (64, 48, 64 * 48 * 16) and rays >= samples
    got = imageio.read_pfm(pfm)
    s = gr.load_xml(ctx, xml)
    img, _ = s.render(16, max_depth=8, seed=5)  # one call of 16 samples = 16 one-sample frames
    ref_pfm = str(tmp_path / "mirror.pfm")
    s.write_image(ref_pfm)
    s.close()
    want = imageio.read_pfm(ref_pfm)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    # PFM rows run bottom to top; the image itself is the mean radiance gr_render returns
    np.testing.assert_allclose(got[::-1], img, rtol=1e-6, atol=0)


@pytest.mark.gpu
def test_render_writes_device_memory_like_host_memory(ctx):
    import torch
    from gr import scenes as sc
    d = sc.glossy_scene(40, 30, level=2, glass_level=1)
    a, b = gr.Scene(ctx, d), gr.Scene(ctx, d)
    host, _ = a.render(4, max_depth=8, seed=9)
    dev = torch.full((30, 40, 3), -1.0, dtype=torch.float32, device="cuda")
    out, st = b.render(4, max_depth=8, seed=9, out=dev)
    assert out is dev and st.device_errors == 0
    np.testing.assert_array_equal(dev.cpu().numpy().view(np.uint32), host.view(np.uint32))
    a.close()
    b.close()
