"""The C-ABI library loads and exports every entry point include/*.h declares."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(gr_\w+)\s*\(", text, flags=re.M):
            syms.add(m.group(1))
    return sorted(syms)


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "gr_trace" in syms and "gr_bvh_build" in syms
    assert len(syms) >= 10


@pytest.mark.parametrize("sym", declared_symbols())
def test_library_exports_symbol(grlib, sym):
    assert hasattr(grlib, sym), "libgr.so does not export %s" % sym


def test_status_strings(grlib):
    for st in range(7):
        assert grlib.gr_status_string(st)
    assert grlib.gr_version() >= 100


def test_context_without_gpu_fails_cleanly(grlib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    st = grlib.gr_context_create(0, None, ctypes.byref(h))
    assert st != 0 and not h.value


def test_bounded_wait_diagnostic_checks_its_context(grlib):
    # host-side argument check only: no context, no device work
    bits = ctypes.c_uint32(7)
    fn = grlib.gr_diag_bounded_wait
    fn.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32)]
    fn.restype = ctypes.c_int
    assert fn(None, 1000, ctypes.byref(bits)) == 1  # GR_ERR_INVALID
    assert bits.value == 7
