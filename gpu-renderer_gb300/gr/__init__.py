"""Python binding of the gr C ABI (include/gr.h) through ctypes.

The library is built in-tree by ``gpu-renderer_gb300/gr_build.py`` into
``gpu-renderer_gb300/lib/libgr.so``. Loading fails loudly when it is missing:
there is no CPU fallback behind these calls.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(_HERE)
LIB_PATH = os.path.join(PKG_ROOT, "lib", "libgr.so")

GR_OK = 0
STATUS = {
    0: "GR_OK", 1: "GR_ERR_INVALID", 2: "GR_ERR_CUDA", 3: "GR_ERR_OOM_BUDGET",
    4: "GR_ERR_PARSE", 5: "GR_ERR_TIMEOUT", 6: "GR_ERR_OVERFLOW",
}

RAY_DTYPE = np.dtype([("o", "<f4", 3), ("d", "<f4", 3), ("tmin", "<f4"), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("t", "<f4"), ("prim", "<i4"), ("u", "<f4"), ("v", "<f4")])

_lib = None
_P = ctypes.c_void_p


class GrError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        super().__init__("%s (%d): %s" % (STATUS.get(status, "?"), status, what))


def load():
    """Loads libgr.so once and declares the C signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libgr.so is not built (%s); run gpu-renderer_gb300/gr_build.py" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    sig = {
        "gr_version": ([], ctypes.c_int),
        "gr_status_string": ([ctypes.c_int], ctypes.c_char_p),
        "gr_context_create": ([ctypes.c_int, ctypes.POINTER(_P)], ctypes.c_int),
        "gr_context_destroy": ([_P], ctypes.c_int),
        "gr_last_error": ([_P], ctypes.c_char_p),
        "gr_bvh_create": ([_P, ctypes.POINTER(_P)], ctypes.c_int),
        "gr_bvh_destroy": ([_P], ctypes.c_int),
        "gr_bvh_build": ([_P, _P, ctypes.c_uint32, _P], ctypes.c_int),
        "gr_bvh_build_host": ([_P, _P, ctypes.c_uint32], ctypes.c_int),
        "gr_bvh_size": ([_P], ctypes.c_uint32),
        "gr_bvh_export": ([_P, _P, _P, _P, _P, _P, _P], ctypes.c_int),
        "gr_trace": ([_P, _P, ctypes.c_uint64, _P, ctypes.c_int, _P], ctypes.c_int),
        "gr_trace_host": ([_P, _P, ctypes.c_uint64, _P, ctypes.c_int], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"]
        return a.ctypes.data_as(_P)
    if isinstance(a, int):
        return _P(a)
    return _P(a.data_ptr())  # torch tensor


class Context:
    """A gr context bound to one CUDA device."""

    def __init__(self, device=0):
        L = load()
        h = _P()
        st = L.gr_context_create(device, ctypes.byref(h))
        if st != GR_OK:
            raise GrError(st, "gr_context_create(%d)" % device)
        self.h = h
        self.device = device

    def check(self, st, what=""):
        if st != GR_OK:
            raise GrError(st, "%s: %s" % (what, load().gr_last_error(self.h).decode()))

    def close(self):
        if self.h:
            load().gr_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BVH:
    """GPU LBVH over a triangle soup (9 floats per triangle)."""

    def __init__(self, ctx):
        self.ctx = ctx
        h = _P()
        ctx.check(load().gr_bvh_create(ctx.h, ctypes.byref(h)), "gr_bvh_create")
        self.h = h

    @property
    def size(self):
        return load().gr_bvh_size(self.h)

    def build_host(self, verts):
        v = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 9)
        self.ctx.check(load().gr_bvh_build_host(self.h, _ptr(v), v.shape[0]), "gr_bvh_build_host")

    def build_device(self, d_verts, n, stream=None):
        self.ctx.check(load().gr_bvh_build(self.h, _ptr(d_verts), n, _P(stream) if stream else None), "gr_bvh_build")

    def export(self):
        n = self.size
        sp = np.zeros(n, np.uint32)
        sc = np.zeros(n, np.uint32)
        rn = np.zeros(max(2 * n - 1, 0) * 8, np.uint32)
        nodes = np.zeros(max(n - 1, 1) * 16, np.uint32)
        tris = np.zeros(12 * n, np.float32)
        root = ctypes.c_uint32()
        self.ctx.check(load().gr_bvh_export(self.h, _ptr(sp), _ptr(sc), _ptr(rn), _ptr(nodes), _ptr(tris),
                                            ctypes.byref(root)), "gr_bvh_export")
        return {"sorted_prim": sp, "sorted_code": sc, "ref_nodes": rn, "nodes": nodes, "tris": tris,
                "root": root.value}

    def trace_host(self, rays, any_hit=False):
        r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        hits = np.zeros((r.shape[0], 4), np.float32)
        self.ctx.check(load().gr_trace_host(self.h, _ptr(r), r.shape[0], _ptr(hits), int(bool(any_hit))),
                       "gr_trace_host")
        return hits

    def trace_device(self, d_rays, n, d_hits, any_hit=False, stream=None):
        self.ctx.check(load().gr_trace(self.h, _ptr(d_rays), n, _ptr(d_hits), int(bool(any_hit)),
                                       _P(stream) if stream else None), "gr_trace")

    def close(self):
        if self.h:
            load().gr_bvh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
