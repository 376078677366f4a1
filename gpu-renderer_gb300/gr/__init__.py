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
LAYOUT_BVH2, LAYOUT_BVH4, LAYOUT_BVH4_Q8, LAYOUT_BVH8_Q8 = 0, 1, 2, 3
LAYOUT_NAMES = {0: "bvh2", 1: "bvh4", 2: "bvh4_q8", 3: "bvh8_q8"}
STATUS = {
    0: "GR_OK", 1: "GR_ERR_INVALID", 2: "GR_ERR_CUDA", 3: "GR_ERR_OOM_BUDGET",
    4: "GR_ERR_PARSE", 5: "GR_ERR_TIMEOUT", 6: "GR_ERR_OVERFLOW", 7: "GR_ERR_IO", 8: "GR_ERR_BUSY",
}
GR_ERR_CUDA, GR_ERR_BUSY = 2, 8
SERVER_FIFO, SERVER_SHORTEST_FIRST = 0, 1

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
        "gr_context_create": ([ctypes.c_int, _P, ctypes.POINTER(_P)], ctypes.c_int),
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
        "gr_bvh_set_layout": ([_P, ctypes.c_int, _P], ctypes.c_int),
        "gr_bvh_export_layout": ([_P, ctypes.c_int, _P], ctypes.c_int),
        "gr_bvh_layout_size": ([_P, ctypes.c_int, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)],
                               ctypes.c_int),
        "gr_bvh_export_layout_tris": ([_P, ctypes.c_int, _P], ctypes.c_int),
        "gr_scene_set_layout": ([_P, ctypes.c_int], ctypes.c_int),
        "gr_bvh_set_tuning": ([_P, _P], ctypes.c_int),
        "gr_bvh_get_tuning": ([_P, _P], ctypes.c_int),
        "gr_bvh_autotune": ([_P, _P, ctypes.c_uint64, ctypes.c_int, _P, _P, ctypes.c_uint32,
                             ctypes.POINTER(ctypes.c_uint32)], ctypes.c_int),
        "gr_scene_autotune": ([_P, _P, _P, ctypes.POINTER(ctypes.c_uint32)], ctypes.c_int),
        "gr_scene_set_tuning": ([_P, _P, ctypes.c_uint32], ctypes.c_int),
        "gr_scene_get_tuning": ([_P, _P, ctypes.POINTER(ctypes.c_uint32)], ctypes.c_int),
        "gr_scene_layout": ([_P], ctypes.c_int),
        "gr_diag_bounded_wait": ([_P, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32)], ctypes.c_int),
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


class Tuning(ctypes.Structure):
    """Traversal launch configuration (gr_trace_tuning)."""
    _fields_ = [("layout", ctypes.c_int32), ("block", ctypes.c_int32), ("short_stack", ctypes.c_int32)]

    def as_dict(self):
        return {"layout": LAYOUT_NAMES[self.layout], "block": self.block, "short_stack": self.short_stack}


class TuningResult(ctypes.Structure):
    _fields_ = [("tuning", Tuning), ("ms", ctypes.c_float)]


class Opts(ctypes.Structure):
    """Context options (gr_opts)."""
    _fields_ = [("default_wave_paths", ctypes.c_uint32), ("flags", ctypes.c_uint32)]


class Context:
    """A gr context bound to one CUDA device. default_wave_paths: the wave
    size of renders that set none (0 = the library's)."""

    def __init__(self, device=0, default_wave_paths=0):
        L = load()
        h = _P()
        opts = Opts(default_wave_paths, 0)
        st = L.gr_context_create(device, ctypes.byref(opts), ctypes.byref(h))
        if st != GR_OK:
            raise GrError(st, "gr_context_create(%d)" % device)
        self.h = h
        self.device = device

    def check(self, st, what=""):
        if st != GR_OK:
            raise GrError(st, "%s: %s" % (what, load().gr_last_error(self.h).decode()))

    def bounded_wait(self, polls):
        """gr_diag_bounded_wait: runs the library's bounded device wait on a flag
        nothing sets, for `polls` polls. Returns (status, device error bits);
        the status is GR_ERR_TIMEOUT (5) with bit 1 set, and the context stays
        usable."""
        bits = ctypes.c_uint32(0)
        st = load().gr_diag_bounded_wait(self.h, polls, ctypes.byref(bits))
        return st, bits.value

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

    def set_layout(self, layout, stream=None):
        self.ctx.check(load().gr_bvh_set_layout(self.h, layout, _P(stream) if stream else None), "gr_bvh_set_layout")

    def set_tuning(self, layout, block=128, short_stack=12):
        t = Tuning(layout, block, short_stack)
        self.ctx.check(load().gr_bvh_set_tuning(self.h, ctypes.byref(t)), "gr_bvh_set_tuning")

    def tuning(self):
        t = Tuning()
        self.ctx.check(load().gr_bvh_get_tuning(self.h, ctypes.byref(t)), "gr_bvh_get_tuning")
        return t.as_dict()

    def autotune(self, d_rays, n, d_hits, any_hit=False):
        """Times every layout x block x short-stack configuration on the rays
        and keeps the fastest; returns [(tuning dict, ms)]."""
        table = (TuningResult * 64)()
        rows = ctypes.c_uint32()
        self.ctx.check(load().gr_bvh_autotune(self.h, _ptr(d_rays), n, int(bool(any_hit)), _ptr(d_hits), table, 64,
                                              ctypes.byref(rows)), "gr_bvh_autotune")
        return [(table[i].tuning.as_dict(), float(table[i].ms)) for i in range(min(rows.value, 64))]

    def export_layout(self, layout):
        n = self.size
        nb, _ = self.layout_size(layout)
        out = np.zeros(nb // 4, np.uint32)
        if n:
            self.ctx.check(load().gr_bvh_export_layout(self.h, layout, _ptr(out)), "gr_bvh_export_layout")
        return out

    def layout_size(self, layout):
        """(node bytes, triangle bytes) of a layout (built if needed)."""
        nb, tb = ctypes.c_uint64(), ctypes.c_uint64()
        self.ctx.check(load().gr_bvh_layout_size(self.h, layout, ctypes.byref(nb), ctypes.byref(tb)),
                       "gr_bvh_layout_size")
        return nb.value, tb.value

    def export_layout_tris(self, layout):
        """The triangles a layout traverses, (m, 12) float32."""
        _, tb = self.layout_size(layout)
        out = np.zeros(tb // 4, np.float32)
        if tb:
            self.ctx.check(load().gr_bvh_export_layout_tris(self.h, layout, _ptr(out)), "gr_bvh_export_layout_tris")
        return out

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


# ---- scene records (include/gr.h) --------------------------------------------------

class Material(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("color", ctypes.c_float * 3), ("emission", ctypes.c_float * 3),
                ("alpha_u", ctypes.c_float), ("alpha_v", ctypes.c_float), ("eta_i", ctypes.c_float * 3),
                ("eta_t", ctypes.c_float * 3), ("k", ctypes.c_float * 3), ("ior", ctypes.c_float),
                ("color_map", _P), ("color_map_width", ctypes.c_uint32), ("color_map_height", ctypes.c_uint32),
                ("uv_offset", ctypes.c_float * 2), ("uv_scale", ctypes.c_float * 2), ("specular", ctypes.c_float * 3)]


class Mesh(ctypes.Structure):
    _fields_ = [("positions", _P), ("num_vertices", ctypes.c_uint32), ("normals", _P), ("indices", _P),
                ("num_triangles", ctypes.c_uint32), ("material", ctypes.c_uint32), ("texcoords", _P)]


class Camera(ctypes.Structure):
    _fields_ = [("to_world", ctypes.c_float * 16), ("fov_deg", ctypes.c_float), ("width", ctypes.c_uint32),
                ("height", ctypes.c_uint32)]


class Environment(ctypes.Structure):
    _fields_ = [("radiance", ctypes.c_float * 3), ("enabled", ctypes.c_int32), ("map", _P),
                ("map_width", ctypes.c_uint32), ("map_height", ctypes.c_uint32), ("to_world", ctypes.c_float * 16)]


class RenderOpts(ctypes.Structure):
    _fields_ = [("spp", ctypes.c_uint32), ("max_depth", ctypes.c_uint32), ("seed", ctypes.c_uint64),
                ("rr_depth", ctypes.c_int32), ("flags", ctypes.c_uint32), ("wave_paths", ctypes.c_uint32)]


class RenderStats(ctypes.Structure):
    _fields_ = [("ms", ctypes.c_double), ("closest_rays", ctypes.c_uint64), ("shadow_rays", ctypes.c_uint64),
                ("samples", ctypes.c_uint64), ("waves", ctypes.c_uint32), ("device_errors", ctypes.c_uint32)]


MAT_DIFFUSE, MAT_DIELECTRIC, MAT_CONDUCTOR, MAT_PLASTIC = 0, 1, 2, 3
RENDER_REFERENCE_COMPAT = 1
RENDER_NO_GRAPH = 2

_SCENE_SIGS = {
    "gr_scene_create": ([_P, _P, ctypes.c_uint32, _P, ctypes.c_uint32, _P, _P, ctypes.POINTER(_P)], ctypes.c_int),
    "gr_scene_destroy": ([_P], ctypes.c_int),
    "gr_scene_info": ([_P, _P, _P, _P, _P], ctypes.c_int),
    "gr_render": ([_P, ctypes.POINTER(RenderOpts), _P, ctypes.POINTER(RenderStats)], ctypes.c_int),
    "gr_scene_accumulation": ([_P, _P, _P], ctypes.c_int),
    "gr_scene_reset": ([_P], ctypes.c_int),
    "gr_scene_get_camera": ([_P, ctypes.POINTER(Camera)], ctypes.c_int),
    "gr_scene_set_camera": ([_P, ctypes.POINTER(Camera)], ctypes.c_int),
    "gr_scene_zoom": ([_P, ctypes.c_float], ctypes.c_int),
    "gr_scene_translate": ([_P, ctypes.c_float, ctypes.c_float], ctypes.c_int),
    "gr_scene_rotate": ([_P, ctypes.c_float, ctypes.c_float], ctypes.c_int),
    "gr_scene_resize": ([_P, ctypes.c_uint32, ctypes.c_uint32], ctypes.c_int),
    "gr_scene_rgba8": ([_P, _P, _P], ctypes.c_int),
    "gr_scene_rgba8_host": ([_P, _P], ctypes.c_int),
    "gr_scene_write_image": ([_P, ctypes.c_char_p], ctypes.c_int),
}

_IMAGE_SIGS = {
    "gr_image_write": ([ctypes.c_char_p, _P, ctypes.c_uint32, ctypes.c_uint32], ctypes.c_int),
}


def image_write(path, img):
    """gr_image_write: a linear RGB image (height, width, 3) to a .png (8-bit
    sRGB, rows flipped as the reference writes them) or .pfm file."""
    a = np.ascontiguousarray(img, np.float32)
    if a.ndim != 3 or a.shape[2] != 3:
        raise ValueError("expected an (height, width, 3) image")
    st = _declare(_IMAGE_SIGS).gr_image_write(os.fsencode(path), _ptr(a), a.shape[1], a.shape[0])
    if st != 0:
        raise GrError(st, "gr_image_write(%s)" % path)


def _declare(sigs):
    L = load()
    for name, (args, res) in sigs.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    return L


def material_record(m):
    """dict -> Material. Keys: type, color, emission, alpha (or alpha_u/alpha_v),
    eta_i, eta_t, k, ior."""
    r = Material()
    r.type = int(m.get("type", MAT_DIFFUSE))
    r.color[:] = [float(x) for x in m.get("color", (0.5, 0.5, 0.5))]
    r.emission[:] = [float(x) for x in m.get("emission", (0.0, 0.0, 0.0))]
    a = m.get("alpha", 0.1)
    r.alpha_u = float(m.get("alpha_u", a))
    r.alpha_v = float(m.get("alpha_v", a))
    r.eta_i[:] = [float(x) for x in m.get("eta_i", (1.0, 1.0, 1.0))]
    r.eta_t[:] = [float(x) for x in m.get("eta_t", (0.200438, 0.924033, 1.10221))]
    r.k[:] = [float(x) for x in m.get("k", (3.91295, 2.45285, 2.14219))]
    r.ior = float(m.get("ior", 1.5))
    cm = m.get("color_map")
    if cm is not None:  # (H, W, 3) float32, kept alive by the caller's dict
        cm = np.ascontiguousarray(cm, np.float32)
        m["color_map"] = cm
        r.color_map = cm.ctypes.data
        r.color_map_height, r.color_map_width = cm.shape[0], cm.shape[1]
    r.uv_offset[:] = [float(x) for x in m.get("uv_offset", (0.0, 0.0))]
    r.uv_scale[:] = [float(x) for x in m.get("uv_scale", (1.0, 1.0))]
    r.specular[:] = [float(x) for x in m.get("specular", (1.0, 1.0, 1.0))]
    return r


def environment_record(env):
    """None / constant radiance / {"map", "to_world"} -> Environment (maps kept alive by the dict)."""
    e = Environment()
    if env is None:
        return e
    e.enabled = 1
    if isinstance(env, dict):
        mp = np.ascontiguousarray(env["map"], np.float32)
        env["map"] = mp
        e.map = mp.ctypes.data
        e.map_height, e.map_width = mp.shape[0], mp.shape[1]
        e.to_world[:] = [float(x) for x in np.asarray(env.get("to_world", np.eye(4)), np.float32).reshape(16)]
    else:
        e.radiance[:] = [float(x) for x in env]
    return e


class Scene:
    """A scene on the GPU (gr_scene): meshes, materials, camera, environment.

    `desc` is a gr.scenes.SceneDesc (meshes as numpy arrays)."""

    def __init__(self, ctx, desc):
        L = _declare(_SCENE_SIGS)
        self.ctx = ctx
        self.desc = desc
        self._keep = []
        meshes = (Mesh * max(len(desc.meshes), 1))()
        for i, m in enumerate(desc.meshes):
            pos = np.ascontiguousarray(m.positions, np.float32)
            idx = np.ascontiguousarray(m.indices, np.uint32)
            nrm = None if m.normals is None else np.ascontiguousarray(m.normals, np.float32)
            self._keep += [pos, idx, nrm]
            meshes[i].positions = pos.ctypes.data
            meshes[i].num_vertices = pos.shape[0]
            meshes[i].normals = None if nrm is None else nrm.ctypes.data
            meshes[i].indices = idx.ctypes.data
            meshes[i].num_triangles = idx.shape[0]
            meshes[i].material = m.material
            if getattr(m, "texcoords", None) is not None:
                tc = np.ascontiguousarray(m.texcoords, np.float32)
                self._keep.append(tc)
                meshes[i].texcoords = tc.ctypes.data
        mats = (Material * max(len(desc.materials), 1))(*[material_record(m) for m in desc.materials])
        cam = Camera()
        cam.to_world[:] = [float(x) for x in np.asarray(desc.camera["to_world"], np.float32).reshape(16)]
        cam.fov_deg = float(desc.camera["fov"])
        cam.width = int(desc.camera["width"])
        cam.height = int(desc.camera["height"])
        env = environment_record(desc.env)
        h = _P()
        ctx.check(L.gr_scene_create(ctx.h, meshes, len(desc.meshes), mats, len(desc.materials), ctypes.byref(cam),
                                    ctypes.byref(env), ctypes.byref(h)), "gr_scene_create")
        self.h = h
        self._keep = []
        self.width, self.height = cam.width, cam.height

    # ---- view operations (PathTracer::zoom / translate / rotate / resize) ----

    def camera(self):
        """The scene's camera as a dict (to_world 4x4, fov, width, height)."""
        c = Camera()
        self.ctx.check(_declare(_SCENE_SIGS).gr_scene_get_camera(self.h, ctypes.byref(c)), "gr_scene_get_camera")
        return {"to_world": np.array(c.to_world[:], np.float32).reshape(4, 4), "fov": float(c.fov_deg),
                "width": int(c.width), "height": int(c.height)}

    def _after_view_change(self, st, what):
        self.ctx.check(st, what)
        cam = self.camera()
        self.width, self.height = cam["width"], cam["height"]

    def set_camera(self, cam):
        c = camera_record(cam)
        self._after_view_change(_declare(_SCENE_SIGS).gr_scene_set_camera(self.h, ctypes.byref(c)),
                                "gr_scene_set_camera")

    def zoom(self, d):
        self._after_view_change(_declare(_SCENE_SIGS).gr_scene_zoom(self.h, d), "gr_scene_zoom")

    def translate(self, x, y):
        self._after_view_change(_declare(_SCENE_SIGS).gr_scene_translate(self.h, x, y), "gr_scene_translate")

    def rotate(self, yaw, pitch):
        self._after_view_change(_declare(_SCENE_SIGS).gr_scene_rotate(self.h, yaw, pitch), "gr_scene_rotate")

    def resize(self, width, height):
        self._after_view_change(_declare(_SCENE_SIGS).gr_scene_resize(self.h, width, height), "gr_scene_resize")

    def rgba8(self):
        """The sRGB 8-bit RGBA image (height, width, 4) uint8 of the mean radiance."""
        out = np.zeros(self.width * self.height, np.uint32)
        self.ctx.check(_declare(_SCENE_SIGS).gr_scene_rgba8_host(self.h, _ptr(out)), "gr_scene_rgba8_host")
        return out.view(np.uint8).reshape(self.height, self.width, 4)

    def write_image(self, path):
        """The accumulated mean radiance to a .png or .pfm file (PathTracer::output)."""
        self.ctx.check(_declare(_SCENE_SIGS).gr_scene_write_image(self.h, os.fsencode(path)), "gr_scene_write_image")

    def rgba8_device(self, d_out, stream=None):
        self.ctx.check(_declare(_SCENE_SIGS).gr_scene_rgba8(self.h, _ptr(d_out), _P(stream) if stream else None),
                       "gr_scene_rgba8")

    def render(self, spp, max_depth=8, seed=0, rr_depth=3, flags=0, wave_paths=0, want_image=True, out=None):
        """Adds spp samples per pixel; returns (mean image, RenderStats). `out`
        may be a device tensor of height x width x 3 floats that gr_render
        fills on the GPU (then it is returned in place of a host image)."""
        L = _declare(_SCENE_SIGS)
        o = RenderOpts(spp, max_depth, seed, rr_depth, flags, wave_paths)
        st = RenderStats()
        img = out if out is not None else (np.zeros((self.height, self.width, 3), np.float32) if want_image else None)
        self.ctx.check(L.gr_render(self.h, ctypes.byref(o), _ptr(img), ctypes.byref(st)), "gr_render")
        return img, st

    def accumulation(self):
        L = _declare(_SCENE_SIGS)
        s = np.zeros((self.height, self.width, 3), np.float64)
        c = np.zeros((self.height, self.width), np.uint32)
        self.ctx.check(L.gr_scene_accumulation(self.h, _ptr(s), _ptr(c)), "gr_scene_accumulation")
        return s, c

    def reset(self):
        self.ctx.check(_declare(_SCENE_SIGS).gr_scene_reset(self.h), "gr_scene_reset")

    def set_layout(self, layout):
        self.ctx.check(load().gr_scene_set_layout(self.h, layout), "gr_scene_set_layout")

    def autotune(self, spp=1, max_depth=8, seed=0, rr_depth=3, flags=0):
        """Render autotuner: traversal configuration and wave size (queue
        capacity) from timed probe renders. Clears the accumulation."""
        o = RenderOpts(spp, max_depth, seed, rr_depth, flags, 0)
        t = Tuning()
        w = ctypes.c_uint32()
        self.ctx.check(load().gr_scene_autotune(self.h, ctypes.byref(o), ctypes.byref(t), ctypes.byref(w)),
                       "gr_scene_autotune")
        return t.as_dict(), w.value

    def set_tuning(self, layout, block=128, short_stack=12, wave_paths=0):
        t = Tuning(layout, block, short_stack)
        self.ctx.check(load().gr_scene_set_tuning(self.h, ctypes.byref(t), wave_paths), "gr_scene_set_tuning")

    def tuning(self):
        t = Tuning()
        w = ctypes.c_uint32()
        self.ctx.check(load().gr_scene_get_tuning(self.h, ctypes.byref(t), ctypes.byref(w)), "gr_scene_get_tuning")
        return t.as_dict(), w.value

    def info(self):
        v = [ctypes.c_uint32() for _ in range(4)]
        self.ctx.check(_declare(_SCENE_SIGS).gr_scene_info(self.h, *[ctypes.byref(x) for x in v]), "gr_scene_info")
        return {"width": v[0].value, "height": v[1].value, "triangles": v[2].value, "lights": v[3].value}

    def close(self):
        if getattr(self, "h", None):
            _declare(_SCENE_SIGS).gr_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PathTracer:
    """The reference's PathTracer interface (src/renderer/pathtracer.h:16-46)
    over a gr scene: render(num) adds `num` samples per pixel, output() writes
    the image, reset() clears the accumulation."""

    def __init__(self, scene, max_path_length=33, seed=0, rr_depth=3, flags=0):
        self.scene = scene
        self.max_path_length = max_path_length
        self.seed = seed
        self.rr_depth = rr_depth
        self.flags = flags
        self.sample_num = 0

    def render(self, num=1):
        img, st = self.scene.render(num, self.max_path_length, self.seed, self.rr_depth, self.flags)
        self.sample_num += num
        self.image = img
        return img, st

    def output(self, filename):
        """PathTracer::output: the accumulated image to a .png (8-bit sRGB,
        flipped as the reference writes it) or .pfm file, by gr_scene_write_image."""
        self.scene.write_image(filename)

    def reset(self):
        self.scene.reset()
        self.sample_num = 0

    # the viewer's camera operations (pathtracer.cu:177-213); each restarts the sample sequence
    def zoom(self, d):
        self.scene.zoom(d)
        self.sample_num = 0

    def translate(self, x, y):
        self.scene.translate(x, y)
        self.sample_num = 0

    def rotate(self, yaw, pitch):
        self.scene.rotate(yaw, pitch)
        self.sample_num = 0

    def resize(self, width, height):
        self.scene.resize(width, height)
        self.sample_num = 0

    def get_resolution(self):
        return self.scene.width, self.scene.height

    def display(self):
        """The 8-bit RGBA display image of render(uint32*) (filter_kernel)."""
        return self.scene.rgba8()


# ---- batched rendering and serving ---------------------------------------------------

class ServerOpts(ctypes.Structure):
    _fields_ = [("budget_bytes", ctypes.c_uint64), ("wave_paths", ctypes.c_uint32), ("max_active", ctypes.c_uint32),
                ("layout", ctypes.c_int32), ("block", ctypes.c_int32), ("short_stack", ctypes.c_int32),
                ("policy", ctypes.c_int32), ("age_cap_s", ctypes.c_double), ("max_wait_s", ctypes.c_double)]


class JobStats(ctypes.Structure):
    _fields_ = [("submit_s", ctypes.c_double), ("admit_s", ctypes.c_double), ("done_s", ctypes.c_double),
                ("samples", ctypes.c_uint64), ("status", ctypes.c_int32), ("waves", ctypes.c_uint32),
                ("first_wave", ctypes.c_uint64), ("last_wave", ctypes.c_uint64)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("admitted", ctypes.c_uint64), ("completed", ctypes.c_uint64),
                ("waves", ctypes.c_uint64), ("closest_rays", ctypes.c_uint64), ("shadow_rays", ctypes.c_uint64),
                ("bytes_in_use", ctypes.c_uint64), ("peak_bytes", ctypes.c_uint64), ("busy_s", ctypes.c_double),
                ("rejected", ctypes.c_uint64)]


_SERVER_SIGS = {
    "gr_render_batch": ([_P, _P, _P, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(RenderStats)], ctypes.c_int),
    "gr_scene_device_bytes": ([_P], ctypes.c_uint64),
    "gr_server_create": ([_P, ctypes.POINTER(ServerOpts), ctypes.POINTER(_P)], ctypes.c_int),
    "gr_server_destroy": ([_P], ctypes.c_int),
    "gr_server_submit": ([_P, _P, _P, ctypes.POINTER(RenderOpts), ctypes.POINTER(ctypes.c_uint64)], ctypes.c_int),
    "gr_server_wait": ([_P, ctypes.c_uint64, ctypes.c_double, ctypes.POINTER(ctypes.c_int), _P,
                        ctypes.POINTER(JobStats)], ctypes.c_int),
    "gr_server_poll": ([_P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_int), _P, ctypes.POINTER(JobStats)],
                       ctypes.c_int),
    "gr_server_now": ([_P], ctypes.c_double),
    "gr_server_stats_get": ([_P, ctypes.POINTER(ServerStats)], ctypes.c_int),
    "gr_diag_server_fail_waves": ([_P, ctypes.c_uint32], ctypes.c_int),
}


def camera_record(cam):
    c = Camera()
    c.to_world[:] = [float(x) for x in np.asarray(cam["to_world"], np.float32).reshape(16)]
    c.fov_deg = float(cam["fov"])
    c.width = int(cam["width"])
    c.height = int(cam["height"])
    return c


def render_batch(ctx, scenes, opts, wave_paths=0):
    """Renders jobs (scene, RenderOpts-like dict) in shared waves; each scene
    accumulates as if rendered alone. Returns RenderStats."""
    L = _declare(_SERVER_SIGS)
    n = len(scenes)
    hs = (_P * max(n, 1))(*[s.h for s in scenes])
    os_ = (RenderOpts * max(n, 1))()
    for i, o in enumerate(opts):
        os_[i] = RenderOpts(o["spp"], o.get("max_depth", 8), o.get("seed", 0), o.get("rr_depth", 3),
                            o.get("flags", 0), 0)
    st = RenderStats()
    ctx.check(L.gr_render_batch(ctx.h, hs, os_, n, wave_paths, ctypes.byref(st)), "gr_render_batch")
    return st


class Server:
    """Continuous-batching render server (gr_server)."""

    def __init__(self, ctx, budget_bytes=0, wave_paths=0, max_active=0, layout=LAYOUT_BVH2, block=0, short_stack=0,
                 policy=SERVER_FIFO, age_cap_s=0.0, max_wait_s=0.0):
        L = _declare(_SERVER_SIGS)
        self.ctx = ctx
        o = ServerOpts(budget_bytes, wave_paths, max_active, layout, block, short_stack, policy, age_cap_s, max_wait_s)
        h = _P()
        ctx.check(L.gr_server_create(ctx.h, ctypes.byref(o), ctypes.byref(h)), "gr_server_create")
        self.h = h

    def submit(self, scene, spp, max_depth=8, seed=0, rr_depth=3, flags=0, camera=None):
        L = _declare(_SERVER_SIGS)
        o = RenderOpts(spp, max_depth, seed, rr_depth, flags, 0)
        t = ctypes.c_uint64()
        cam = None if camera is None else camera_record(camera)
        self.ctx.check(L.gr_server_submit(self.h, scene.h, None if cam is None else ctypes.byref(cam), ctypes.byref(o),
                                          ctypes.byref(t)), "gr_server_submit")
        return t.value

    def wait(self, ticket, timeout=-1.0, image_shape=None):
        L = _declare(_SERVER_SIGS)
        done = ctypes.c_int()
        js = JobStats()
        img = None if image_shape is None else np.zeros(tuple(image_shape) + (3,), np.float32)
        st = L.gr_server_wait(self.h, ticket, timeout, ctypes.byref(done), _ptr(img), ctypes.byref(js))
        self.ctx.check(st, "gr_server_wait")
        return bool(done.value), img, js

    def poll(self, ticket, image_shape=None):
        """wait() without waiting: (done, image or None, JobStats)."""
        L = _declare(_SERVER_SIGS)
        done = ctypes.c_int()
        js = JobStats()
        img = None if image_shape is None else np.zeros(tuple(image_shape) + (3,), np.float32)
        self.ctx.check(L.gr_server_poll(self.h, ticket, ctypes.byref(done), _ptr(img), ctypes.byref(js)),
                       "gr_server_poll")
        return bool(done.value), img, js

    def now(self):
        return _declare(_SERVER_SIGS).gr_server_now(self.h)

    def fail_waves(self, count):
        """Host-side fault injection: the next `count` waves report a failed
        launch without running (gr_diag_server_fail_waves)."""
        self.ctx.check(_declare(_SERVER_SIGS).gr_diag_server_fail_waves(self.h, count), "gr_diag_server_fail_waves")

    def stats(self):
        s = ServerStats()
        self.ctx.check(_declare(_SERVER_SIGS).gr_server_stats_get(self.h, ctypes.byref(s)), "gr_server_stats_get")
        return s

    def close(self):
        if getattr(self, "h", None):
            _declare(_SERVER_SIGS).gr_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- scene files ---------------------------------------------------------------

_DESC_SIGS = {
    "gr_scene_desc_load_xml": ([ctypes.c_char_p, ctypes.POINTER(_P)], ctypes.c_int),
    "gr_scene_desc_destroy": ([_P], ctypes.c_int),
    "gr_scene_desc_error": ([_P], ctypes.c_char_p),
    "gr_scene_desc_warnings": ([_P], ctypes.c_char_p),
    "gr_scene_desc_info": ([_P, _P, _P, _P, ctypes.POINTER(Camera), ctypes.POINTER(Environment)], ctypes.c_int),
    "gr_scene_desc_triangles": ([_P, _P, _P, _P], ctypes.c_int),
    "gr_scene_desc_mesh": ([_P, ctypes.c_uint32, _P, _P, _P, _P, _P, _P], ctypes.c_int),
    "gr_scene_desc_mesh_texcoords": ([_P, ctypes.c_uint32, _P, _P], ctypes.c_int),
    "gr_scene_create_from_desc": ([_P, _P, ctypes.POINTER(_P)], ctypes.c_int),
    "gr_scene_load_xml": ([_P, ctypes.c_char_p, ctypes.POINTER(_P)], ctypes.c_int),
}


class ParsedScene:
    """A Mitsuba-XML scene parsed by the library (no GPU needed)."""

    def __init__(self, path):
        L = _declare(_DESC_SIGS)
        h = _P()
        st = L.gr_scene_desc_load_xml(os.fsencode(path), ctypes.byref(h))
        self.h = h
        if st != GR_OK:
            msg = L.gr_scene_desc_error(h).decode() if h else "out of memory"
            self.close()
            raise GrError(st, msg)
        self.warnings = [w for w in L.gr_scene_desc_warnings(h).decode().splitlines() if w]
        m, t, li = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        cam, env = Camera(), Environment()
        L.gr_scene_desc_info(h, ctypes.byref(m), ctypes.byref(t), ctypes.byref(li), ctypes.byref(cam),
                             ctypes.byref(env))
        self.num_meshes, self.num_triangles, self.num_light_triangles = m.value, t.value, li.value
        self.camera = {"to_world": np.array(cam.to_world[:], np.float32).reshape(4, 4), "fov": cam.fov_deg,
                       "width": cam.width, "height": cam.height}
        self.env = tuple(env.radiance[:]) if env.enabled else None
        self.env_map_size = (int(env.map_width), int(env.map_height)) if env.enabled and env.map else None

    def triangles(self):
        L = _declare(_DESC_SIGS)
        v = np.zeros((self.num_triangles, 9), np.float32)
        mesh = np.zeros(self.num_triangles, np.uint32)
        mats = (Material * max(self.num_meshes, 1))()
        L.gr_scene_desc_triangles(self.h, _ptr(v), _ptr(mesh), mats)
        return v, mesh, [mats[i] for i in range(self.num_meshes)]

    def triangle_attributes(self):
        """Per triangle, in the flattened order of triangles(): shading
        normals (n x 9 floats) and texture coordinates (n x 6 floats), NaN
        where the triangle's mesh has none."""
        L = _declare(_DESC_SIGS)
        nrm = np.full((self.num_triangles, 9), np.nan, np.float32)
        uvs = np.full((self.num_triangles, 6), np.nan, np.float32)
        off = 0
        for i in range(self.num_meshes):
            nv, nt, hn, ht = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_int(), ctypes.c_int()
            L.gr_scene_desc_mesh(self.h, i, ctypes.byref(nv), ctypes.byref(nt), ctypes.byref(hn), None, None, None)
            L.gr_scene_desc_mesh_texcoords(self.h, i, ctypes.byref(ht), None)
            idx = np.zeros((nt.value, 3), np.uint32)
            n = np.zeros((nv.value, 3), np.float32) if hn.value else None
            t = np.zeros((nv.value, 2), np.float32) if ht.value else None
            L.gr_scene_desc_mesh(self.h, i, None, None, None, None, _ptr(n), _ptr(idx))
            if t is not None:
                L.gr_scene_desc_mesh_texcoords(self.h, i, None, _ptr(t))
                uvs[off:off + nt.value] = t[idx].reshape(-1, 6)
            if n is not None:
                nrm[off:off + nt.value] = n[idx].reshape(-1, 9)
            off += nt.value
        return nrm, uvs

    def scene_desc(self):
        """The parsed scene as a gr.scenes.SceneDesc (one mesh per shape, each
        with its own material), e.g. to build the same scene from records."""
        from .scenes import MeshDesc, SceneDesc
        L = _declare(_DESC_SIGS)
        _, _, mats = self.triangles()
        meshes, materials = [], []
        for i in range(self.num_meshes):
            nv, nt, hn = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_int()
            L.gr_scene_desc_mesh(self.h, i, ctypes.byref(nv), ctypes.byref(nt), ctypes.byref(hn), None, None, None)
            pos = np.zeros((nv.value, 3), np.float32)
            nrm = np.zeros((nv.value, 3), np.float32) if hn.value else None
            idx = np.zeros((nt.value, 3), np.uint32)
            L.gr_scene_desc_mesh(self.h, i, None, None, None, _ptr(pos), _ptr(nrm), _ptr(idx))
            meshes.append(MeshDesc(pos, idx, i, normals=nrm))
            r = mats[i]
            if r.color_map:
                raise ValueError("textured materials have no record form here")
            materials.append({"type": r.type, "color": tuple(r.color), "emission": tuple(r.emission),
                              "alpha_u": r.alpha_u, "alpha_v": r.alpha_v, "eta_i": tuple(r.eta_i),
                              "eta_t": tuple(r.eta_t), "k": tuple(r.k), "ior": r.ior, "specular": tuple(r.specular)})
        return SceneDesc(meshes, materials, dict(self.camera), self.env)

    def create(self, ctx):
        h = _P()
        ctx.check(_declare(_DESC_SIGS).gr_scene_create_from_desc(ctx.h, self.h, ctypes.byref(h)),
                  "gr_scene_create_from_desc")
        return _wrap_scene(ctx, h, self.camera["width"], self.camera["height"])

    def close(self):
        if getattr(self, "h", None):
            _declare(_DESC_SIGS).gr_scene_desc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _wrap_scene(ctx, h, width, height):
    s = Scene.__new__(Scene)
    s.ctx, s.desc, s._keep, s.h, s.width, s.height = ctx, None, [], h, width, height
    return s


def load_xml(ctx, path):
    """gr_scene_load_xml: the drop-in for the reference's PathTracer(filename)."""
    h = _P()
    ctx.check(_declare(_DESC_SIGS).gr_scene_load_xml(ctx.h, os.fsencode(path), ctypes.byref(h)), "gr_scene_load_xml")
    info = [ctypes.c_uint32() for _ in range(4)]
    _declare(_SCENE_SIGS).gr_scene_info(h, *[ctypes.byref(x) for x in info])
    return _wrap_scene(ctx, h, info[0].value, info[1].value)
