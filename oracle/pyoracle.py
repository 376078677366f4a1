"""ctypes wrapper of the CPU oracle (oracle/build/liboracle.so).

Test infrastructure: imported only by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py. The product (libgr.so) never uses it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_lbvh.so")
_P = ctypes.c_void_p
_lib = None
_ref = None


def build():
    r = subprocess.run(["make", "-s", "-C", HERE, "-j4"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        _lib = ctypes.CDLL(LIB)
    return _lib


def ref_available():
    return os.path.exists(REF_LIB)


def load_ref():
    global _ref
    if _ref is None:
        _ref = ctypes.CDLL(REF_LIB)
    return _ref


def _p(a):
    return None if a is None else a.ctypes.data_as(_P)


def threads():
    return os.cpu_count() or 1


def morton(verts):
    v = np.ascontiguousarray(verts, np.float32).reshape(-1, 9)
    codes = np.zeros(v.shape[0], np.uint32)
    cbox = np.zeros(6, np.float32)
    load().or_morton(_p(v), v.shape[0], _p(codes), _p(cbox))
    return codes, cbox


def lbvh(verts):
    v = np.ascontiguousarray(verts, np.float32).reshape(-1, 9)
    n = v.shape[0]
    out = {
        "sorted_prim": np.zeros(n, np.uint32), "sorted_code": np.zeros(n, np.uint32),
        "ref_nodes": np.zeros(max(2 * n - 1, 0) * 8, np.uint32),
        "nodes": np.zeros(max(n - 1, 1) * 16, np.uint32), "tris": np.zeros(12 * n, np.float32),
    }
    root = ctypes.c_uint32()
    load().or_lbvh_build(_p(v), n, _p(out["sorted_prim"]), _p(out["sorted_code"]), _p(out["ref_nodes"]),
                         _p(out["nodes"]), _p(out["tris"]), ctypes.byref(root))
    out["root"] = root.value
    return out


def trace(bvh, rays, any_hit=False, stats=False, nthreads=None):
    r = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    m = r.shape[0]
    hits = np.zeros((m, 4), np.float32)
    st = np.zeros((m, 2), np.uint32) if stats else None
    load().or_trace(_p(bvh["nodes"]), _p(bvh["tris"]), ctypes.c_uint32(bvh["root"]), _p(r), ctypes.c_uint64(m),
                    int(any_hit), _p(hits), _p(st), nthreads or threads())
    return (hits, st) if stats else hits


def bvh4(bvh, quant):
    """4-wide layout collapsed from the oracle's binary nodes."""
    n = bvh["tris"].size // 12
    out = np.zeros(max(n - 1, 1) * (16 if quant else 32), np.uint32)
    load().or_bvh4_build(_p(bvh["nodes"]), ctypes.c_uint32(n), int(quant), _p(out))
    return out


def bvh8(bvh):
    """8-wide quantised layout collapsed from the oracle's binary nodes:
    (nodes as uint32 words, 24 per node; node-order triangles, 12 floats each)."""
    n = bvh["tris"].size // 12
    if n == 0:
        return np.zeros(0, np.uint32), np.zeros(0, np.float32)
    cap_n, cap_t = max(n - 1, 1), max(n, 2)
    nodes = np.zeros(cap_n * 24, np.uint32)
    tris = np.zeros(cap_t * 12, np.float32)
    nt = ctypes.c_uint32()
    L = load()
    L.or_bvh8_build.restype = ctypes.c_uint32
    count = L.or_bvh8_build(_p(bvh["nodes"]), _p(bvh["tris"]), ctypes.c_uint32(n), ctypes.c_uint32(bvh["root"]),
                            _p(nodes), ctypes.c_uint32(cap_n), _p(tris), ctypes.c_uint32(cap_t), ctypes.byref(nt))
    return nodes[:24 * count].copy(), tris[:12 * nt.value].copy()


def trace8(bvh, nodes8, tris8, rays, any_hit=False, stats=False, nthreads=None):
    r = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    m = r.shape[0]
    hits = np.zeros((m, 4), np.float32)
    st = np.zeros((m, 2), np.uint32) if stats else None
    load().or_trace8(_p(nodes8), _p(tris8), ctypes.c_uint32(bvh["root"]), _p(r), ctypes.c_uint64(m), int(any_hit),
                     _p(hits), _p(st), nthreads or threads())
    return (hits, st) if stats else hits


def trace4(bvh, nodes4, quant, rays, any_hit=False, stats=False, nthreads=None):
    r = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    m = r.shape[0]
    hits = np.zeros((m, 4), np.float32)
    st = np.zeros((m, 2), np.uint32) if stats else None
    load().or_trace4(_p(nodes4), int(quant), _p(bvh["tris"]), ctypes.c_uint32(bvh["root"]), _p(r), ctypes.c_uint64(m),
                     int(any_hit), _p(hits), _p(st), nthreads or threads())
    return (hits, st) if stats else hits


def trace_brute(verts, rays, any_hit=False, nthreads=None):
    v = np.ascontiguousarray(verts, np.float32).reshape(-1, 9)
    r = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    hits = np.zeros((r.shape[0], 4), np.float32)
    load().or_trace_brute(_p(v), v.shape[0], _p(r), ctypes.c_uint64(r.shape[0]), int(any_hit), _p(hits),
                          nthreads or threads())
    return hits


def trace_ref(ref_nodes, verts, rays, any_hit=False, stats=False, nthreads=None):
    v = np.ascontiguousarray(verts, np.float32).reshape(-1, 9)
    r = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    m = r.shape[0]
    hits = np.zeros((m, 4), np.float32)
    st = np.zeros((m, 2), np.uint32) if stats else None
    load().or_trace_ref(_p(ref_nodes), _p(v), v.shape[0], _p(r), ctypes.c_uint64(m), int(any_hit), _p(hits),
                        _p(st), nthreads or threads())
    return (hits, st) if stats else hits


def fp64_check(ref_nodes, verts, rays, prim, rel_gap=1e-6, bary_margin=1e-6, edge_rel=1e-6, nthreads=None):
    v = np.ascontiguousarray(verts, np.float32).reshape(-1, 9)
    r = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    p = np.ascontiguousarray(prim, np.int32)
    m = r.shape[0]
    t64 = np.zeros(m, np.float64)
    amb = np.zeros(m, np.uint8)
    load().or_fp64_check(_p(ref_nodes), _p(v), v.shape[0], _p(r), ctypes.c_uint64(m), _p(p), _p(t64), _p(amb),
                         ctypes.c_double(rel_gap), ctypes.c_double(bary_margin), ctypes.c_double(edge_rel),
                         nthreads or threads())
    return t64, amb.astype(bool)


def ref_lbvh(verts):
    """The reference's own host LBVH_build (bvh.h), compiled from its sources."""
    v = np.ascontiguousarray(verts, np.float32).reshape(-1, 9)
    n = v.shape[0]
    nodes = np.zeros(max(2 * n - 1, 0) * 8, np.uint32)
    codes = np.zeros(n, np.uint32)
    load_ref().ref_lbvh_build(_p(v), n, _p(nodes), _p(codes))
    return nodes, codes


class _OrMaterial(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("color", ctypes.c_float * 3), ("emission", ctypes.c_float * 3),
                ("ax", ctypes.c_float), ("ay", ctypes.c_float), ("eta_i", ctypes.c_float * 3),
                ("eta_t", ctypes.c_float * 3), ("k", ctypes.c_float * 3), ("ior", ctypes.c_float),
                ("emissive", ctypes.c_uint32), ("tex_off", ctypes.c_uint32), ("tex_w", ctypes.c_uint32),
                ("tex_h", ctypes.c_uint32), ("tuo", ctypes.c_float), ("tvo", ctypes.c_float), ("tus", ctypes.c_float),
                ("tvs", ctypes.c_float), ("spec", ctypes.c_float * 3)]


class _OrEnvmap(ctypes.Structure):
    _fields_ = [("texels", ctypes.c_void_p), ("w", ctypes.c_uint32), ("h", ctypes.c_uint32),
                ("m", ctypes.c_float * 9), ("c", ctypes.c_float * 3)]


class _OrCamera(ctypes.Structure):
    _fields_ = [("m", ctypes.c_float * 12), ("fov_deg", ctypes.c_float), ("width", ctypes.c_uint32),
                ("height", ctypes.c_uint32)]


def render(desc, spp, max_depth=8, seed=0, rr_depth=3, flags=0, sample_base=0, nthreads=None):
    """The integrator restated on the CPU; returns (sum of radiance per pixel
    as float64 (H, W, 3), spp). `desc` is a gr.scenes.SceneDesc."""
    import gr
    soup, nrm, tmat = desc.flatten()
    uvs, uv_bits = desc.flatten_uv()
    tmat = tmat | uv_bits
    texels = []
    n_texels = 0
    mats = (_OrMaterial * max(len(desc.materials), 1))()
    for i, m in enumerate(desc.materials):
        r = gr.material_record(m)
        o = mats[i]
        o.type = r.type
        o.color[:] = r.color[:]
        o.emission[:] = r.emission[:]
        o.ax, o.ay = r.alpha_u, r.alpha_v
        o.eta_i[:] = r.eta_i[:]
        o.eta_t[:] = r.eta_t[:]
        o.k[:] = r.k[:]
        o.ior = r.ior
        o.emissive = 1 if any(x != 0.0 for x in r.emission) else 0
        o.spec[:] = r.specular[:]
        cm = m.get("color_map")
        o.tuo, o.tvo = r.uv_offset[0], r.uv_offset[1]
        o.tus, o.tvs = r.uv_scale[0], r.uv_scale[1]
        if cm is not None:
            cm = np.ascontiguousarray(cm, np.float32).reshape(-1, 3)
            o.tex_off, o.tex_w, o.tex_h = n_texels, r.color_map_width, r.color_map_height
            texels.append(cm)
            n_texels += cm.shape[0]
    cam = _OrCamera()
    M = np.asarray(desc.camera["to_world"], np.float32).reshape(4, 4)
    cam.m[:] = [float(x) for x in M[:3].reshape(12)]
    cam.fov_deg = float(desc.camera["fov"])
    cam.width = int(desc.camera["width"])
    cam.height = int(desc.camera["height"])
    envmap = None
    if isinstance(desc.env, dict):
        env = np.zeros(3, np.float32)
        mp = np.ascontiguousarray(desc.env["map"], np.float32)
        envmap = _OrEnvmap()
        envmap.texels = mp.ctypes.data
        envmap.h, envmap.w = mp.shape[0], mp.shape[1]
        # inverse of the upper 3x3 by cofactors in double, as the library computes it
        M = np.asarray(desc.env.get("to_world", np.eye(4)), np.float32).reshape(4, 4)
        a, b, c, d, e, f, g, h, i = (float(M[r, k]) for r in range(3) for k in range(3))
        det = a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g)
        inv = [(e * i - f * h) / det, (c * h - b * i) / det, (b * f - c * e) / det,
               (f * g - d * i) / det, (a * i - c * g) / det, (c * d - a * f) / det,
               (d * h - e * g) / det, (b * g - a * h) / det, (a * e - b * d) / det]
        envmap.m[:] = [float(np.float32(x)) for x in inv]
        lo, hi = soup.reshape(-1, 3).min(axis=0), soup.reshape(-1, 3).max(axis=0)
        envmap.c[:] = [float(x) for x in ((lo + hi) * np.float32(0.5)).astype(np.float32)]
    else:
        env = np.zeros(3, np.float32) if desc.env is None else np.asarray(desc.env, np.float32)
    tex = np.ascontiguousarray(np.concatenate(texels), np.float32) if texels else None
    fb = np.zeros((cam.height, cam.width, 3), np.float64)
    load().or_render(_p(soup), _p(nrm), _p(tmat), ctypes.c_uint32(soup.shape[0]), mats,
                     ctypes.c_uint32(len(desc.materials)), ctypes.byref(cam), _p(env), int(desc.env is not None),
                     ctypes.c_uint32(spp), ctypes.c_uint32(sample_base), ctypes.c_uint32(max_depth),
                     ctypes.c_uint64(seed), ctypes.c_int32(rr_depth), ctypes.c_uint32(flags), _p(fb),
                     nthreads or threads(), _p(uvs), _p(tex), ctypes.byref(envmap) if envmap is not None else None)
    return fb
