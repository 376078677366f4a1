"""The reference's own scene loading (test infrastructure): a ctypes wrapper
around oracle/_ref/libref_loader.so, which build_ref.sh compiles from the
reference's loader sources where they lie (Scene::Scene, scene.cpp:4-27:
load_mitsuba_file / load_obj_file and the flattening of its meshes into
m_cpu_triangles).

load(path) returns what the reference's loader produced, per triangle in
m_cpu_triangles order and per mesh; material_fields() maps one reference
material record onto the gr_material fields it determines, so that a test
compares only what the reference's material type uses (the reference reuses
one "current material" object between shapes, so unused fields keep whatever
an earlier material left there).
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libref_loader.so")

_lib = None
_P = ctypes.c_void_p

# reference MaterialType (material.h:6-13) -> gr_material_type
REF_TO_GR_TYPE = {0: 0, 1: 1, 2: 2, 4: 3}
# texture slots of a reference material record, in ref_materials' order
_SLOTS = ("color", "color1", "eta_i", "eta_t", "k", "ior", "alpha_x", "alpha_y")


def available():
    return os.path.exists(LIB)


def _load_lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(LIB)
        L.ref_load.argtypes = [ctypes.c_char_p, ctypes.POINTER(_P), ctypes.POINTER(ctypes.c_uint32)]
        L.ref_load.restype = ctypes.c_int
        L.ref_triangles.argtypes = [_P, _P, _P, _P, _P]
        L.ref_materials.argtypes = [_P, _P]
        L.ref_camera_env.argtypes = [_P, _P, _P]
        L.ref_free.argtypes = [_P]
        L.ref_material_floats.restype = ctypes.c_int
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(_P)


def load(path):
    """The reference loader's result for the scene file `path`:
    verts (n, 9), normals (n, 9) and uvs (n, 6) (NaN where a triangle's mesh
    has none), mesh (n,) mesh index of each triangle, materials (meshes, 48)
    raw records (see ref_loader.cpp), camera (19,) = cameraToWorld row-major,
    fov in radians, width, height, env (6,) = has, first texel rgb, width,
    height."""
    L = _load_lib()
    h, nm = _P(), ctypes.c_uint32()
    n = L.ref_load(os.fsencode(path), ctypes.byref(h), ctypes.byref(nm))
    if n < 0:
        raise RuntimeError("the reference loader failed on " + path)
    try:
        out = {"verts": np.zeros((n, 9), np.float32), "normals": np.zeros((n, 9), np.float32),
               "uvs": np.zeros((n, 6), np.float32), "mesh": np.zeros(n, np.uint32),
               "materials": np.zeros((nm.value, L.ref_material_floats()), np.float32),
               "camera": np.zeros(19, np.float32), "env": np.zeros(6, np.float32)}
        L.ref_triangles(h, _ptr(out["verts"]), _ptr(out["normals"]), _ptr(out["uvs"]), _ptr(out["mesh"]))
        if nm.value:
            L.ref_materials(h, _ptr(out["materials"]))
        L.ref_camera_env(h, _ptr(out["camera"]), _ptr(out["env"]))
    finally:
        L.ref_free(h)
    return out


def material_fields(rec):
    """The gr_material fields one reference material record determines, as a
    dict of float32 arrays (what a loader must reproduce for that type)."""
    rec = np.asarray(rec, np.float32)
    slot = {name: rec[4 + 5 * k: 9 + 5 * k] for k, name in enumerate(_SLOTS)}  # rgb, width, height
    t = REF_TO_GR_TYPE[int(rec[0])]
    f = {"type": np.float32(t), "emission": rec[1:4]}
    col = slot["color"]
    if col[3] * col[4] > 1:
        f["color_map_size"] = col[3:5]
        f["color_map_first"] = col[0:3]
    else:
        f["color"] = col[0:3]
    if t == 1:  # smooth dielectric: the "ior" texture
        f["ior"] = slot["ior"][0:1]
    elif t == 2:  # GGX conductor
        f.update(eta_i=slot["eta_i"][0:3], eta_t=slot["eta_t"][0:3], k=slot["k"][0:3],
                 alpha=np.array([slot["alpha_x"][0], slot["alpha_y"][0]], np.float32))
    elif t == 3:  # rough plastic: color1 is the specular lobe's reflectance
        f.update(specular=slot["color1"][0:3], eta_i=slot["eta_i"][0:3], eta_t=slot["eta_t"][0:3],
                 alpha=np.array([slot["alpha_x"][0], slot["alpha_y"][0]], np.float32))
    return f


def gr_material_fields(m):
    """The same fields read from a gr_material record (gr.Material)."""
    f = {"type": np.float32(m.type), "emission": np.array(m.emission[:], np.float32)}
    if m.color_map:
        w, h = m.color_map_width, m.color_map_height
        first = ctypes.cast(m.color_map, ctypes.POINTER(ctypes.c_float))
        f["color_map_size"] = np.array([w, h], np.float32)
        f["color_map_first"] = np.array([first[0], first[1], first[2]], np.float32)
    else:
        f["color"] = np.array(m.color[:], np.float32)
    if m.type == 1:
        f["ior"] = np.array([m.ior], np.float32)
    elif m.type == 2:
        f.update(eta_i=np.array(m.eta_i[:], np.float32), eta_t=np.array(m.eta_t[:], np.float32),
                 k=np.array(m.k[:], np.float32), alpha=np.array([m.alpha_u, m.alpha_v], np.float32))
    elif m.type == 3:
        f.update(specular=np.array(m.specular[:], np.float32), eta_i=np.array(m.eta_i[:], np.float32),
                 eta_t=np.array(m.eta_t[:], np.float32), alpha=np.array([m.alpha_u, m.alpha_v], np.float32))
    return f


def deg_to_rad(fov_deg):
    """The reference's degToRad (fwd.h:29-32) in FP32: deg / 180 * PI."""
    return np.float32(np.float32(fov_deg) / np.float32(180.0)) * np.float32(3.14159265358979323846)
