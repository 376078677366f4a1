"""Runs the reference's own device kernels on the GPU — test and bench
infrastructure, never the product.

The kernels of src/renderer/pathtracer_kernel.h (primary rays, trace_kernel,
shade_hit_with_MIS_kernel, trace_shadow_kernel, the light- and BSDF-sampling
accumulation kernels, finish_sample_kernel) are compiled from the reference
sources by oracle/ref/build_ref.sh into two cubins under oracle/_ref/: `stock`
(nvcc's default device flags, as the reference's own build compiles them) and
`nofma` (--fmad=false: every float operation rounded as written, the arithmetic
the CPU restatement in oracle/trace.cpp follows). This module loads a cubin
through the CUDA driver API and lays out the kernels' argument and scene
records from oracle/_ref/ref_layout.json (the byte layout the reference headers
give them, printed at build time):

* traversal (`RefKernels.trace`, `RefScene`): launched as the reference's
  trace() / trace_shadow() wrappers do, 32-thread blocks, one thread per ray
  (pathtracer_kernel.h:235-246, 310-321); the scene follows the reference's own
  harness shape: one mesh whose corner k of triangle j is vertex 3j+k;
* whole frames (`RefRender`): the scene records the reference's loader and
  Scene constructor build from an exported scene (mitsubaloader.cpp:274-530,
  scene.cpp:4-61, camera.h:21-38, texture.cpp, environment.cpp) restated here
  from our scene description, and the frame loop of PathTracer::render
  (pathtracer.cu:41-150) run by oracle/ref_frame.cpp with the reference's
  launch shapes and host synchronisation.

Before any launch the host checks every index the kernels will follow: child
and triangle indices in range, and the tree no deeper than the kernels'
64-entry traversal stack (pathtracer_kernel.h:192,265); every pointer in a
record is one of this module's own device allocations.
"""
import ctypes
import json
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
CUBINS = {"stock": "ref_kernels.cubin", "nofma": "ref_kernels_nofma.cubin"}
LAYOUT = os.path.join(REF_DIR, "ref_layout.json")
FRAME_LIB = os.path.join(HERE, "build", "libref_frame.so")
# Itanium-mangled names of the kernels (uint32 is unsigned int, utility/types.h:4)
_PT = "9PTContext9SceneView15FrameBufferView"
KERNEL_NAMES = {
    "generate": "_Z28generate_primary_rays_kernel" + _PT,
    "trace": "_Z12trace_kernel9SceneViewjP3RayP3Hit",
    "shade": "_Z25shade_hit_with_MIS_kernelj" + _PT,
    "trace_shadow": "_Z19trace_shadow_kernel9SceneViewjP3RayP3Hit",
    "accumulate_light": "_Z45accumulate_light_sampling_contribution_kernelj" + _PT,
    "accumulate_bsdf": "_Z44accumulate_BSDF_sampling_contribution_kernelj" + _PT,
    "finish": "_Z20finish_sample_kernelj15FrameBufferView",
}
FRAME_ORDER = ("generate", "trace", "shade", "trace_shadow", "accumulate_light", "accumulate_bsdf", "finish")
STACK_ENTRIES = 64
BLOCK = 32
# the reference loader's roughconductor defaults (mitsubaloader.cpp:350-357)
CONDUCTOR_ETA = (0.200438, 0.924033, 1.10221)
CONDUCTOR_K = (3.91295, 2.45285, 2.14219)


def available(build="stock"):
    return os.path.exists(os.path.join(REF_DIR, CUBINS[build])) and os.path.exists(LAYOUT)


def render_available(build="stock"):
    return available(build) and os.path.exists(FRAME_LIB)


# ---------------------------------------------------------------------------
# Scene descriptions as files (the reference's own fixture scenes, parsed here
# where its tree is, travel to the GPU machine this way)
# ---------------------------------------------------------------------------
CBOX_SCENE = os.path.join(REF_DIR, "cbox_scene.npz")
# the same fixture as the reference's own loader produces it (refloader.py)
CBOX_REFLOADER_SCENE = os.path.join(REF_DIR, "cbox_refloader_scene.npz")


def save_refloader_scene(xml_path, out_path):
    """The scene the reference's own loader builds from `xml_path`, as a
    SceneDesc file: one mesh per reference mesh with its triangles' corners as
    separate vertices (m_cpu_triangles order), its shading normals, and the
    material fields its type uses. The camera's field of view is kept in
    degrees as this library parses it, after checking that the reference's
    radians are exactly its degToRad."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "gpu-renderer_gb300"))
    import gr
    import refloader
    from gr.scenes import MeshDesc, SceneDesc
    r = refloader.load(xml_path)
    parsed = gr.ParsedScene(xml_path)
    fov = parsed.camera["fov"]
    parsed.close()
    if refloader.deg_to_rad(fov).view(np.uint32) != r["camera"][16:17].view(np.uint32)[0]:
        raise RuntimeError("field of view differs from the reference loader's")
    meshes, mats = [], []
    for i in range(r["materials"].shape[0]):
        sel = r["mesh"] == i
        k = int(sel.sum())
        nrm = r["normals"][sel].reshape(-1, 3)
        meshes.append(MeshDesc(r["verts"][sel].reshape(-1, 3), np.arange(3 * k, dtype=np.uint32).reshape(k, 3), i,
                               normals=None if np.isnan(nrm).any() else nrm))
        f = refloader.material_fields(r["materials"][i])
        if "color_map_size" in f:
            raise ValueError("textured materials have no record form here")
        m = {"type": int(f["type"]), "color": tuple(map(float, f["color"])), "emission": tuple(map(float, f["emission"])),
             "alpha_u": 0.0, "alpha_v": 0.0, "eta_i": (0.0, 0.0, 0.0), "eta_t": (0.0, 0.0, 0.0), "k": (0.0, 0.0, 0.0),
             "ior": 0.0, "specular": (0.0, 0.0, 0.0)}
        if "ior" in f:
            m["ior"] = float(f["ior"][0])
        for key in ("eta_i", "eta_t", "k", "specular"):
            if key in f:
                m[key] = tuple(map(float, f[key]))
        if "alpha" in f:
            m["alpha_u"], m["alpha_v"] = float(f["alpha"][0]), float(f["alpha"][1])
        mats.append(m)
    cam = {"to_world": r["camera"][:16].reshape(4, 4).copy(), "fov": fov, "width": int(r["camera"][17]),
           "height": int(r["camera"][18])}
    env = tuple(map(float, r["env"][1:4])) if r["env"][0] else None
    save_desc(SceneDesc(meshes, mats, cam, env), out_path)


def save_desc(desc, path):
    """A gr.scenes.SceneDesc (constant or no environment) to an .npz file."""
    arrays = {"camera_to_world": np.asarray(desc.camera["to_world"], np.float32),
              "camera": np.array([desc.camera["fov"], desc.camera["width"], desc.camera["height"]], np.float64),
              "materials": np.array(json.dumps(desc.materials)), "n_meshes": np.array(len(desc.meshes))}
    if desc.env is not None:
        arrays["env"] = np.asarray(desc.env, np.float32)
    for i, m in enumerate(desc.meshes):
        arrays["p%d" % i] = m.positions
        arrays["i%d" % i] = m.indices
        arrays["m%d" % i] = np.array(m.material)
        if m.normals is not None:
            arrays["n%d" % i] = m.normals
    np.savez_compressed(path, **arrays)


def load_desc(path, width=None, height=None):
    """The SceneDesc save_desc wrote; width / height replace the camera's
    resolution (the field of view stays)."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "gpu-renderer_gb300"))
    from gr.scenes import MeshDesc, SceneDesc
    z = np.load(path)
    meshes = [MeshDesc(z["p%d" % i], z["i%d" % i], int(z["m%d" % i]), normals=z["n%d" % i] if "n%d" % i in z else None)
              for i in range(int(z["n_meshes"]))]
    fov, w, h = z["camera"]
    cam = {"to_world": z["camera_to_world"], "fov": float(fov), "width": int(width or w), "height": int(height or h)}
    mats = [{k: (tuple(v) if isinstance(v, list) else v) for k, v in m.items()} for m in json.loads(str(z["materials"]))]
    return SceneDesc(meshes, mats, cam, tuple(z["env"]) if "env" in z else None)


def load_layout():
    with open(LAYOUT) as f:
        L = json.load(f)
    sizes = {k: L[k]["size"] for k in ("Ray", "Hit", "BVHLinearNode", "Spectrum", "Transform", "TextureView")}
    if sizes != {"Ray": 32, "Hit": 16, "BVHLinearNode": 32, "Spectrum": 12, "Transform": 128, "TextureView": 40}:
        raise RuntimeError("unexpected reference record sizes: %r" % sizes)
    if L["Hit"]["triangle_id"] != 4:
        raise RuntimeError("unexpected Hit layout")
    ptr_fields = [("SceneView", "m_triangles"), ("SceneView", "m_lights"), ("SceneView", "m_bvh"),
                  ("TriangleMeshView", "m_p"), ("TriangleMeshView", "m_n"), ("TriangleMeshView", "m_uv"),
                  ("TriangleMeshView", "m_index"), ("TextureView", "m_buffer"), ("EnvironmentLightView", "m_buffer"),
                  ("FrameBufferView", "m_buffer"), ("FrameBufferView", "m_sample_num")]
    for t, f in ptr_fields:
        if L[t][f] % 8:
            raise RuntimeError("unaligned pointer field %s::%s" % (t, f))
    for t in ("Triangle", "TriangleMeshView", "Material", "SceneView", "PTContext", "RayQueue"):
        if L[t]["size"] % 8:
            raise RuntimeError("unexpected size of " + t)
    return L


def tree_depth(ref_nodes, n):
    """Checks a reference-layout node array (8 words per node: box, index,
    leaf byte) over n triangles and returns its depth in edges (a single leaf
    has depth 0). Raises ValueError on any index the kernels would follow out
    of range."""
    w = np.ascontiguousarray(ref_nodes, np.uint32).reshape(-1, 8)
    m = w.shape[0]
    if n == 0 or m != 2 * n - 1:
        raise ValueError("expected %d nodes for %d triangles, got %d" % (max(2 * n - 1, 0), n, m))
    leaf = (w[:, 7] & 0xFF) != 0
    idx = w[:, 6].astype(np.int64)
    if np.any(idx[leaf] >= n):
        raise ValueError("leaf triangle index out of range")
    inner = np.nonzero(~leaf)[0]
    if np.any(inner + 1 >= m) or np.any(idx[inner] >= m) or np.any(idx[inner] <= inner + 1):
        raise ValueError("child index out of range or not after its parent")
    depth, frontier = 0, np.array([0], np.int64)
    seen = 1
    while True:
        f = frontier[~leaf[frontier]]
        if f.size == 0:
            break
        frontier = np.concatenate([f + 1, idx[f]])
        seen += frontier.size
        depth += 1
        if seen > m:
            raise ValueError("node array is not a tree")
    if seen != m:
        raise ValueError("node array is not a tree (%d of %d nodes reachable)" % (seen, m))
    return depth


# ---------------------------------------------------------------------------
# Record builders (bytes in the reference layout)
# ---------------------------------------------------------------------------
def _put(buf, off, dtype, values):
    a = np.asarray(values, dtype).reshape(-1)
    buf[off:off + a.nbytes] = np.frombuffer(a.tobytes(), np.uint8)


def _transform(buf, off, m):
    """Transform (transform.h:87-148): the matrix and its inverse, row-major."""
    m = np.asarray(m, np.float64).reshape(4, 4)
    _put(buf, off, np.float32, m)
    _put(buf, off + 64, np.float32, np.linalg.inv(m))


def _transform_pair(buf, off, m, minv):
    _put(buf, off, np.float32, np.asarray(m, np.float64).reshape(4, 4))
    _put(buf, off + 64, np.float32, np.asarray(minv, np.float64).reshape(4, 4))


def camera_record(L, to_world, fov_deg, width, height):
    """Camera() followed by Camera::setup(toWorld, fov, w, h, free = false)
    (camera.h:10-38): the matrices computed in double precision and stored as
    float, where the reference computes them in float (a few ulp apart)."""
    C = L["Camera"]
    b = np.zeros(C["size"], np.uint8)
    d = np.array([0.0, -0.2, -1.0], np.float32)
    _put(b, C["m_eye"], np.float32, [0, 2, 7])
    _put(b, C["m_dir"], np.float32, d)
    _put(b, C["m_up"], np.float32, [0, 1, 0])
    _put(b, C["m_yaw"], np.float32, [math.atan2(float(d[0]), float(d[2]))])
    _put(b, C["m_pitch"], np.float32, [math.asin(float(d[1]))])
    fov = np.float32(np.float32(fov_deg) / np.float32(180) * np.float32(math.pi))
    _put(b, C["m_fov"], np.float32, [fov, fov])
    _put(b, C["m_resolution_x"], np.uint32, [width])
    _put(b, C["m_resolution_y"], np.uint32, [height])
    aspect = float(np.float32(np.float32(width) / np.float32(height)))
    _put(b, C["m_aspect_ratio"], np.float32, [aspect])
    _transform(b, C["m_cameraToWorld"], to_world)
    # CameraToRaster = Scale(w, h, 1) * Scale(-0.5, 0.5 aspect, 1) *
    # Translate(-1, 1 / aspect, 0) * Perspective(fov, 1e-4, 1e4); the camera
    # keeps its inverse (camera.h:31-36, transform.cpp:105-151, 251-259)
    inv_tan = 1.0 / math.tan(float(fov) * 0.5)
    n, f = 1e-4, 1e4
    persp = np.array([[inv_tan, 0, 0, 0], [0, inv_tan, 0, 0], [0, 0, f / (f - n), -f * n / (f - n)], [0, 0, 1, 0]])
    s1 = np.diag([float(width), float(height), 1.0, 1.0])
    s2 = np.diag([-0.5, 0.5 * aspect, 1.0, 1.0])
    tr = np.eye(4)
    tr[0, 3], tr[1, 3] = -1.0, 1.0 / aspect
    cam_to_raster = s1 @ s2 @ tr @ persp
    _transform_pair(b, C["m_rasterToCamera"], np.linalg.inv(cam_to_raster), cam_to_raster)
    b[C["m_free"]] = 0
    return b


def env_record(L, radiance, world_center):
    """EnvironmentLight::setup(radiance) viewed as EnvironmentLightView
    (environment.cpp:3-9, 40-46); radiance None: no environment (m_has false).
    Returns the record and the texel array its buffer pointer must name; the
    pointer field is left zero."""
    E = L["EnvironmentLightView"]
    b = np.zeros(E["size"], np.uint8)
    b[E["m_has"]] = 1 if radiance is not None else 0
    texels = np.asarray(radiance if radiance is not None else (0.0, 0.0, 0.0), np.float32).reshape(1, 3)
    _put(b, E["m_width"], np.int32, [1 if radiance is not None else 0])
    _put(b, E["m_height"], np.int32, [1 if radiance is not None else 0])
    _transform_pair(b, E["m_o2w"], np.eye(4), np.eye(4))
    _transform_pair(b, E["m_w2o"], np.eye(4), np.eye(4))
    _put(b, E["m_world_center"], np.float32, world_center)
    return b, texels


def material_records(L, materials):
    """The Material of every shape, in shape order, as the reference's loader
    builds them from an exported scene (mitsubaloader.cpp:288-440 for the BSDF,
    the area emitter's radiance as m_emission, :481-516). `materials` holds
    gr material dicts. The loader reuses one material across shapes and sets
    only the textures a BSDF type names, so the others carry over from the
    shape before (none of the reference's BSDFs reads them, bxdf.h:160-215);
    before the first assignment they name a 1x1 black texture here instead of
    the reference's null, empty view. Every texture is a 1x1 constant
    (texture.cpp:15-27). Returns [(record bytes, {TextureView offset: texel
    (3,)})] with the buffer pointers left zero."""
    import gr
    M, T, E = L["Material"], L["TextureView"], L["enums"]
    cur = np.zeros(M["size"], np.uint8)
    tex = {}

    def set_view(field, value, kind):
        off = M[field]
        _put(cur, off + T["m_uvoffset"], np.float32, [0, 0])
        _put(cur, off + T["m_uvscale"], np.float32, [1, 1])
        _put(cur, off + T["m_width"], np.uint32, [1])
        _put(cur, off + T["m_height"], np.uint32, [1])
        _put(cur, off + T["m_type"], np.int32, [E[kind]])
        v = np.asarray(value, np.float32).reshape(-1)
        tex[off] = np.repeat(v, 3) if v.size == 1 else v

    for field in ("m_color", "m_color1", "m_etaI", "m_etaT", "m_k", "m_ior", "m_alpha_x", "m_alpha_y"):
        set_view(field, (0.0, 0.0, 0.0), "TEXTURE_SPECTRUM")
    out = []
    for m in materials:
        r = gr.material_record(m)
        if r.type == gr.MAT_DIFFUSE:
            set_view("m_color", tuple(r.color), "TEXTURE_SPECTRUM")
            mtype = "MATERIAL_DIFFUSE"
        elif r.type == gr.MAT_DIELECTRIC:
            set_view("m_color", tuple(r.color), "TEXTURE_SPECTRUM")
            set_view("m_ior", [r.ior], "TEXTURE_FLOAT")
            mtype = "MATERIAL_SPECULAR"
        elif r.type == gr.MAT_CONDUCTOR:
            set_view("m_color", tuple(r.color), "TEXTURE_SPECTRUM")
            set_view("m_etaI", (1.0, 1.0, 1.0), "TEXTURE_SPECTRUM")
            set_view("m_etaT", tuple(r.eta_t), "TEXTURE_SPECTRUM")
            set_view("m_k", tuple(r.k), "TEXTURE_SPECTRUM")
            set_view("m_alpha_x", [r.alpha_u], "TEXTURE_FLOAT")
            set_view("m_alpha_y", [r.alpha_u], "TEXTURE_FLOAT")
            mtype = "MATERIAL_ROUGH_CONDUCTOR"
        else:
            raise ValueError("material type %d has no exported counterpart" % r.type)
        _put(cur, M["m_type"], np.int32, [E[mtype]])
        _put(cur, M["m_emission"], np.float32, tuple(m.get("emission", (0.0, 0.0, 0.0))))
        out.append((cur.copy(), dict(tex)))
    return out


# ---------------------------------------------------------------------------
# Driver API
# ---------------------------------------------------------------------------
class _Driver:
    """The few CUDA driver API calls this module needs, through ctypes."""

    def __init__(self):
        self.lib = ctypes.CDLL("libcuda.so.1")
        self.lib.cuGetErrorString.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
        self.lib.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 7 + [
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]

    def check(self, rc, what):
        if rc != 0:
            s = ctypes.c_char_p()
            self.lib.cuGetErrorString(rc, ctypes.byref(s))
            raise RuntimeError("%s failed: %s (%d)" % (what, (s.value or b"?").decode(), rc))


class RefKernels:
    """One loaded cubin (`stock` or `nofma`) on one device."""

    def __init__(self, build="stock", device=0):
        import torch
        if not available(build):
            raise FileNotFoundError("reference kernels not built (oracle/_ref/%s)" % CUBINS[build])
        self.layout = load_layout()
        self.build = build
        self.device = device
        torch.cuda.set_device(device)
        torch.zeros(1, device="cuda")  # the runtime makes the primary context current
        self.d = _Driver()
        lib = self.d.lib
        self.d.check(lib.cuInit(0), "cuInit")
        dev = ctypes.c_int()
        self.d.check(lib.cuDeviceGet(ctypes.byref(dev), device), "cuDeviceGet")
        self.ctx = ctypes.c_void_p()
        self.d.check(lib.cuDevicePrimaryCtxRetain(ctypes.byref(self.ctx), dev), "cuDevicePrimaryCtxRetain")
        self.dev = dev
        self.d.check(lib.cuCtxSetCurrent(self.ctx), "cuCtxSetCurrent")
        self.mod = ctypes.c_void_p()
        path = os.path.join(REF_DIR, CUBINS[build]).encode()
        self.d.check(lib.cuModuleLoad(ctypes.byref(self.mod), path), "cuModuleLoad")
        self.fn = {}
        for key, name in KERNEL_NAMES.items():
            f = ctypes.c_void_p()
            self.d.check(lib.cuModuleGetFunction(ctypes.byref(f), self.mod, name.encode()),
                         "cuModuleGetFunction(%s)" % key)
            self.fn[key] = f

    def close(self):
        if self.mod:
            self.d.lib.cuModuleUnload(self.mod)
            self.mod = ctypes.c_void_p()
            self.d.lib.cuDevicePrimaryCtxRelease_v2(self.dev)

    def scene(self, ref_nodes, verts):
        return RefScene(self, ref_nodes, verts)

    def trace(self, scene, rays, hits, any_hit=False, stream=None):
        """Launches the reference traversal kernel on device tensors: rays
        (m, 8) float32 in the reference Ray layout, hits (m, 4) 32-bit (t,
        triangle id, u, v). Misses get id -1; their t, u, v are whatever the
        kernel leaves there."""
        import torch
        m = rays.shape[0]
        if m == 0:
            return
        if m >= 2 ** 32 - BLOCK:
            raise ValueError("too many rays")
        for t, name, width in ((rays, "rays", 8), (hits, "hits", 4)):
            if not (t.is_cuda and t.is_contiguous() and t.element_size() == 4 and t.dim() == 2
                    and t.shape[1] == width):
                raise ValueError(name + ": expected a contiguous (m, %d) 32-bit CUDA tensor" % width)
        if hits.shape[0] < m:
            raise ValueError("hits shorter than rays")
        if stream is None:
            stream = torch.cuda.current_stream().cuda_stream
        sv = (ctypes.c_uint8 * scene.scene_view.size).from_buffer_copy(scene.scene_view.tobytes())
        size = ctypes.c_uint32(m)
        rp = ctypes.c_uint64(rays.data_ptr())
        hp = ctypes.c_uint64(hits.data_ptr())
        params = (ctypes.c_void_p * 4)(ctypes.addressof(sv), ctypes.addressof(size), ctypes.addressof(rp),
                                       ctypes.addressof(hp))
        grid = (m + BLOCK - 1) // BLOCK
        fn = self.fn["trace_shadow" if any_hit else "trace"]
        self.d.check(self.d.lib.cuLaunchKernel(fn, grid, 1, 1, BLOCK, 1, 1, 0, ctypes.c_void_p(stream), params,
                                               None), "cuLaunchKernel")

    def trace_host(self, scene, rays, any_hit=False):
        import torch
        r = torch.from_numpy(np.ascontiguousarray(rays, np.float32).reshape(-1, 8)).cuda()
        h = torch.zeros((r.shape[0], 4), dtype=torch.float32, device="cuda")
        self.trace(scene, r, h, any_hit)
        torch.cuda.synchronize()
        return h.cpu().numpy()


def _mesh_view(L, n_tris, n_p, n_n, p_ptr, n_ptr, index_ptr, material):
    V = L["TriangleMeshView"]
    b = np.zeros(V["size"], np.uint8)
    _put(b, V["m_triangle_num"], np.uint32, [n_tris])
    _put(b, V["m_p_num"], np.uint32, [n_p])
    _put(b, V["m_n_num"], np.uint32, [n_n])
    _put(b, V["m_uv_num"], np.uint32, [0])
    _put(b, V["m_index_num"], np.uint32, [3 * n_tris])
    _put(b, V["m_p"], np.uint64, [p_ptr])
    _put(b, V["m_n"], np.uint64, [n_ptr])
    _put(b, V["m_uv"], np.uint64, [0])
    _put(b, V["m_index"], np.uint64, [index_ptr])
    b[V["m_material"]:V["m_material"] + material.size] = material
    return b


def _triangles(L, view, n_tris, out=None):
    """Triangle records j = 0..n-1 of one mesh view: the view and m_index = 3j
    (scene.cpp:8-12), written into `out` (n_tris, Triangle size) if given."""
    T = L["Triangle"]
    rec = np.zeros((n_tris, T["size"]), np.uint8) if out is None else out
    rec[:] = 0
    rec[:, T["m_mesh"]:T["m_mesh"] + view.size] = view
    rec.view(np.uint32)[:, T["m_index"] // 4] = 3 * np.arange(n_tris, dtype=np.uint32)
    return rec


class RefScene:
    """Device copies of one triangle soup in the reference's records, for the
    traversal kernels alone."""

    def __init__(self, rk, ref_nodes, verts):
        import torch
        L = rk.layout
        v = np.ascontiguousarray(verts, np.float32).reshape(-1, 9)
        n = v.shape[0]
        self.depth = tree_depth(ref_nodes, n)
        if self.depth > STACK_ENTRIES:
            raise ValueError("tree depth %d exceeds the reference kernels' %d-entry stack" %
                             (self.depth, STACK_ENTRIES))
        dev = torch.device("cuda", rk.device)
        self.nodes = torch.from_numpy(np.ascontiguousarray(ref_nodes, np.uint32).reshape(-1)).to(dev)
        self.p = torch.from_numpy(v.reshape(-1)).to(dev)  # 3n float3 corners
        corner = np.full((3 * n, 3), -1, np.int32)
        corner[:, 0] = np.arange(3 * n, dtype=np.int32)
        self.index = torch.from_numpy(corner.reshape(-1)).to(dev)  # int3 (p, uv, n) per corner
        view = _mesh_view(L, n, 3 * n, 0, self.p.data_ptr(), 0, self.index.data_ptr(),
                          np.zeros(L["Material"]["size"], np.uint8))
        self.triangles = torch.from_numpy(_triangles(L, view, n).reshape(-1)).to(dev)
        S = L["SceneView"]
        sv = np.zeros(S["size"], np.uint8)
        _put(sv, S["m_triangles"], np.uint64, [self.triangles.data_ptr()])
        _put(sv, S["m_triangles_num"], np.uint32, [n])
        _put(sv, S["m_bvh"], np.uint64, [self.nodes.data_ptr()])
        self.scene_view = sv
        self.n = n


class RefRender:
    """One scene description rendered by the reference's kernels: the scene
    records of the reference's loader and Scene constructor, its framebuffer
    and its three ray queues (pathtracer_kernel.h:24-57), on the device."""

    def __init__(self, rk, desc, ref_nodes):
        import torch
        if not os.path.exists(FRAME_LIB):
            raise FileNotFoundError("oracle/build/libref_frame.so not built")
        self.rk = rk
        L = rk.layout
        dev = torch.device("cuda", rk.device)
        self.keep = []

        def upload(a):
            t = torch.from_numpy(np.ascontiguousarray(a)).to(dev)
            self.keep.append(t)
            return t.data_ptr()

        cam = desc.camera
        W, H = int(cam["width"]), int(cam["height"])
        mats = material_records(L, [desc.materials[m.material] for m in desc.meshes])
        # geometry and per-mesh views, in shape order (scene.cpp:6-13)
        n_total = desc.num_triangles
        triangles = np.empty((n_total, L["Triangle"]["size"]), np.uint8)
        lights = []
        first = 0
        for m, (mat_bytes, tex) in zip(desc.meshes, mats):
            for off, texel in tex.items():
                ptr = upload(np.asarray(texel, np.float32).reshape(1, 3))
                _put(mat_bytes, off + L["TextureView"]["m_buffer"], np.uint64, [ptr])
            pos = np.ascontiguousarray(m.positions, np.float32).reshape(-1, 3)
            tri = np.ascontiguousarray(m.indices, np.int32).reshape(-1, 3)
            if tri.size and (tri.min() < 0 or tri.max() >= pos.shape[0]):
                raise ValueError("mesh index out of range")
            corner = np.full((tri.size, 3), -1, np.int32)
            corner[:, 0] = tri.reshape(-1)
            n_ptr, n_n = 0, 0
            if m.normals is not None:
                nrm = np.ascontiguousarray(m.normals, np.float32).reshape(-1, 3)
                if nrm.shape[0] != pos.shape[0]:
                    raise ValueError("one normal per vertex expected")
                corner[:, 2] = tri.reshape(-1)
                n_ptr, n_n = upload(nrm), nrm.shape[0]
            view = _mesh_view(L, tri.shape[0], pos.shape[0], n_n, upload(pos), n_ptr, upload(corner), mat_bytes)
            r = _triangles(L, view, tri.shape[0], triangles[first:first + tri.shape[0]])
            em = desc.materials[m.material].get("emission", (0.0, 0.0, 0.0))
            if any(float(x) != 0.0 for x in em):
                lights.append(r.copy())
            first += tri.shape[0]
        if not lights:
            raise ValueError("the reference's light sampling needs an emissive triangle (sample_lights)")
        light_recs = np.concatenate(lights)
        self.depth = tree_depth(ref_nodes, n_total)
        if self.depth > STACK_ENTRIES:
            raise ValueError("tree depth %d exceeds the reference kernels' %d-entry stack" %
                             (self.depth, STACK_ENTRIES))
        box = np.ascontiguousarray(ref_nodes, np.uint32).reshape(-1, 8)[0, :6].view(np.float32)
        center = (box[:3] + box[3:]) * np.float32(0.5)  # AABB::centroid of the root (scene.cpp:23-24)
        env, env_texels = env_record(L, desc.env, center)
        _put(env, L["EnvironmentLightView"]["m_buffer"], np.uint64, [upload(env_texels)])
        S = L["SceneView"]
        sv = np.zeros(S["size"], np.uint8)
        camb = camera_record(L, np.asarray(cam["to_world"], np.float64).reshape(4, 4), float(cam["fov"]), W, H)
        sv[S["m_camera"]:S["m_camera"] + camb.size] = camb
        _put(sv, S["m_triangles"], np.uint64, [upload(triangles.reshape(-1))])
        _put(sv, S["m_triangles_num"], np.uint32, [n_total])
        _put(sv, S["m_lights"], np.uint64, [upload(light_recs.reshape(-1))])
        _put(sv, S["m_lights_num"], np.uint32, [light_recs.shape[0]])
        sv[S["m_environment_light"]:S["m_environment_light"] + env.size] = env
        _put(sv, S["m_bvh"], np.uint64, [upload(np.ascontiguousarray(ref_nodes, np.uint32).reshape(-1))])
        del triangles
        # framebuffer (framebuffer.h:8-35) and queues sized to the pixel count
        npix = W * H
        self.fb = torch.zeros((npix, 3), dtype=torch.float32, device=dev)
        self.fb_count = torch.zeros(npix, dtype=torch.int32, device=dev)
        F = L["FrameBufferView"]
        fbv = np.zeros(F["size"], np.uint8)
        _put(fbv, F["m_resolution_x"], np.uint32, [W])
        _put(fbv, F["m_resolution_y"], np.uint32, [H])
        _put(fbv, F["m_buffer"], np.uint64, [self.fb.data_ptr()])
        _put(fbv, F["m_sample_num"], np.uint64, [self.fb_count.data_ptr()])
        Q, P = L["RayQueue"], L["PTContext"]
        ctxb = np.zeros(P["size"], np.uint8)
        self.queues = []
        for which in ("m_in_queue", "m_shadow_queue", "m_scatter_queue"):
            # zeroed: the reference's scatter queue is read before it is
            # written (its seeds are not copied on append, rayqueue.h:19-47)
            q = {k: torch.zeros(npix * s, dtype=torch.uint8, device=dev)
                 for k, s in (("m_rays", 32), ("m_hits", 16), ("m_weight", 12), ("m_pdf", 4), ("m_specular", 1),
                              ("m_idx", 4), ("m_seed", 4))}
            q["m_size"] = torch.zeros(4, dtype=torch.uint8, device=dev)
            self.queues.append(q)
            for k, t in q.items():
                _put(ctxb, P[which] + Q[k], np.uint64, [t.data_ptr()])
        self.scene_view, self.fb_view, self.context = sv, fbv, ctxb
        self.width, self.height = W, H
        self.samples = 0
        self.triangles = n_total
        self.lights = light_recs.shape[0]

    def render(self, frames, max_path_length):
        """Renders `frames` 1-spp frames; returns (seconds, rays traced)."""
        import torch
        lib = ctypes.CDLL(FRAME_LIB)
        lib.ref_render_frames.restype = ctypes.c_int
        L = self.rk.layout
        P, Q = L["PTContext"], L["RayQueue"]
        ctx = np.array([P["size"], P["m_bounce"], P["m_sample_num"], P["m_in_queue"], P["m_shadow_queue"],
                        P["m_scatter_queue"], Q["size"], Q["m_rays"], Q["m_hits"], Q["m_size"]], np.uint32)
        fns = (ctypes.c_void_p * 7)(*[self.rk.fn[k].value for k in FRAME_ORDER])
        secs = ctypes.c_double()
        rays = ctypes.c_uint64()
        torch.cuda.synchronize()
        rc = lib.ref_render_frames(fns, self.scene_view.ctypes.data_as(ctypes.c_void_p),
                                   ctypes.c_uint32(self.scene_view.size),
                                   self.fb_view.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint32(self.fb_view.size),
                                   self.context.ctypes.data_as(ctypes.c_void_p),
                                   ctx.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint32(self.width),
                                   ctypes.c_uint32(self.height), ctypes.c_uint32(frames),
                                   ctypes.c_uint32(self.samples), ctypes.c_uint32(max_path_length),
                                   ctypes.byref(secs), ctypes.byref(rays))
        if rc != 0:
            self.rk.d.check(rc, "reference frame loop")
        self.samples += frames
        return secs.value, rays.value

    def image(self):
        """Mean radiance per pixel, (H, W, 3) float64: the framebuffer sum over
        the per-pixel sample count (framebuffer.h:8-35)."""
        s = self.fb.double().cpu().numpy().reshape(self.height, self.width, 3)
        c = self.fb_count.cpu().numpy().reshape(self.height, self.width, 1)
        return s / np.maximum(c, 1)
