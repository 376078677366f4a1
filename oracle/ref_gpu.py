"""Runs the reference's own traversal kernels on the GPU — test and bench
infrastructure, never the product.

`trace_kernel` and `trace_shadow_kernel` (src/renderer/pathtracer_kernel.h:
175-321) are compiled from the reference sources by oracle/ref/build_ref.sh
into two cubins under oracle/_ref/: `stock` (nvcc's default device flags, as
the reference's own build compiles them) and `nofma` (--fmad=false: every
float operation rounded as written, the arithmetic the CPU restatement in
oracle/trace.cpp follows). This module loads a cubin through the CUDA driver
API, lays out the kernels' argument records from oracle/_ref/ref_layout.json
(SceneView, scene.h:15-30; Triangle / TriangleMeshView, triangle.h:10-60) and
launches them as the reference's trace() / trace_shadow() wrappers do:
32-thread blocks, one thread per ray (pathtracer_kernel.h:235-246, 310-321).

Scene data follow the reference's own harness shape: one mesh whose corner k
of triangle j is vertex 3j+k (index records (3j+k, -1, -1)), Triangle j with
m_index = 3j, and the BVH in the reference's BVHLinearNode layout.

Before any launch the host checks every index the kernels will follow: child
and triangle indices in range, and the tree no deeper than the kernels'
64-entry traversal stack (pathtracer_kernel.h:192,265).
"""
import ctypes
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
CUBINS = {"stock": "ref_kernels.cubin", "nofma": "ref_kernels_nofma.cubin"}
LAYOUT = os.path.join(REF_DIR, "ref_layout.json")
# Itanium-mangled names of trace_kernel(SceneView, uint32, Ray*, Hit*) and
# trace_shadow_kernel(SceneView, uint32, Ray*, Hit*); uint32 is unsigned int
# (utility/types.h:4).
KERNELS = {False: b"_Z12trace_kernel9SceneViewjP3RayP3Hit",
           True: b"_Z19trace_shadow_kernel9SceneViewjP3RayP3Hit"}
STACK_ENTRIES = 64
BLOCK = 32


def available(build="stock"):
    return os.path.exists(os.path.join(REF_DIR, CUBINS[build])) and os.path.exists(LAYOUT)


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
        with open(LAYOUT) as f:
            self.layout = json.load(f)
        L = self.layout
        if (L["ray_size"], L["hit_size"], L["hit_id"], L["node_size"]) != (32, 16, 4, 32):
            raise RuntimeError("unexpected reference record sizes: %r" % L)
        for k in ("mesh_p", "mesh_n", "mesh_uv", "mesh_index"):
            if (L["tri_mesh"] + L[k]) % 8:
                raise RuntimeError("unaligned pointer field " + k)
        if L["triangle_size"] % 8 or L["sv_triangles"] % 8 or L["sv_bvh"] % 8 or L["sv_triangles_num"] % 4:
            raise RuntimeError("unexpected record alignment: %r" % L)
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
        for any_hit, name in KERNELS.items():
            f = ctypes.c_void_p()
            self.d.check(lib.cuModuleGetFunction(ctypes.byref(f), self.mod, name), "cuModuleGetFunction")
            self.fn[any_hit] = f

    def close(self):
        if self.mod:
            self.d.lib.cuModuleUnload(self.mod)
            self.mod = ctypes.c_void_p()
            self.d.lib.cuDevicePrimaryCtxRelease_v2(self.dev)

    def scene(self, ref_nodes, verts):
        return RefScene(self, ref_nodes, verts)

    def trace(self, scene, rays, hits, any_hit=False, stream=None):
        """Launches the reference kernel on device tensors: rays (m, 8) float32
        in the reference Ray layout, hits (m, 4) 32-bit (t, triangle id, u, v).
        Misses get id -1; their t, u, v are whatever the kernel leaves there."""
        import torch
        m = rays.shape[0]
        if m == 0:
            return
        if m >= 2 ** 32 - BLOCK:
            raise ValueError("too many rays")
        for t, name in ((rays, "rays"), (hits, "hits")):
            if not (t.is_cuda and t.is_contiguous() and t.element_size() == 4 and t.dim() == 2
                    and t.shape[1] == (8 if name == "rays" else 4)):
                raise ValueError(name + ": expected a contiguous (m, %d) 32-bit CUDA tensor" %
                                 (8 if name == "rays" else 4))
        if hits.shape[0] < m:
            raise ValueError("hits shorter than rays")
        if stream is None:
            stream = torch.cuda.current_stream().cuda_stream
        sv = (ctypes.c_uint8 * self.layout["scene_view_size"]).from_buffer_copy(scene.scene_view.tobytes())
        size = ctypes.c_uint32(m)
        rp = ctypes.c_uint64(rays.data_ptr())
        hp = ctypes.c_uint64(hits.data_ptr())
        params = (ctypes.c_void_p * 4)(ctypes.addressof(sv), ctypes.addressof(size), ctypes.addressof(rp),
                                       ctypes.addressof(hp))
        grid = (m + BLOCK - 1) // BLOCK
        self.d.check(self.d.lib.cuLaunchKernel(self.fn[bool(any_hit)], grid, 1, 1, BLOCK, 1, 1, 0,
                                               ctypes.c_void_p(stream), params, None), "cuLaunchKernel")

    def trace_host(self, scene, rays, any_hit=False):
        import torch
        r = torch.from_numpy(np.ascontiguousarray(rays, np.float32).reshape(-1, 8)).cuda()
        h = torch.zeros((r.shape[0], 4), dtype=torch.float32, device="cuda")
        self.trace(scene, r, h, any_hit)
        torch.cuda.synchronize()
        return h.cpu().numpy()


class RefScene:
    """Device copies of one triangle soup in the reference's records."""

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
        rec = np.zeros((n, L["triangle_size"]), np.uint8)
        r64 = rec.view(np.uint64)
        r32 = rec.view(np.uint32)
        r64[:, (L["tri_mesh"] + L["mesh_p"]) // 8] = self.p.data_ptr()
        r64[:, (L["tri_mesh"] + L["mesh_index"]) // 8] = self.index.data_ptr()
        r32[:, (L["tri_mesh"] + L["mesh_triangle_num"]) // 4] = n
        r32[:, L["tri_index"] // 4] = 3 * np.arange(n, dtype=np.uint32)
        self.triangles = torch.from_numpy(rec.reshape(-1)).to(dev)
        del rec
        sv = np.zeros(L["scene_view_size"], np.uint8)
        sv[L["sv_triangles"]:L["sv_triangles"] + 8].view(np.uint64)[0] = self.triangles.data_ptr()
        sv[L["sv_triangles_num"]:L["sv_triangles_num"] + 4].view(np.uint32)[0] = n
        sv[L["sv_bvh"]:L["sv_bvh"] + 8].view(np.uint64)[0] = self.nodes.data_ptr()
        self.scene_view = sv
        self.n = n
