// Test and bench infrastructure: the reference's frame driver,
// PathTracer::render(uint32*) (pathtracer.cu:41-150), restated in C++ over the
// CUDA driver API so that the reference's own kernels — compiled from its
// sources into a cubin and loaded by ref_gpu.py — render frames on the GPU with
// the reference's launch shapes and its host synchronisation: every kernel is
// followed by a device synchronise and every queue size is read back with a
// blocking copy, as the reference does (pathtracer.cu:75-145). The product
// never loads this library.
//
// The kernel argument records (PTContext, SceneView, FrameBufferView) arrive as
// bytes laid out by ref_gpu.py from the reference headers' layout; this file
// only swaps the queue records between bounces and patches the two counters.
#include <dlfcn.h>

#include <chrono>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

typedef int CUresult;
typedef unsigned long long CUdeviceptr;
typedef CUresult (*LaunchFn)(void*, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, void*,
                             void**, void**);
typedef CUresult (*DtoHFn)(void*, CUdeviceptr, size_t);
typedef CUresult (*MemsetFn)(CUdeviceptr, unsigned, size_t);
typedef CUresult (*SyncFn)();

struct Driver {
    LaunchFn launch = nullptr;
    DtoHFn dtoh = nullptr;
    MemsetFn memset32 = nullptr;
    SyncFn sync = nullptr;
    bool ok = false;
    Driver() {
        void* h = dlopen("libcuda.so.1", RTLD_NOW | RTLD_GLOBAL);
        if (!h) return;
        launch = (LaunchFn)dlsym(h, "cuLaunchKernel");
        dtoh = (DtoHFn)dlsym(h, "cuMemcpyDtoH_v2");
        memset32 = (MemsetFn)dlsym(h, "cuMemsetD32_v2");
        sync = (SyncFn)dlsym(h, "cuCtxSynchronize");
        ok = launch && dtoh && memset32 && sync;
    }
};

Driver& drv() {
    static Driver d;
    return d;
}

uint32_t div_up(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

uint64_t read_u64(const uint8_t* p) {
    uint64_t v;
    std::memcpy(&v, p, 8);
    return v;
}

}  // namespace

extern "C" {

// Offsets the driver needs, from the reference layout (in bytes):
// ctx: [0] PTContext size, [1] m_bounce, [2] m_sample_num, [3] m_in_queue,
//      [4] m_shadow_queue, [5] m_scatter_queue, [6] RayQueue size,
//      [7] RayQueue::m_rays, [8] RayQueue::m_hits, [9] RayQueue::m_size.
// fns: generate_primary_rays_kernel, trace_kernel, shade_hit_with_MIS_kernel,
//      trace_shadow_kernel, accumulate_light_sampling_contribution_kernel,
//      accumulate_BSDF_sampling_contribution_kernel, finish_sample_kernel.
// Renders `frames` frames starting at sample number first_sample; returns 0 on
// success, else the first failing CUresult (or -1 without a driver). seconds:
// wall time of the frames; rays: the rays traced (camera, shadow and scatter).
int ref_render_frames(void* const* fns, const uint8_t* scene_view, uint32_t scene_view_size,
                      const uint8_t* fb_view, uint32_t fb_view_size, const uint8_t* context_in,
                      const uint32_t* ctx, uint32_t width, uint32_t height, uint32_t frames, uint32_t first_sample,
                      uint32_t max_path_length, double* seconds, uint64_t* rays) {
    Driver& d = drv();
    if (!d.ok) return -1;
    const uint32_t ctx_size = ctx[0], off_bounce = ctx[1], off_sample = ctx[2], off_in = ctx[3],
                   off_scatter = ctx[5], q_size = ctx[6], q_rays = ctx[7], q_hits = ctx[8], q_count = ctx[9];
    const uint32_t off_shadow = ctx[4];
    std::vector<uint8_t> sv(scene_view, scene_view + scene_view_size);
    std::vector<uint8_t> fb(fb_view, fb_view + fb_view_size);
    std::vector<uint8_t> c(context_in, context_in + ctx_size);
    std::vector<uint8_t> tmp(q_size);
    const uint32_t pixels = width * height;
    uint64_t ray_count = 0;

#define CK(x)                          \
    do {                               \
        const CUresult r__ = (x);      \
        if (r__ != 0) return (int)r__; \
    } while (0)

    auto queue_count = [&](uint32_t off_queue, uint32_t* n) -> CUresult {
        return d.dtoh(n, (CUdeviceptr)read_u64(&c[off_queue + q_count]), 4);
    };
    auto trace = [&](void* fn, uint32_t off_queue, uint32_t n) -> CUresult {
        if (n == 0) return 0;  // trace() returns at once for an empty queue (pathtracer_kernel.h:237-240)
        CUdeviceptr r = (CUdeviceptr)read_u64(&c[off_queue + q_rays]);
        CUdeviceptr h = (CUdeviceptr)read_u64(&c[off_queue + q_hits]);
        void* args[] = {sv.data(), &n, &r, &h};
        CUresult e = d.launch(fn, div_up(n, 32), 1, 1, 32, 1, 1, 0, nullptr, args, nullptr);
        return e ? e : d.sync();
    };
    auto stage = [&](void* fn, uint32_t n) -> CUresult {
        // shade_hit / accumulate_*: 32-thread blocks over the queue
        // (pathtracer_kernel.h:630-640, 666-682, 751-767); the accumulate
        // wrappers return at once for an empty queue, and shade_hit is only
        // reached with a non-empty one
        if (n == 0) return 0;
        void* args[] = {&n, c.data(), sv.data(), fb.data()};
        CUresult e = d.launch(fn, div_up(n, 32), 1, 1, 32, 1, 1, 0, nullptr, args, nullptr);
        return e ? e : d.sync();
    };

    const auto t0 = std::chrono::steady_clock::now();
    for (uint32_t f = 0; f < frames; ++f) {
        const uint32_t bounce0 = 0, sample = first_sample + f;
        std::memcpy(&c[off_bounce], &bounce0, 4);
        std::memcpy(&c[off_sample], &sample, 4);
        // generate_primary_rays: 32x32 blocks over the image (pathtracer_kernel.h:106-117)
        {
            void* args[] = {c.data(), sv.data(), fb.data()};
            CK(d.launch(fns[0], div_up(width, 32), div_up(height, 32), 1, 32, 32, 1, 0, nullptr, args, nullptr));
            CK(d.sync());
        }
        uint32_t n_in = 0;
        CK(queue_count(off_in, &n_in));
        ray_count += n_in;
        CK(trace(fns[1], off_in, n_in));
        for (uint32_t b = 0; b < max_path_length; ++b) {
            std::memcpy(&c[off_bounce], &b, 4);
            CK(queue_count(off_in, &n_in));
            if (n_in == 0) break;
            CK(d.memset32((CUdeviceptr)read_u64(&c[off_scatter + q_count]), 0, 1));
            CK(d.memset32((CUdeviceptr)read_u64(&c[off_shadow + q_count]), 0, 1));
            CK(stage(fns[2], n_in));
            uint32_t n_shadow = 0;
            CK(queue_count(off_shadow, &n_shadow));
            ray_count += n_shadow;
            CK(trace(fns[3], off_shadow, n_shadow));
            CK(stage(fns[4], n_shadow));
            uint32_t n_scatter = 0;
            CK(queue_count(off_scatter, &n_scatter));
            ray_count += n_scatter;
            CK(trace(fns[1], off_scatter, n_scatter));
            CK(stage(fns[5], n_scatter));
            // std::swap(m_scatter_queue, m_in_queue) (pathtracer.cu:141)
            std::memcpy(tmp.data(), &c[off_in], q_size);
            std::memcpy(&c[off_in], &c[off_scatter], q_size);
            std::memcpy(&c[off_scatter], tmp.data(), q_size);
        }
        // finish_sample: 32-thread blocks over the pixels (pathtracer_kernel.h:782-790)
        {
            uint32_t n = pixels;
            void* args[] = {&n, fb.data()};
            CK(d.launch(fns[6], div_up(n, 32), 1, 1, 32, 1, 1, 0, nullptr, args, nullptr));
            CK(d.sync());
        }
        // each frame starts from the queues as allocated (pathtracer.cu:55-72)
        std::memcpy(c.data(), context_in, ctx_size);
    }
    const auto t1 = std::chrono::steady_clock::now();
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    if (rays) *rays = ray_count;
    return 0;
#undef CK
}

}  // extern "C"
