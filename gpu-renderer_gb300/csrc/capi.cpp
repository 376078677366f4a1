// C ABI: context, BVH and traversal entry points (include/gr.h).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "gr_internal.h"
#include "render.h"

namespace gr {

cudaError_t DevBuf::ensure(size_t want) {
    if (want <= bytes && p) return cudaSuccess;
    release();
    cudaError_t e = cudaMalloc(&p, want ? want : 256);
    if (e != cudaSuccess) {
        p = nullptr;
        bytes = 0;
        return e;
    }
    bytes = want;
    return cudaSuccess;
}

void DevBuf::release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

void context_free(gr_ctx* ctx) {
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->batch_pool && ctx->batch_pool_free) ctx->batch_pool_free(ctx->batch_pool);
    ctx->batch_pool = nullptr;
    ctx->counter.release();
    ctx->scratch8.release();
    ctx->stage_in.release();
    ctx->stage_out.release();
    if (ctx->stream2) cudaStreamSynchronize(ctx->stream2);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->stream2) cudaStreamDestroy(ctx->stream2);
    delete ctx;
}

void ctx_retain(gr_ctx* ctx) { ++ctx->refs; }

void ctx_release(gr_ctx* ctx) {
    if (--ctx->refs == 0 && ctx->destroyed) context_free(ctx);
}

}  // namespace gr

namespace {

gr_status fail(gr_ctx* ctx, gr_status st, const char* what) {
    if (ctx) ctx->last_error = what;
    return st;
}

gr_status cuda_fail(gr_ctx* ctx, cudaError_t e, const char* where) {
    cudaGetLastError();  // clear a sticky launch error so the context stays usable
    if (ctx) {
        ctx->last_error = std::string(where) + ": " + cudaGetErrorString(e);
    }
    return e == cudaErrorMemoryAllocation ? GR_ERR_OOM_BUDGET : GR_ERR_CUDA;
}

#define GR_CUDA(ctx, call)                                   \
    do {                                                     \
        cudaError_t e__ = (call);                            \
        if (e__ != cudaSuccess) return cuda_fail(ctx, e__, #call); \
    } while (0)

cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

gr_status check_device_errors(gr_bvh* bvh, uint32_t err) {
    if (err & gr::ERR_TIMEOUT) return fail(bvh->ctx, GR_ERR_TIMEOUT, "device wait timed out");
    if (err & gr::ERR_STACK) return fail(bvh->ctx, GR_ERR_OVERFLOW, "traversal stack overflow");
    if (err & gr::ERR_QUEUE) return fail(bvh->ctx, GR_ERR_OVERFLOW, "queue capacity exceeded");
    if (err & gr::ERR_RANGE) return fail(bvh->ctx, GR_ERR_INVALID, "out-of-range index skipped on device");
    return GR_OK;
}

gr::BvhDevice device_view(gr_bvh* bvh) {
    gr::BvhDevice v;
    v.nodes = (const gr::Node*)bvh->buf.nodes.p;
    v.tris = (const gr::Tri*)bvh->buf.tris.p;
    v.meta = (const gr::BvhMeta*)bvh->buf.meta.p;
    v.n = bvh->n;
    return v;
}

// Builds the derived node layout `layout` if it is not current (binary nodes
// are always built). The 8-wide build waits for `s`.
cudaError_t ensure_layout(gr_bvh* bvh, int layout, cudaStream_t s) {
    if (!bvh->built || layout == gr::kLayoutBvh2) return cudaSuccess;
    if (layout == gr::kLayoutBvh8Q8) {
        if (bvh->built8) return cudaSuccess;
        std::lock_guard<std::mutex> lock(bvh->ctx->scratch8_mu);
        const cudaError_t e = gr::bvh8_build(bvh->buf, bvh->n, bvh->ctx->scratch8, bvh->ctx->num_sms, s);
        if (e == cudaSuccess) bvh->built8 = true;
        return e;
    }
    bool& done = layout == gr::kLayoutBvh4 ? bvh->built4 : bvh->built4q;
    if (done) return cudaSuccess;
    const cudaError_t e = gr::bvh4_build(bvh->buf, bvh->n, layout, s);
    if (e == cudaSuccess) done = true;
    return e;
}

}  // namespace

namespace gr {

const void* layout_nodes(const gr_bvh* bvh, int layout) {
    switch (layout) {
        case kLayoutBvh4: return bvh->buf.nodes4.p;
        case kLayoutBvh4Q8: return bvh->buf.nodes4q.p;
        case kLayoutBvh8Q8: return bvh->buf.nodes8.p;
        default: return bvh->buf.nodes.p;
    }
}

const Tri* layout_tris(const gr_bvh* bvh, int layout) {
    return (const Tri*)(layout == kLayoutBvh8Q8 ? bvh->buf.tris8.p : bvh->buf.tris.p);
}

}  // namespace gr

namespace {

gr_status read_meta(gr_bvh* bvh, gr::BvhMeta* m) {
    GR_CUDA(bvh->ctx, cudaMemcpy(m, bvh->buf.meta.p, sizeof(gr::BvhMeta), cudaMemcpyDeviceToHost));
    return GR_OK;
}

}  // namespace

extern "C" {

int gr_version(void) { return 100; }

const char* gr_status_string(int st) {
    switch (st) {
        case GR_OK: return "ok";
        case GR_ERR_INVALID: return "invalid argument";
        case GR_ERR_CUDA: return "CUDA error";
        case GR_ERR_OOM_BUDGET: return "out of memory or over budget";
        case GR_ERR_PARSE: return "parse error";
        case GR_ERR_TIMEOUT: return "device wait timed out";
        case GR_ERR_OVERFLOW: return "device capacity exceeded";
        case GR_ERR_IO: return "file could not be written";
        case GR_ERR_BUSY: return "server busy: job refused";
        default: return "unknown status";
    }
}

gr_status gr_context_create(int device, const gr_opts* opts, gr_ctx** out) {
    if (!out) return GR_ERR_INVALID;
    *out = nullptr;
    if (opts && opts->flags != 0) return GR_ERR_INVALID;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
        cudaGetLastError();
        return GR_ERR_CUDA;
    }
    gr_ctx* ctx = new (std::nothrow) gr_ctx();
    if (!ctx) return GR_ERR_OOM_BUDGET;
    ctx->device = device;
    ctx->default_wave_paths = opts && opts->default_wave_paths ? opts->default_wave_paths : gr::kDefaultWavePaths;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = ctx->counter.ensure(256);
    if (e == cudaSuccess) e = cudaMemset(ctx->counter.p, 0, 256);
    if (e != cudaSuccess) {
        cudaGetLastError();
        delete ctx;
        return GR_ERR_CUDA;
    }
    *out = ctx;
    return GR_OK;
}

gr_status gr_context_destroy(gr_ctx* ctx) {
    if (!ctx || ctx->destroyed) return GR_ERR_INVALID;
    ctx->destroyed = true;
    if (ctx->refs == 0) gr::context_free(ctx);
    return GR_OK;
}

const char* gr_last_error(const gr_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "no context"; }

gr_status gr_bvh_create(gr_ctx* ctx, gr_bvh** out) {
    if (!ctx || !out) return GR_ERR_INVALID;
    gr_bvh* b = new (std::nothrow) gr_bvh();
    if (!b) return fail(ctx, GR_ERR_OOM_BUDGET, "host allocation failed");
    b->ctx = ctx;
    gr::ctx_retain(ctx);
    *out = b;
    return GR_OK;
}

gr_status gr_bvh_destroy(gr_bvh* bvh) {
    if (!bvh) return GR_ERR_INVALID;
    gr_ctx* ctx = bvh->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    delete bvh;
    gr::ctx_release(ctx);
    return GR_OK;
}

uint32_t gr_bvh_size(const gr_bvh* bvh) { return bvh ? bvh->n : 0; }

gr_status gr_bvh_build(gr_bvh* bvh, const float* d_verts, uint32_t n, void* stream) {
    if (!bvh) return GR_ERR_INVALID;
    if (n > gr::kMaxTriangles) return fail(bvh->ctx, GR_ERR_INVALID, "too many triangles");
    if (n > 0 && !d_verts) return fail(bvh->ctx, GR_ERR_INVALID, "null vertex pointer");
    GR_CUDA(bvh->ctx, cudaSetDevice(bvh->ctx->device));
    bvh->built = false;
    bvh->built4 = bvh->built4q = bvh->built8 = false;
    GR_CUDA(bvh->ctx, gr::lbvh_build(bvh->buf, d_verts, n, bvh->ctx->num_sms, as_stream(stream)));
    bvh->n = n;
    bvh->built = true;
    // keep the requested traversal layout current
    GR_CUDA(bvh->ctx, ensure_layout(bvh, bvh->layout, as_stream(stream)));
    return GR_OK;
}

gr_status gr_bvh_build_host(gr_bvh* bvh, const float* h_verts, uint32_t n) {
    if (!bvh) return GR_ERR_INVALID;
    if (n > 0 && !h_verts) return fail(bvh->ctx, GR_ERR_INVALID, "null vertex pointer");
    GR_CUDA(bvh->ctx, cudaSetDevice(bvh->ctx->device));
    cudaStream_t s = bvh->ctx->stream;
    gr::DevBuf& staging = bvh->ctx->stage_in;
    GR_CUDA(bvh->ctx, staging.ensure(36ull * (n ? n : 1)));
    if (n) GR_CUDA(bvh->ctx, cudaMemcpyAsync(staging.p, h_verts, 36ull * n, cudaMemcpyHostToDevice, s));
    gr_status st = gr_bvh_build(bvh, (const float*)staging.p, n, s);
    if (st != GR_OK) return st;
    GR_CUDA(bvh->ctx, cudaStreamSynchronize(s));
    gr::BvhMeta m;
    st = read_meta(bvh, &m);
    if (st != GR_OK) return st;
    return check_device_errors(bvh, m.err);
}

gr_status gr_bvh_export(gr_bvh* bvh, uint32_t* h_sorted_prim, uint32_t* h_sorted_code, uint32_t* h_ref_nodes,
                        uint32_t* h_nodes, float* h_tris, uint32_t* h_root) {
    if (!bvh || !bvh->built) return GR_ERR_INVALID;
    GR_CUDA(bvh->ctx, cudaSetDevice(bvh->ctx->device));
    GR_CUDA(bvh->ctx, cudaDeviceSynchronize());
    gr::BvhMeta m;
    gr_status st = read_meta(bvh, &m);
    if (st != GR_OK) return st;
    st = check_device_errors(bvh, m.err);
    if (st != GR_OK) return st;
    const uint32_t n = bvh->n;
    if (h_root) *h_root = m.root;
    if (n == 0) return GR_OK;
    if (h_sorted_prim) GR_CUDA(bvh->ctx, cudaMemcpy(h_sorted_prim, bvh->buf.prim.p, 4ull * n, cudaMemcpyDeviceToHost));
    if (h_sorted_code) GR_CUDA(bvh->ctx, cudaMemcpy(h_sorted_code, bvh->buf.code.p, 4ull * n, cudaMemcpyDeviceToHost));
    if (h_nodes)
        GR_CUDA(bvh->ctx, cudaMemcpy(h_nodes, bvh->buf.nodes.p, sizeof(gr::Node) * (n > 1 ? n - 1 : 1),
                                     cudaMemcpyDeviceToHost));
    if (h_tris) GR_CUDA(bvh->ctx, cudaMemcpy(h_tris, bvh->buf.tris.p, sizeof(gr::Tri) * n, cudaMemcpyDeviceToHost));
    if (h_ref_nodes) {
        gr::DevBuf out;
        const size_t bytes = 32ull * (2ull * n - 1);
        GR_CUDA(bvh->ctx, out.ensure(bytes));
        GR_CUDA(bvh->ctx, gr::lbvh_export_ref(bvh->buf, n, (uint32_t*)out.p, bvh->ctx->stream));
        GR_CUDA(bvh->ctx, cudaMemcpyAsync(h_ref_nodes, out.p, bytes, cudaMemcpyDeviceToHost, bvh->ctx->stream));
        GR_CUDA(bvh->ctx, cudaStreamSynchronize(bvh->ctx->stream));
    }
    return GR_OK;
}

}  // extern "C"

namespace {

// One traversal launch with the work counter at `counter_offset` of the
// context's counter buffer.
gr_status trace_on(gr_bvh* bvh, const gr_ray* d_rays, uint64_t n, gr_hit* d_hits, int any_hit, cudaStream_t s,
                   size_t counter_offset) {
    gr_ctx* ctx = bvh->ctx;
    unsigned long long* counter = (unsigned long long*)((char*)ctx->counter.p + counter_offset);
    uint32_t* err = (uint32_t*)((char*)ctx->counter.p + 64);
    gr::TraceTuning tune;
    tune.layout = bvh->layout;
    tune.block = bvh->block;
    tune.sstack = bvh->sstack;
    gr::BvhDevice view = device_view(bvh);
    view.tris = gr::layout_tris(bvh, bvh->layout);
    GR_CUDA(ctx, gr::trace_launch(view, gr::layout_nodes(bvh, bvh->layout), tune, d_rays, n, d_hits, any_hit, counter,
                                  err, ctx->num_sms, s));
    return GR_OK;
}

}  // namespace

extern "C" {

gr_status gr_trace(gr_bvh* bvh, const gr_ray* d_rays, uint64_t n, gr_hit* d_hits, int any_hit, void* stream) {
    if (!bvh || !bvh->built) return GR_ERR_INVALID;
    if (n > 0 && (!d_rays || !d_hits)) return fail(bvh->ctx, GR_ERR_INVALID, "null ray or hit pointer");
    GR_CUDA(bvh->ctx, cudaSetDevice(bvh->ctx->device));
    return trace_on(bvh, d_rays, n, d_hits, any_hit, as_stream(stream), 0);
}

// Host-memory traversal. When both buffers are page-locked host memory the
// device can address (cudaHostGetDevicePointer succeeds), one traversal reads
// the rays and writes the hits there directly: on NVLink-C2C systems the
// transfers ride inside the kernel at no measurable cost (4 Mi rays: 1,064
// Mrays/s against 1,069 for device buffers). Otherwise the rays are cut into
// chunks of at least 1 Mi rays (at most 8); chunk k goes to one of two streams
// (k & 1) as copy-in, traversal, copy-out, so one chunk's copies overlap
// another chunk's traversal; each stream has its own work counter.
gr_status gr_trace_host(gr_bvh* bvh, const gr_ray* h_rays, uint64_t n, gr_hit* h_hits, int any_hit) {
    if (!bvh || !bvh->built) return GR_ERR_INVALID;
    if (n > 0 && (!h_rays || !h_hits)) return fail(bvh->ctx, GR_ERR_INVALID, "null ray or hit pointer");
    gr_ctx* ctx = bvh->ctx;
    GR_CUDA(ctx, cudaSetDevice(ctx->device));
    if (n == 0) return GR_OK;
    void* mapped_rays = nullptr;
    void* mapped_hits = nullptr;
    if (cudaHostGetDevicePointer(&mapped_rays, (void*)h_rays, 0) == cudaSuccess &&
        cudaHostGetDevicePointer(&mapped_hits, (void*)h_hits, 0) == cudaSuccess) {
        const gr_status st =
            trace_on(bvh, (const gr_ray*)mapped_rays, n, (gr_hit*)mapped_hits, any_hit, ctx->stream, 128);
        if (st != GR_OK) return st;
        GR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        uint32_t err = 0;
        GR_CUDA(ctx, cudaMemcpy(&err, (char*)ctx->counter.p + 64, 4, cudaMemcpyDeviceToHost));
        return check_device_errors(bvh, err);
    }
    cudaGetLastError();  // not page-locked: clear the lookup's error and stage through device memory
    gr::DevBuf& dr = ctx->stage_in;
    gr::DevBuf& dh = ctx->stage_out;
    GR_CUDA(ctx, dr.ensure(sizeof(gr_ray) * n));
    GR_CUDA(ctx, dh.ensure(sizeof(gr_hit) * n));
    const uint64_t chunk = std::max<uint64_t>(1ull << 20, (n + 7) / 8);
    cudaStream_t st[2] = {ctx->stream, ctx->stream2};
    const size_t counter_at[2] = {128, 192};
    // both streams start after any work already queued on the context stream
    cudaEvent_t start;
    GR_CUDA(ctx, cudaEventCreateWithFlags(&start, cudaEventDisableTiming));
    gr_status status = GR_OK;
    cudaError_t e = cudaEventRecord(start, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->stream2, start, 0);
    for (uint64_t off = 0, k = 0; e == cudaSuccess && status == GR_OK && off < n; off += chunk, ++k) {
        const uint64_t m = std::min(chunk, n - off);
        cudaStream_t s = st[k & 1];
        gr_ray* r = (gr_ray*)dr.p + off;
        gr_hit* h = (gr_hit*)dh.p + off;
        e = cudaMemcpyAsync(r, h_rays + off, sizeof(gr_ray) * m, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) status = trace_on(bvh, r, m, h, any_hit, s, counter_at[k & 1]);
        if (e == cudaSuccess && status == GR_OK)
            e = cudaMemcpyAsync(h_hits + off, h, sizeof(gr_hit) * m, cudaMemcpyDeviceToHost, s);
    }
    const cudaError_t e1 = cudaStreamSynchronize(ctx->stream2);
    const cudaError_t e0 = cudaStreamSynchronize(ctx->stream);
    cudaEventDestroy(start);
    if (status != GR_OK) return status;
    GR_CUDA(ctx, e);
    GR_CUDA(ctx, e1);
    GR_CUDA(ctx, e0);
    uint32_t err = 0;
    GR_CUDA(ctx, cudaMemcpy(&err, (char*)ctx->counter.p + 64, 4, cudaMemcpyDeviceToHost));
    return check_device_errors(bvh, err);
}

}  // extern "C"

extern "C" gr_status gr_bvh_build_noalloc(gr_ctx* ctx, const float* d_verts, uint32_t n, void* d_nodes, void* d_tris,
                                          uint32_t* d_sorted_prim, uint32_t* d_sorted_code, void* d_header,
                                          void* stream) {
    if (!ctx) return GR_ERR_INVALID;
    const uint32_t limit = gr::lbvh_static_max_triangles();
    if (n > limit) {
        ctx->last_error = "gr_bvh_build_noalloc: " + std::to_string(n) +
                          " triangles exceed the fixed scratch limit of " + std::to_string(limit) +
                          "; use gr_bvh_build";
        return GR_ERR_INVALID;
    }
    if (!d_header || (n > 0 && (!d_verts || !d_nodes || !d_tris || !d_sorted_prim || !d_sorted_code))) {
        ctx->last_error = "gr_bvh_build_noalloc: null pointer";
        return GR_ERR_INVALID;
    }
    GR_CUDA(ctx, cudaSetDevice(ctx->device));
    GR_CUDA(ctx, gr::lbvh_build_static(d_verts, n, (gr::Node*)d_nodes, (gr::Tri*)d_tris, d_sorted_code, d_sorted_prim,
                                       (gr::BvhMeta*)d_header, ctx->device, ctx->num_sms, as_stream(stream)));
    return GR_OK;
}

extern "C" gr_status gr_diag_bounded_wait(gr_ctx* ctx, uint32_t polls, uint32_t* err_bits) {
    if (!ctx) return GR_ERR_INVALID;
    GR_CUDA(ctx, cudaSetDevice(ctx->device));
    uint32_t bits = 0;
    GR_CUDA(ctx, gr::lookback_probe(polls, &bits, ctx->stream));
    if (err_bits) *err_bits = bits;
    if (bits & gr::ERR_TIMEOUT) return fail(ctx, GR_ERR_TIMEOUT, "gr_diag_bounded_wait: the wait gave up");
    return GR_OK;
}

extern "C" gr_status gr_bvh_set_layout(gr_bvh* bvh, int layout, void* stream) {
    if (!bvh || layout < 0 || layout >= gr::kNumLayouts) return GR_ERR_INVALID;
    GR_CUDA(bvh->ctx, cudaSetDevice(bvh->ctx->device));
    GR_CUDA(bvh->ctx, ensure_layout(bvh, layout, as_stream(stream)));
    bvh->layout = layout;
    return GR_OK;
}

extern "C" gr_status gr_bvh_layout_size(gr_bvh* bvh, int layout, uint64_t* node_bytes, uint64_t* tri_bytes) {
    if (!bvh || !bvh->built || layout < 0 || layout >= gr::kNumLayouts) return GR_ERR_INVALID;
    GR_CUDA(bvh->ctx, cudaSetDevice(bvh->ctx->device));
    GR_CUDA(bvh->ctx, ensure_layout(bvh, layout, bvh->ctx->stream));
    const uint64_t count = bvh->n == 0 ? 0 : (bvh->n > 1 ? bvh->n - 1 : 1);
    uint64_t nb = 0, tb = sizeof(gr::Tri) * (uint64_t)bvh->n;
    switch (layout) {
        case gr::kLayoutBvh4: nb = count * sizeof(gr::Node4); break;
        case gr::kLayoutBvh4Q8: nb = count * sizeof(gr::Node4Q); break;
        case gr::kLayoutBvh8Q8:
            nb = (uint64_t)bvh->buf.count8 * sizeof(gr::Node8Q);
            tb = (uint64_t)bvh->buf.tris8_count * sizeof(gr::Tri);
            break;
        default: nb = count * sizeof(gr::Node); break;
    }
    if (node_bytes) *node_bytes = nb;
    if (tri_bytes) *tri_bytes = tb;
    return GR_OK;
}

extern "C" gr_status gr_bvh_export_layout(gr_bvh* bvh, int layout, void* h_nodes) {
    if (!bvh || !bvh->built || layout < 1 || layout >= gr::kNumLayouts || !h_nodes) return GR_ERR_INVALID;
    uint64_t nb = 0;
    gr_status st = gr_bvh_layout_size(bvh, layout, &nb, nullptr);
    if (st != GR_OK) return st;
    GR_CUDA(bvh->ctx, cudaStreamSynchronize(bvh->ctx->stream));
    GR_CUDA(bvh->ctx, cudaDeviceSynchronize());
    if (nb) GR_CUDA(bvh->ctx, cudaMemcpy(h_nodes, gr::layout_nodes(bvh, layout), nb, cudaMemcpyDeviceToHost));
    return GR_OK;
}

extern "C" gr_status gr_bvh_export_layout_tris(gr_bvh* bvh, int layout, float* h_tris) {
    if (!bvh || !bvh->built || layout < 0 || layout >= gr::kNumLayouts || !h_tris) return GR_ERR_INVALID;
    uint64_t tb = 0;
    gr_status st = gr_bvh_layout_size(bvh, layout, nullptr, &tb);
    if (st != GR_OK) return st;
    GR_CUDA(bvh->ctx, cudaStreamSynchronize(bvh->ctx->stream));
    GR_CUDA(bvh->ctx, cudaDeviceSynchronize());
    if (tb) GR_CUDA(bvh->ctx, cudaMemcpy(h_tris, gr::layout_tris(bvh, layout), tb, cudaMemcpyDeviceToHost));
    return GR_OK;
}

extern "C" gr_status gr_bvh_set_tuning(gr_bvh* bvh, const gr_trace_tuning* t) {
    if (!bvh || !t) return GR_ERR_INVALID;
    gr::TraceTuning tt;
    tt.layout = t->layout;
    tt.block = t->block;
    tt.sstack = t->short_stack;
    if (!gr::tuning_valid(tt)) return fail(bvh->ctx, GR_ERR_INVALID, "gr_bvh_set_tuning: unsupported configuration");
    gr_status st = gr_bvh_set_layout(bvh, t->layout, bvh->ctx->stream);
    if (st != GR_OK) return st;
    bvh->block = t->block;
    bvh->sstack = t->short_stack;
    return GR_OK;
}

extern "C" gr_status gr_bvh_get_tuning(const gr_bvh* bvh, gr_trace_tuning* t) {
    if (!bvh || !t) return GR_ERR_INVALID;
    t->layout = bvh->layout;
    t->block = bvh->block;
    t->short_stack = bvh->sstack;
    return GR_OK;
}

extern "C" gr_status gr_bvh_autotune(gr_bvh* bvh, const gr_ray* d_rays, uint64_t n, int any_hit, gr_hit* d_hits,
                                     gr_tuning_result* h_table, uint32_t max_results, uint32_t* n_results) {
    if (!bvh || !bvh->built || !d_rays || !d_hits || n == 0) return GR_ERR_INVALID;
    gr_ctx* ctx = bvh->ctx;
    GR_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    cudaEvent_t e0, e1;
    GR_CUDA(ctx, cudaEventCreate(&e0));
    GR_CUDA(ctx, cudaEventCreate(&e1));
    const int layouts[] = {0, 1, 2, 3}, blocks[] = {64, 128, 256}, stacks[] = {8, 12, 16};
    gr_trace_tuning best{bvh->layout, bvh->block, bvh->sstack};
    float best_ms = 1e30f;
    uint32_t rows = 0;
    gr_status st = GR_OK;
    for (int lay : layouts) {
        if ((st = gr_bvh_set_layout(bvh, lay, s)) != GR_OK) break;
        for (int blk : blocks)
            for (int ss : stacks) {
                bvh->block = blk;
                bvh->sstack = ss;
                float ms = 0.0f;
                // one warm-up launch, then the faster of two timed launches
                float m = 1e30f;
                for (int rep = 0; rep < 3 && st == GR_OK; ++rep) {
                    cudaEventRecord(e0, s);
                    st = gr_trace(bvh, d_rays, n, d_hits, any_hit, s);
                    cudaEventRecord(e1, s);
                    cudaEventSynchronize(e1);
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (rep > 0) m = std::min(m, ms);
                }
                if (st != GR_OK) break;
                if (h_table && rows < max_results) {
                    h_table[rows].tuning = gr_trace_tuning{lay, blk, ss};
                    h_table[rows].ms = m;
                }
                ++rows;
                if (m < best_ms) {
                    best_ms = m;
                    best = gr_trace_tuning{lay, blk, ss};
                }
            }
        if (st != GR_OK) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (n_results) *n_results = rows;
    if (st != GR_OK) return st;
    return gr_bvh_set_tuning(bvh, &best);
}
