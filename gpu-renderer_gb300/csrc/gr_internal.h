// Internal declarations shared by the host C++ and the CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "gr.h"

namespace gr {

// Device-side error word bits (kernels never trap; they set a bit and return).
enum : uint32_t {
    ERR_TIMEOUT = 1u << 0,   // a bounded spin gave up
    ERR_STACK = 1u << 1,     // traversal stack overflow
    ERR_QUEUE = 1u << 2,     // queue capacity exceeded
    ERR_RANGE = 1u << 3,     // an index out of range was seen and skipped
};

// Bounded spin limit for decoupled look-back waits (each iteration is an L2
// load, so this is far more than any predecessor tile can take).
constexpr uint32_t kSpinLimit = 1u << 22;

// Largest triangle count a BVH accepts: look-back words pack a 30-bit count.
constexpr uint32_t kMaxTriangles = (1u << 30) - 1;
// Largest image (width x height, counted in 64 bits): pixel indices and the
// 4-byte per-pixel arrays stay within 32-bit offsets.
constexpr uint64_t kMaxPixels = 0xFFFFFFFFull / 4;
inline bool pixels_ok(uint32_t width, uint32_t height) {
    return width != 0 && height != 0 && (uint64_t)width * height <= kMaxPixels;
}

// Traversal-node layout, 64 bytes (four 16-byte words):
//   q0 = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   q1 = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   q2 = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   q3 = (child0, child1, parent, 0) as int32; child < 0 is leaf ~p, where p
//        is the sorted position of a triangle in the leaf-order triangle array.
// Node index = the gap between sorted positions g and g+1 that the node splits.
struct Node {
    float4 q0, q1, q2;
    int4 q3;
};
static_assert(sizeof(Node) == 64, "node layout");

// 4-wide node with FP32 child boxes, 128 bytes: boxes in SoA order
// (lo.x[4], hi.x[4], lo.y[4], hi.y[4], lo.z[4], hi.z[4]), child references
// (same encoding as Node), and the valid-child mask in w[0].
struct Node4 {
    float4 lox, hix, loy, hiy, loz, hiz;
    int4 child;
    uint4 meta;  // x: child mask (bit k = slot k valid)
};
static_assert(sizeof(Node4) == 128, "node4 layout");

// 4-wide node with 8-bit quantised child boxes, 64 bytes. A child plane is
// origin + q * 2^e (one FMA), with q rounded outward so the decoded box
// contains the FP32 child box:
//   q0 = (origin.x, origin.y, origin.z, meta): meta bits 0-7 / 8-15 / 16-23 are
//        the biased exponents ex, ey, ez (e + 127), bits 24-27 the child mask
//   q1 = bytes qlo.x[4], qhi.x[4], qlo.y[4], qhi.y[4]
//   q2 = bytes qlo.z[4], qhi.z[4], 0, 0
//   q3 = child references
struct Node4Q {
    float4 q0;
    uint4 q1;
    uint4 q2;
    int4 child;
};
static_assert(sizeof(Node4Q) == 64, "node4q layout");

// 8-wide node with 8-bit quantised child boxes, 96 bytes (three 32-byte
// loads). Slots are assigned so that, for a ray whose direction has sign bits
// oct (bit a set = negative along axis a), visiting inner children in order of
// (slot ^ oct) is near to far. Inner children are stored contiguously from
// child_base in slot order, leaf triangles contiguously from tri_base (in the
// layout's own triangle array) in slot order.
//   meta:  bits 0-7 / 8-15 / 16-23 biased exponents (x, y, z), bits 24-31
//          inner-child mask (slot k holds an inner node)
//   valid: bits 0-7 slot k holds a child
//   q:     per axis two words of 8 bytes (byte k = slot k): lo.x, hi.x, lo.y,
//          hi.y, lo.z, hi.z; a plane decodes as fma(q, 2^e, origin)
struct Node8Q {
    float ox, oy, oz;
    uint32_t meta;
    uint32_t child_base;
    uint32_t tri_base;
    uint32_t valid;
    uint32_t pad0;
    uint32_t q[12];
    uint32_t pad1[4];
};
static_assert(sizeof(Node8Q) == 96, "node8q layout");

enum Layout : int { kLayoutBvh2 = 0, kLayoutBvh4 = 1, kLayoutBvh4Q8 = 2, kLayoutBvh8Q8 = 3 };
constexpr int kNumLayouts = 4;

// Traversal launch configuration chosen by the autotuner (or by the caller).
struct TraceTuning {
    int layout = kLayoutBvh2;
    int block = 128;   // threads per block: 64, 128 or 256
    int sstack = 12;   // stack entries per thread kept in shared memory: 8, 12 or 16
};
bool tuning_valid(const TraceTuning& t);

// Leaf-order triangle: three 16-byte words (v0, prim bits), (v1, 0), (v2, 0).
struct Tri {
    float4 a, b, c;
};
static_assert(sizeof(Tri) == 48, "triangle layout");

constexpr uint32_t kNoNode = 0xFFFFFFFFu;

// Device buffer owned by an object; grows on demand, never shrinks.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t want);
    void release();
    ~DevBuf() { release(); }
};

struct BvhMeta;

// What a traversal kernel needs; the root index is read on the device from the
// BVH header so no host synchronisation sits between build and trace.
struct BvhDevice {
    const Node* nodes;
    const Tri* tris;
    const BvhMeta* meta;  // meta->root is kNoNode when the BVH is empty
    uint32_t n;
};

// Build scratch + outputs, sliced from a few allocations.
struct BvhBuffers {
    DevBuf nodes, tris, code, prim;  // outputs kept for traversal / export
    DevBuf nodes4, nodes4q;          // 4-wide layouts (built on request), indexed like `nodes`
    DevBuf nodes8, tris8;            // 8-wide layout (built on request): nodes from 0 (root), leaf-order triangles
    uint32_t count8 = 0;             // 8-wide nodes
    uint32_t tris8_count = 0;        // triangles in tris8
    DevBuf scratch;                  // transient build state
    DevBuf meta;                     // small device header (root, error word, centroid bounds)
};

// Host-visible layout of the small per-BVH device header.
struct BvhMeta {
    uint32_t root;
    uint32_t pad0;
    uint32_t err;
    uint32_t pad;
    float cbox[6];  // centroid bounds used for the Morton codes
    float pad2[2];
};

// lbvh.cu
// Runs the build's bounded look-back wait on a status word nothing publishes,
// for `polls` polls (at most kSpinLimit); *h_err receives the error bits it set
// (ERR_TIMEOUT when the wait gave up, as it must).
cudaError_t lookback_probe(uint32_t polls, uint32_t* h_err, cudaStream_t s);
cudaError_t lbvh_build(BvhBuffers& b, const float* d_verts, uint32_t n, int num_sms, cudaStream_t s);
cudaError_t lbvh_export_ref(const BvhBuffers& b, uint32_t n, uint32_t* d_ref_nodes, cudaStream_t s);
// build whose scratch is a file-scope device array (no allocation); see lbvh.cu
uint32_t lbvh_static_max_triangles();
cudaError_t lbvh_build_static(const float* d_verts, uint32_t n, Node* nodes, Tri* tris, uint32_t* code,
                              uint32_t* prim, BvhMeta* meta, int device, int num_sms, cudaStream_t s);

// bvh4.cu: 4-wide layouts collapsed from the binary nodes (every node at
// even depth becomes a 4-wide node at the same index)
cudaError_t bvh4_build(BvhBuffers& b, uint32_t n, int layout, cudaStream_t s);
// bvh8.cu: level by level, one host read of the level size per level (waits for `s`)
// `scratch` holds the build's level state (about 144 bytes per triangle); it
// is the context's, kept between builds, and the caller holds its lock.
cudaError_t bvh8_build(BvhBuffers& b, uint32_t n, DevBuf& scratch, int num_sms, cudaStream_t s);

// trace.cu
cudaError_t trace_launch(const BvhDevice& bvh, const void* nodes, const TraceTuning& tune, const gr_ray* d_rays,
                         uint64_t n, gr_hit* d_hits, int any_hit, unsigned long long* d_counter, uint32_t* d_err,
                         int num_sms, cudaStream_t s);

}  // namespace gr

// Context and object definitions (host side).
// A context is freed when it has been destroyed and no object created from it
// is alive any more, so objects may outlive a gr_context_destroy call.
struct gr_ctx {
    int refs = 0;
    bool destroyed = false;
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;  // second stream of the pipelined host-memory traversal
    std::string last_error;
    // traversal work counters: offset 0 (gr_trace), 128 and 192 (the two streams
    // of gr_trace_host's pipeline); error word at offset 64
    gr::DevBuf counter;
    gr::DevBuf stage_in, stage_out;  // device staging for the host-memory entry points
    // 8-wide layout build state, reused by every BVH of the context (grown,
    // never shrunk, until the context is destroyed); the render server's
    // thread may build too, so it is taken under its lock
    gr::DevBuf scratch8;
    std::mutex scratch8_mu;
    uint32_t default_wave_paths = 0;     // wave size when neither a call nor its scene sets one (gr_opts)
    void* batch_pool = nullptr;          // wave pool of gr_render_batch (owned; freed with the context)
    void (*batch_pool_free)(void*) = nullptr;
};

namespace gr {
// reference counting of contexts by the objects created from them
void ctx_retain(gr_ctx* ctx);
void ctx_release(gr_ctx* ctx);
void context_free(gr_ctx* ctx);
}  // namespace gr

struct gr_bvh;
namespace gr {
// capi.cpp: the node and triangle arrays a layout's traversal reads.
const void* layout_nodes(const gr_bvh* bvh, int layout);
const Tri* layout_tris(const gr_bvh* bvh, int layout);
}  // namespace gr

struct gr_bvh {
    gr_ctx* ctx = nullptr;
    // not copyable: owns device memory
    uint32_t n = 0;
    bool built = false;
    int layout = 0;       // traversal layout gr_trace uses
    int block = 128;      // gr_trace launch shape (autotuned or set)
    int sstack = 12;
    bool built4 = false, built4q = false, built8 = false;
    gr::BvhBuffers buf;
};
