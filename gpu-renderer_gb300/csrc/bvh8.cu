// 8-wide BVH with 8-bit quantised child boxes (Node8Q), collapsed from the
// binary LBVH level by level.
//
// Each 8-wide node starts from one binary node's two children and repeatedly
// opens the inner child with the largest surface area, until it has 8
// children or only leaves (the greedy collapse of wide-BVH builders). Its
// children are then assigned to slots by position: slot bit a means "on the
// high side along axis a", chosen greedily by the score
// sum_a (+/-)(child centre - node centre)_a, so that a ray visiting inner
// children in order of (slot ^ octant) goes roughly near to far. Boxes are
// quantised outward against the exact planes q * 2^e + lo (lo the node's
// lower corner), whose ray distances the traversal measures with one FMA per
// plane.
//
// Nodes are numbered breadth first, level by level: a level's nodes are
// collapsed (eight lanes each), their inner-child and leaf counts are prefix-
// summed, and the children become the next level at consecutive indices, so
// a node's inner children are contiguous from child_base and its leaf
// triangles contiguous from tri_base (copied into the layout's own triangle
// array). The numbering is deterministic; the host reads one level size per
// level.
#include <algorithm>

#include "gr_internal.h"
#include "quant.cuh"

namespace gr {
namespace {

using namespace q8;

constexpr int kBlock8 = 256;
constexpr int kLanesPerNode = 8;            // lanes collapsing one 8-wide node
constexpr int kNodesPerCollapseBlock = 32;  // nodes per collapse block: one emit warp
constexpr int kCollapseThreads = kNodesPerCollapseBlock * kLanesPerNode;
constexpr int kScanThreads = 1024;
constexpr int32_t kEmptySlot = INT32_MIN;
constexpr int kMaxLevels8 = 72;
constexpr int kLevelsPerSync = 4;        // levels launched per host read-back of the level state
constexpr int kCollapseBlocksPerSm = 5;  // grid of the collapse (its loop covers any level size)
constexpr int kEmitBlocksPerSm = 4;

// 8-wide planes: plane(q) = q * 2^e + lo, taken EXACTLY (the traversal
// measures it as fma(q, 2^e / d, (lo - o) / d) with error margins, never
// rounding the plane itself); e grows until plane(255) >= hi. q * 2^e is a
// float, so each comparison of a plane with a coordinate is decided exactly
// from the rounded sum and its two-sum error.
constexpr int kMaxExp8 = 119;  // 255 * 2^e stays finite

__device__ __forceinline__ float pow2f(int e) { return __uint_as_float((uint32_t)(e + 127) << 23); }

// Sign of (a + b) - v, exactly: -1, 0 or +1.
__device__ __forceinline__ int cmp_sum(float a, float b, float v) {
    const float s = __fadd_rn(a, b);
    if (s != v) return s < v ? -1 : 1;
    const float bp = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
    return e < 0.0f ? -1 : (e > 0.0f ? 1 : 0);
}

__device__ __forceinline__ int cmp_plane(int q, float scale, float lo, float v) {
    return cmp_sum(__fmul_rn((float)q, scale), lo, v);
}

__device__ __forceinline__ int pick_exponent8(float lo, float hi, uint32_t* err) {
    const float extent = __fsub_rn(hi, lo);
    int e = -126;
    if (extent > 0.0f) {
        int ex;
        frexpf(__fdiv_rn(extent, 255.0f), &ex);
        e = max(-126, min(kMaxExp8, ex - 1));
    }
    while (cmp_plane(255, pow2f(e), lo, hi) < 0) {
        if (e >= kMaxExp8) {
            atomicOr(err, ERR_RANGE);  // extent beyond about 2^127: not representable
            break;
        }
        ++e;
    }
    return e;
}

__device__ __forceinline__ uint32_t quant_lo8(float v, float scale, float lo) {
    int q = 0;
    for (int step = 128; step > 0; step >>= 1)  // largest q with plane(q) <= v (plane(0) = lo <= v)
        if (q + step <= 255 && cmp_plane(q + step, scale, lo, v) <= 0) q += step;
    return (uint32_t)q;
}

__device__ __forceinline__ uint32_t quant_hi8(float v, float scale, float lo) {
    int q = 255;
    for (int step = 128; step > 0; step >>= 1)  // smallest q with plane(q) >= v (plane(255) >= v)
        if (q - step >= 0 && cmp_plane(q - step, scale, lo, v) >= 0) q -= step;
    return (uint32_t)q;
}

__device__ __forceinline__ float half_area(const CBox& b) {
    const float dx = __fsub_rn(b.hi[0], b.lo[0]);
    const float dy = __fsub_rn(b.hi[1], b.lo[1]);
    const float dz = __fsub_rn(b.hi[2], b.lo[2]);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dy), __fmul_rn(dy, dz)), __fmul_rn(dz, dx));
}

// One level of the build as the device sees it: its node count, where its
// nodes start in the output, where its leaf triangles start, and whether a
// capacity was exceeded (the build then stops with no more writes). Level l's
// scan writes level l + 1's state, so the host launches levels without reading
// their sizes back.
struct Level8 {
    uint32_t n, out_base, tri_cursor, overflow;
};

__global__ void k8_init(const BvhMeta* __restrict__ meta, uint32_t* frontier, Level8* level,
                        unsigned long long* bsum) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        frontier[0] = meta->root;
        level[0] = Level8{1u, 0u, 0u, 0u};
        bsum[0] = 0ull;
    }
}

__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// Order-preserving 32-bit key of a float (larger float, larger key); -0 and +0
// share one key, as they compare equal.
__device__ __forceinline__ uint32_t order_key(float x) {
    const uint32_t b = __float_as_uint(x == 0.0f ? 0.0f : x);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// Eight lanes per 8-wide node, four nodes per warp: lane k of a group holds
// candidate child k. Every choice is made exactly as one thread scanning the
// candidates in order would make it (first largest on ties), so the node does
// not depend on the lanes' arithmetic order. Loops run the same number of
// times in every group, so each shuffle has the whole warp. Writes the node
// (without its bases) and its 8 slot references when `have`; returns the
// counts (inner | leaf << 32).
__device__ unsigned long long collapse_group(const Node* __restrict__ nodes, bool have, uint32_t root_id,
                                             Node8Q* __restrict__ out, int32_t* __restrict__ sref_out, uint32_t* err) {
    constexpr uint32_t kAll = 0xFFFFFFFFu;
    constexpr int W = kLanesPerNode;
    const int k = threadIdx.x & (W - 1);
    int32_t ref = kEmptySlot;
    CBox box = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};
    int cnt8 = 0;
    if (have) {
        const Node root = nodes[root_id];
        box = child_box(root, k & 1);
        if (k < 2) ref = k ? root.q3.y : root.q3.x;
        cnt8 = 2;
    }
    // an inner candidate's node is fetched towards L2 as soon as it becomes a
    // candidate, so opening it later waits on L2 rather than DRAM
    if (ref >= 0) prefetch_l2(nodes + ref);
    // open the inner candidate with the largest surface area (at most 6 times)
    for (int step = 0; step < 6; ++step) {
        const float area = half_area(box);
        int best = -1;
        float best_a = 0.0f;
        for (int j = 0; j < W; ++j) {
            const float aj = __shfl_sync(kAll, area, j, W);
            const int32_t rj = __shfl_sync(kAll, ref, j, W);
            if (j < cnt8 && rj >= 0 && (best < 0 || aj > best_a)) {
                best = j;
                best_a = aj;
            }
        }
        const int32_t rb = __shfl_sync(kAll, ref, best < 0 ? 0 : best, W);
        if (best >= 0 && cnt8 < 8) {
            const Node cn = nodes[rb];
            if (k == best) {
                ref = cn.q3.x;
                box = child_box(cn, 0);
            }
            if (k == cnt8) {
                ref = cn.q3.y;
                box = child_box(cn, 1);
            }
            if ((k == best || k == cnt8) && ref >= 0) prefetch_l2(nodes + ref);
            ++cnt8;
        }
    }
    // node box (folded in candidate order) and centre (lo + hi)
    float lo[3], hi[3], nc[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        lo[a] = __shfl_sync(kAll, box.lo[a], 0, W);
        hi[a] = __shfl_sync(kAll, box.hi[a], 0, W);
    }
#pragma unroll
    for (int j = 1; j < W; ++j) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float l = __shfl_sync(kAll, box.lo[a], j, W), h = __shfl_sync(kAll, box.hi[a], j, W);
            if (j < cnt8) {
                lo[a] = fminf(lo[a], l);
                hi[a] = fmaxf(hi[a], h);
            }
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) nc[a] = __fadd_rn(lo[a], hi[a]);
    // this lane's child scored against every slot
    const float dx = __fsub_rn(__fadd_rn(box.lo[0], box.hi[0]), nc[0]);
    const float dy = __fsub_rn(__fadd_rn(box.lo[1], box.hi[1]), nc[1]);
    const float dz = __fsub_rn(__fadd_rn(box.lo[2], box.hi[2]), nc[2]);
    float sc[8];
    bool nan_score = false;
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        sc[s] = __fadd_rn(__fadd_rn((s & 1) ? dx : -dx, (s & 2) ? dy : -dy), (s & 4) ? dz : -dz);
        nan_score |= isnan(sc[s]);
    }
    const bool slow = __any_sync(kAll, k < cnt8 && nan_score);
    // greedy assignment: the best (score, then lowest child, then lowest slot) first
    uint32_t used = 0;
    bool taken = false;
    int my_slot = -1;
    for (int it = 0; it < 8; ++it) {
        int win = -1;
        if (!slow) {
            // this lane's first largest free slot, then the group's largest
            // score with the lowest pair 8 k + s on ties (-0 and +0 tie)
            const bool cand = k < cnt8 && !taken;
            int bs = -1;
            float bsc = 0.0f;
#pragma unroll
            for (int s = 0; s < 8; ++s)
                if (cand && !(used >> s & 1u) && (bs < 0 || sc[s] > bsc)) {
                    bs = s;
                    bsc = sc[s];
                }
            uint32_t key = bs >= 0 ? order_key(bsc) : 0u;
            int p = bs >= 0 ? 8 * k + bs : 0xFF;
#pragma unroll
            for (int d = 1; d < W; d <<= 1) {
                const uint32_t ok = __shfl_xor_sync(kAll, key, d, W);
                const int op = __shfl_xor_sync(kAll, p, d, W);
                if (ok > key || (ok == key && op < p)) {
                    key = ok;
                    p = op;
                }
            }
            win = p;
        } else {
            // a NaN score in the warp: fold the group's pairs in order, as one thread would
            float wsc = 0.0f;
            for (int j = 0; j < W; ++j) {
                const bool tj = __shfl_sync(kAll, (int)taken, j, W) != 0;
#pragma unroll
                for (int s = 0; s < 8; ++s) {
                    const float x = __shfl_sync(kAll, sc[s], j, W);
                    if (j < cnt8 && !tj && !(used >> s & 1u) && (win < 0 || x > wsc)) {
                        win = 8 * j + s;
                        wsc = x;
                    }
                }
            }
        }
        if (it < cnt8) {
            if (win < 0 || win >= 64) {  // no free pair: cannot happen while it < cnt8 <= 8
                if (k == 0) atomicOr(err, ERR_RANGE);
            } else {
                used |= 1u << (win & 7);
                if (k == (win >> 3)) {
                    taken = true;
                    my_slot = win & 7;
                }
            }
        }
    }
    // quantise: per-axis exponents (lanes 0-2), then this lane's child's six planes
    uint32_t my_be = 0;
    if (have && k < 3) my_be = (uint32_t)(pick_exponent8(k == 0 ? lo[0] : (k == 1 ? lo[1] : lo[2]),
                                                         k == 0 ? hi[0] : (k == 1 ? hi[1] : hi[2]), err) + 127);
    uint32_t be[3];
    float scale[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        be[a] = __shfl_sync(kAll, my_be, a, W);
        scale[a] = __uint_as_float(be[a] << 23);
    }
    uint32_t wq[12];
#pragma unroll
    for (int w = 0; w < 12; ++w) wq[w] = 0;
    if (k < cnt8 && my_slot >= 0) {
        const int sh = 8 * (my_slot & 3), half = my_slot >> 2;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const uint32_t ql = quant_lo8(box.lo[a], scale[a], lo[a]) << sh;
            const uint32_t qh = quant_hi8(box.hi[a], scale[a], lo[a]) << sh;
            wq[4 * a + 0] = half ? 0u : ql;
            wq[4 * a + 1] = half ? ql : 0u;
            wq[4 * a + 2] = half ? 0u : qh;
            wq[4 * a + 3] = half ? qh : 0u;
        }
    }
    uint32_t imask = (k < cnt8 && ref >= 0 && my_slot >= 0) ? 1u << my_slot : 0u;
#pragma unroll
    for (int d = 1; d < W; d <<= 1) {
        imask |= __shfl_xor_sync(kAll, imask, d, W);
#pragma unroll
        for (int w = 0; w < 12; ++w) wq[w] |= __shfl_xor_sync(kAll, wq[w], d, W);
    }
    if (!have) return 0ull;
    // the node's 24 words: lane k writes words k, k + 8 and k + 16
    uint32_t w0 = 0, w1 = 0, w2 = 0;
    if (k < 3) w0 = __float_as_uint(k == 0 ? lo[0] : (k == 1 ? lo[1] : lo[2]));
    if (k == 3) w0 = be[0] | (be[1] << 8) | (be[2] << 16) | (imask << 24);
    if (k == 6) w0 = used;
#pragma unroll
    for (int w = 0; w < 8; ++w) {
        if (k == w) w1 = wq[w];
        if (k == w && w < 4) w2 = wq[8 + w];
    }
    uint32_t* o = reinterpret_cast<uint32_t*>(out);
    o[k] = w0;
    o[k + 8] = w1;
    o[k + 16] = w2;
    // slot references: each child at its slot, empty slots marked
    if (k < cnt8 && my_slot >= 0) sref_out[my_slot] = ref;
    if (!(used >> k & 1u)) sref_out[k] = kEmptySlot;
    const uint32_t n_inner = __popc(imask);
    return (unsigned long long)n_inner | ((unsigned long long)(cnt8 - n_inner) << 32);
}

// The level's nodes, eight lanes each (four per warp), over a grid of any
// size; each node's counts go to cnt[i] and are added into the sum of its
// 32-node tile (bsum, zeroed by the previous level's scan).
__global__ void __launch_bounds__(kCollapseThreads) k8_collapse(const Node* __restrict__ nodes,
                                                              const uint32_t* __restrict__ frontier,
                                                              const Level8* __restrict__ level,
                                                              Node8Q* __restrict__ out, int32_t* __restrict__ slots,
                                                              unsigned long long* __restrict__ cnt,
                                                              unsigned long long* __restrict__ bsum, uint32_t* err) {
    const Level8 L = *level;
    constexpr uint32_t kPerWarp = 32 / kLanesPerNode;
    const uint32_t warps = gridDim.x * (kCollapseThreads / 32);
    const uint32_t g = (threadIdx.x & 31) / kLanesPerNode;
    for (uint32_t w = blockIdx.x * (kCollapseThreads / 32) + threadIdx.x / 32; (uint64_t)w * kPerWarp < L.n;
         w += warps) {  // the same trip count for the whole warp
        const uint32_t i = w * kPerWarp + g;
        const bool have = i < L.n;
        const unsigned long long c =
            collapse_group(nodes, have, have ? frontier[i] : 0u, out + L.out_base + i, slots + 8ull * i, err);
        if (have && (threadIdx.x & (kLanesPerNode - 1)) == 0) {
            cnt[i] = c;
            atomicAdd(&bsum[i / kNodesPerCollapseBlock], c);
        }
    }
}

// Exclusive scan of the level's tile sums in place (one block); writes the
// next level's state and zeroes the next level's tile sums.
__global__ void __launch_bounds__(kScanThreads) k8_scan_blocks(unsigned long long* bsum, const Level8* level,
                                                               Level8* next, unsigned long long* next_bsum,
                                                               uint32_t max_nodes, uint32_t max_tris) {
    __shared__ unsigned long long s_warp[32];
    __shared__ uint32_t s_next_tiles;
    const Level8 L = *level;
    const uint32_t nblocks = (L.n + kNodesPerCollapseBlock - 1) / kNodesPerCollapseBlock;
    const uint32_t per = (nblocks + kScanThreads - 1) / kScanThreads;
    const uint32_t b0 = threadIdx.x * per, b1 = min(nblocks, b0 + per);
    unsigned long long sum = 0;
    for (uint32_t b = b0; b < b1; ++b) sum += bsum[b];
    // exclusive scan of the threads' sums: within each warp, then over the warp totals
    static_assert(kScanThreads == 1024, "32 warps of 32");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long x = sum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = s_warp[lane];
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, w, d);
            if (lane >= d) w += y;
        }
        s_warp[lane] = w;
    }
    __syncthreads();
    unsigned long long run = (warp ? s_warp[warp - 1] : 0ull) + x - sum;
    for (uint32_t b = b0; b < b1; ++b) {
        const unsigned long long v = bsum[b];
        bsum[b] = run;
        run += v;
    }
    if (threadIdx.x == 0) {
        const unsigned long long total = s_warp[31];
        Level8 nx;
        nx.n = (uint32_t)total;
        nx.out_base = L.out_base + L.n;
        nx.tri_cursor = L.tri_cursor + (uint32_t)(total >> 32);
        nx.overflow = L.overflow;
        if ((uint64_t)nx.out_base + nx.n > max_nodes || nx.tri_cursor > max_tris) {
            nx.overflow = 1u;
            nx.n = 0u;
        }
        *next = nx;
        s_next_tiles = (nx.n + kNodesPerCollapseBlock - 1) / kNodesPerCollapseBlock;
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < s_next_tiles; b += kScanThreads) next_bsum[b] = 0ull;
}

// Writes each node's bases, the next level's binary ids (inner children in
// slot order) and the leaf triangles (in slot order) into the layout's
// triangle array. A node's offsets are its tile's exclusive count sum plus the
// counts of the nodes before it in the tile, whose 32 nodes are one warp here
// (a warp scan). Nothing is written once a capacity was exceeded.
__global__ void __launch_bounds__(kBlock8) k8_emit(const Level8* __restrict__ level, const Level8* __restrict__ next,
                                                   Node8Q* __restrict__ out, const int32_t* __restrict__ slots,
                                                   const unsigned long long* __restrict__ cnt,
                                                   const unsigned long long* __restrict__ bsum,
                                                   uint32_t* __restrict__ next_frontier, const Tri* __restrict__ tris,
                                                   Tri* __restrict__ tris8) {
    static_assert(kNodesPerCollapseBlock == 32, "a tile's nodes are one emit warp");
    const Level8 L = *level;
    if (next->overflow) return;
    const uint32_t next_base = L.out_base + L.n;
    const int lane = threadIdx.x & 31;
    for (uint32_t base = blockIdx.x * kBlock8; base < L.n; base += gridDim.x * kBlock8) {  // block-uniform
        const uint32_t i = base + threadIdx.x;
        const unsigned long long c = i < L.n ? cnt[i] : 0ull;
        unsigned long long x = c;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, x, d);
            if (lane >= d) x += y;
        }
        if (i >= L.n) continue;
        const unsigned long long pre = bsum[i / kNodesPerCollapseBlock] + (x - c);
        const uint32_t inner0 = (uint32_t)pre, leaf0 = (uint32_t)(pre >> 32);
        out[L.out_base + i].child_base = next_base + inner0;
        out[L.out_base + i].tri_base = L.tri_cursor + leaf0;
        uint32_t ri = 0, rl = 0;
        for (int s = 0; s < 8; ++s) {
            const int32_t r = slots[8ull * i + s];
            if (r == kEmptySlot) continue;
            if (r >= 0) {
                next_frontier[inner0 + ri++] = (uint32_t)r;
            } else {
                tris8[L.tri_cursor + leaf0 + rl++] = tris[(uint32_t)(~r)];
            }
        }
    }
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

cudaError_t bvh8_build(BvhBuffers& b, uint32_t n, DevBuf& scratch, int num_sms, cudaStream_t s) {
    b.count8 = 0;
    b.tris8_count = 0;
    if (n == 0) return cudaSuccess;
    const size_t maxnodes = n > 1 ? n - 1 : 1;
    const size_t maxtris = std::max<size_t>(n, 2);  // a lone triangle fills both children of its node
    const size_t maxtiles = (maxnodes + kNodesPerCollapseBlock - 1) / kNodesPerCollapseBlock;
    // scratch: two frontiers, slot refs, counts, two sets of tile sums, the
    // level states, and the nodes before compaction
    size_t off = 0;
    const size_t o_f0 = off; off += align256(4 * maxnodes);
    const size_t o_f1 = off; off += align256(4 * maxnodes);
    const size_t o_sl = off; off += align256(32 * maxnodes);
    const size_t o_cn = off; off += align256(8 * maxnodes);
    const size_t o_b0 = off; off += align256(8 * maxtiles);
    const size_t o_b1 = off; off += align256(8 * maxtiles);
    const size_t o_lv = off; off += align256(sizeof(Level8) * (kMaxLevels8 + 1));
    const size_t o_nd = off; off += align256(sizeof(Node8Q) * maxnodes);
    cudaError_t e;
    if ((e = scratch.ensure(off)) != cudaSuccess) return e;
    if ((e = b.tris8.ensure(sizeof(Tri) * maxtris)) != cudaSuccess) return e;
    char* base = (char*)scratch.p;
    uint32_t* frontier[2] = {(uint32_t*)(base + o_f0), (uint32_t*)(base + o_f1)};
    int32_t* slots = (int32_t*)(base + o_sl);
    unsigned long long* cnt = (unsigned long long*)(base + o_cn);
    unsigned long long* tile_sums[2] = {(unsigned long long*)(base + o_b0), (unsigned long long*)(base + o_b1)};
    Level8* level_state = (Level8*)(base + o_lv);
    Node8Q* staged = (Node8Q*)(base + o_nd);
    const Node* nodes = (const Node*)b.nodes.p;
    uint32_t* err = &((BvhMeta*)b.meta.p)->err;
    const int sms = std::max(1, num_sms);
    k8_init<<<1, 32, 0, s>>>((const BvhMeta*)b.meta.p, frontier[0], level_state, tile_sums[0]);
    // levels are launched kLevelsPerSync at a time; the host reads the state
    // after each batch and stops at the first empty level (launches past it do
    // nothing)
    Level8 h{};
    int level = 0;
    for (;;) {
        for (int j = 0; j < kLevelsPerSync && level < kMaxLevels8; ++j, ++level) {
            const int c = level & 1;
            k8_collapse<<<sms * kCollapseBlocksPerSm, kCollapseThreads, 0, s>>>(
                nodes, frontier[c], level_state + level, staged, slots, cnt, tile_sums[c], err);
            k8_scan_blocks<<<1, kScanThreads, 0, s>>>(tile_sums[c], level_state + level, level_state + level + 1,
                                                      tile_sums[c ^ 1], (uint32_t)maxnodes, (uint32_t)maxtris);
            k8_emit<<<sms * kEmitBlocksPerSm, kBlock8, 0, s>>>(level_state + level, level_state + level + 1, staged,
                                                              slots, cnt, tile_sums[c], frontier[c ^ 1],
                                                              (const Tri*)b.tris.p, (Tri*)b.tris8.p);
        }
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(&h, level_state + level, sizeof(h), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
            return e;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
        if (h.overflow) return cudaErrorInvalidValue;
        if (h.n == 0) break;
        if (level >= kMaxLevels8) return cudaErrorInvalidValue;
    }
    const uint32_t out_base = h.out_base, tri_cursor = h.tri_cursor;
    if ((e = b.nodes8.ensure(sizeof(Node8Q) * out_base)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(b.nodes8.p, staged, sizeof(Node8Q) * out_base, cudaMemcpyDeviceToDevice, s)) !=
        cudaSuccess)
        return e;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    b.count8 = out_base;
    b.tris8_count = tri_cursor;
    return cudaSuccess;
}

}  // namespace gr
