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
// collapsed (one thread each), their inner-child and leaf counts are prefix-
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
constexpr int kScanThreads = 1024;
constexpr int32_t kEmptySlot = INT32_MIN;
constexpr int kMaxLevels8 = 72;

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

// Exclusive scan of one 64-bit value per thread over a kBlock8-thread block.
__device__ unsigned long long block_exclusive(unsigned long long v, unsigned long long* block_total) {
    __shared__ unsigned long long s_warp[kBlock8 / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = lane < kBlock8 / 32 ? s_warp[lane] : 0ull;
#pragma unroll
        for (int d = 1; d < kBlock8 / 32; d <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, w, d);
            if (lane >= d) w += y;
        }
        if (lane < kBlock8 / 32) s_warp[lane] = w;
    }
    __syncthreads();
    const unsigned long long before = warp ? s_warp[warp - 1] : 0ull;
    if (block_total) *block_total = s_warp[kBlock8 / 32 - 1];
    return before + x - v;
}

__global__ void k8_init(const BvhMeta* __restrict__ meta, uint32_t* frontier) {
    if (threadIdx.x == 0 && blockIdx.x == 0) frontier[0] = meta->root;
}

// One thread per 8-wide node of the level: collapse, assign slots, quantise.
// Writes the node (without its bases), its 8 slot references and its counts
// (inner | leaf << 32); one partial sum per block.
__global__ void __launch_bounds__(kBlock8) k8_collapse(const Node* __restrict__ nodes,
                                                       const uint32_t* __restrict__ frontier, uint32_t level_n,
                                                       uint32_t out_base, Node8Q* __restrict__ out,
                                                       int32_t* __restrict__ slots, unsigned long long* __restrict__ cnt,
                                                       unsigned long long* __restrict__ bsum, uint32_t* err) {
    const uint32_t i = blockIdx.x * kBlock8 + threadIdx.x;
    unsigned long long c = 0;
    if (i < level_n) {
        const Node root = nodes[frontier[i]];
        CBox box[8];
        int32_t ref[8];
        int cnt8 = 2;
        ref[0] = root.q3.x;
        box[0] = child_box(root, 0);
        ref[1] = root.q3.y;
        box[1] = child_box(root, 1);
        while (cnt8 < 8) {
            int best = -1;
            float best_a = 0.0f;
            for (int k = 0; k < cnt8; ++k)
                if (ref[k] >= 0) {
                    const float a = half_area(box[k]);
                    if (best < 0 || a > best_a) {
                        best = k;
                        best_a = a;
                    }
                }
            if (best < 0) break;
            const Node cn = nodes[ref[best]];
            ref[best] = cn.q3.x;
            box[best] = child_box(cn, 0);
            ref[cnt8] = cn.q3.y;
            box[cnt8] = child_box(cn, 1);
            ++cnt8;
        }
        // node box and centre (sums lo + hi, the factor 1/2 cancels)
        float lo[3], hi[3], nc[3];
        for (int a = 0; a < 3; ++a) {
            lo[a] = box[0].lo[a];
            hi[a] = box[0].hi[a];
            for (int k = 1; k < cnt8; ++k) {
                lo[a] = fminf(lo[a], box[k].lo[a]);
                hi[a] = fmaxf(hi[a], box[k].hi[a]);
            }
            nc[a] = __fadd_rn(lo[a], hi[a]);
        }
        // greedy slot assignment: best (score, then lowest child, then lowest slot) first
        int slot_of[8];
        uint32_t used = 0;
        for (int k = 0; k < 8; ++k) slot_of[k] = -1;
        for (int it = 0; it < cnt8; ++it) {
            int bk = -1, bs = -1;
            float bsc = 0.0f;
            for (int k = 0; k < cnt8; ++k) {
                if (slot_of[k] >= 0) continue;
                const float dx = __fsub_rn(__fadd_rn(box[k].lo[0], box[k].hi[0]), nc[0]);
                const float dy = __fsub_rn(__fadd_rn(box[k].lo[1], box[k].hi[1]), nc[1]);
                const float dz = __fsub_rn(__fadd_rn(box[k].lo[2], box[k].hi[2]), nc[2]);
                for (int s = 0; s < 8; ++s) {
                    if (used & (1u << s)) continue;
                    const float sc = __fadd_rn(__fadd_rn((s & 1) ? dx : -dx, (s & 2) ? dy : -dy), (s & 4) ? dz : -dz);
                    if (bk < 0 || sc > bsc) {
                        bk = k;
                        bs = s;
                        bsc = sc;
                    }
                }
            }
            slot_of[bk] = bs;
            used |= 1u << bs;
        }
        // quantise
        float scale[3];
        uint32_t be[3];
        for (int a = 0; a < 3; ++a) {
            const int e = pick_exponent8(lo[a], hi[a], err);
            be[a] = (uint32_t)(e + 127);
            scale[a] = __uint_as_float(be[a] << 23);
        }
        Node8Q o;
        o.ox = lo[0];
        o.oy = lo[1];
        o.oz = lo[2];
        for (int w = 0; w < 12; ++w) o.q[w] = 0;
        uint32_t imask = 0;
        int32_t sref[8];
        for (int s = 0; s < 8; ++s) sref[s] = kEmptySlot;
        uint32_t n_inner = 0, n_leaf = 0;
        for (int k = 0; k < cnt8; ++k) {
            const int s = slot_of[k];
            sref[s] = ref[k];
            if (ref[k] >= 0) {
                imask |= 1u << s;
                ++n_inner;
            } else {
                ++n_leaf;
            }
            for (int a = 0; a < 3; ++a) {
                o.q[4 * a + (s >> 2)] |= quant_lo8(box[k].lo[a], scale[a], lo[a]) << (8 * (s & 3));
                o.q[4 * a + 2 + (s >> 2)] |= quant_hi8(box[k].hi[a], scale[a], lo[a]) << (8 * (s & 3));
            }
        }
        o.meta = be[0] | (be[1] << 8) | (be[2] << 16) | (imask << 24);
        o.child_base = 0;
        o.tri_base = 0;
        o.valid = used;
        o.pad0 = 0;
        for (int w = 0; w < 4; ++w) o.pad1[w] = 0;
        out[out_base + i] = o;
        for (int s = 0; s < 8; ++s) slots[8ull * i + s] = sref[s];
        c = (unsigned long long)n_inner | ((unsigned long long)n_leaf << 32);
        cnt[i] = c;
    }
    unsigned long long total;
    block_exclusive(c, &total);
    if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

// Exclusive scan of the block sums in place (one block); level totals to *total.
__global__ void __launch_bounds__(kScanThreads) k8_scan_blocks(unsigned long long* bsum, uint32_t nblocks,
                                                               unsigned long long* total) {
    __shared__ unsigned long long s_part[kScanThreads];
    const uint32_t per = (nblocks + kScanThreads - 1) / kScanThreads;
    const uint32_t b0 = threadIdx.x * per, b1 = min(nblocks, b0 + per);
    unsigned long long sum = 0;
    for (uint32_t b = b0; b < b1; ++b) sum += bsum[b];
    s_part[threadIdx.x] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long run = 0;
        for (int t = 0; t < kScanThreads; ++t) {
            const unsigned long long v = s_part[t];
            s_part[t] = run;
            run += v;
        }
        *total = run;
    }
    __syncthreads();
    unsigned long long run = s_part[threadIdx.x];
    for (uint32_t b = b0; b < b1; ++b) {
        const unsigned long long v = bsum[b];
        bsum[b] = run;
        run += v;
    }
}

// Writes each node's bases, the next level's binary ids (inner children in
// slot order) and the leaf triangles (in slot order) into the layout's
// triangle array.
__global__ void __launch_bounds__(kBlock8) k8_emit(uint32_t level_n, uint32_t out_base, uint32_t next_base,
                                                   uint32_t tri_cursor, Node8Q* __restrict__ out,
                                                   const int32_t* __restrict__ slots,
                                                   const unsigned long long* __restrict__ cnt,
                                                   const unsigned long long* __restrict__ bsum,
                                                   uint32_t* __restrict__ next_frontier, const Tri* __restrict__ tris,
                                                   Tri* __restrict__ tris8) {
    const uint32_t i = blockIdx.x * kBlock8 + threadIdx.x;
    const unsigned long long c = i < level_n ? cnt[i] : 0ull;
    const unsigned long long pre = block_exclusive(c, nullptr) + bsum[blockIdx.x];
    if (i >= level_n) return;
    const uint32_t inner0 = (uint32_t)pre, leaf0 = (uint32_t)(pre >> 32);
    out[out_base + i].child_base = next_base + inner0;
    out[out_base + i].tri_base = tri_cursor + leaf0;
    uint32_t ri = 0, rl = 0;
    for (int s = 0; s < 8; ++s) {
        const int32_t r = slots[8ull * i + s];
        if (r == kEmptySlot) continue;
        if (r >= 0) {
            next_frontier[inner0 + ri++] = (uint32_t)r;
        } else {
            tris8[tri_cursor + leaf0 + rl++] = tris[(uint32_t)(~r)];
        }
    }
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

cudaError_t bvh8_build(BvhBuffers& b, uint32_t n, cudaStream_t s) {
    b.count8 = 0;
    b.tris8_count = 0;
    if (n == 0) return cudaSuccess;
    const size_t maxnodes = n > 1 ? n - 1 : 1;
    const size_t maxtris = std::max<size_t>(n, 2);  // a lone triangle fills both children of its node
    const size_t maxblocks = (maxnodes + kBlock8 - 1) / kBlock8;
    // scratch: two frontiers, slot refs, counts, block sums, totals, and the nodes before compaction
    size_t off = 0;
    const size_t o_f0 = off; off += align256(4 * maxnodes);
    const size_t o_f1 = off; off += align256(4 * maxnodes);
    const size_t o_sl = off; off += align256(32 * maxnodes);
    const size_t o_cn = off; off += align256(8 * maxnodes);
    const size_t o_bs = off; off += align256(8 * maxblocks);
    const size_t o_tt = off; off += align256(16);
    const size_t o_nd = off; off += align256(sizeof(Node8Q) * maxnodes);
    cudaError_t e;
    if ((e = b.scratch8.ensure(off)) != cudaSuccess) return e;
    if ((e = b.tris8.ensure(sizeof(Tri) * maxtris)) != cudaSuccess) return e;
    char* base = (char*)b.scratch8.p;
    uint32_t* frontier[2] = {(uint32_t*)(base + o_f0), (uint32_t*)(base + o_f1)};
    int32_t* slots = (int32_t*)(base + o_sl);
    unsigned long long* cnt = (unsigned long long*)(base + o_cn);
    unsigned long long* bsum = (unsigned long long*)(base + o_bs);
    unsigned long long* total = (unsigned long long*)(base + o_tt);
    Node8Q* staged = (Node8Q*)(base + o_nd);
    k8_init<<<1, 32, 0, s>>>((const BvhMeta*)b.meta.p, frontier[0]);
    uint32_t level_n = 1, out_base = 0, tri_cursor = 0;
    int cur = 0;
    for (int level = 0; level_n > 0; ++level) {
        if (level >= kMaxLevels8 || out_base + (size_t)level_n > maxnodes) return cudaErrorInvalidValue;
        const uint32_t nb = (level_n + kBlock8 - 1) / kBlock8;
        k8_collapse<<<nb, kBlock8, 0, s>>>((const Node*)b.nodes.p, frontier[cur], level_n, out_base, staged, slots, cnt,
                                           bsum, &((BvhMeta*)b.meta.p)->err);
        k8_scan_blocks<<<1, kScanThreads, 0, s>>>(bsum, nb, total);
        k8_emit<<<nb, kBlock8, 0, s>>>(level_n, out_base, out_base + level_n, tri_cursor, staged, slots, cnt, bsum,
                                       frontier[cur ^ 1], (const Tri*)b.tris.p, (Tri*)b.tris8.p);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        unsigned long long h[1];
        if ((e = cudaMemcpyAsync(h, total, sizeof(h), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
        out_base += level_n;
        tri_cursor += (uint32_t)(h[0] >> 32);
        level_n = (uint32_t)h[0];
        cur ^= 1;
        if (tri_cursor > maxtris) return cudaErrorInvalidValue;
    }
    if ((e = b.nodes8.ensure(sizeof(Node8Q) * out_base)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(b.nodes8.p, staged, sizeof(Node8Q) * out_base, cudaMemcpyDeviceToDevice, s)) !=
        cudaSuccess)
        return e;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    b.scratch8.release();
    b.count8 = out_base;
    b.tris8_count = tri_cursor;
    return cudaSuccess;
}

}  // namespace gr
