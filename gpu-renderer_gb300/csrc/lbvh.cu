// GPU LBVH build: Morton codes -> LSD radix sort -> the split level of
// each gap between sorted codes (the radix tree's over unique codes, midpoint
// subtrees inside runs of equal codes) -> one bottom-up pass that links the
// nodes and fits their boxes. Produces the same tree as the reference's host
// LBVH_build (src/renderer/bvh.h:186-221) with ties kept in input order.
//
// Every float operation that feeds a Morton code is written with an explicit
// round-to-nearest intrinsic so nvcc cannot contract it into an FMA: the codes
// must equal the reference host computation (bvh.h:193-204) bit for bit.
#include <algorithm>
#include <mutex>

#include <cuda.h>  // CUcontext / CUresult: the driver entry points are reached through the runtime

#include "gr_internal.h"

namespace gr {
namespace {

constexpr int kBlock = 256;
// sorted positions (and gaps) per block in the bottom-up pass's first part: one per thread
constexpr int kRefitChunk = 256;

// ---- small device helpers ---------------------------------------------------

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

struct Box3 {
    float lo[3], hi[3];
};

__device__ __forceinline__ Box3 tri_box(const float* __restrict__ v, uint64_t i) {
    const float* p = v + 9ull * i;
    float a[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) a[k] = __ldg(p + k);
    Box3 b;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        b.lo[k] = fminf(fminf(a[k], a[3 + k]), a[6 + k]);
        b.hi[k] = fmaxf(fmaxf(a[k], a[3 + k]), a[6 + k]);
    }
    return b;
}

// Standard 10-bit spread: bit i moves to bit 3i.
__device__ __forceinline__ uint32_t spread10(uint32_t x) {
    x &= 0x3FFu;
    x = (x | (x << 16)) & 0x030000FFu;
    x = (x | (x << 8)) & 0x0300F00Fu;
    x = (x | (x << 4)) & 0x030C30C3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

// Block-wide exclusive scan of one value per thread (blockDim.x <= 1024);
// `s_warp` holds THREADS / 32 values.
template <int THREADS, class T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* s_warp, T* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        constexpr int W = THREADS / 32;
        T w = lane < W ? s_warp[lane] : T(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < W) s_warp[lane] = w;  // inclusive warp totals
    }
    __syncthreads();
    T base = warp > 0 ? s_warp[warp - 1] : T(0);
    *total = s_warp[THREADS / 32 - 1];
    __syncthreads();
    return base + x - v;
}

// ---- 1. centroid bounds -------------------------------------------------------

// Min / max of the six bound values over the block (lo in 0-2, hi in 3-5);
// threads 0-5 return them.
__device__ __forceinline__ float block_bounds(float lo[3], float hi[3]) {
    __shared__ float s[6][kBlock / 32];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xFFFFFFFFu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xFFFFFFFFu, hi[k], o));
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        for (int k = 0; k < 3; ++k) { s[k][warp] = lo[k]; s[3 + k][warp] = hi[k]; }
    }
    __syncthreads();
    float r = 0.0f;
    if (threadIdx.x < 6) {
        const int k = threadIdx.x;
        r = s[k][0];
        for (int w = 1; w < kBlock / 32; ++w) r = k < 3 ? fminf(r, s[k][w]) : fmaxf(r, s[k][w]);
    }
    return r;
}

// Centroid bounds: each block reduces its share of the triangles to a partial
// box; the last block to finish (counted on `done`) folds the partials into
// the header (min / max do not depend on the order).
__global__ void __launch_bounds__(kBlock) k_centroid(const float* __restrict__ verts, uint32_t n,
                                                     float* __restrict__ partial, uint32_t* __restrict__ done,
                                                     BvhMeta* meta) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = blockIdx.x * kBlock + threadIdx.x; i < n; i += gridDim.x * kBlock) {
        Box3 b = tri_box(verts, i);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float c = __fmul_rn(__fadd_rn(b.lo[k], b.hi[k]), 0.5f);  // AABB::centroid
            lo[k] = fminf(lo[k], c);
            hi[k] = fmaxf(hi[k], c);
        }
    }
    const float r = block_bounds(lo, hi);
    __shared__ bool s_last;
    if (threadIdx.x < 6) {
        partial[6 * blockIdx.x + threadIdx.x] = r;
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    for (int k = 0; k < 3; ++k) { lo[k] = INFINITY; hi[k] = -INFINITY; }
    for (uint32_t p = threadIdx.x; p < gridDim.x; p += kBlock) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], __ldcg(partial + 6 * p + k));
            hi[k] = fmaxf(hi[k], __ldcg(partial + 6 * p + 3 + k));
        }
    }
    __syncthreads();  // block_bounds' shared words are reused
    const float f = block_bounds(lo, hi);
    if (threadIdx.x < 6) meta->cbox[threadIdx.x] = f;
}

// ---- 2. Morton codes + the four digit histograms ------------------------------

// Also clears the sort's status words (`status`, `nstatus` words), which the
// look-back passes need at zero.
__global__ void __launch_bounds__(kBlock) k_morton_hist(const float* __restrict__ verts, uint32_t n,
                                                        const BvhMeta* __restrict__ meta, uint32_t* __restrict__ keys,
                                                        uint32_t* __restrict__ vals, uint32_t* __restrict__ hist,
                                                        uint32_t* __restrict__ status, uint32_t nstatus) {
    __shared__ uint32_t s_hist[4 * 256];
    for (int i = threadIdx.x; i < 4 * 256; i += kBlock) s_hist[i] = 0;
    for (uint32_t i = blockIdx.x * kBlock + threadIdx.x; i < nstatus; i += gridDim.x * kBlock) status[i] = 0;
    __syncthreads();
    float blo[3], bhi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) { blo[k] = meta->cbox[k]; bhi[k] = meta->cbox[3 + k]; }
    for (uint32_t i = blockIdx.x * kBlock + threadIdx.x; i < n; i += gridDim.x * kBlock) {
        Box3 b = tri_box(verts, i);
        uint32_t cell[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float c = __fmul_rn(__fadd_rn(b.lo[k], b.hi[k]), 0.5f);
            float q = __fmul_rn(__fdiv_rn(__fsub_rn(c, blo[k]), __fsub_rn(bhi[k], blo[k])), 1024.0f);
            uint32_t x = __float2uint_rz(q);  // truncation; NaN -> 0
            cell[k] = x > 1023u ? 1023u : x;  // 1024 -> 1023 (bvh.h:15)
        }
        uint32_t code = (spread10(cell[2]) << 2) | (spread10(cell[1]) << 1) | spread10(cell[0]);
        keys[i] = code;
        vals[i] = i;
        atomicAdd(&s_hist[code & 0xFF], 1u);
        atomicAdd(&s_hist[256 + ((code >> 8) & 0xFF)], 1u);
        atomicAdd(&s_hist[512 + ((code >> 16) & 0xFF)], 1u);
        atomicAdd(&s_hist[768 + (code >> 24)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 4 * 256; i += kBlock)
        if (s_hist[i]) atomicAdd(&hist[i], s_hist[i]);
}

// ---- 3. radix sort ----------------------------------------------------------------
// Four passes of one 8-bit digit each. Tiles of 4096 keys are ranked in shared
// memory (warp multi-split by ballots, stable in input order), the tile's
// per-digit counts are prefixed over the tiles before it, and keys are written
// out grouped by digit. The prefix comes from a grid barrier and a scan of every
// tile's counts when all tiles fit on the GPU at once (all four passes in one
// cooperative launch), else from decoupled look-back (one launch per pass).

constexpr int kOsThreads = 512;
constexpr int kOsItems = 8;
constexpr int kOsTile = kOsThreads * kOsItems;
constexpr int kOsWarps = kOsThreads / 32;
constexpr uint32_t kFlagAgg = 1u << 30, kFlagInc = 2u << 30, kCountMask = (1u << 30) - 1;

// Decoupled look-back over the tiles before `tile` (their status words `stride`
// apart): sums their published counts until a tile with its inclusive prefix.
// A tile that has not published yet is polled again; after `limit` polls in all
// the wait gives up, sets ERR_TIMEOUT and returns what it has summed (the result
// is then wrong and the host reports the error bit).
__device__ __forceinline__ uint32_t lookback(const uint32_t* status, size_t stride, int64_t tile, uint32_t limit,
                                             uint32_t* err) {
    uint32_t excl = 0, spins = 0;
    int64_t t = tile - 1;
    while (t >= 0) {
        const uint32_t v = ld_acquire(status + (size_t)t * stride);
        const uint32_t flag = v & ~kCountMask;
        if (flag == 0) {
            if (++spins > limit) {
                atomicOr(err, ERR_TIMEOUT);
                break;
            }
            continue;
        }
        excl += v & kCountMask;
        if (flag == kFlagInc) break;
        --t;
    }
    return excl;
}
// Lanes of the warp holding the same 8-bit digit as this lane (digit 256 marks
// a key past the end: those lanes match only each other). Nine ballots at full
// issue rate in place of one match instruction, whose throughput made the
// ranking the longest phase of a pass.
__device__ __forceinline__ uint32_t match_digit(uint32_t d) {
    uint32_t peers = __ballot_sync(0xFFFFFFFFu, d < 256u);
    if (d >= 256u) peers = ~peers;
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        const bool bit = (d >> b) & 1u;
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, bit);
        peers &= bit ? m : ~m;
    }
    return peers;
}

// Cooperative sort: up to this many tiles each tile sums the earlier tiles'
// digit counts itself (one grid barrier); more tiles scan the counts first.
constexpr uint32_t kSumTiles = 64;

constexpr size_t kOsSmem = sizeof(uint32_t) * (kOsWarps * 256 + 256 + 256 + 2 * kOsTile + 2 * kOsWarps + 1);

// Grid-wide barrier of a cooperative launch (every block resident): block
// arrivals are counted on `ctr`, and the k-th barrier of the launch waits for
// (k + 1) * gridDim.x arrivals, at most `limit` polls (then ERR_TIMEOUT).
// The block barrier before the fence puts every thread's writes ahead of the
// arrival; the block barrier after it puts the other blocks' writes ahead of
// every thread's later reads (which go to L2: __ldcg).
__device__ __forceinline__ void grid_barrier(uint32_t* ctr, uint32_t target, uint32_t* err,
                                             uint32_t limit = kSpinLimit) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(ctr, 1u);
        uint32_t spins = 0;
        while (ld_acquire(ctr) < target) {
            if (++spins > limit) {
                atomicOr(err, ERR_TIMEOUT);
                break;
            }
        }
        __threadfence();
    }
    __syncthreads();
}

// One tile of one sort pass: ranks the tile's keys by the pass's digit, finds
// where each digit's run of the tile starts in the output, and writes the
// tile out grouped by digit. The runs' output starts come from the pass's
// digit histogram plus the counts of the tiles before this one, by decoupled
// look-back over `status` (COOP false) or, in a cooperative launch (COOP
// true), from the counts every tile publishes in `status` (digit-major) before
// a grid barrier (`barrier` is its index in the launch): up to kSumTiles tiles
// each tile sums the columns itself; beyond, the blocks scan the columns over
// the tiles and a second grid barrier follows.
template <bool COOP>
__device__ __forceinline__ void sort_tile(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                          uint32_t* __restrict__ kout, uint32_t* __restrict__ vout, uint32_t n,
                                          int pass, const uint32_t* __restrict__ hist, uint32_t tile,
                                          uint32_t* __restrict__ status, uint32_t* sync_ctr, uint32_t barrier,
                                          uint32_t* __restrict__ err, uint32_t* smem) {
    uint32_t* s_wcnt = smem;                       // [warps][256]
    uint32_t* s_dstart = s_wcnt + kOsWarps * 256;  // [256] tile-local digit starts
    uint32_t* s_gbase = s_dstart + 256;            // [256] global digit bases
    uint32_t* s_keys = s_gbase + 256;              // [tile]
    uint32_t* s_vals = s_keys + kOsTile;           // [tile]
    unsigned long long* s_warp = reinterpret_cast<unsigned long long*>(s_vals + kOsTile);  // [warps] scan scratch

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int shift = 8 * pass;
    for (int i = threadIdx.x; i < kOsWarps * 256; i += kOsThreads) s_wcnt[i] = 0;
    __syncthreads();
    const uint64_t base = (uint64_t)tile * kOsTile;

    uint32_t key[kOsItems], val[kOsItems], rank[kOsItems], dig[kOsItems];
#pragma unroll
    for (int j = 0; j < kOsItems; ++j) {
        const uint64_t idx = base + warp * (32 * kOsItems) + j * 32 + lane;
        const bool ok = idx < n;
        key[j] = ok ? (COOP ? __ldcg(kin + idx) : kin[idx]) : 0u;
        val[j] = ok ? (COOP ? __ldcg(vin + idx) : vin[idx]) : 0u;
        dig[j] = ok ? ((key[j] >> shift) & 0xFFu) : 256u;
    }
    const uint32_t ltmask = lanemask_lt();
    uint32_t* wc = s_wcnt + warp * 256;
#pragma unroll
    for (int j = 0; j < kOsItems; ++j) {
        const uint32_t d = dig[j];
        const uint32_t peers = match_digit(d);
        const uint32_t lt = __popc(peers & ltmask);
        const uint32_t before = d < 256u ? wc[d] : 0u;
        __syncwarp();
        if (d < 256u && lt == 0) wc[d] = before + __popc(peers);
        __syncwarp();
        rank[j] = before + lt;
    }
    __syncthreads();

    uint32_t cnt = 0;
    if (threadIdx.x < 256) {
        const int d = threadIdx.x;
        uint32_t run = 0;
        for (int w = 0; w < kOsWarps; ++w) {
            const uint32_t t = s_wcnt[w * 256 + d];
            s_wcnt[w * 256 + d] = run;
            run += t;
        }
        cnt = run;
    }
    __syncthreads();
    // one scan gives the tile-local digit starts (low word) and the pass's
    // global digit starts from the histogram (high word; the tile's counts sum
    // to at most kOsTile, so the low word never carries)
    unsigned long long tot;
    const unsigned long long both = block_exclusive_scan<kOsThreads>(
        threadIdx.x < 256 ? ((unsigned long long)hist[256 * pass + threadIdx.x] << 32) | cnt : 0ull, s_warp, &tot);
    const uint32_t dstart = (uint32_t)both;
    if (COOP) {
        // counts digit-major: column d holds digit d's count of every tile
        const uint32_t tiles = gridDim.x;
        if (threadIdx.x < 256) status[(size_t)threadIdx.x * tiles + tile] = cnt;
        grid_barrier(sync_ctr, (barrier + 1) * gridDim.x, err);
        if (tiles <= kSumTiles) {
            // few tiles: each warp sums 16 digits' columns up to this tile,
            // 32 tiles per coalesced load
            constexpr int kDigitsPerWarp = 256 / kOsWarps, kRound = 8;
#pragma unroll
            for (int r = 0; r < kDigitsPerWarp; r += kRound) {
                uint32_t acc[kRound];
#pragma unroll
                for (int k = 0; k < kRound; ++k) acc[k] = 0;
                for (uint32_t t = lane; t < tile; t += 32) {
#pragma unroll
                    for (int k = 0; k < kRound; ++k)
                        acc[k] += __ldcg(status + (size_t)(warp * kDigitsPerWarp + r + k) * tiles + t);
                }
#pragma unroll
                for (int k = 0; k < kRound; ++k) {
                    const uint32_t sum = __reduce_add_sync(0xFFFFFFFFu, acc[k]);
                    if (lane == 0) s_gbase[warp * kDigitsPerWarp + r + k] = sum;
                }
            }
            __syncthreads();
            if (threadIdx.x < 256) {
                s_dstart[threadIdx.x] = dstart;
                s_gbase[threadIdx.x] += (uint32_t)(both >> 32);
            }
        } else {
            // many tiles: each block turns some columns into exclusive prefixes
            // over the tiles, then every tile reads its own (summing every
            // column in every tile moved tens of MB through L2 per pass)
            for (uint32_t d = blockIdx.x; d < 256; d += gridDim.x) {
                uint32_t* col = status + (size_t)d * tiles;
                uint32_t carry = 0;
                for (uint32_t t0 = 0; t0 < tiles; t0 += kOsThreads) {
                    const uint32_t t = t0 + threadIdx.x;
                    const uint32_t v = t < tiles ? __ldcg(col + t) : 0u;
                    unsigned long long sum;
                    const uint32_t ex =
                        (uint32_t)block_exclusive_scan<kOsThreads>((unsigned long long)v, s_warp, &sum);
                    if (t < tiles) col[t] = carry + ex;
                    carry += (uint32_t)sum;
                }
            }
            grid_barrier(sync_ctr, (barrier + 2) * gridDim.x, err);
            if (threadIdx.x < 256) {
                s_dstart[threadIdx.x] = dstart;
                s_gbase[threadIdx.x] = (uint32_t)(both >> 32) + __ldcg(status + (size_t)threadIdx.x * tiles + tile);
            }
        }
    } else if (threadIdx.x < 256) {
        const int d = threadIdx.x;
        s_dstart[d] = dstart;
        uint32_t* st = status + (size_t)tile * 256 + d;
        uint32_t excl = 0;
        if (tile == 0) {
            st_release(st, kFlagInc | cnt);
        } else {
            st_release(st, kFlagAgg | cnt);
            excl = lookback(status + d, 256, (int64_t)tile, kSpinLimit, err);
            st_release(st, kFlagInc | ((excl + cnt) & kCountMask));
        }
        s_gbase[d] = (uint32_t)(both >> 32) + excl;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kOsItems; ++j) {
        const uint32_t d = dig[j];
        if (d < 256u) {
            const uint32_t r = s_dstart[d] + s_wcnt[warp * 256 + d] + rank[j];
            s_keys[r] = key[j];
            s_vals[r] = val[j];
        }
    }
    __syncthreads();
    const uint64_t left = (uint64_t)n - base;
    const uint32_t valid = left < (uint64_t)kOsTile ? (uint32_t)left : (uint32_t)kOsTile;
    for (uint32_t i = threadIdx.x; i < valid; i += kOsThreads) {
        const uint32_t k = s_keys[i];
        const uint32_t d = (k >> shift) & 0xFFu;
        const uint32_t pos = s_gbase[d] + (i - s_dstart[d]);
        if (pos < n) {
            kout[pos] = k;
            vout[pos] = s_vals[i];
        } else {
            atomicOr(err, ERR_RANGE);
        }
    }
}

// One sort pass, tiles taken in launch order from `tile_ctr` (so a tile's
// predecessors have started: the look-back's waits end).
__global__ void __launch_bounds__(kOsThreads, 2) k_onesweep(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                         uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                         uint32_t n, int pass, const uint32_t* __restrict__ hist,
                                                         uint32_t* __restrict__ status, uint32_t* __restrict__ tile_ctr,
                                                         uint32_t* __restrict__ err) {
    extern __shared__ uint32_t smem[];
    __shared__ uint32_t s_tile;
    if (threadIdx.x == 0) s_tile = atomicAdd(tile_ctr + pass, 1u);
    __syncthreads();
    sort_tile<false>(kin, vin, kout, vout, n, pass, hist, s_tile, status, nullptr, 0, err, smem);
}

// All four sort passes in one cooperative launch, one block per tile (every
// tile resident): keys and values go from (key_a, val_a) to (key_b, val_b)
// and back, twice. Grid barriers a pass: after the tiles publish their counts,
// after the counts are scanned (more than kSumTiles tiles), and after the
// tiles are written (before the next pass reads them and overwrites the
// counts).
__global__ void __launch_bounds__(kOsThreads, 2) k_sort_coop(uint32_t* key_a, uint32_t* val_a, uint32_t* key_b,
                                                          uint32_t* val_b, uint32_t n,
                                                          const uint32_t* __restrict__ hist, uint32_t* counts,
                                                          uint32_t* sync_ctr, uint32_t* err) {
    extern __shared__ uint32_t smem[];
    const uint32_t per_pass = gridDim.x <= kSumTiles ? 2 : 3;  // grid barriers a pass
    for (int pass = 0; pass < 4; ++pass) {
        const bool even = (pass & 1) == 0;
        sort_tile<true>(even ? key_a : key_b, even ? val_a : val_b, even ? key_b : key_a, even ? val_b : val_a, n,
                        pass, hist, blockIdx.x, counts, sync_ctr, per_pass * pass, err, smem);
        if (pass < 3) grid_barrier(sync_ctr, per_pass * (pass + 1) * gridDim.x, err);
    }
}

// ---- 4. split levels of the gaps -----------------------------------------------------
// Gap g lies between sorted positions g and g + 1; internal nodes are stored at
// the gap they split. Its level orders the gaps by depth in the tree:
//   - codes differ: the length of their common prefix, clz(code[g] ^ code[g + 1])
//     (2..31: the codes have 30 bits), the radix tree's split level (Karras,
//     HPG 2012; the reference's split search, bvh.h:125-160);
//   - codes equal (a run of equal codes, split at its midpoint recursively,
//     bvh.h:162-165): 32 + the depth of g's node in the run's midpoint subtree,
//     so every gap inside a run ranks below the run's outer gaps.
// A node covering positions [lo, hi] is a child of the node at one of its two
// outer gaps, lo - 1 or hi: in a binary tree over ordered leaves both outer gaps
// belong to ancestors, the parent is the deeper one, and two outer gaps never
// tie (for distinct codes the shared prefix of lo - 1 and hi + 1 with the
// range would have to differ at the same bit in opposite directions). So the
// level of the two outer gaps alone picks every node's parent (the bottom-up
// form of the same radix tree: Apetrei, EG 2014).

// Depth of gap g (codes g and g + 1 equal) in the midpoint subtree of its run:
// the run's ends by exponential then binary search over the sorted codes, then
// a descent from the run's root split.
__device__ __forceinline__ uint32_t run_depth(const uint32_t* __restrict__ code, uint32_t n, uint32_t g,
                                              uint32_t* __restrict__ err) {
    const uint32_t c = code[g];
    int64_t good = g, bad = -1;  // code[good] == c; code[bad] < c (or bad = -1)
    for (int64_t step = 1;; step <<= 1) {
        const int64_t t = good - step;
        if (t < 0) break;
        if (code[t] != c) { bad = t; break; }
        good = t;
    }
    while (good - bad > 1) {
        const int64_t mid = bad + ((good - bad) >> 1);
        if (code[mid] == c) good = mid; else bad = mid;
    }
    const uint32_t s = (uint32_t)good;
    int64_t good_r = (int64_t)g + 1, bad_r = n;  // code[good_r] == c; code[bad_r] > c (or n)
    for (int64_t step = 1;; step <<= 1) {
        const int64_t t = good_r + step;
        if (t >= (int64_t)n) break;
        if (code[t] != c) { bad_r = t; break; }
        good_r = t;
    }
    while (bad_r - good_r > 1) {
        const int64_t mid = good_r + ((bad_r - good_r) >> 1);
        if (code[mid] == c) good_r = mid; else bad_r = mid;
    }
    uint32_t a = s, b = (uint32_t)good_r;  // the run, inclusive
    uint32_t G = a + ((b - a + 1) >> 1) - 1, depth = 0;
    while (G != g) {
        if (g < G) b = G; else a = G + 1;
        G = a + ((b - a + 1) >> 1) - 1;
        if (++depth > 32) {
            atomicOr(err, ERR_RANGE);
            break;
        }
    }
    return depth;
}

// Also clears the node counters of the bottom-up pass.
__global__ void __launch_bounds__(kBlock) k_gaps(const uint32_t* __restrict__ code, uint32_t n,
                                                 uint8_t* __restrict__ level, uint32_t* __restrict__ counters,
                                                 uint32_t* __restrict__ err) {
    for (uint32_t g = blockIdx.x * kBlock + threadIdx.x; g + 1 < n; g += gridDim.x * kBlock) {
        const uint32_t c0 = code[g], c1 = code[g + 1];
        level[g] = (uint8_t)(c0 != c1 ? (uint32_t)__clz(c0 ^ c1) : 32u + run_depth(code, n, g, err));
        counters[g] = 0;
    }
}

// ---- 5. hierarchy, boxes and leaf-order triangles in one bottom-up pass ------------

__device__ __forceinline__ void put_child_box(Node* nd, int slot, const Box3& b) {
    float4* q = reinterpret_cast<float4*>(nd);
    q[slot] = make_float4(b.lo[0], b.hi[0], b.lo[1], b.hi[1]);
    reinterpret_cast<float2*>(&nd->q2)[slot] = make_float2(b.lo[2], b.hi[2]);
}

__device__ __forceinline__ Box3 get_child_box_l2(const Node* nd, int slot) {
    const float4 xy = __ldcg(reinterpret_cast<const float4*>(nd) + slot);
    const float2 z = __ldcg(reinterpret_cast<const float2*>(&nd->q2) + slot);
    Box3 b;
    b.lo[0] = xy.x; b.hi[0] = xy.y; b.lo[1] = xy.z; b.hi[1] = xy.w; b.lo[2] = z.x; b.hi[2] = z.y;
    return b;
}

// Counter increment with acquire-release semantics at GPU scope: this thread's
// earlier writes (its child box and link) are visible to the thread that sees
// the incremented count, and the sibling's, written before its own increment,
// are visible to this thread's later reads. One ordered atomic in place of two
// full fences around a relaxed one.
__device__ __forceinline__ uint32_t atomic_add_acq_rel(uint32_t* p, uint32_t v) {
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

__device__ __forceinline__ void box_union(Box3& a, const Box3& b) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        a.lo[k] = fminf(a.lo[k], b.lo[k]);
        a.hi[k] = fmaxf(a.hi[k], b.hi[k]);
    }
}

// A finished subtree on its way up: its id (~position for a leaf, else its
// gap), the sorted positions it covers, the levels of its two outer gaps
// lo - 1 and hi (-1 where the range ends the sequence) and its box.
struct Sub {
    int32_t me;
    uint32_t lo, hi;
    int32_t llo, lhi;
    Box3 box;
};

// Where the climb writes: the node array, the parent of each leaf, per
// internal node and child slot the child's outer end and that end's outer-gap
// level (far[2G] = the left child's first position and the level of the gap
// before it, far[2G + 1] = the right child's last position and the level of
// the gap after it), the node counters, and per chunk the subtree left to
// attach across the chunk's left border.
struct ClimbOut {
    Node* nodes;
    uint32_t* parent_leaf;
    unsigned long long* far;
    BvhMeta* meta;
    uint32_t* counters;
    Sub* pend;
    uint32_t* err;
};

// Slot of the parent of a subtree that is not the whole range: the outer gap
// with the higher level (0: the gap after it, the subtree is a left child).
__device__ __forceinline__ int parent_slot(const Sub& s) { return s.lhi > s.llo ? 0 : 1; }

__device__ __forceinline__ unsigned long long far_word(const Sub& s, int slot) {
    const uint32_t end = slot == 0 ? s.lo : s.hi;
    const int32_t lv = slot == 0 ? s.llo : s.lhi;
    return ((unsigned long long)(uint32_t)(lv & 0xFF) << 32) | end;
}

// Takes the sibling's outer end (and its gap level) from its far word: the
// subtree becomes its parent's range.
__device__ __forceinline__ void widen(Sub& s, int slot, unsigned long long w) {
    const uint32_t end = (uint32_t)w;
    const uint32_t lb = (uint32_t)(w >> 32) & 0xFFu;
    const int32_t lv = lb == 0xFFu ? -1 : (int32_t)lb;
    if (slot == 0) { s.hi = end; s.lhi = lv; } else { s.lo = end; s.llo = lv; }
}

// The finished subtree `s` hangs below gap `G` in slot `slot` (0 = left): its
// box and id go into the parent's record, its far word into far, and the
// parent's index into its own record.
__device__ __forceinline__ void attach(const ClimbOut& o, const Sub& s, uint32_t G, int slot) {
    Node* pn = o.nodes + G;
    put_child_box(pn, slot, s.box);
    reinterpret_cast<int32_t*>(&pn->q3)[slot] = s.me;
    o.far[2 * G + slot] = far_word(s, slot);
    if (s.me >= 0) *reinterpret_cast<int2*>(&o.nodes[s.me].q3.z) = make_int2((int32_t)G, 0);
    else o.parent_leaf[~s.me] = G;
}

// The whole range is finished: `s` is the root.
__device__ __forceinline__ void set_root(const ClimbOut& o, const Sub& s) {
    *reinterpret_cast<int2*>(&o.nodes[s.me].q3.z) = make_int2((int32_t)kNoNode, 0);
    o.meta->root = (uint32_t)s.me;
}

// Climb from finished subtree `s` with GPU-scope counters: at each parent the
// first arrival stops, the second unions its sibling's box and range and goes
// on up. Two round trips a level: the counter, then the sibling's box and far
// word (which carries the level the next step needs).
__device__ __forceinline__ void climb_global(const ClimbOut& o, Sub s) {
    for (int guard = 0;; ++guard) {
        if (s.llo < 0 && s.lhi < 0) {
            set_root(o, s);
            return;
        }
        if (guard > 128) {
            atomicOr(o.err, ERR_RANGE);
            return;
        }
        const int slot = parent_slot(s);
        const uint32_t G = slot == 0 ? s.hi : s.lo - 1;
        attach(o, s, G, slot);
        if (atomic_add_acq_rel(&o.counters[G], 1u) == 0) return;  // sibling not done yet
        box_union(s.box, get_child_box_l2(o.nodes + G, slot ^ 1));
        widen(s, slot, __ldcg(&o.far[2 * G + (slot ^ 1)]));
        s.me = (int32_t)G;
    }
}

// Writes a finished node's whole 64-byte record (two 32-byte stores): the
// children's boxes, their ids, the parent's index.
__device__ __forceinline__ void write_node(Node* nd, const Box3& b0, const Box3& b1, int32_t l0, int32_t l1,
                                           uint32_t parent) {
    float* q = reinterpret_cast<float*>(nd);
    asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(q), "f"(b0.lo[0]), "f"(b0.hi[0]),
                 "f"(b0.lo[1]), "f"(b0.hi[1]), "f"(b1.lo[0]), "f"(b1.hi[0]), "f"(b1.lo[1]), "f"(b1.hi[1])
                 : "memory");
    asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(q + 8), "f"(b0.lo[2]),
                 "f"(b0.hi[2]), "f"(b1.lo[2]), "f"(b1.hi[2]), "f"(__int_as_float(l0)), "f"(__int_as_float(l1)),
                 "f"(__uint_as_float(parent)), "f"(0.0f)
                 : "memory");
}

// Bit-or with acquire-release semantics at CTA scope on a shared-memory word
// (the arrival mask of a node: bit = child slot).
__device__ __forceinline__ uint32_t atomic_or_acq_rel_cta(uint32_t* p, uint32_t v) {
    uint32_t old;
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("atom.acq_rel.cta.shared.or.b32 %0, [%1], %2;" : "=r"(old) : "r"(a), "r"(v) : "memory");
    return old;
}

// Bottom-up pass, part 1: a block takes kRefitChunk sorted positions, one per
// thread; the thread climbs while its subtree's parent is one of the chunk's
// gaps [base, base + kRefitChunk). The climb touches shared memory only:
// arrivals are marked with an ordered bit-or at block scope (bit = child
// slot), each child's box, id and far word wait there for the sibling, and
// the second arrival records the node's parent. A subtree inside the chunk can
// have its parent outside only at gap base - 1 (its range starts at base), so
// at most one subtree per chunk is left over: it goes to `pend`. After the
// block barrier each thread writes, coalesced, its position's triangle and
// leaf parent and its gap's node: the whole record if both children arrived,
// else the one child's slot, far word and arrival count for part 2.
__global__ void __launch_bounds__(kRefitChunk) k_climb_chunk(const float* __restrict__ verts, uint32_t n,
                                                             const uint32_t* __restrict__ prim,
                                                             const uint8_t* __restrict__ level, ClimbOut o,
                                                             Tri* __restrict__ tris) {
    __shared__ uint32_t s_mask[kRefitChunk];
    __shared__ uint32_t s_parent[kRefitChunk];
    __shared__ __align__(16) float s_box[kRefitChunk][2][6];  // per gap and slot: lo.xyz, hi.xyz
    __shared__ unsigned long long s_far[kRefitChunk][2];
    __shared__ int32_t s_link[kRefitChunk][2];
    __shared__ Sub s_pend;
    const uint32_t chunks = (n + kRefitChunk - 1) / kRefitChunk;
    for (uint32_t c = blockIdx.x; c < chunks; c += gridDim.x) {  // block-uniform
        const uint32_t base = c * kRefitChunk;
        s_mask[threadIdx.x] = 0;
        if (threadIdx.x == 0) s_pend.lo = 0;  // no subtree left over (a left-over range starts at base > 0)
        __syncthreads();
        const uint32_t p = base + threadIdx.x;  // one sorted position per thread
        Tri t;
        uint32_t leaf_parent = kNoNode;
        if (p < n) {
            const uint32_t id = prim[p];
            const float* v = verts + 9ull * id;
            float a[9];
#pragma unroll
            for (int k = 0; k < 9; ++k) a[k] = __ldg(v + k);
            t.a = make_float4(a[0], a[1], a[2], __uint_as_float(id));
            t.b = make_float4(a[3], a[4], a[5], 0.0f);
            t.c = make_float4(a[6], a[7], a[8], 0.0f);
            Sub s;
            s.me = ~(int32_t)p;
            s.lo = s.hi = p;
            s.llo = p > 0 ? (int32_t)__ldg(level + p - 1) : -1;
            s.lhi = p + 1 < n ? (int32_t)__ldg(level + p) : -1;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                s.box.lo[k] = fminf(fminf(a[k], a[3 + k]), a[6 + k]);
                s.box.hi[k] = fmaxf(fmaxf(a[k], a[3 + k]), a[6 + k]);
            }
            if (n == 1) {
                // one triangle: a single node whose two children are the same leaf
                write_node(o.nodes, s.box, s.box, ~0, ~0, kNoNode);
                o.meta->root = 0;
            } else {
                // s is finished and is not the root
                for (int guard = 0;; ++guard) {
                    if (guard > 128) {
                        atomicOr(o.err, ERR_RANGE);
                        break;
                    }
                    const int slot = parent_slot(s);
                    const uint32_t P = slot == 0 ? s.hi : s.lo - 1;
                    if (s.me < 0) leaf_parent = P;
                    if (slot == 1 && s.lo == base) {  // parent at gap base - 1, another chunk's
                        s_pend = s;
                        break;
                    }
                    const uint32_t g = P - base;
                    float2* sb2 = reinterpret_cast<float2*>(s_box[g][slot]);
                    sb2[0] = make_float2(s.box.lo[0], s.box.lo[1]);
                    sb2[1] = make_float2(s.box.lo[2], s.box.hi[0]);
                    sb2[2] = make_float2(s.box.hi[1], s.box.hi[2]);
                    s_far[g][slot] = far_word(s, slot);
                    s_link[g][slot] = s.me;
                    if (atomic_or_acq_rel_cta(&s_mask[g], 1u << slot) == 0) break;  // sibling not done yet
                    const float2* ob2 = reinterpret_cast<const float2*>(s_box[g][slot ^ 1]);
                    const float2 u0 = ob2[0], u1 = ob2[1], u2 = ob2[2];
                    Box3 sb;
                    sb.lo[0] = u0.x; sb.lo[1] = u0.y; sb.lo[2] = u1.x; sb.hi[0] = u1.y; sb.hi[1] = u2.x; sb.hi[2] = u2.y;
                    box_union(s.box, sb);
                    widen(s, slot, s_far[g][slot ^ 1]);
                    s.me = (int32_t)P;
                    if (s.llo < 0 && s.lhi < 0) {  // the root
                        s_parent[g] = kNoNode;
                        o.meta->root = P;
                        break;
                    }
                    s_parent[g] = parent_slot(s) == 0 ? s.hi : s.lo - 1;
                }
            }
        }
        __syncthreads();
        if (p < n) {
            tris[p] = t;
            if (n > 1) o.parent_leaf[p] = leaf_parent;
        }
        if (p + 1 < n) {
            const uint32_t m = s_mask[threadIdx.x];
            const int j = threadIdx.x;
            const float4* sb4 = reinterpret_cast<const float4*>(s_box[j]);
            const float4 u = sb4[0], w = sb4[1], z = sb4[2];
            Box3 b0, b1;
            b0.lo[0] = u.x; b0.lo[1] = u.y; b0.lo[2] = u.z; b0.hi[0] = u.w; b0.hi[1] = w.x; b0.hi[2] = w.y;
            b1.lo[0] = w.z; b1.lo[1] = w.w; b1.lo[2] = z.x; b1.hi[0] = z.y; b1.hi[1] = z.z; b1.hi[2] = z.w;
            if (m == 3u) {  // finished here: the whole record
                write_node(o.nodes + p, b0, b1, s_link[j][0], s_link[j][1], s_parent[j]);
            } else if (m != 0u) {  // one child arrived: its slot, far word and count for part 2
                const int slot = m == 1u ? 0 : 1;
                Node* nd = o.nodes + p;
                put_child_box(nd, slot, slot == 0 ? b0 : b1);
                reinterpret_cast<int32_t*>(&nd->q3)[slot] = s_link[j][slot];
                o.far[2 * p + slot] = s_far[j][slot];
                o.counters[p] = 1;
            }
        }
        if (threadIdx.x == 0) o.pend[c] = s_pend;
        __syncthreads();
    }
}

// Bottom-up pass, part 2: one thread per chunk attaches the chunk's left-over
// subtree (if any) across the chunk's left border and climbs with GPU-scope
// counters. Part 1's writes are complete and visible (kernel boundary); every
// node still open has exactly its missing arrivals left.
constexpr int kUpThreads = 64;  // small blocks: the climbs spread over many SMs

__global__ void __launch_bounds__(kUpThreads) k_climb_up(uint32_t chunks, ClimbOut o) {
    for (uint32_t c = blockIdx.x * kUpThreads + threadIdx.x; c < chunks; c += gridDim.x * kUpThreads) {
        const Sub* ps = o.pend + c;
        Sub s;
        s.lo = ps->lo;
        if (s.lo == 0) continue;
        s.me = ps->me;
        s.hi = ps->hi;
        s.llo = ps->llo;
        s.lhi = ps->lhi;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            s.box.lo[k] = ps->box.lo[k];
            s.box.hi[k] = ps->box.hi[k];
        }
        climb_global(o, s);
    }
}

// ---- 6. reference-layout export (parity only) -------------------------------------
// Preorder index of a node covering leaves [first, ...] = 2*first + number of
// left turns on the path from the root.

__global__ void __launch_bounds__(kBlock) k_export_ref(const Node* __restrict__ nodes, const Tri* __restrict__ tris,
                                                       const uint32_t* __restrict__ parent_leaf, uint32_t n,
                                                       uint32_t* __restrict__ out) {
    const uint64_t total = 2ull * n - 1;
    for (uint64_t x = blockIdx.x * (uint64_t)kBlock + threadIdx.x; x < total; x += (uint64_t)gridDim.x * kBlock) {
        uint32_t w[8];
        uint32_t first, parent;
        int32_t me;
        if (x < n) {  // leaf at sorted position x
            const uint32_t p = (uint32_t)x;
            const Tri t = tris[p];
            const float a[9] = {t.a.x, t.a.y, t.a.z, t.b.x, t.b.y, t.b.z, t.c.x, t.c.y, t.c.z};
            for (int k = 0; k < 3; ++k) {
                w[k] = __float_as_uint(fminf(fminf(a[k], a[3 + k]), a[6 + k]));
                w[3 + k] = __float_as_uint(fmaxf(fmaxf(a[k], a[3 + k]), a[6 + k]));
            }
            w[6] = __float_as_uint(t.a.w);
            w[7] = 1;
            first = p;
            me = ~(int32_t)p;
            parent = n == 1 ? kNoNode : parent_leaf[p];
        } else {  // internal node at gap G
            const uint32_t G = (uint32_t)(x - n);
            const Node nd = nodes[G];
            w[0] = __float_as_uint(fminf(nd.q0.x, nd.q1.x));
            w[1] = __float_as_uint(fminf(nd.q0.z, nd.q1.z));
            w[2] = __float_as_uint(fminf(nd.q2.x, nd.q2.z));
            w[3] = __float_as_uint(fmaxf(nd.q0.y, nd.q1.y));
            w[4] = __float_as_uint(fmaxf(nd.q0.w, nd.q1.w));
            w[5] = __float_as_uint(fmaxf(nd.q2.y, nd.q2.w));
            int32_t c = nd.q3.x;
            int guard = 0;
            while (c >= 0 && ++guard < 128) c = nodes[c].q3.x;
            first = (uint32_t)~c;
            w[7] = 0;
            me = (int32_t)G;
            parent = (uint32_t)nd.q3.z;
            w[6] = 0;  // filled below once the preorder index is known
        }
        uint32_t left_turns = 0;
        int guard = 0;
        while (parent != kNoNode && ++guard < 128) {
            const int4 q = nodes[parent].q3;
            if (q.x == me) ++left_turns;
            me = (int32_t)parent;
            parent = (uint32_t)q.z;
        }
        const uint32_t pre = 2 * first + left_turns;
        if (x >= n) {
            const uint32_t G = (uint32_t)(x - n);
            w[6] = pre + 2 * (G - first + 1);
        }
        uint4* o = reinterpret_cast<uint4*>(out + 8ull * pre);
        o[0] = make_uint4(w[0], w[1], w[2], w[3]);
        o[1] = make_uint4(w[4], w[5], w[6], w[7]);
    }
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct Scratch {
    uint32_t *keys_alt, *vals_alt, *parent_leaf, *counters;
    unsigned long long* far;
    Sub* pend;
    uint8_t* level;
    uint32_t *hist, *os_status, *tile_ctr, *err;
    float* partial;
    size_t zero_bytes;  // bytes from the histograms up to the end of the zeroed region
    void* zero_base;
};

constexpr int kPartials = 1024;

size_t scratch_layout(uint32_t n, char* base, Scratch* s) {
    const uint64_t os_tiles = ((uint64_t)n + kOsTile - 1) / kOsTile;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char* p = base ? base + off : nullptr;
        off += align256(bytes);
        return p;
    };
    const size_t w = 4ull * n;
    s->keys_alt = (uint32_t*)take(w);
    s->vals_alt = (uint32_t*)take(w);
    s->parent_leaf = (uint32_t*)take(w);
    s->far = (unsigned long long*)take(16ull * n);
    s->pend = (Sub*)take(sizeof(Sub) * (((uint64_t)n + kRefitChunk - 1) / kRefitChunk));
    s->level = (uint8_t*)take(n);
    s->partial = (float*)take(sizeof(float) * 6 * kPartials);
    s->counters = (uint32_t*)take(w);                            // cleared by k_gaps
    s->os_status = (uint32_t*)take(4ull * os_tiles * 256 * 4);  // cleared by k_morton_hist
    // everything from here on is zeroed before each build
    const size_t zstart = off;
    s->hist = (uint32_t*)take(4 * 256 * 4);
    s->tile_ctr = (uint32_t*)take(16 * 4);
    s->err = (uint32_t*)take(4);
    s->zero_base = base ? base + zstart : nullptr;
    s->zero_bytes = off - zstart;
    return off;
}

// The build's bounded waits on their own: tile 1 looks back at tile 0, whose
// status word nothing publishes, and a one-block grid barrier waits for a
// second block that does not exist, so both waits run out after `limit` polls.
__global__ void k_lookback_probe(const uint32_t* status, uint32_t limit, uint32_t* err, uint32_t* out,
                                 uint32_t* ctr) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *out = lookback(status, 1, 1, limit, err);
    grid_barrier(ctr, 2, err, limit);
}

}  // namespace

cudaError_t lookback_probe(uint32_t polls, uint32_t* h_err, cudaStream_t s) {
    uint32_t* d = nullptr;
    cudaError_t e = cudaMalloc(&d, 4 * sizeof(uint32_t));  // status word, error word, result, barrier counter
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(d, 0, 4 * sizeof(uint32_t), s);
    if (e == cudaSuccess) {
        k_lookback_probe<<<1, 32, 0, s>>>(d, std::min(polls, kSpinLimit), d + 1, d + 2, d + 3);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_err, d + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d);
    return e;
}

namespace {

// How many sort tiles one cooperative launch can hold on the current device
// (resident blocks of k_sort_coop per SM times the SMs; 0 without cooperative
// launch), looked up once per device.
cudaError_t sort_coop_capacity(int num_sms, int* tiles) {
    static std::mutex mu;
    static int cached[64];
    static bool known[64];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 0 || dev >= 64 || !known[dev]) {
        int coop = 0, per_sm = 0;
        if ((e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev)) != cudaSuccess) return e;
        if ((e = cudaFuncSetAttribute(k_sort_coop, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kOsSmem)) !=
            cudaSuccess)
            return e;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sort_coop, kOsThreads, kOsSmem)) !=
            cudaSuccess)
            return e;
        const int cap = coop ? per_sm * num_sms : 0;
        if (dev < 0 || dev >= 64) {
            *tiles = cap;
            return cudaSuccess;
        }
        cached[dev] = cap;
        known[dev] = true;
    }
    *tiles = cached[dev];
    return cudaSuccess;
}

// The build's launch sequence over laid-out scratch `s` (scratch_layout): the
// one both the allocating build and the no-allocation build run. Zeroes the
// scratch region that must start at zero, then centroid bounds, Morton codes
// and histograms, four onesweep passes (the sorted codes and triangle ids end
// in `code` / `prim`), the gaps' split levels and the bottom-up pass that links
// the nodes and fits their boxes, and folds the build's error word into the
// header.
cudaError_t launch_build(const float* d_verts, uint32_t n, const Scratch& s, Node* nodes, Tri* tris, uint32_t* code,
                         uint32_t* prim, BvhMeta* meta, int num_sms, cudaStream_t st) {
    cudaError_t e;
    if ((e = cudaMemsetAsync(s.zero_base, 0, s.zero_bytes, st)) != cudaSuccess) return e;
    const int grid = (int)std::min<uint64_t>(((uint64_t)n + kBlock - 1) / kBlock, (uint64_t)num_sms * 8);
    const int parts = std::min(grid, kPartials);
    k_centroid<<<parts, kBlock, 0, st>>>(d_verts, n, s.partial, s.tile_ctr + 4, meta);
    const uint32_t os_tiles = (n + kOsTile - 1) / kOsTile;
    k_morton_hist<<<std::min(grid, num_sms * 2), kBlock, 0, st>>>(d_verts, n, meta, code, prim, s.hist, s.os_status,
                                                                  4 * os_tiles * 256);
    if ((e = cudaFuncSetAttribute(k_onesweep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kOsSmem)) !=
        cudaSuccess)
        return e;
    int coop_tiles = 0;
    if ((e = sort_coop_capacity(num_sms, &coop_tiles)) != cudaSuccess) return e;
    bool sorted = false;
    if (os_tiles <= (uint32_t)coop_tiles) {
        // every tile resident: the four passes in one cooperative launch (a
        // launch the device refuses as too large, e.g. a client held to part of
        // the SMs, falls back to the look-back passes)
        uint32_t* sync_ctr = s.tile_ctr + 8;
        void* args[] = {&code, &prim, (void*)&s.keys_alt, (void*)&s.vals_alt, &n, (void*)&s.hist,
                        (void*)&s.os_status, &sync_ctr, (void*)&s.err};
        e = cudaLaunchCooperativeKernel((const void*)k_sort_coop, dim3(os_tiles), dim3(kOsThreads), args, kOsSmem, st);
        if (e == cudaSuccess) {
            sorted = true;
        } else if (e == cudaErrorCooperativeLaunchTooLarge) {
            (void)cudaGetLastError();
        } else {
            return e;
        }
    }
    if (!sorted) {
        uint32_t* kin = code;
        uint32_t* vin = prim;
        uint32_t* kout = s.keys_alt;
        uint32_t* vout = s.vals_alt;
        for (int pass = 0; pass < 4; ++pass) {
            k_onesweep<<<os_tiles, kOsThreads, kOsSmem, st>>>(kin, vin, kout, vout, n, pass, s.hist,
                                                              s.os_status + (size_t)pass * os_tiles * 256,
                                                              s.tile_ctr, s.err);
            std::swap(kin, kout);
            std::swap(vin, vout);
        }
    }
    // four passes: the sorted data is back in code/prim
    k_gaps<<<grid, kBlock, 0, st>>>(code, n, s.level, s.counters, s.err);
    const uint32_t chunks = (n + kRefitChunk - 1) / kRefitChunk;
    const ClimbOut out{nodes, s.parent_leaf, s.far, meta, s.counters, s.pend, s.err};
    k_climb_chunk<<<chunks, kRefitChunk, 0, st>>>(d_verts, n, prim, s.level, out, tris);
    k_climb_up<<<(chunks + kUpThreads - 1) / kUpThreads, kUpThreads, 0, st>>>(chunks, out);
    // fold the build's error word into the header the host reads
    if ((e = cudaMemcpyAsync(&meta->err, s.err, 4, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
    return cudaGetLastError();
}

}  // namespace

cudaError_t lbvh_build(BvhBuffers& b, const float* d_verts, uint32_t n, int num_sms, cudaStream_t st) {
    cudaError_t e;
    if ((e = b.meta.ensure(sizeof(BvhMeta))) != cudaSuccess) return e;
    BvhMeta* meta = (BvhMeta*)b.meta.p;
    if ((e = cudaMemsetAsync(meta, 0, sizeof(BvhMeta), st)) != cudaSuccess) return e;
    if (n == 0) {
        const uint32_t none = kNoNode;
        return cudaMemcpyAsync(&meta->root, &none, 4, cudaMemcpyHostToDevice, st);
    }
    const size_t nn = n > 1 ? n - 1 : 1;
    if ((e = b.nodes.ensure(nn * sizeof(Node))) != cudaSuccess) return e;
    if ((e = b.tris.ensure((size_t)n * sizeof(Tri))) != cudaSuccess) return e;
    if ((e = b.code.ensure(4ull * n)) != cudaSuccess) return e;
    if ((e = b.prim.ensure(4ull * n)) != cudaSuccess) return e;
    Scratch s;
    const size_t need = scratch_layout(n, nullptr, &s);
    if ((e = b.scratch.ensure(need)) != cudaSuccess) return e;
    scratch_layout(n, (char*)b.scratch.p, &s);
    return launch_build(d_verts, n, s, (Node*)b.nodes.p, (Tri*)b.tris.p, (uint32_t*)b.code.p, (uint32_t*)b.prim.p,
                        meta, num_sms, st);
}

cudaError_t lbvh_export_ref(const BvhBuffers& b, uint32_t n, uint32_t* d_ref_nodes, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    Scratch s;
    scratch_layout(n, (char*)b.scratch.p, &s);
    const uint64_t total = 2ull * n - 1;
    const int grid = (int)std::min<uint64_t>((total + kBlock - 1) / kBlock, 4096);
    k_export_ref<<<grid, kBlock, 0, st>>>((const Node*)b.nodes.p, (const Tri*)b.tris.p, s.parent_leaf, n, d_ref_nodes);
    return cudaGetLastError();
}

}  // namespace gr

// ---- build without allocation ------------------------------------------------------
// Some callers cannot call cudaMalloc: plug-ins whose host application owns
// every byte of device memory (and hands the plug-in only the buffers of a
// call), and latency-critical loops in which a cudaMalloc / cudaFree would
// synchronise the device. For them the build's scratch (sort buffers, split
// levels, parent links, node counters, look-back words) lives in one
// file-scope device array, sized for kStaticMaxTriangles triangles; the caller
// passes the input soup and every output buffer.
//
// Every call shares this one array and it keeps the last call's contents: the
// part that must start at zero is cleared at the start of each call, and two
// calls that overlap on the GPU (different streams, no ordering between them)
// race on it.

namespace gr {
namespace {

constexpr uint32_t kStaticMaxTriangles = 1u << 17;  // 131,072 triangles

constexpr size_t round256(size_t x) { return (x + 255) & ~size_t(255); }

// Upper bound of scratch_layout(kStaticMaxTriangles): four per-triangle word
// arrays (sort buffers, leaf parents, node counters), the two far words per
// node, the left-over subtree per chunk, one level byte per gap, the centroid
// partials, the histograms, the sort's look-back words (per tile of each
// pass), tile counters and the error word, each rounded up to 256 bytes as
// scratch_layout rounds them.
constexpr size_t kStaticOsTiles = (kStaticMaxTriangles + kOsTile - 1) / kOsTile;
constexpr size_t kStaticChunks = (kStaticMaxTriangles + kRefitChunk - 1) / kRefitChunk;
constexpr size_t kStaticScratchBytes =
    4 * round256((size_t)kStaticMaxTriangles * 4) + round256((size_t)kStaticMaxTriangles * 16) +
    round256(sizeof(Sub) * kStaticChunks) + round256(kStaticMaxTriangles) +
    round256(sizeof(float) * 6 * kPartials) + 4096 + round256(4 * kStaticOsTiles * 256 * 4) + round256(16 * 4) +
    round256(4);

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

// Identity of the calling thread's current CUDA context (cuCtxGetCurrent +
// cuCtxGetId, reached through the runtime's driver entry points so the library
// does not link the driver library). A context's id is unique for the life of
// the process, so a device whose primary context was destroyed and created
// again (cudaDeviceReset) shows a new id.
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

cudaError_t current_context_id(unsigned long long* id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    if (!get_current || !get_id) {
        void* a = nullptr;
        void* b = nullptr;
        cudaDriverEntryPointQueryResult qa = cudaDriverEntryPointSymbolNotFound, qb = qa;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa);
        if (e == cudaSuccess) e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb);
        if (e != cudaSuccess) return e;
        if (qa != cudaDriverEntryPointSuccess || qb != cudaDriverEntryPointSuccess || !a || !b)
            return cudaErrorNotSupported;
        get_current = reinterpret_cast<CtxGetCurrentFn>(a);
        get_id = reinterpret_cast<CtxGetIdFn>(b);
    }
    CUcontext c = nullptr;
    if (get_current(&c) != CUDA_SUCCESS || !c) return cudaErrorDeviceUninitialized;
    if (get_id(c, id) != CUDA_SUCCESS) return cudaErrorDeviceUninitialized;
    return cudaSuccess;
}

constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
struct StaticScratch {
    unsigned long long ctx_id = 0;
    void* ptr = nullptr;
};
StaticScratch g_static[kMaxDevices];

// Device address of g_static_scratch on the current device (the caller has
// made `device` current). The array's name in host code is only a host-side
// stand-in, so its address is looked up with cudaGetSymbolAddress once per
// device at set-up, and again only if the device's context changed since.
cudaError_t static_scratch(int device, void** out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_static_mu);
    unsigned long long id = 0;
    cudaError_t e = current_context_id(&id);
    if (e != cudaSuccess) return e;
    StaticScratch& c = g_static[device];
    if (!c.ptr || c.ctx_id != id) {
        void* p = nullptr;
        if ((e = cudaGetSymbolAddress(&p, g_static_scratch)) != cudaSuccess) return e;
        c.ptr = p;
        c.ctx_id = id;
    }
    *out = c.ptr;
    return cudaSuccess;
}

}  // namespace

uint32_t lbvh_static_max_triangles() { return kStaticMaxTriangles; }

cudaError_t lbvh_build_static(const float* d_verts, uint32_t n, Node* nodes, Tri* tris, uint32_t* code,
                              uint32_t* prim, BvhMeta* meta, int device, int num_sms, cudaStream_t st) {
    cudaError_t e;
    void* base = nullptr;
    if ((e = static_scratch(device, &base)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(meta, 0, sizeof(BvhMeta), st)) != cudaSuccess) return e;
    if (n == 0) return cudaMemsetAsync(&meta->root, 0xFF, 4, st);
    Scratch s;
    if (scratch_layout(n, nullptr, &s) > kStaticScratchBytes) return cudaErrorInvalidValue;
    scratch_layout(n, (char*)base, &s);
    return launch_build(d_verts, n, s, nodes, tris, code, prim, meta, num_sms, st);
}

}  // namespace gr
