// Closest-hit and any-hit traversal (binary, 4-wide FP32, 4-wide and 8-wide
// 8-bit quantised node layouts).
//
// Replaces trace_kernel / trace_shadow_kernel (src/renderer/pathtracer_kernel.h
// :175-308). Differences by design:
//   - persistent warps with dynamic refill: a fixed grid of warps pulls rays
//     from a global counter, and a warp refills its idle lanes whenever at
//     least kRefillRays of them have finished, until the queue is drained;
//   - child boxes live in the parent node and are fetched as 32-byte vector
//     loads; all children are tested at once and the nearest is visited first;
//   - a short per-thread stack in shared memory (8, 12 or 16 entries, chosen by
//     the autotuner with the block size), spilling to local memory past it;
//   - the FP32 watertight triangle test (Woop, Benthin, Wald, JCGT 2013) on
//     leaf-order triangle copies instead of the reference's FP64
//     Moller-Trumbore through 408-byte Triangle records.
// Every float operation is an explicit round-to-nearest intrinsic so the
// result is reproducible by the host oracle bit for bit.
#include <algorithm>

#include "gr_internal.h"
#include "traverse.cuh"

namespace gr {
namespace {

struct RaySrc {
    const float4* __restrict__ rays;
    float4* __restrict__ hits;
    uint64_t n;
    const void* nodes;
    const Tri* tris;
    uint32_t root;
    __device__ __forceinline__ uint32_t load(uint64_t i, float4& r0, float4& r1, const void*& nd, const Tri*& tr) const {
        r0 = __ldg(rays + 2 * i);
        r1 = __ldg(rays + 2 * i + 1);
        nd = nodes;
        tr = tris;
        return root;
    }
    __device__ __forceinline__ void finish(uint64_t i, const trav::Lane& L) const {
        hits[i] = L.best_prim == 0xFFFFFFFFu ? make_float4(L.p.tmax, __int_as_float(-1), 0.0f, 0.0f)
                                             : make_float4(L.best_t, __uint_as_float(L.best_prim), L.bu, L.bv);
    }
};

template <bool ANY, int LAYOUT, int SSTACK>
__global__ void __launch_bounds__(trav::kMaxTraceThreads, 4) k_trace(const void* __restrict__ nodes, const Tri* __restrict__ tris,
                                                                  const BvhMeta* __restrict__ meta,
                                                                  const float4* __restrict__ rays, uint64_t n,
                                                                  float4* __restrict__ hits, unsigned long long* counter,
                                                                  uint32_t* err) {
    extern __shared__ int2 s_stack[];
    RaySrc src{rays, hits, n, nodes, tris, meta->root};
    trav::traverse_loop<ANY, LAYOUT, SSTACK, trav::kRefillRays>(src, counter, err, s_stack);
}

template <bool ANY, int LAYOUT, int SSTACK>
cudaError_t launch(const BvhDevice& bvh, const void* nodes, int block, const float4* r, uint64_t n, float4* h,
                   unsigned long long* counter, uint32_t* err, int num_sms, cudaStream_t s) {
    static int occ[3] = {0, 0, 0};  // per block size 64 / 128 / 256
    const int bi = block == 64 ? 0 : (block == 128 ? 1 : 2);
    const size_t smem = trav::traverse_smem(LAYOUT, SSTACK, block);
    if (occ[bi] == 0) {
        const cudaError_t e =
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[bi], k_trace<ANY, LAYOUT, SSTACK>, block, smem);
        if (e != cudaSuccess) return e;
        if (occ[bi] < 1) occ[bi] = 1;
    }
    const uint64_t warps_needed = (n + 31) / 32;
    const uint64_t blocks_needed = (warps_needed + block / 32 - 1) / (block / 32);
    const int grid = (int)std::min<uint64_t>((uint64_t)num_sms * occ[bi], blocks_needed);
    k_trace<ANY, LAYOUT, SSTACK><<<grid, block, smem, s>>>(nodes, bvh.tris, bvh.meta, r, n, h, counter, err);
    return cudaGetLastError();
}

template <bool ANY, int LAYOUT>
cudaError_t launch_s(const BvhDevice& bvh, const void* nodes, const TraceTuning& t, const float4* r, uint64_t n,
                     float4* h, unsigned long long* c, uint32_t* err, int num_sms, cudaStream_t s) {
    if (t.sstack == 8) return launch<ANY, LAYOUT, 8>(bvh, nodes, t.block, r, n, h, c, err, num_sms, s);
    if (t.sstack == 16) return launch<ANY, LAYOUT, 16>(bvh, nodes, t.block, r, n, h, c, err, num_sms, s);
    return launch<ANY, LAYOUT, 12>(bvh, nodes, t.block, r, n, h, c, err, num_sms, s);
}

}  // namespace

bool tuning_valid(const TraceTuning& t) {
    return t.layout >= 0 && t.layout < kNumLayouts && (t.block == 64 || t.block == 128 || t.block == 256) &&
           (t.sstack == 8 || t.sstack == 12 || t.sstack == 16);
}

cudaError_t trace_launch(const BvhDevice& bvh, const void* nodes, const TraceTuning& tune, const gr_ray* d_rays,
                         uint64_t n, gr_hit* d_hits, int any_hit, unsigned long long* d_counter, uint32_t* d_err,
                         int num_sms, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if (!tuning_valid(tune)) return cudaErrorInvalidValue;
    if (reinterpret_cast<uintptr_t>(nodes) & 31) return cudaErrorMisalignedAddress;  // 32-byte node loads
    cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    const float4* r = reinterpret_cast<const float4*>(d_rays);
    float4* h = reinterpret_cast<float4*>(d_hits);
    switch (tune.layout * 2 + (any_hit ? 1 : 0)) {
        case 0: return launch_s<false, kLayoutBvh2>(bvh, nodes, tune, r, n, h, d_counter, d_err, num_sms, s);
        case 1: return launch_s<true, kLayoutBvh2>(bvh, nodes, tune, r, n, h, d_counter, d_err, num_sms, s);
        case 2: return launch_s<false, kLayoutBvh4>(bvh, nodes, tune, r, n, h, d_counter, d_err, num_sms, s);
        case 3: return launch_s<true, kLayoutBvh4>(bvh, nodes, tune, r, n, h, d_counter, d_err, num_sms, s);
        case 4: return launch_s<false, kLayoutBvh4Q8>(bvh, nodes, tune, r, n, h, d_counter, d_err, num_sms, s);
        case 5: return launch_s<true, kLayoutBvh4Q8>(bvh, nodes, tune, r, n, h, d_counter, d_err, num_sms, s);
        case 6: return launch_s<false, kLayoutBvh8Q8>(bvh, nodes, tune, r, n, h, d_counter, d_err, num_sms, s);
        case 7: return launch_s<true, kLayoutBvh8Q8>(bvh, nodes, tune, r, n, h, d_counter, d_err, num_sms, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace gr
