// Device helpers shared by the wide-node builders (bvh4.cu, bvh8.cu): child
// boxes of a binary node and the outward 8-bit quantisation of box planes.
// A quantised plane decodes as fma(q, 2^e, origin); the builders pick, for
// every child, the largest q whose decoded lower plane is <= the FP32 box and
// the smallest q whose decoded upper plane is >= it, using that same decode,
// so a decoded box always contains its FP32 box.
#pragma once

#include "gr_internal.h"

namespace gr {
namespace q8 {

struct CBox {
    float lo[3], hi[3];
};

__device__ __forceinline__ CBox child_box(const Node& nd, int slot) {
    CBox b;
    const float4 xy = slot == 0 ? nd.q0 : nd.q1;
    b.lo[0] = xy.x; b.hi[0] = xy.y; b.lo[1] = xy.z; b.hi[1] = xy.w;
    b.lo[2] = slot == 0 ? nd.q2.x : nd.q2.z;
    b.hi[2] = slot == 0 ? nd.q2.y : nd.q2.w;
    return b;
}

__device__ __forceinline__ float decode(int q, float scale, float origin) { return __fmaf_rn((float)q, scale, origin); }

// Exponent e (2^e per quantisation step) so 255 steps from lo reach hi.
__device__ __forceinline__ int pick_exponent(float lo, float hi) {
    const float extent = __fsub_rn(hi, lo);
    int e = -126;
    if (extent > 0.0f) {
        int ex;
        frexpf(__fdiv_rn(extent, 255.0f), &ex);
        e = max(-126, min(127, ex));
    }
    while (e < 127 && decode(255, __uint_as_float((uint32_t)(e + 127) << 23), lo) < hi) ++e;
    return e;
}

__device__ __forceinline__ uint32_t quant_lo(float v, float scale, float origin) {
    int q = (int)fminf(fmaxf(floorf(__fdiv_rn(__fsub_rn(v, origin), scale)), 0.0f), 255.0f);
    while (q > 0 && decode(q, scale, origin) > v) --q;
    while (q < 255 && decode(q + 1, scale, origin) <= v) ++q;
    return (uint32_t)q;
}

__device__ __forceinline__ uint32_t quant_hi(float v, float scale, float origin) {
    int q = (int)fminf(fmaxf(ceilf(__fdiv_rn(__fsub_rn(v, origin), scale)), 0.0f), 255.0f);
    while (q < 255 && decode(q, scale, origin) < v) ++q;
    while (q > 0 && decode(q - 1, scale, origin) >= v) --q;
    return (uint32_t)q;
}

}  // namespace q8
}  // namespace gr
