// 4-wide BVH layouts collapsed from the binary LBVH.
//
// Every binary node at even depth becomes a 4-wide node stored at its own
// (gap) index; its slots are its two children, each internal child replaced
// by that child's two children. Internal slot references are therefore nodes
// at even depth again, and the tree is the binary tree with every other level
// folded. Odd-depth indices stay unused, so no compaction pass is needed.
//
// Two encodings (gr_internal.h): FP32 child boxes (Node4, 128 B) and 8-bit
// quantised child boxes (Node4Q, 64 B). A quantised plane decodes as
// fma(q, 2^e, origin); the builder picks, for every child, the largest q whose
// decoded lower plane is <= the FP32 box and the smallest q whose decoded
// upper plane is >= it, using that same decode, so the decoded box always
// contains the FP32 box and a watertight hit inside it is never culled.
#include <algorithm>

#include "gr_internal.h"
#include "quant.cuh"

namespace gr {
namespace {

using namespace q8;

constexpr int kBlock = 256;

__global__ void __launch_bounds__(kBlock) k_bvh4(const Node* __restrict__ nodes, uint32_t n, Node4* out4, Node4Q* outq,
                                                 int quant, uint32_t* __restrict__ err) {
    const uint32_t count = n > 1 ? n - 1 : 1;
    for (uint32_t G = blockIdx.x * kBlock + threadIdx.x; G < count; G += gridDim.x * kBlock) {
        uint32_t depth = 0, x = G;
        int guard = 0;
        for (;;) {
            const uint32_t par = (uint32_t)nodes[x].q3.z;
            if (par == kNoNode) break;
            x = par;
            ++depth;
            if (++guard > 128) {
                atomicOr(err, ERR_RANGE);
                break;
            }
        }
        if (depth & 1u) continue;
        const Node nd = nodes[G];
        CBox box[4];
        int32_t ref[4] = {0, 0, 0, 0};
        int ns = 0;
        for (int k = 0; k < 2; ++k) {
            const int32_t c = k == 0 ? nd.q3.x : nd.q3.y;
            if (c < 0) {
                box[ns] = child_box(nd, k);
                ref[ns++] = c;
            } else {
                const Node cn = nodes[c];
                box[ns] = child_box(cn, 0);
                ref[ns++] = cn.q3.x;
                box[ns] = child_box(cn, 1);
                ref[ns++] = cn.q3.y;
            }
        }
        const uint32_t mask = (1u << ns) - 1u;
        if (!quant) {
            Node4 o;
            float lx[4] = {0, 0, 0, 0}, hx[4] = {0, 0, 0, 0}, ly[4] = {0, 0, 0, 0}, hy[4] = {0, 0, 0, 0};
            float lz[4] = {0, 0, 0, 0}, hz[4] = {0, 0, 0, 0};
            for (int k = 0; k < ns; ++k) {
                lx[k] = box[k].lo[0]; hx[k] = box[k].hi[0];
                ly[k] = box[k].lo[1]; hy[k] = box[k].hi[1];
                lz[k] = box[k].lo[2]; hz[k] = box[k].hi[2];
            }
            o.lox = make_float4(lx[0], lx[1], lx[2], lx[3]);
            o.hix = make_float4(hx[0], hx[1], hx[2], hx[3]);
            o.loy = make_float4(ly[0], ly[1], ly[2], ly[3]);
            o.hiy = make_float4(hy[0], hy[1], hy[2], hy[3]);
            o.loz = make_float4(lz[0], lz[1], lz[2], lz[3]);
            o.hiz = make_float4(hz[0], hz[1], hz[2], hz[3]);
            o.child = make_int4(ref[0], ref[1], ref[2], ref[3]);
            o.meta = make_uint4(mask, 0, 0, 0);
            out4[G] = o;
        } else {
            float org[3], scale[3];
            uint32_t be[3];
            for (int a = 0; a < 3; ++a) {
                float lo = box[0].lo[a], hi = box[0].hi[a];
                for (int k = 1; k < ns; ++k) {
                    lo = fminf(lo, box[k].lo[a]);
                    hi = fmaxf(hi, box[k].hi[a]);
                }
                const int e = pick_exponent(lo, hi);
                org[a] = lo;
                be[a] = (uint32_t)(e + 127);
                scale[a] = __uint_as_float(be[a] << 23);
            }
            uint32_t w[6] = {0, 0, 0, 0, 0, 0};  // qlo.x, qhi.x, qlo.y, qhi.y, qlo.z, qhi.z
            for (int k = 0; k < ns; ++k)
                for (int a = 0; a < 3; ++a) {
                    w[2 * a] |= quant_lo(box[k].lo[a], scale[a], org[a]) << (8 * k);
                    w[2 * a + 1] |= quant_hi(box[k].hi[a], scale[a], org[a]) << (8 * k);
                }
            Node4Q o;
            o.q0 = make_float4(org[0], org[1], org[2], __uint_as_float(be[0] | (be[1] << 8) | (be[2] << 16) | (mask << 24)));
            o.q1 = make_uint4(w[0], w[1], w[2], w[3]);
            o.q2 = make_uint4(w[4], w[5], 0, 0);
            o.child = make_int4(ref[0], ref[1], ref[2], ref[3]);
            outq[G] = o;
        }
    }
}

}  // namespace

cudaError_t bvh4_build(BvhBuffers& b, uint32_t n, int layout, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const size_t count = n > 1 ? n - 1 : 1;
    cudaError_t e;
    const bool quant = layout == kLayoutBvh4Q8;
    DevBuf& out = quant ? b.nodes4q : b.nodes4;
    if ((e = out.ensure(count * (quant ? sizeof(Node4Q) : sizeof(Node4)))) != cudaSuccess) return e;
    // odd-depth slots are never read; clear them so exports are deterministic
    if ((e = cudaMemsetAsync(out.p, 0, count * (quant ? sizeof(Node4Q) : sizeof(Node4)), s)) != cudaSuccess) return e;
    const int grid = (int)std::min<size_t>((count + kBlock - 1) / kBlock, 4096);
    k_bvh4<<<grid, kBlock, 0, s>>>((const Node*)b.nodes.p, n, (Node4*)b.nodes4.p, (Node4Q*)b.nodes4q.p, quant ? 1 : 0,
                                   &((BvhMeta*)b.meta.p)->err);
    return cudaGetLastError();
}

}  // namespace gr
