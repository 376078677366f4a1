// Traversal core shared by the ray-query kernels (trace.cu) and the
// integrator's queue kernels (render.cu): ray set-up, child-box slab test,
// FP32 watertight triangle test, one traversal step, and the persistent
// dynamic-fetch loop. Every float operation is an explicit round-to-nearest
// intrinsic so the host oracle reproduces hits bit for bit.
#pragma once

#include "gr_internal.h"

namespace gr {
namespace trav {

constexpr int kTraceThreads = 128;
constexpr int kShortStack = 12;
constexpr int kStackMax = 64;

struct RayW {
    float ox, oy, oz, tmin, tmax;
    float sx, sy, sz;
    int kx, ky, kz;
    float ix, iy, iz;     // reciprocal direction (near-zero components clamped)
    float nox, noy, noz;  // -origin * reciprocal direction
};

__device__ __forceinline__ float pick(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }

__device__ __forceinline__ RayW prepare(const float4 r0, const float4 r1) {
    RayW p;
    p.ox = r0.x; p.oy = r0.y; p.oz = r0.z;
    const float dx = r0.w, dy = r1.x, dz = r1.y;
    p.tmin = r1.z;
    p.tmax = r1.w;
    const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
    int kz = 0;
    float m = ax;
    if (ay > m) { kz = 1; m = ay; }
    if (az > m) kz = 2;
    int kx = kz == 2 ? 0 : kz + 1;
    int ky = kx == 2 ? 0 : kx + 1;
    const float dkz = pick(dx, dy, dz, kz);
    if (dkz < 0.0f) { const int t = kx; kx = ky; ky = t; }
    p.kx = kx; p.ky = ky; p.kz = kz;
    p.sx = __fdiv_rn(pick(dx, dy, dz, kx), dkz);
    p.sy = __fdiv_rn(pick(dx, dy, dz, ky), dkz);
    p.sz = __frcp_rn(dkz);
    const float eps = 0x1p-80f;
    const float cx = fabsf(dx) > eps ? dx : copysignf(eps, dx);
    const float cy = fabsf(dy) > eps ? dy : copysignf(eps, dy);
    const float cz = fabsf(dz) > eps ? dz : copysignf(eps, dz);
    p.ix = __frcp_rn(cx); p.iy = __frcp_rn(cy); p.iz = __frcp_rn(cz);
    p.nox = -__fmul_rn(p.ox, p.ix); p.noy = -__fmul_rn(p.oy, p.iy); p.noz = -__fmul_rn(p.oz, p.iz);
    return p;
}

__device__ __forceinline__ bool slab(const RayW& p, float lox, float hix, float loy, float hiy, float loz, float hiz,
                                     float tbest, float& tn) {
    const float x0 = __fmaf_rn(lox, p.ix, p.nox), x1 = __fmaf_rn(hix, p.ix, p.nox);
    const float y0 = __fmaf_rn(loy, p.iy, p.noy), y1 = __fmaf_rn(hiy, p.iy, p.noy);
    const float z0 = __fmaf_rn(loz, p.iz, p.noz), z1 = __fmaf_rn(hiz, p.iz, p.noz);
    const float tnear = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), p.tmin));
    const float tfar = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fminf(fmaxf(z0, z1), tbest));
    tn = tnear;
    return tnear <= tfar;
}

__device__ __forceinline__ bool tri_test(const RayW& p, const float4 a, const float4 b, const float4 c, float tbest,
                                         float& t, float& u, float& v) {
    const float Ax0 = __fsub_rn(a.x, p.ox), Ay0 = __fsub_rn(a.y, p.oy), Az0 = __fsub_rn(a.z, p.oz);
    const float Bx0 = __fsub_rn(b.x, p.ox), By0 = __fsub_rn(b.y, p.oy), Bz0 = __fsub_rn(b.z, p.oz);
    const float Cx0 = __fsub_rn(c.x, p.ox), Cy0 = __fsub_rn(c.y, p.oy), Cz0 = __fsub_rn(c.z, p.oz);
    const float Akz = pick(Ax0, Ay0, Az0, p.kz), Bkz = pick(Bx0, By0, Bz0, p.kz), Ckz = pick(Cx0, Cy0, Cz0, p.kz);
    const float Ax = __fmaf_rn(-p.sx, Akz, pick(Ax0, Ay0, Az0, p.kx));
    const float Ay = __fmaf_rn(-p.sy, Akz, pick(Ax0, Ay0, Az0, p.ky));
    const float Bx = __fmaf_rn(-p.sx, Bkz, pick(Bx0, By0, Bz0, p.kx));
    const float By = __fmaf_rn(-p.sy, Bkz, pick(Bx0, By0, Bz0, p.ky));
    const float Cx = __fmaf_rn(-p.sx, Ckz, pick(Cx0, Cy0, Cz0, p.kx));
    const float Cy = __fmaf_rn(-p.sy, Ckz, pick(Cx0, Cy0, Cz0, p.ky));
    const float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    const float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    const float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.0f) return false;
    const float Az = __fmul_rn(p.sz, Akz), Bz = __fmul_rn(p.sz, Bkz), Cz = __fmul_rn(p.sz, Ckz);
    const float T = __fmaf_rn(U, Az, __fmaf_rn(V, Bz, __fmul_rn(W, Cz)));
    const float rcp = __frcp_rn(det);
    const float tt = __fmul_rn(T, rcp);
    if (!(tt >= p.tmin && tt <= tbest)) return false;
    t = tt;
    u = __fmul_rn(V, rcp);
    v = __fmul_rn(W, rcp);
    return true;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Per-lane traversal state. A lane owns one ray at a time; when its ray
// finishes the lane goes idle and is refilled with a new ray once enough lanes
// of the warp are idle, so long-tailed rays do not hold a whole warp.
struct Lane {
    const Node* nodes;  // BVH of this lane's ray (rays of one queue may belong to different scenes)
    const Tri* tris;
    RayW p;
    float best_t, bu, bv;
    uint32_t best_prim;
    uint64_t ray;
    int32_t node;
    int sp;
};

// Processes one node for the lane; returns true when the ray is finished.
template <bool ANY>
__device__ __forceinline__ bool trace_step(Lane& L, int2 (*s_stack)[kTraceThreads], int2* l_stack, uint32_t* err) {
    const int tid = threadIdx.x;
    const Node* __restrict__ nodes = L.nodes;
    const Tri* __restrict__ tris = L.tris;
    const float4* q = reinterpret_cast<const float4*>(nodes + L.node);
    const float4 q0 = __ldg(q), q1 = __ldg(q + 1), q2 = __ldg(q + 2);
    const int4 q3 = __ldg(reinterpret_cast<const int4*>(q + 3));
    float tn0, tn1;
    const bool h0 = slab(L.p, q0.x, q0.y, q0.z, q0.w, q2.x, q2.y, L.best_t, tn0);
    const bool h1 = slab(L.p, q1.x, q1.y, q1.z, q1.w, q2.z, q2.w, L.best_t, tn1);
    const bool swap = h0 && h1 && tn1 < tn0;
    const int32_t cn = swap ? q3.y : q3.x, cf = swap ? q3.x : q3.y;
    const float tnf = swap ? tn0 : tn1;
    const bool hn = swap ? h1 : h0, hf = swap ? h0 : h1;
    int32_t next = -1;
    bool have = false;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
        const bool h = s == 0 ? hn : hf;
        const int32_t c = s == 0 ? cn : cf;
        if (!h) continue;
        if (c < 0) {
            const Tri* tr = tris + (uint32_t)(~c);
            const float4 a = __ldg(&tr->a), b = __ldg(&tr->b), cc = __ldg(&tr->c);
            float t, u, v;
            if (tri_test(L.p, a, b, cc, L.best_t, t, u, v)) {
                const uint32_t prim = __float_as_uint(a.w);
                if (ANY) {
                    L.best_t = t; L.bu = u; L.bv = v; L.best_prim = prim;
                    return true;
                }
                if (t < L.best_t || prim < L.best_prim) {
                    L.best_t = t; L.bu = u; L.bv = v; L.best_prim = prim;
                }
            }
        } else if (!have) {
            next = c;
            have = true;
        } else {
            if (L.sp < kShortStack) {
                s_stack[L.sp][tid] = make_int2(c, __float_as_int(tnf));
            } else if (L.sp < kStackMax) {
                l_stack[L.sp - kShortStack] = make_int2(c, __float_as_int(tnf));
            } else {
                atomicOr(err, ERR_STACK);
                return true;
            }
            ++L.sp;
        }
    }
    if (!have) {
        for (;;) {
            if (L.sp == 0) return true;
            --L.sp;
            const int2 e = L.sp < kShortStack ? s_stack[L.sp][tid] : l_stack[L.sp - kShortStack];
            if (ANY || __int_as_float(e.y) <= L.best_t) { next = e.x; break; }
        }
    }
    L.node = next;
    return false;
}

// Refill when at least this many lanes of a warp are idle.
constexpr int kRefillLanes = 8;


// Persistent dynamic-fetch loop. `Src` supplies the work:
//   uint64_t n                                        number of rays
//   uint32_t load(uint64_t i, float4& r0, float4& r1, const Node*& nodes,
//                 const Tri*& tris)                   ray i (reference Ray layout) and
//                                                     its BVH; returns the root node
//   void finish(uint64_t i, const Lane& L)            ray i is done (L.best_prim ==
//                                                     0xFFFFFFFF means a miss)
template <bool ANY, class Src>
__device__ __forceinline__ void traverse_loop(Src& src, unsigned long long* counter, uint32_t* err,
                                              int2 (*s_stack)[kTraceThreads]) {
    int2 l_stack[kStackMax - kShortStack];
    const int lane = threadIdx.x & 31;
    const uint32_t ltmask = lanemask_lt();
    const uint64_t n = src.n;
    Lane L;
    bool active = false;
    bool exhausted = false;
    for (;;) {
        const uint32_t idle = __ballot_sync(0xFFFFFFFFu, !active);
        const int nidle = __popc(idle);
        if (!exhausted && (nidle >= kRefillLanes || nidle == 32)) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(counter, (unsigned long long)nidle);
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (base + nidle >= n) exhausted = true;
            if (!active) {
                const uint64_t i = base + __popc(idle & ltmask);
                if (i < n) {
                    float4 r0, r1;
                    const uint32_t root = src.load(i, r0, r1, L.nodes, L.tris);
                    L.p = prepare(r0, r1);
                    L.best_t = L.p.tmax;
                    L.bu = 0.0f;
                    L.bv = 0.0f;
                    L.best_prim = 0xFFFFFFFFu;
                    L.ray = i;
                    L.node = (int32_t)root;
                    L.sp = 0;
                    active = true;
                    if (root == kNoNode) {
                        src.finish(i, L);
                        active = false;
                    }
                }
            }
        }
        if (__ballot_sync(0xFFFFFFFFu, active) == 0) {
            if (exhausted) break;
            continue;
        }
        if (active && trace_step<ANY>(L, s_stack, l_stack, err)) {
            src.finish(L.ray, L);
            active = false;
        }
    }
}

}  // namespace trav
}  // namespace gr
