// Traversal core shared by the ray-query kernels (trace.cu) and the
// integrator's queue kernels (render.cu): ray set-up, child-box slab test,
// FP32 watertight triangle test, one traversal step, and the persistent
// dynamic-fetch loop. Every float operation is an explicit round-to-nearest
// intrinsic so the host oracle reproduces hits bit for bit.
#pragma once

#include "gr_internal.h"

namespace gr {
namespace trav {

// Launch shape and short-stack depth are tuning parameters (the autotuner
// picks them per device and workload); these are the defaults.
constexpr int kTraceThreads = 128;
constexpr int kShortStack = 12;
constexpr int kStackMax = 64;
constexpr int kMaxTraceThreads = 256;

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

// Relative slack on every cull: a box (or a deferred stack entry) is kept
// while its entry distance is within (1 + 2^-20) of the exit / closest-hit
// distance, so a triangle whose hit distance rounds an ulp below its box's
// entry distance is still reached and the closest hit does not depend on the
// order boxes are visited in.
constexpr float kCullSlack = 1.00000095367431640625f;  // 1 + 2^-20

__device__ __forceinline__ bool slab(const RayW& p, float lox, float hix, float loy, float hiy, float loz, float hiz,
                                     float tbest, float& tn) {
    const float x0 = __fmaf_rn(lox, p.ix, p.nox), x1 = __fmaf_rn(hix, p.ix, p.nox);
    const float y0 = __fmaf_rn(loy, p.iy, p.noy), y1 = __fmaf_rn(hiy, p.iy, p.noy);
    const float z0 = __fmaf_rn(loz, p.iz, p.noz), z1 = __fmaf_rn(hiz, p.iz, p.noz);
    const float tnear = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), p.tmin));
    const float tfar = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fminf(fmaxf(z0, z1), tbest));
    tn = tnear;
    return tnear <= __fmul_rn(tfar, kCullSlack);
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

// 32-byte read-only load (ld.global.nc.v8, sm_100 and later): one L1 sector
// per lane per request instead of two 16-byte requests. `p` must be 32-byte
// aligned; node arrays are separate allocations with 64- or 128-byte records.
__device__ __forceinline__ void ldg32B(const void* p, float4& a, float4& b) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

__device__ __forceinline__ int4 as_int4(const float4 f) {
    return make_int4(__float_as_int(f.x), __float_as_int(f.y), __float_as_int(f.z), __float_as_int(f.w));
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
    const void* nodes;  // BVH of this lane's ray (rays of one queue may belong to different scenes)
    const Tri* tris;
    RayW p;
    float best_t, bu, bv;
    uint32_t best_prim;
    uint64_t ray;
    int32_t node;
    int sp;
};

// Tests leaf triangle `c` (~sorted position); returns true when an any-hit
// query is answered. Closest-hit ties at equal t go to the smaller prim id.
template <bool ANY>
__device__ __forceinline__ bool leaf(Lane& L, int32_t c) {
    const Tri* tr = L.tris + (uint32_t)(~c);
    const float4 a = __ldg(&tr->a), b = __ldg(&tr->b), cc = __ldg(&tr->c);
    float t, u, v;
    if (!tri_test(L.p, a, b, cc, L.best_t, t, u, v)) return false;
    const uint32_t prim = __float_as_uint(a.w);
    if (ANY) {
        L.best_t = t; L.bu = u; L.bv = v; L.best_prim = prim;
        return true;
    }
    if (t < L.best_t || prim < L.best_prim) {
        L.best_t = t; L.bu = u; L.bv = v; L.best_prim = prim;
    }
    return false;
}

// Pushes a deferred node with its entry distance; false on overflow. The
// first SSTACK entries of a thread live in shared memory ([entry][thread],
// conflict-free), deeper entries in a local array.
template <int SSTACK>
__device__ __forceinline__ bool push(Lane& L, int32_t c, float tn, int2* s_stack, int2* l_stack, uint32_t* err) {
    if (L.sp < SSTACK) {
        s_stack[L.sp * blockDim.x + threadIdx.x] = make_int2(c, __float_as_int(tn));
    } else if (L.sp < kStackMax) {
        l_stack[L.sp - SSTACK] = make_int2(c, __float_as_int(tn));
    } else {
        atomicOr(err, ERR_STACK);
        return false;
    }
    ++L.sp;
    return true;
}

// Pops the next deferred node still in front of the closest hit; false when
// the stack is empty (the ray is finished).
template <bool ANY, int SSTACK>
__device__ __forceinline__ bool pop(Lane& L, const int2* s_stack, const int2* l_stack, int32_t& next) {
    for (;;) {
        if (L.sp == 0) return false;
        --L.sp;
        const int2 e = L.sp < SSTACK ? s_stack[L.sp * blockDim.x + threadIdx.x] : l_stack[L.sp - SSTACK];
        if (ANY || __int_as_float(e.y) <= __fmul_rn(L.best_t, kCullSlack)) {
            next = e.x;
            return true;
        }
    }
}

// One binary node: both child boxes, nearer first; leaves tested inline.
// Returns true when the ray is finished.
template <bool ANY, int SSTACK>
__device__ __forceinline__ bool trace_step2(Lane& L, int2* s_stack, int2* l_stack, uint32_t* err) {
    const float4* q = reinterpret_cast<const float4*>(static_cast<const Node*>(L.nodes) + L.node);
    float4 q0, q1, q2, q3f;
    ldg32B(q, q0, q1);
    ldg32B(q + 2, q2, q3f);
    const int4 q3 = as_int4(q3f);
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
            if (leaf<ANY>(L, c)) return true;
        } else if (!have) {
            next = c;
            have = true;
        } else if (!push<SSTACK>(L, c, tnf, s_stack, l_stack, err)) {
            return true;
        }
    }
    if (!have && !pop<ANY, SSTACK>(L, s_stack, l_stack, next)) return true;
    L.node = next;
    return false;
}

// Decoded quantised plane: origin + q * 2^e in one rounding.
__device__ __forceinline__ float qplane(uint32_t word, int k, float scale, float origin) {
    return __fmaf_rn((float)((word >> (8 * k)) & 0xFFu), scale, origin);
}

// One 4-wide node (FP32 or 8-bit quantised boxes): the hit children are
// visited in order of (entry distance, slot); leaves tested inline, the nearest
// inner child visited next, the other inner children pushed so the nearer pop
// first. Returns true when the ray is finished.
template <bool ANY, bool QUANT, int SSTACK>
__device__ __forceinline__ bool trace_step4(Lane& L, int2* s_stack, int2* l_stack, uint32_t* err) {
    float tn[4];
    bool h[4];
    int32_t c[4];
    if (QUANT) {
        const Node4Q* nd = static_cast<const Node4Q*>(L.nodes) + L.node;
        float4 q0, q1f, q2f, chf;
        ldg32B(&nd->q0, q0, q1f);
        ldg32B(&nd->q2, q2f, chf);
        const int4 q1i = as_int4(q1f), q2i = as_int4(q2f), ch = as_int4(chf);
        const uint4 q1 = make_uint4(q1i.x, q1i.y, q1i.z, q1i.w), q2 = make_uint4(q2i.x, q2i.y, q2i.z, q2i.w);
        const uint32_t meta = __float_as_uint(q0.w);
        const float sx = __uint_as_float((meta & 0xFFu) << 23);
        const float sy = __uint_as_float(((meta >> 8) & 0xFFu) << 23);
        const float sz = __uint_as_float(((meta >> 16) & 0xFFu) << 23);
        const uint32_t mask = meta >> 24;
        c[0] = ch.x; c[1] = ch.y; c[2] = ch.z; c[3] = ch.w;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            h[k] = false;
            tn[k] = 0.0f;
            if (mask & (1u << k))
                h[k] = slab(L.p, qplane(q1.x, k, sx, q0.x), qplane(q1.y, k, sx, q0.x), qplane(q1.z, k, sy, q0.y),
                            qplane(q1.w, k, sy, q0.y), qplane(q2.x, k, sz, q0.z), qplane(q2.y, k, sz, q0.z),
                            L.best_t, tn[k]);
        }
    } else {
        const Node4* nd = static_cast<const Node4*>(L.nodes) + L.node;
        float4 lox, hix, loy, hiy, loz, hiz, chf, metaf;
        ldg32B(&nd->lox, lox, hix);
        ldg32B(&nd->loy, loy, hiy);
        ldg32B(&nd->loz, loz, hiz);
        ldg32B(&nd->child, chf, metaf);
        const int4 ch = as_int4(chf);
        const uint32_t mask = __float_as_uint(metaf.x);
        c[0] = ch.x; c[1] = ch.y; c[2] = ch.z; c[3] = ch.w;
        const float lx[4] = {lox.x, lox.y, lox.z, lox.w}, hx[4] = {hix.x, hix.y, hix.z, hix.w};
        const float ly[4] = {loy.x, loy.y, loy.z, loy.w}, hy[4] = {hiy.x, hiy.y, hiy.z, hiy.w};
        const float lz[4] = {loz.x, loz.y, loz.z, loz.w}, hz[4] = {hiz.x, hiz.y, hiz.z, hiz.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            h[k] = false;
            tn[k] = 0.0f;
            if (mask & (1u << k)) h[k] = slab(L.p, lx[k], hx[k], ly[k], hy[k], lz[k], hz[k], L.best_t, tn[k]);
        }
    }
    int rank[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        int r = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (j != k && h[j] && (tn[j] < tn[k] || (tn[j] == tn[k] && j < k))) ++r;
        rank[k] = r;
    }
    int32_t next = -1;
    bool have = false;
    int np = 0;
    int32_t pc0 = 0, pc1 = 0, pc2 = 0;
    float pt0 = 0.0f, pt1 = 0.0f, pt2 = 0.0f;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        int32_t cr = 0;
        float tr = 0.0f;
        bool hr = false;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (h[k] && rank[k] == r) {
                cr = c[k];
                tr = tn[k];
                hr = true;
            }
        if (!hr) continue;
        if (cr < 0) {
            if (leaf<ANY>(L, cr)) return true;
        } else if (!have) {
            next = cr;
            have = true;
        } else {
            if (np == 0) { pc0 = cr; pt0 = tr; }
            else if (np == 1) { pc1 = cr; pt1 = tr; }
            else { pc2 = cr; pt2 = tr; }
            ++np;
        }
    }
    if (np > 2 && !push<SSTACK>(L, pc2, pt2, s_stack, l_stack, err)) return true;
    if (np > 1 && !push<SSTACK>(L, pc1, pt1, s_stack, l_stack, err)) return true;
    if (np > 0 && !push<SSTACK>(L, pc0, pt0, s_stack, l_stack, err)) return true;
    if (!have && !pop<ANY, SSTACK>(L, s_stack, l_stack, next)) return true;
    L.node = next;
    return false;
}

template <bool ANY, int LAYOUT, int SSTACK>
__device__ __forceinline__ bool trace_step(Lane& L, int2* s_stack, int2* l_stack, uint32_t* err) {
    if (LAYOUT == kLayoutBvh2) return trace_step2<ANY, SSTACK>(L, s_stack, l_stack, err);
    return trace_step4<ANY, LAYOUT == kLayoutBvh4Q8, SSTACK>(L, s_stack, l_stack, err);
}

// Refill when at least this many lanes of a warp are idle.
constexpr int kRefillLanes = 8;

// Persistent dynamic-fetch loop. `Src` supplies the work:
//   uint64_t n                                        number of rays
//   uint32_t load(uint64_t i, float4& r0, float4& r1, const void*& nodes,
//                 const Tri*& tris)                   ray i (reference Ray layout) and
//                                                     its BVH (nodes of layout LAYOUT);
//                                                     returns the root node
//   void finish(uint64_t i, const Lane& L)            ray i is done (L.best_prim ==
//                                                     0xFFFFFFFF means a miss)
// The shared stack has SSTACK x blockDim.x int2 entries (dynamic shared memory).
template <bool ANY, int LAYOUT, int SSTACK, class Src>
__device__ __forceinline__ void traverse_loop(Src& src, unsigned long long* counter, uint32_t* err, int2* s_stack) {
    int2 l_stack[kStackMax - SSTACK];
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
        if (active && trace_step<ANY, LAYOUT, SSTACK>(L, s_stack, l_stack, err)) {
            src.finish(L.ray, L);
            active = false;
        }
    }
}

}  // namespace trav
}  // namespace gr
