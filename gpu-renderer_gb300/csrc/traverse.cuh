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
// Traversal kernels are declared __launch_bounds__(kMaxTraceThreads, 4): at
// most 64 registers, so 4 blocks of 256 threads stay resident per SM (the
// packed plane arithmetic would otherwise take 80 and lose a block: measured
// 3 % slower than the scalar version, 7 % faster with the bound).

struct RayW {
    float ox, oy, oz, tmin, tmax;
    float sx, sy, sz;
    int kx, ky, kz;
    float ix, iy, iz;     // reciprocal direction (near-zero components clamped)
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
    return p;
}

// Relative slack on every cull: a box (or a deferred stack entry) is kept
// while its entry distance is within (1 + 2^-16) of the exit / closest-hit
// distance. A plane's distance is (plane - o) * (1/d), three roundings and so
// within 3 ulps of the exact value relative to itself, so a box that contains
// a hit point is never culled by rounding, and a triangle whose computed hit
// distance is a few ulps below its box's entry distance is still reached: the
// closest hit does not depend on the order boxes are visited in or on the
// node layout. (A form like fma(plane, 1/d, -o/d) has an absolute error of
// order ulp(o/d), which culled grazing rays that start on a surface.)
constexpr float kCullSlack = 1.0000152587890625f;  // 1 + 2^-16

__device__ __forceinline__ float plane_t(float plane, float o, float inv) {
    return __fmul_rn(__fsub_rn(plane, o), inv);
}

__device__ __forceinline__ bool slab(const RayW& p, float lox, float hix, float loy, float hiy, float loz, float hiz,
                                     float tbest, float& tn) {
    const float x0 = plane_t(lox, p.ox, p.ix), x1 = plane_t(hix, p.ox, p.ix);
    const float y0 = plane_t(loy, p.oy, p.iy), y1 = plane_t(hiy, p.oy, p.iy);
    const float z0 = plane_t(loz, p.oz, p.iz), z1 = plane_t(hiz, p.oz, p.iz);
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

// ---- 8-wide quantised nodes ----------------------------------------------------

__device__ __forceinline__ float max3(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

__device__ __forceinline__ float min3(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Plane distances of slots b and b + 4 of one plane set. Byte b of w0 and of
// w1 becomes the mantissa byte of v = 1 + q * 2^-15 (one byte permute each:
// 0x3F80qq00, exact), and the distance is one packed two-lane FMA,
// fma(v, S', C') with S' = 2^15 * S and C' = C - S' from the node's terms
// (axis_terms8): v * S' + C' = q * S + C up to the rounding of C', which the
// node's margins cover. Each lane rounds exactly as a scalar __fmaf_rn would.
__device__ __forceinline__ float2 plane_pair(uint32_t w0, uint32_t w1, int b, float Sp, float Cp) {
    const float v0 = __uint_as_float(__byte_perm(w0, 0x3F800000u, 0x7604u | ((uint32_t)b << 4)));
    const float v1 = __uint_as_float(__byte_perm(w1, 0x3F800000u, 0x7604u | ((uint32_t)b << 4)));
    float2 t;
    asm("{\n\t"
        ".reg .b64 v, s, c, r;\n\t"
        "mov.b64 v, {%2, %3};\n\t"
        "mov.b64 s, {%4, %4};\n\t"
        "mov.b64 c, {%5, %5};\n\t"
        "fma.rn.f32x2 r, v, s, c;\n\t"
        "mov.b64 {%0, %1}, r;\n\t"
        "}"
        : "=f"(t.x), "=f"(t.y)
        : "f"(v0), "f"(v1), "f"(Sp), "f"(Cp));
    return t;
}

// Per node and axis, with S = 2^e * (1/d) and C = (lo - o) * (1/d): the
// plane scale S' = 2^15 * S (exact) and the near / far offsets C' -+ m with
// C' = C - S' and m = |C| * 2^-20 + |S| * 2^-7. The roundings of C, C', the
// offsets and the final FMA stay below 2.5 * 2^-23 * |C| + (2^-8 + 2^-16) * |S|
// (C' = C - S' is rounded at the size of S', 2^15 |S|, and so is C' -+ m), so
// the measured interval [near, far] always contains the quantised box's.
__device__ __forceinline__ void axis_terms8(uint32_t biased_e, float lo, float o, float inv, float& Sp, float& cn,
                                            float& cf) {
    const float S = __fmul_rn(__uint_as_float(biased_e << 23), inv);
    const float C = __fmul_rn(__fsub_rn(lo, o), inv);
    Sp = __fmul_rn(S, 32768.0f);
    const float Cp = __fsub_rn(C, Sp);
    const float m = __fmaf_rn(fabsf(C), 0x1p-20f, __fmul_rn(fabsf(S), 0x1p-7f));
    cn = __fsub_rn(Cp, m);
    cf = __fadd_rn(Cp, m);
}

// axis_terms8 for the x and y axes at once, in packed two-lane FP32
// (mul / sub / fma / add .rn.f32x2, |.| as a mask of the sign bits): each lane
// rounds exactly as the scalar form.
__device__ __forceinline__ void axis_terms8_xy(uint32_t ex, uint32_t ey, float lox, float loy, float ox, float oy,
                                               float ix, float iy, float& Sx, float& Sy, float& cnx, float& cny,
                                               float& cfx, float& cfy) {
    asm("{\n\t"
        ".reg .b64 e, inv, S, Sp, lo, o, C, Cp, aS, aC, k7, k15, k20, t, m, cn, cf;\n\t"
        "mov.b64 e, {%6, %7};\n\t"
        "mov.b64 inv, {%12, %13};\n\t"
        "mul.rn.f32x2 S, e, inv;\n\t"
        "mov.b64 lo, {%8, %9};\n\t"
        "mov.b64 o, {%10, %11};\n\t"
        "sub.rn.f32x2 C, lo, o;\n\t"
        "mul.rn.f32x2 C, C, inv;\n\t"
        "mov.b64 k15, 0x4700000047000000;\n\t"  // {2^15, 2^15}
        "mul.rn.f32x2 Sp, S, k15;\n\t"
        "sub.rn.f32x2 Cp, C, Sp;\n\t"
        "and.b64 aS, S, 0x7FFFFFFF7FFFFFFF;\n\t"
        "and.b64 aC, C, 0x7FFFFFFF7FFFFFFF;\n\t"
        "mov.b64 k7, 0x3C0000003C000000;\n\t"   // {2^-7, 2^-7}
        "mov.b64 k20, 0x3580000035800000;\n\t"  // {2^-20, 2^-20}
        "mul.rn.f32x2 t, aS, k7;\n\t"
        "fma.rn.f32x2 m, aC, k20, t;\n\t"
        "sub.rn.f32x2 cn, Cp, m;\n\t"
        "add.rn.f32x2 cf, Cp, m;\n\t"
        "mov.b64 {%0, %1}, Sp;\n\t"
        "mov.b64 {%2, %3}, cn;\n\t"
        "mov.b64 {%4, %5}, cf;\n\t"
        "}"
        : "=f"(Sx), "=f"(Sy), "=f"(cnx), "=f"(cny), "=f"(cfx), "=f"(cfy)
        : "f"(__uint_as_float(ex << 23)), "f"(__uint_as_float(ey << 23)), "f"(lox), "f"(loy), "f"(ox), "f"(oy),
          "f"(ix), "f"(iy));
}

// Bit k of an 8-bit mask moved to bit k ^ oct.
__device__ __forceinline__ uint32_t xor_permute8(uint32_t x, uint32_t oct) {
    if (oct & 1u) x = ((x & 0x55u) << 1) | ((x >> 1) & 0x55u);
    if (oct & 2u) x = ((x & 0x33u) << 2) | ((x >> 2) & 0x33u);
    if (oct & 4u) x = ((x & 0x0Fu) << 4) | ((x >> 4) & 0x0Fu);
    return x;
}

constexpr uint32_t kPerm8Bytes = 8 * 256;

// Dynamic shared memory of a traversal kernel: the short stacks, and for the
// 8-wide layout the octant permutation table.
inline size_t traverse_smem(int layout, int sstack, int block) {
    return sizeof(int2) * (size_t)sstack * block + (layout == kLayoutBvh8Q8 ? kPerm8Bytes : 0);
}

template <int SSTACK>
__device__ __forceinline__ int2 stack_at(int i, const int2* s_stack, const int2* l_stack) {
    return i < SSTACK ? s_stack[i * blockDim.x + threadIdx.x] : l_stack[i - SSTACK];
}

template <int SSTACK>
__device__ __forceinline__ void stack_put(int i, int2 v, int2* s_stack, int2* l_stack) {
    if (i < SSTACK) s_stack[i * blockDim.x + threadIdx.x] = v;
    else l_stack[i - SSTACK] = v;
}

// Leaf triangle `idx` of the layout's own triangle array.
template <bool ANY>
__device__ __forceinline__ bool leaf_at(Lane& L, uint32_t idx) { return leaf<ANY>(L, ~(int32_t)idx); }

// One 8-wide node. A child plane is q * 2^e + lo, taken exactly; its ray
// distance q * S + C, with S = 2^e / d (exact: a power-of-two scaling) and
// C = (lo - o) / d, is measured as one FMA from per-node terms
// (axis_terms8, plane_pair), near planes with the offset C' - m and far
// planes with C' + m, so the measured interval always contains the quantised
// box's. The near plane of an axis is lo when d >= 0, else hi.
// A child is hit when max(near, tmin) <= min(far, best_t * slack). Hit leaf
// triangles are tested in slot order; hit inner children are ranked by
// slot ^ octant and the lowest rank is visited next. The remaining inner hits
// stay on the stack as one group entry (child_base, inner mask | hits << 8),
// taken one child at a time. Returns true when the ray is finished.
template <bool ANY, int SSTACK>
__device__ __forceinline__ bool trace_step8(Lane& L, int2* s_stack, int2* l_stack, uint32_t* err,
                                            const unsigned char* perm8) {
    const float4* q = reinterpret_cast<const float4*>(static_cast<const Node8Q*>(L.nodes) + L.node);
    float4 h0, h1, b0, b1, c0, c1;
    ldg32B(q, h0, h1);
    ldg32B(q + 2, b0, b1);
    ldg32B(q + 4, c0, c1);
    const uint32_t meta = __float_as_uint(h0.w);
    const uint32_t child_base = __float_as_uint(h1.x), tri_base = __float_as_uint(h1.y);
    const uint32_t valid = __float_as_uint(h1.z), imask = meta >> 24;
    const uint32_t sx = __float_as_uint(L.p.ix) >> 31, sy = __float_as_uint(L.p.iy) >> 31;
    const uint32_t sz = __float_as_uint(L.p.iz) >> 31;
    const uint32_t oct = sx | (sy << 1) | (sz << 2);
    float Sx, Sy, Sz, cnx, cfx, cny, cfy, cnz, cfz;
    axis_terms8_xy(meta & 0xFFu, (meta >> 8) & 0xFFu, h0.x, h0.y, L.p.ox, L.p.oy, L.p.ix, L.p.iy, Sx, Sy, cnx, cny,
                   cfx, cfy);
    axis_terms8((meta >> 16) & 0xFFu, h0.z, L.p.oz, L.p.iz, Sz, cnz, cfz);
    const float bound = __fmul_rn(L.best_t, kCullSlack);
    // words: b0 = (lo.x[0-3], lo.x[4-7], hi.x[0-3], hi.x[4-7]), b1 the same for y, c0 for z
    const uint32_t lx0 = __float_as_uint(b0.x), lx1 = __float_as_uint(b0.y);
    const uint32_t hx0 = __float_as_uint(b0.z), hx1 = __float_as_uint(b0.w);
    const uint32_t ly0 = __float_as_uint(b1.x), ly1 = __float_as_uint(b1.y);
    const uint32_t hy0 = __float_as_uint(b1.z), hy1 = __float_as_uint(b1.w);
    const uint32_t lz0 = __float_as_uint(c0.x), lz1 = __float_as_uint(c0.y);
    const uint32_t hz0 = __float_as_uint(c0.z), hz1 = __float_as_uint(c0.w);
    const uint32_t nx0 = sx ? hx0 : lx0, nx1 = sx ? hx1 : lx1, fx0 = sx ? lx0 : hx0, fx1 = sx ? lx1 : hx1;
    const uint32_t ny0 = sy ? hy0 : ly0, ny1 = sy ? hy1 : ly1, fy0 = sy ? ly0 : hy0, fy1 = sy ? ly1 : hy1;
    const uint32_t nz0 = sz ? hz0 : lz0, nz1 = sz ? hz1 : lz1, fz0 = sz ? lz0 : hz0, fz1 = sz ? lz1 : hz1;
    uint32_t hm = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) {  // slots b and b + 4
        const float2 tnx = plane_pair(nx0, nx1, b, Sx, cnx);
        const float2 tfx = plane_pair(fx0, fx1, b, Sx, cfx);
        const float2 tny = plane_pair(ny0, ny1, b, Sy, cny);
        const float2 tfy = plane_pair(fy0, fy1, b, Sy, cfy);
        const float2 tnz = plane_pair(nz0, nz1, b, Sz, cnz);
        const float2 tfz = plane_pair(fz0, fz1, b, Sz, cfz);
        const float tnear0 = fmaxf(max3(tnx.x, tny.x, tnz.x), L.p.tmin);
        const float tfar0 = fminf(min3(tfx.x, tfy.x, tfz.x), bound);
        const float tnear1 = fmaxf(max3(tnx.y, tny.y, tnz.y), L.p.tmin);
        const float tfar1 = fminf(min3(tfx.y, tfy.y, tfz.y), bound);
        hm |= (tnear0 <= tfar0 ? 1u : 0u) << b;
        hm |= (tnear1 <= tfar1 ? 1u : 0u) << (b + 4);
    }
    hm &= valid;
    uint32_t thits = hm & ~imask;
    const uint32_t ihits = perm8[(oct << 8) | (hm & imask)];  // xor_permute8(hm & imask, oct)
    // The next node does not depend on this node's leaf tests (group entries are
    // not culled by distance), so the stack is updated and the next node chosen
    // before the triangles are tested: the visit order and every test are
    // unchanged (measured: any hit 1,020 -> 1,057 Mrays/s, closest hit the same;
    // also starting the next node's fetch into L1 here made both far slower).
    bool last = false;
    uint32_t gbase = child_base, gmask = imask, hits = ihits;
    if (hits) {
        if (hits & (hits - 1u)) {
            if (L.sp >= kStackMax) {
                atomicOr(err, ERR_STACK);
                last = true;
            } else {
                stack_put<SSTACK>(L.sp, make_int2((int32_t)child_base, (int32_t)(imask | ((hits & (hits - 1u)) << 8))),
                                  s_stack, l_stack);
                ++L.sp;
            }
        }
    } else if (L.sp == 0) {
        last = true;
    } else {
        const int2 e = stack_at<SSTACK>(L.sp - 1, s_stack, l_stack);
        gbase = (uint32_t)e.x;
        gmask = (uint32_t)e.y & 0xFFu;
        hits = (uint32_t)e.y >> 8;
        const uint32_t rest = hits & (hits - 1u);
        if (rest) stack_put<SSTACK>(L.sp - 1, make_int2(e.x, (int32_t)(gmask | (rest << 8))), s_stack, l_stack);
        else --L.sp;
    }
    if (!last) {
        const uint32_t slot = (uint32_t)(__ffs(hits) - 1) ^ oct;
        L.node = (int32_t)(gbase + __popc(gmask & ((1u << slot) - 1u)));
    }
    if (thits) {
        const uint32_t leafmask = valid & ~imask;
        do {
            const int k = __ffs(thits) - 1;
            thits &= thits - 1u;
            if (leaf_at<ANY>(L, tri_base + __popc(leafmask & ((1u << k) - 1u)))) return true;
        } while (thits);
    }
    return last;
}

template <bool ANY, int LAYOUT, int SSTACK>
__device__ __forceinline__ bool trace_step(Lane& L, int2* s_stack, int2* l_stack, uint32_t* err,
                                           const unsigned char* perm8) {
    if (LAYOUT == kLayoutBvh2) return trace_step2<ANY, SSTACK>(L, s_stack, l_stack, err);
    if (LAYOUT == kLayoutBvh8Q8) return trace_step8<ANY, SSTACK>(L, s_stack, l_stack, err, perm8);
    return trace_step4<ANY, LAYOUT == kLayoutBvh4Q8, SSTACK>(L, s_stack, l_stack, err);
}

// A warp refills its idle lanes once at least REFILL of them are idle. The
// ray-query kernels use 4 (a ray loads in two 16-byte reads; 2, 6 and 8
// measured slower); the render's queue kernels use 12 (a queued path also looks
// up its job and scene; 4, 6, 8, 16 and 20 measured slower on the Cornell and
// glossy renders).
constexpr int kRefillRays = 4;
constexpr int kRefillQueue = 12;

// Persistent dynamic-fetch loop. `Src` supplies the work:
//   uint64_t n                                        number of rays
//   uint32_t load(uint64_t i, float4& r0, float4& r1, const void*& nodes,
//                 const Tri*& tris)                   ray i (reference Ray layout) and
//                                                     its BVH (nodes and triangles of
//                                                     layout LAYOUT); returns the binary
//                                                     root (kNoNode when empty)
//   void finish(uint64_t i, const Lane& L)            ray i is done (L.best_prim ==
//                                                     0xFFFFFFFF means a miss)
// The shared stack has SSTACK x blockDim.x int2 entries (dynamic shared memory),
// followed for the 8-wide layout by the octant permutation table
// (traverse_smem). Every thread of the block calls it (the table is filled
// behind a block barrier).
template <bool ANY, int LAYOUT, int SSTACK, int REFILL, class Src>
__device__ __forceinline__ void traverse_loop(Src& src, unsigned long long* counter, uint32_t* err, int2* s_stack) {
    int2 l_stack[kStackMax - SSTACK];
    // 8-wide layout: xor_permute8 as a table (octant x mask, 2 KB after the
    // short stacks), filled once per block
    unsigned char* perm8 = reinterpret_cast<unsigned char*>(s_stack + SSTACK * blockDim.x);
    if (LAYOUT == kLayoutBvh8Q8) {
        for (uint32_t i = threadIdx.x; i < kPerm8Bytes; i += blockDim.x) perm8[i] = (unsigned char)xor_permute8(i & 255u, i >> 8);
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    const uint32_t ltmask = lanemask_lt();
    const uint64_t n = src.n;
    Lane L;
    bool active = false;
    bool exhausted = false;
    for (;;) {
        const uint32_t idle = __ballot_sync(0xFFFFFFFFu, !active);
        const int nidle = __popc(idle);
        if (exhausted) {
            if (nidle == 32) break;  // a refill that found no rays leaves every lane idle
        } else if (nidle >= REFILL || nidle == 32) {
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
                    L.node = (LAYOUT == kLayoutBvh8Q8 && root != kNoNode) ? 0 : (int32_t)root;  // 8-wide root is node 0
                    L.sp = 0;
                    active = true;
                    if (root == kNoNode) {
                        src.finish(i, L);
                        active = false;
                    }
                }
            }
        }
        if (active && trace_step<ANY, LAYOUT, SSTACK>(L, s_stack, l_stack, err, perm8)) {
            src.finish(L.ray, L);
            active = false;
        }
    }
}

}  // namespace trav
}  // namespace gr
