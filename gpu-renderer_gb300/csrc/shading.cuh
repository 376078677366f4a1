// Device shading math for the wavefront integrator: RNG, shading frame,
// Lambert / GGX conductor / smooth dielectric BSDFs, light sampling.
//
// The formulas restate the reference's HOST_DEVICE code (slongle/GPU-Renderer
// src/renderer/sampling.h, bsdf.h, bsdfs/*.h, triangle.h), which itself follows
// pbrt-v3; names and argument meaning are kept so the two can be read side by
// side. Compiled with --fmad=false so each operation rounds as written, as the
// host oracle does (with contraction, chains of refractions turn last-bit
// differences into different paths).
#pragma once

#include <stdint.h>

namespace gr {
namespace sh {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.31830988618379067154f;

// ---- small vector helpers ------------------------------------------------------
struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ V3 operator/(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ V3 normalize(V3 v) { return v * (1.0f / sqrtf(dot(v, v))); }
__device__ __forceinline__ float maxc(V3 v) { return fmaxf(v.x, fmaxf(v.y, v.z)); }
__device__ __forceinline__ bool black(V3 v) { return v.x == 0.0f && v.y == 0.0f && v.z == 0.0f; }
__device__ __forceinline__ V3 vsqrt(V3 v) { return {sqrtf(v.x), sqrtf(v.y), sqrtf(v.z)}; }
__device__ __forceinline__ V3 vs(float s) { return {s, s, s}; }

// ---- PCG32 (O'Neill 2014), one stream per path ------------------------------------
// State advances by the 64-bit LCG; the increment is derived from the pixel
// index so it need not be stored.
__device__ __forceinline__ uint64_t pcg_inc(uint64_t seq) { return (seq << 1) | 1ull; }
__device__ __forceinline__ uint32_t pcg_next(uint64_t& state, uint64_t inc) {
    const uint64_t old = state;
    state = old * 6364136223846793005ull + inc;
    const uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
    const uint32_t rot = (uint32_t)(old >> 59);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
}
__device__ __forceinline__ uint64_t pcg_seed(uint64_t initstate, uint64_t inc) {
    uint64_t st = 0;
    pcg_next(st, inc);
    st += initstate;
    pcg_next(st, inc);
    return st;
}
// 24-bit uniform float in [0, 1)
__device__ __forceinline__ float pcg_float(uint64_t& state, uint64_t inc) {
    return (float)(pcg_next(state, inc) >> 8) * 0x1p-24f;
}

// ---- shading frame (sampling.h:124-164) --------------------------------------------
struct Frame {
    V3 s, t, n;
};
__device__ __forceinline__ Frame make_frame(V3 n) {
    Frame f;
    f.n = n;
    if (fabsf(n.x) > fabsf(n.y)) {
        const float inv = 1.0f / sqrtf(n.x * n.x + n.z * n.z);
        f.s = v3(n.z * inv, 0.0f, -n.x * inv);
    } else {
        const float inv = 1.0f / sqrtf(n.y * n.y + n.z * n.z);
        f.s = v3(0.0f, n.z * inv, -n.y * inv);
    }
    f.t = cross(f.s, n);
    return f;
}
__device__ __forceinline__ V3 to_local(const Frame& f, V3 v) { return normalize(v3(dot(v, f.s), dot(v, f.t), dot(v, f.n))); }
__device__ __forceinline__ V3 to_world(const Frame& f, V3 v) { return normalize(f.s * v.x + f.t * v.y + f.n * v.z); }

// ---- trigonometric helpers on local directions (sampling.h:84-121) ------------------
__device__ __forceinline__ float cos2t(V3 w) { return w.z * w.z; }
__device__ __forceinline__ float sin2t(V3 w) { return fmaxf(0.0f, 1.0f - cos2t(w)); }
__device__ __forceinline__ float sint(V3 w) { return sqrtf(sin2t(w)); }
__device__ __forceinline__ float tant(V3 w) { return sint(w) / w.z; }
__device__ __forceinline__ float tan2t(V3 w) { return sin2t(w) / cos2t(w); }
__device__ __forceinline__ float clampf(float a, float l, float r) { return a > r ? r : (a < l ? l : a); }
__device__ __forceinline__ float cosp(V3 w) {
    const float st = sint(w);
    return st == 0.0f ? 1.0f : clampf(w.x / st, -1.0f, 1.0f);
}
__device__ __forceinline__ float sinp(V3 w) {
    const float st = sint(w);
    return st == 0.0f ? 0.0f : clampf(w.y / st, -1.0f, 1.0f);
}

__device__ __forceinline__ V3 cosine_hemisphere(float u0, float u1) {
    const float a = sqrtf(u0);
    const float b = kPi * 2.0f * u1;
    return v3(a * cosf(b), a * sinf(b), sqrtf(fmaxf(0.0f, 1.0f - u0)));
}

// ---- Fresnel (bsdfs/optical.h) -------------------------------------------------------
__device__ __forceinline__ float fr_dielectric(float cos_i, float eta_i, float eta_t) {
    cos_i = clampf(cos_i, -1.0f, 1.0f);
    if (!(cos_i > 0.0f)) {
        const float t = eta_t;
        eta_t = eta_i;
        eta_i = t;
        cos_i = fabsf(cos_i);
    }
    const float sin_i = sqrtf(fmaxf(0.0f, 1.0f - cos_i * cos_i));
    const float sin_t = eta_i / eta_t * sin_i;
    if (sin_t >= 1.0f) return 1.0f;
    const float cos_t = sqrtf(fmaxf(0.0f, 1.0f - sin_t * sin_t));
    const float par = ((eta_t * cos_i) - (eta_i * cos_t)) / ((eta_t * cos_i) + (eta_i * cos_t));
    const float perp = ((eta_i * cos_i) - (eta_t * cos_t)) / ((eta_i * cos_i) + (eta_t * cos_t));
    return (par * par + perp * perp) * 0.5f;
}

__device__ __forceinline__ V3 fr_conductor(float cos_i, V3 eta_i, V3 eta_t, V3 k) {
    cos_i = clampf(cos_i, -1.0f, 1.0f);
    const V3 eta = eta_t / eta_i;
    const V3 etak = k / eta_i;
    const float c2 = cos_i * cos_i;
    const float s2 = 1.0f - c2;
    const V3 eta2 = eta * eta, etak2 = etak * etak;
    const V3 t0 = eta2 - etak2 - vs(s2);
    const V3 a2b2 = vsqrt(t0 * t0 + eta2 * etak2 * 4.0f);
    const V3 t1 = a2b2 + vs(c2);
    const V3 a = vsqrt((a2b2 + t0) * 0.5f);
    const V3 t2 = a * 2.0f * cos_i;
    const V3 rs = (t1 - t2) / (t1 + t2);
    const V3 t3 = a2b2 * c2 + vs(s2 * s2);
    const V3 t4 = t2 * s2;
    const V3 rp = rs * (t3 - t4) / (t3 + t4);
    return (rp + rs) * 0.5f;
}

// ---- Trowbridge-Reitz (GGX) microfacet distribution (bsdfs/microfacet.h) ---------
__device__ __forceinline__ float ggx_lambda(V3 w, float ax, float ay) {
    const float abs_tan = fabsf(tant(w));
    if (isinf(abs_tan)) return 0.0f;
    const float cp = cosp(w), sp = sinp(w);
    const float alpha = sqrtf(cp * cp * ax * ax + sp * sp * ay * ay);
    const float a2t2 = (alpha * abs_tan) * (alpha * abs_tan);
    return (-1.0f + sqrtf(1.0f + a2t2)) / 2.0f;
}
__device__ __forceinline__ float ggx_g1(V3 w, float ax, float ay) { return 1.0f / (1.0f + ggx_lambda(w, ax, ay)); }
__device__ __forceinline__ float ggx_g(V3 wo, V3 wi, float ax, float ay) {
    return 1.0f / (1.0f + ggx_lambda(wo, ax, ay) + ggx_lambda(wi, ax, ay));
}
__device__ __forceinline__ float ggx_d(V3 wh, float ax, float ay) {
    const float t2 = tan2t(wh);
    if (isinf(t2)) return 0.0f;
    const float c4 = cos2t(wh) * cos2t(wh);
    const float cp = cosp(wh), sp = sinp(wh);
    const float e = (cp * cp / (ax * ax) + sp * sp / (ay * ay)) * t2;
    return 1.0f / (kPi * ax * ay * c4 * (1.0f + e) * (1.0f + e));
}

// Visible-normal slope sampling for a unit-roughness distribution (pbrt-v3,
// after Heitz & d'Eon 2014), including its rational fit for the y slope.
__device__ __forceinline__ void ggx_sample11(float cos_t, float u1, float u2, float& sx, float& sy) {
    if (cos_t > 0.9999f) {
        const float r = sqrtf(u1 / (1.0f - u1));
        const float phi = 6.28318530718f * u2;
        sx = r * cosf(phi);
        sy = r * sinf(phi);
        return;
    }
    const float sin_t = sqrtf(fmaxf(0.0f, 1.0f - cos_t * cos_t));
    const float tan_t = sin_t / cos_t;
    const float a = 1.0f / tan_t;
    const float g1 = 2.0f / (1.0f + sqrtf(1.0f + 1.0f / (a * a)));
    const float A = 2.0f * u1 / g1 - 1.0f;
    float tmp = 1.0f / (A * A - 1.0f);
    if (tmp > 1e10f) tmp = 1e10f;
    const float B = tan_t;
    const float D = sqrtf(fmaxf(B * B * tmp * tmp - (A * A - B * B) * tmp, 0.0f));
    const float x1 = B * tmp - D, x2 = B * tmp + D;
    sx = (A < 0.0f || x2 > 1.0f / tan_t) ? x1 : x2;
    float S;
    if (u2 > 0.5f) {
        S = 1.0f;
        u2 = 2.0f * (u2 - 0.5f);
    } else {
        S = -1.0f;
        u2 = 2.0f * (0.5f - u2);
    }
    const float z = (u2 * (u2 * (u2 * 0.27385f - 0.73369f) + 0.46341f)) /
                    (u2 * (u2 * (u2 * 0.093073f + 0.309420f) - 1.000000f) + 0.597999f);
    sy = S * z * sqrtf(1.0f + sx * sx);
}

__device__ __forceinline__ V3 ggx_sample_wh(V3 wo, float u0, float u1, float ax, float ay) {
    const bool flip = wo.z < 0.0f;
    const V3 wi = flip ? -wo : wo;
    const V3 st = normalize(v3(ax * wi.x, ay * wi.y, wi.z));
    float sx, sy;
    ggx_sample11(st.z, u0, u1, sx, sy);
    const float cp = cosp(st), sp = sinp(st);
    const float tmp = cp * sx - sp * sy;
    sy = sp * sx + cp * sy;
    sx = tmp;
    sx = ax * sx;
    sy = ay * sy;
    V3 wh = normalize(v3(-sx, -sy, 1.0f));
    return flip ? -wh : wh;
}

__device__ __forceinline__ V3 reflect(V3 wo, V3 n) { return -wo + n * 2.0f * dot(wo, n); }

__device__ __forceinline__ bool refract(V3 wi, V3 n, float eta, V3& wt) {
    const float cos_i = dot(n, wi);
    const float sin2_i = fmaxf(0.0f, 1.0f - cos_i * cos_i);
    const float sin2_t = eta * eta * sin2_i;
    if (sin2_t >= 1.0f) return false;
    const float cos_t = sqrtf(1.0f - sin2_t);
    wt = -wi * eta + n * (eta * cos_i - cos_t);
    return true;
}

}  // namespace sh
}  // namespace gr
