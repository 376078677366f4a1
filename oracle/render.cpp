// CPU oracle: the wavefront integrator restated one path at a time.
// Test infrastructure only (see oracle_render.h). Compiled with
// -ffp-contract=off like the product's shading kernels (--fmad=false).
#include "oracle_render.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "oracle.h"

namespace {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.31830988618379067154f;

struct V3 {
    float x, y, z;
};
inline V3 v3(float x, float y, float z) { return {x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline V3 operator/(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline V3 normalize(V3 v) { return v * (1.0f / std::sqrt(dot(v, v))); }
inline float maxc(V3 v) { return std::fmax(v.x, std::fmax(v.y, v.z)); }
inline bool black(V3 v) { return v.x == 0.0f && v.y == 0.0f && v.z == 0.0f; }
inline V3 vsqrt(V3 v) { return {std::sqrt(v.x), std::sqrt(v.y), std::sqrt(v.z)}; }
inline V3 vs(float s) { return {s, s, s}; }

// PCG32 (O'Neill 2014): LCG state, XSH-RR output
struct Pcg {
    uint64_t st, inc;
    uint32_t next() {
        const uint64_t old = st;
        st = old * 6364136223846793005ull + inc;
        const uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
        const uint32_t rot = (uint32_t)(old >> 59);
        return (xs >> rot) | (xs << ((32u - rot) & 31u));
    }
    float uniform() { return (float)(next() >> 8) * 0x1p-24f; }
};

Pcg pcg_for(uint64_t seed, uint32_t pixel, uint32_t sample) {
    Pcg r;
    r.inc = ((uint64_t)pixel << 1) | 1ull;
    r.st = 0;
    r.next();
    r.st += seed + (uint64_t)sample * 0x9E3779B97F4A7C15ull;
    r.next();
    return r;
}

struct Frame {
    V3 s, t, n;
};
Frame make_frame(V3 n) {  // sampling.h:130-144
    Frame f;
    f.n = n;
    if (std::fabs(n.x) > std::fabs(n.y)) {
        const float inv = 1.0f / std::sqrt(n.x * n.x + n.z * n.z);
        f.s = v3(n.z * inv, 0.0f, -n.x * inv);
    } else {
        const float inv = 1.0f / std::sqrt(n.y * n.y + n.z * n.z);
        f.s = v3(0.0f, n.z * inv, -n.y * inv);
    }
    f.t = cross(f.s, n);
    return f;
}
V3 to_local(const Frame& f, V3 v) { return normalize(v3(dot(v, f.s), dot(v, f.t), dot(v, f.n))); }
V3 to_world(const Frame& f, V3 v) { return normalize(f.s * v.x + f.t * v.y + f.n * v.z); }

float cos2t(V3 w) { return w.z * w.z; }
float sin2t(V3 w) { return std::fmax(0.0f, 1.0f - cos2t(w)); }
float sint(V3 w) { return std::sqrt(sin2t(w)); }
float tant(V3 w) { return sint(w) / w.z; }
float tan2t(V3 w) { return sin2t(w) / cos2t(w); }
float clampf(float a, float l, float r) { return a > r ? r : (a < l ? l : a); }
float cosp(V3 w) {
    const float st = sint(w);
    return st == 0.0f ? 1.0f : clampf(w.x / st, -1.0f, 1.0f);
}
float sinp(V3 w) {
    const float st = sint(w);
    return st == 0.0f ? 0.0f : clampf(w.y / st, -1.0f, 1.0f);
}

V3 cosine_hemisphere(float u0, float u1) {  // sampling.h:63-70
    const float a = std::sqrt(u0);
    const float b = kPi * 2.0f * u1;
    return v3(a * std::cos(b), a * std::sin(b), std::sqrt(std::fmax(0.0f, 1.0f - u0)));
}

float fr_dielectric(float ci, float ei, float et) {  // optical.h:42-69
    ci = clampf(ci, -1.0f, 1.0f);
    if (!(ci > 0.0f)) {
        std::swap(ei, et);
        ci = std::fabs(ci);
    }
    const float si = std::sqrt(std::fmax(0.0f, 1.0f - ci * ci));
    const float st = ei / et * si;
    if (st >= 1.0f) return 1.0f;
    const float ct = std::sqrt(std::fmax(0.0f, 1.0f - st * st));
    const float par = ((et * ci) - (ei * ct)) / ((et * ci) + (ei * ct));
    const float perp = ((ei * ci) - (et * ct)) / ((ei * ci) + (et * ct));
    return (par * par + perp * perp) * 0.5f;
}

V3 fr_conductor(float ci, V3 ei, V3 et, V3 k) {  // optical.h:72-100
    ci = clampf(ci, -1.0f, 1.0f);
    const V3 eta = et / ei, etak = k / ei;
    const float c2 = ci * ci, s2 = 1.0f - c2;
    const V3 eta2 = eta * eta, etak2 = etak * etak;
    const V3 t0 = eta2 - etak2 - vs(s2);
    const V3 a2b2 = vsqrt(t0 * t0 + eta2 * etak2 * 4.0f);
    const V3 t1 = a2b2 + vs(c2);
    const V3 a = vsqrt((a2b2 + t0) * 0.5f);
    const V3 t2 = a * 2.0f * ci;
    const V3 rs = (t1 - t2) / (t1 + t2);
    const V3 t3 = a2b2 * c2 + vs(s2 * s2);
    const V3 t4 = t2 * s2;
    const V3 rp = rs * (t3 - t4) / (t3 + t4);
    return (rp + rs) * 0.5f;
}

float lambda(V3 w, float ax, float ay) {  // microfacet.h:7-20
    const float at = std::fabs(tant(w));
    if (std::isinf(at)) return 0.0f;
    const float cp = cosp(w), sp = sinp(w);
    const float alpha = std::sqrt(cp * cp * ax * ax + sp * sp * ay * ay);
    const float q = (alpha * at) * (alpha * at);
    return (-1.0f + std::sqrt(1.0f + q)) / 2.0f;
}
float g1(V3 w, float ax, float ay) { return 1.0f / (1.0f + lambda(w, ax, ay)); }
float gg(V3 wo, V3 wi, float ax, float ay) { return 1.0f / (1.0f + lambda(wo, ax, ay) + lambda(wi, ax, ay)); }
float ggx_d(V3 wh, float ax, float ay) {  // microfacet.h:126-139
    const float t2 = tan2t(wh);
    if (std::isinf(t2)) return 0.0f;
    const float c4 = cos2t(wh) * cos2t(wh);
    const float cp = cosp(wh), sp = sinp(wh);
    const float e = (cp * cp / (ax * ax) + sp * sp / (ay * ay)) * t2;
    return 1.0f / (kPi * ax * ay * c4 * (1.0f + e) * (1.0f + e));
}

void sample11(float ct, float u1, float u2, float& sx, float& sy) {  // microfacet.h:38-84
    if (ct > 0.9999f) {
        const float r = std::sqrt(u1 / (1.0f - u1));
        const float phi = 6.28318530718f * u2;
        sx = r * std::cos(phi);
        sy = r * std::sin(phi);
        return;
    }
    const float st = std::sqrt(std::fmax(0.0f, 1.0f - ct * ct));
    const float tt = st / ct;
    const float a = 1.0f / tt;
    const float G1 = 2.0f / (1.0f + std::sqrt(1.0f + 1.0f / (a * a)));
    const float A = 2.0f * u1 / G1 - 1.0f;
    float tmp = 1.0f / (A * A - 1.0f);
    if (tmp > 1e10f) tmp = 1e10f;
    const float B = tt;
    const float D = std::sqrt(std::fmax(B * B * tmp * tmp - (A * A - B * B) * tmp, 0.0f));
    const float x1 = B * tmp - D, x2 = B * tmp + D;
    sx = (A < 0.0f || x2 > 1.0f / tt) ? x1 : x2;
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
    sy = S * z * std::sqrt(1.0f + sx * sx);
}

V3 sample_wh(V3 wo, float u0, float u1, float ax, float ay) {  // microfacet.h:86-124
    const bool flip = wo.z < 0.0f;
    const V3 wi = flip ? -wo : wo;
    const V3 st = normalize(v3(ax * wi.x, ay * wi.y, wi.z));
    float sx, sy;
    sample11(st.z, u0, u1, sx, sy);
    const float cp = cosp(st), sp = sinp(st);
    const float tmp = cp * sx - sp * sy;
    sy = sp * sx + cp * sy;
    sx = tmp;
    sx = ax * sx;
    sy = ay * sy;
    const V3 wh = normalize(v3(-sx, -sy, 1.0f));
    return flip ? -wh : wh;
}

V3 reflect(V3 wo, V3 n) { return -wo + n * 2.0f * dot(wo, n); }
bool refract(V3 wi, V3 n, float eta, V3& wt) {
    const float ci = dot(n, wi);
    const float s2i = std::fmax(0.0f, 1.0f - ci * ci);
    const float s2t = eta * eta * s2i;
    if (s2t >= 1.0f) return false;
    const float ct = std::sqrt(1.0f - s2t);
    wt = -wi * eta + n * (eta * ci - ct);
    return true;
}

V3 mf_eval(const or_material& m, V3 color, V3 wo, V3 wi) {
    const float co = std::fabs(wo.z), ci = std::fabs(wi.z);
    V3 wh = wi + wo;
    if (ci == 0.0f || co == 0.0f) return vs(0.0f);
    if (wh.x == 0.0f && wh.y == 0.0f && wh.z == 0.0f) return vs(0.0f);
    wh = normalize(wh);
    const V3 F = m.type == 3 ? vs(fr_dielectric(dot(wi, wh), m.eta_i[0], m.eta_t[0]))
                             : fr_conductor(std::fabs(dot(wi, wh)), v3(m.eta_i[0], m.eta_i[1], m.eta_i[2]),
                                            v3(m.eta_t[0], m.eta_t[1], m.eta_t[2]), v3(m.k[0], m.k[1], m.k[2]));
    return color * ggx_d(wh, m.ax, m.ay) * gg(wo, wi, m.ax, m.ay) * F / (4.0f * co);
}
float mf_pdf_wh(const or_material& m, V3 wo, V3 wh, bool compat) {
    if (compat) return ggx_d(wh, m.ax, m.ay) * std::fabs(wh.z) / (4.0f * dot(wo, wh));
    return g1(wo, m.ax, m.ay) * ggx_d(wh, m.ax, m.ay) / (4.0f * std::fabs(wo.z));
}

struct Bsdf {
    Frame fr;
    const or_material* m;
    bool compat;
    V3 color;  // the material color at the shading point
};

// rough plastic (bsdf.h:33-39): Lambert + GGX with dielectric Fresnel; lobes picked with probability 1/2
V3 plastic_eval(const Bsdf& b, V3 wo, V3 wi) {
    return b.color * kInvPi * std::fabs(wi.z) + mf_eval(*b.m, v3(b.m->spec[0], b.m->spec[1], b.m->spec[2]), wo, wi);
}
float plastic_pdf(const Bsdf& b, V3 wo, V3 wi) {
    const float p = std::fabs(wi.z) * kInvPi + mf_pdf_wh(*b.m, wo, normalize(wo + wi), b.compat);
    return b.compat ? p : 0.5f * p;  // the reference sums the lobe densities
}

V3 bsdf_eval(const Bsdf& b, V3 wo_w, V3 wi_w) {
    const V3 wo = to_local(b.fr, wo_w), wi = to_local(b.fr, wi_w);
    if (wo.z == 0.0f) return vs(0.0f);
    if (!(wo.z * wi.z > 0.0f)) return vs(0.0f);
    if (b.m->type == 0) return b.color * kInvPi * std::fabs(wi.z);
    if (b.m->type == 2) return mf_eval(*b.m, b.color, wo, wi);
    if (b.m->type == 3) return plastic_eval(b, wo, wi);
    return vs(0.0f);
}
float bsdf_pdf(const Bsdf& b, V3 wo_w, V3 wi_w) {
    const V3 wo = to_local(b.fr, wo_w), wi = to_local(b.fr, wi_w);
    if (wo.z == 0.0f) return 0.0f;
    if (!(wo.z * wi.z > 0.0f)) return 0.0f;
    if (b.m->type == 0) return std::fabs(wi.z) * kInvPi;
    if (b.m->type == 2) return mf_pdf_wh(*b.m, wo, normalize(wo + wi), b.compat);
    if (b.m->type == 3) return plastic_pdf(b, wo, wi);
    return 0.0f;
}

struct Smp {
    V3 wi, f;
    float pdf;
    bool specular;
};
Smp bsdf_sample(const Bsdf& b, V3 wo_w, float u0, float u1) {  // bsdf.h:112-167
    Smp s;
    s.f = vs(0.0f);
    s.pdf = 0.0f;
    s.wi = vs(0.0f);
    s.specular = b.m->type == 1;
    const V3 wo = to_local(b.fr, wo_w);
    if (wo.z == 0.0f) return s;
    V3 wi = vs(0.0f);
    if (b.m->type == 0) {
        wi = cosine_hemisphere(u0, u1);
        if (wo.z < 0.0f) wi.z = -wi.z;
        s.f = b.color * kInvPi * std::fabs(wi.z);
        s.pdf = std::fabs(wi.z) * kInvPi;
    } else if (b.m->type == 2) {
        const V3 wh = sample_wh(wo, u0, u1, b.m->ax, b.m->ay);
        wi = reflect(wo, wh);
        if (!(wo.z * wi.z > 0.0f)) return s;
        s.pdf = mf_pdf_wh(*b.m, wo, wh, b.compat);
        s.f = mf_eval(*b.m, b.color, wo, wi);
    } else if (b.m->type == 3) {
        const int lobe = std::min((int)std::floor(u0 * 2.0f), 1);
        const float v0 = u0 * 2.0f - (float)lobe;
        if (lobe == 0) {
            wi = cosine_hemisphere(v0, u1);
            if (wo.z < 0.0f) wi.z = -wi.z;
        } else {
            wi = reflect(wo, sample_wh(wo, v0, u1, b.m->ax, b.m->ay));
        }
        if (!(wo.z * wi.z > 0.0f)) return s;
        s.pdf = plastic_pdf(b, wo, wi);
        s.f = plastic_eval(b, wo, wi);
    } else {
        const float F = fr_dielectric(wo.z, 1.0f, b.m->ior);
        if (u0 < F) {
            wi = v3(-wo.x, -wo.y, wo.z);
            s.pdf = F;
            s.f = b.color * F;
        } else {
            const bool entering = wo.z > 0.0f;
            const float ei = entering ? 1.0f : b.m->ior, et = entering ? b.m->ior : 1.0f;
            const V3 n = wo.z < 0.0f ? v3(0.0f, 0.0f, -1.0f) : v3(0.0f, 0.0f, 1.0f);
            if (!refract(wo, n, ei / et, wi)) return s;
            s.f = b.color * (1.0f - F) * ((ei * ei) / (et * et));
            s.pdf = 1.0f - F;
        }
    }
    if (s.pdf == 0.0f) return s;
    s.wi = to_world(b.fr, wi);
    if (!s.specular) {
        if (!(wo.z * wi.z > 0.0f)) s.f = vs(0.0f);
        else if (b.m->type == 0) s.f = b.color * kInvPi * std::fabs(wi.z);
        else if (b.m->type == 3) s.f = plastic_eval(b, wo, wi);
        else s.f = mf_eval(*b.m, b.color, wo, wi);
    }
    return s;
}

struct Scene {
    const float* verts;
    const float* normals;
    const uint32_t* tri_mat;
    uint32_t ntri;
    const or_material* mats;
    const or_camera* cam;
    V3 env;
    bool has_env;
    const float* uvs;
    const float* texels;
    const or_envmap* envmap;
    std::vector<uint32_t> lights;
    std::vector<uint32_t> nodes;
    std::vector<float> tris;
    uint32_t root;
};

struct Surf {
    V3 p, ng, ns;
    float tu, tv;
};
V3 vert(const Scene& sc, uint32_t t, int k) {
    const float* p = sc.verts + 9ull * t + 3 * k;
    return v3(p[0], p[1], p[2]);
}
Surf surface(const Scene& sc, uint32_t prim, float u, float v) {  // triangle.h:103-138
    const V3 p0 = vert(sc, prim, 0), p1 = vert(sc, prim, 1), p2 = vert(sc, prim, 2);
    const float w = 1.0f - u - v;
    Surf s;
    s.p = p0 * w + p1 * u + p2 * v;
    s.ng = normalize(cross(p0 - p2, p1 - p2));
    if (sc.tri_mat[prim] & 0x80000000u) {
        const float* n = sc.normals + 12ull * prim;
        s.ns = normalize(v3(n[0], n[1], n[2]) * w + v3(n[4], n[5], n[6]) * u + v3(n[8], n[9], n[10]) * v);
    } else {
        s.ns = s.ng;
    }
    if (sc.tri_mat[prim] & 0x40000000u) {
        const float* q = sc.uvs + 6ull * prim;
        s.tu = q[0] * w + q[2] * u + q[4] * v;
        s.tv = q[1] * w + q[3] * u + q[5] * v;
    } else {
        s.tu = u;
        s.tv = v;
    }
    return s;
}

// Nearest texel (TextureView::evalSpectrum, texture.h:37-44), wrapped into [0, size).
int wrap_texel(float x, uint32_t size) {
    const float f = std::fmin(std::fmax(x * (float)size, -1073741824.0f), 1073741824.0f);
    const int i = (int)f % (int)size;
    return i < 0 ? i + (int)size : i;
}

V3 color_at(const Scene& sc, const or_material& m, float tu, float tv) {
    if (m.tex_w == 0) return v3(m.color[0], m.color[1], m.color[2]);
    const int x = wrap_texel(tu * m.tus + m.tuo, m.tex_w);
    const int y = wrap_texel(tv * m.tvs + m.tvo, m.tex_h);
    const float* c = sc.texels + 3ull * (m.tex_off + (uint32_t)y * m.tex_w + (uint32_t)x);
    return v3(c[0], c[1], c[2]);
}

// EnvironmentLightView::Le (environment.h:15-27).
V3 env_radiance(const Scene& sc, V3 o, V3 d) {
    const or_envmap* e = sc.envmap;
    if (!e || e->w == 0) return sc.env;
    V3 w = normalize(o + d * 100000.0f - v3(e->c[0], e->c[1], e->c[2]));
    const float* M = e->m;
    w = normalize(v3(M[0] * w.x + M[1] * w.y + M[2] * w.z, M[3] * w.x + M[4] * w.y + M[5] * w.z,
                     M[6] * w.x + M[7] * w.y + M[8] * w.z));
    const float theta = std::acos(std::fmin(std::fmax(w.z, -1.0f), 1.0f));
    float phi = std::atan2(w.y, w.x);
    if (phi < 0.0f) phi += 6.28318530717958647692f;
    const float uu = phi * 0.15915494309189533577f, vv = theta * 0.31830988618379067154f;
    const uint32_t x = std::min(e->w - 1, (uint32_t)(int)(uu * (float)e->w));
    const uint32_t y = std::min(e->h - 1, (uint32_t)(int)(vv * (float)e->h));
    const float* c = e->texels + 3ull * (y * e->w + x);
    return v3(c[0], c[1], c[2]);
}
float area(const Scene& sc, uint32_t prim) {
    const V3 p0 = vert(sc, prim, 0), p1 = vert(sc, prim, 1), p2 = vert(sc, prim, 2);
    const V3 c = cross(p1 - p0, p2 - p0);
    return std::sqrt(dot(c, c)) * 0.5f;
}
const or_material& mat_of(const Scene& sc, uint32_t prim) { return sc.mats[sc.tri_mat[prim] & 0x3FFFFFFFu]; }

struct Hit {
    float t, u, v;
    int32_t prim;
};
Hit trace(const Scene& sc, const float ray[8], bool any) {
    float h[4];
    or_trace(sc.nodes.data(), sc.tris.data(), sc.root, ray, 1, any ? 1 : 0, h, nullptr, 1);
    Hit r;
    r.t = h[0];
    std::memcpy(&r.prim, h + 1, 4);
    r.u = h[2];
    r.v = h[3];
    return r;
}

V3 path(const Scene& sc, uint32_t pixel, uint32_t sample, uint32_t D, uint64_t seed, int32_t rr_depth, bool compat) {
    Pcg rng = pcg_for(seed, pixel, sample);
    const or_camera& c = *sc.cam;
    // Camera::setup (camera.h:21-38) with degToRad (fwd.h:28-31)
    const float fov = c.fov_deg / 180.0f * 3.14159265358979323846f;
    const float tan_half = std::tan(fov * 0.5f);
    const float aspect = (float)c.width / (float)c.height;
    const float j0 = rng.uniform(), j1 = rng.uniform();
    const float rx = (float)(pixel % c.width) + j0;
    const float ry = (float)(pixel / c.width) + j1;
    const V3 dc = normalize(v3((1.0f - 2.0f * rx / (float)c.width) * tan_half,
                               (2.0f * ry / (float)c.height - 1.0f) * tan_half / aspect, 1.0f));
    const V3 d0 = normalize(v3(c.m[0] * dc.x + c.m[1] * dc.y + c.m[2] * dc.z,
                               c.m[4] * dc.x + c.m[5] * dc.y + c.m[6] * dc.z,
                               c.m[8] * dc.x + c.m[9] * dc.y + c.m[10] * dc.z));
    float ray[8] = {c.m[3], c.m[7], c.m[11], d0.x, d0.y, d0.z, 0.0f, 1e34f};
    V3 thr = vs(1.0f);
    float pdf_prev = 0.0f;
    bool spec = false;
    V3 L = vs(0.0f);
    Hit hit = trace(sc, ray, false);
    for (uint32_t b = 0; b <= D; ++b) {
        const V3 rd = v3(ray[3], ray[4], ray[5]);
        bool as_miss = false;
        if (b > 0) {  // finish the ray scattered by step b-1
            const float rr = rng.uniform();
            if (hit.prim >= 0 && !spec) {
                const or_material& lm = mat_of(sc, (uint32_t)hit.prim);
                if (lm.emissive) {
                    const Surf ls = surface(sc, (uint32_t)hit.prim, hit.u, hit.v);
                    float lpdf = (1.0f / area(sc, (uint32_t)hit.prim)) / (float)sc.lights.size();
                    lpdf *= hit.t * hit.t / std::fabs(dot(rd, ls.ns));
                    const V3 Le = dot(-rd, ls.ns) > 0.0f ? v3(lm.emission[0], lm.emission[1], lm.emission[2]) : vs(0.0f);
                    const float w = (pdf_prev * pdf_prev) / (pdf_prev * pdf_prev + lpdf * lpdf);
                    L = L + thr * Le * w;
                }
            }
            if (rr_depth >= 0 && (int)(b - 1) > rr_depth && maxc(thr) < 1.0f) {
                const float q = std::fmax(0.05f, 1.0f - maxc(thr));
                if (rr < q) {
                    if (compat) as_miss = true;
                    else break;
                } else if (!compat) {
                    thr = thr / (1.0f - q);
                }
            }
        }
        if (b == D) break;
        float s[8];
        for (int k = 0; k < 8; ++k) s[k] = rng.uniform();
        if (hit.prim < 0 || as_miss) {
            if (sc.has_env) L = L + thr * env_radiance(sc, v3(ray[0], ray[1], ray[2]), rd);
            break;
        }
        const or_material& m = mat_of(sc, (uint32_t)hit.prim);
        const Surf sf = surface(sc, (uint32_t)hit.prim, hit.u, hit.v);
        const V3 wo = -normalize(rd);
        if ((b == 0 || spec) && m.emissive && dot(wo, sf.ns) > 0.0f)
            L = L + thr * v3(m.emission[0], m.emission[1], m.emission[2]);
        Bsdf bs{make_frame(sf.ns), &m, compat, color_at(sc, m, sf.tu, sf.tv)};
        if (m.type != 1 && !sc.lights.empty()) {
            const uint32_t nl = (uint32_t)sc.lights.size();
            const uint32_t lid = std::min((uint32_t)(s[0] * (float)nl), nl - 1);
            const uint32_t lt = sc.lights[lid];
            const float a = std::sqrt(s[1]);
            const Surf ls = surface(sc, lt, 1.0f - a, s[2] * a);
            float lpdf = (1.0f / area(sc, lt)) / (float)nl;
            V3 wi = ls.p - sf.p;
            const float d2 = dot(wi, wi);
            wi = wi / std::sqrt(d2);
            lpdf *= d2 / std::fabs(dot(wi, ls.ns));
            if (std::isinf(lpdf)) lpdf = 0.0f;
            const or_material& lm = mat_of(sc, lt);
            const V3 Le = dot(-wi, ls.ns) > 0.0f ? v3(lm.emission[0], lm.emission[1], lm.emission[2]) : vs(0.0f);
            const V3 f = bsdf_eval(bs, wo, wi);
            const float bp = bsdf_pdf(bs, wo, wi);
            const float w = (lpdf * lpdf) / (lpdf * lpdf + bp * bp);
            if (lpdf > 0.0f) {
                const V3 cst = thr * Le * f * w / lpdf;
                if (!black(cst)) {
                    const V3 so = sf.p - rd * 1.0e-4f;
                    const V3 sd = ls.p - so;
                    const float sray[8] = {so.x, so.y, so.z, sd.x, sd.y, sd.z, 0.0f, 0.9999f};
                    if (trace(sc, sray, true).prim < 0) L = L + cst;
                }
            }
        }
        const Smp smp = bsdf_sample(bs, wo, s[5], s[6]);
        const V3 wgt = smp.pdf == 0.0f ? vs(0.0f) : thr * smp.f / smp.pdf;
        if (black(wgt)) break;
        ray[0] = sf.p.x; ray[1] = sf.p.y; ray[2] = sf.p.z;
        ray[3] = smp.wi.x; ray[4] = smp.wi.y; ray[5] = smp.wi.z;
        ray[6] = 1e-4f; ray[7] = 1e38f;
        thr = wgt;
        pdf_prev = smp.pdf;
        spec = smp.specular;
        hit = trace(sc, ray, false);
    }
    return L;
}

}  // namespace

extern "C" int or_render(const float* verts, const float* normals, const uint32_t* tri_mat, uint32_t ntri,
                         const or_material* mats, uint32_t nmat, const or_camera* cam, const float* env, int has_env,
                         uint32_t spp, uint32_t sample_base, uint32_t max_depth, uint64_t seed, int32_t rr_depth,
                         uint32_t flags, double* fb, int threads, const float* uvs, const float* texels,
                         const or_envmap* envmap) {
    Scene sc;
    sc.uvs = uvs;
    sc.texels = texels;
    sc.envmap = envmap;
    sc.verts = verts;
    sc.normals = normals;
    sc.tri_mat = tri_mat;
    sc.ntri = ntri;
    sc.mats = mats;
    sc.cam = cam;
    sc.env = env ? v3(env[0], env[1], env[2]) : vs(0.0f);
    sc.has_env = has_env != 0;
    for (uint32_t t = 0; t < ntri; ++t)
        if (mats[tri_mat[t] & 0x3FFFFFFFu].emissive) sc.lights.push_back(t);
    sc.nodes.assign(16ull * (ntri > 1 ? ntri - 1 : 1), 0);
    sc.tris.assign(12ull * (ntri ? ntri : 1), 0.0f);
    or_lbvh_build(verts, ntri, nullptr, nullptr, nullptr, sc.nodes.data(), sc.tris.data(), &sc.root);
    const uint32_t npix = cam->width * cam->height;
    const bool compat = (flags & 1u) != 0;
    std::atomic<uint32_t> next{0};
    auto work = [&] {
        for (;;) {
            const uint32_t p0 = next.fetch_add(64);
            if (p0 >= npix) break;
            const uint32_t p1 = std::min(npix, p0 + 64);
            for (uint32_t p = p0; p < p1; ++p) {
                for (uint32_t s = 0; s < spp; ++s) {
                    const V3 L = path(sc, p, sample_base + s, max_depth, seed, rr_depth, compat);
                    fb[3ull * p] += (double)L.x;
                    fb[3ull * p + 1] += (double)L.y;
                    fb[3ull * p + 2] += (double)L.z;
                }
            }
        }
    };
    const int nt = std::max(1, threads);
    std::vector<std::thread> pool;
    for (int i = 0; i < nt; ++i) pool.emplace_back(work);
    for (auto& t : pool) t.join();
    (void)nmat;
    return 0;
}
