// CPU oracle: ray traversal. Test infrastructure only (see oracle.h).
//
// Three traversals live here:
//   1. or_trace       — the product's FP32 watertight traversal, restated from
//                       its specification (not from the CUDA source) so that
//                       hit ids, t, u, v can be compared bit for bit.
//   2. or_trace_ref   — the reference's traversal (pathtracer_kernel.h:175-308)
//                       over its own node layout with its mixed-precision
//                       Moller-Trumbore test (:119-152) and slab test (:154-173).
//   3. or_fp64_check  — an FP64 distance oracle with an ambiguity classifier.
// Compiled with -ffp-contract=off: every a*b+c below rounds twice unless it
// is written as fmaf().
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

template <class F>
void parallel_rays(uint64_t nrays, int threads, F&& fn) {
    if (threads <= 1 || nrays < 4096) {
        fn(0, nrays);
        return;
    }
    std::atomic<uint64_t> next{0};
    const uint64_t chunk = 1024;
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        pool.emplace_back([&] {
            for (;;) {
                uint64_t b = next.fetch_add(chunk);
                if (b >= nrays) break;
                fn(b, std::min(nrays, b + chunk));
            }
        });
    }
    for (auto& th : pool) th.join();
}

inline float f_of(uint32_t w) { float f; std::memcpy(&f, &w, 4); return f; }
inline uint32_t w_of(float f) { uint32_t w; std::memcpy(&w, &f, 4); return w; }

// ---------------------------------------------------------------------------
// Product traversal specification
// ---------------------------------------------------------------------------
struct RayPre {
    float o[3], d[3], tmin, tmax;
    int kx, ky, kz;
    float sx, sy, sz;
    float idir[3];
};

inline void prepare(const float* r, RayPre& p) {
    for (int k = 0; k < 3; ++k) { p.o[k] = r[k]; p.d[k] = r[3 + k]; }
    p.tmin = r[6];
    p.tmax = r[7];
    // watertight set-up (Woop, Benthin, Wald, JCGT 2013): kz = dominant axis,
    // ties resolved toward the lower axis index
    float ax = std::fabs(p.d[0]), ay = std::fabs(p.d[1]), az = std::fabs(p.d[2]);
    int kz = 0;
    float m = ax;
    if (ay > m) { kz = 1; m = ay; }
    if (az > m) { kz = 2; }
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    if (p.d[kz] < 0.0f) { int t = kx; kx = ky; ky = t; }
    p.kx = kx; p.ky = ky; p.kz = kz;
    p.sx = p.d[kx] / p.d[kz];
    p.sy = p.d[ky] / p.d[kz];
    p.sz = 1.0f / p.d[kz];
    // slab set-up: near-zero components become +-2^-80 so no product is inf*0
    const float eps = 0x1p-80f;
    for (int k = 0; k < 3; ++k) {
        float dk = std::fabs(p.d[k]) > eps ? p.d[k] : std::copysign(eps, p.d[k]);
        p.idir[k] = 1.0f / dk;
    }
}

// Every cull keeps a box (or a deferred entry) while its entry distance is
// within (1 + 2^-16) of the exit / closest-hit distance; plane distances are
// (plane - o) * (1/d), within 3 ulps relative to themselves.
constexpr float kCullSlack = 1.0000152587890625f;

inline float plane_t(float plane, float o, float inv) { return (plane - o) * inv; }

// Child-box slab test; returns entry distance through *tn.
inline bool slab(const RayPre& p, float lox, float hix, float loy, float hiy, float loz, float hiz, float tbest,
                 float* tn) {
    float x0 = plane_t(lox, p.o[0], p.idir[0]), x1 = plane_t(hix, p.o[0], p.idir[0]);
    float y0 = plane_t(loy, p.o[1], p.idir[1]), y1 = plane_t(hiy, p.o[1], p.idir[1]);
    float z0 = plane_t(loz, p.o[2], p.idir[2]), z1 = plane_t(hiz, p.o[2], p.idir[2]);
    float tnear = std::fmax(std::fmax(std::fmin(x0, x1), std::fmin(y0, y1)), std::fmax(std::fmin(z0, z1), p.tmin));
    float tfar = std::fmin(std::fmin(std::fmax(x0, x1), std::fmax(y0, y1)), std::fmin(std::fmax(z0, z1), tbest));
    *tn = tnear;
    return tnear <= tfar * kCullSlack;
}

// Watertight FP32 test. Edge functions are plain products and differences so a
// shared edge evaluates to exactly opposite values in both triangles.
inline bool tri_test(const RayPre& p, const float* v0, const float* v1, const float* v2, float tbest, float* t_out,
                     float* u_out, float* v_out) {
    float A[3], B[3], C[3];
    for (int k = 0; k < 3; ++k) { A[k] = v0[k] - p.o[k]; B[k] = v1[k] - p.o[k]; C[k] = v2[k] - p.o[k]; }
    float Ax = std::fmaf(-p.sx, A[p.kz], A[p.kx]), Ay = std::fmaf(-p.sy, A[p.kz], A[p.ky]);
    float Bx = std::fmaf(-p.sx, B[p.kz], B[p.kx]), By = std::fmaf(-p.sy, B[p.kz], B[p.ky]);
    float Cx = std::fmaf(-p.sx, C[p.kz], C[p.kx]), Cy = std::fmaf(-p.sy, C[p.kz], C[p.ky]);
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = (U + V) + W;
    if (det == 0.0f) return false;
    float Az = p.sz * A[p.kz], Bz = p.sz * B[p.kz], Cz = p.sz * C[p.kz];
    float T = std::fmaf(U, Az, std::fmaf(V, Bz, W * Cz));
    float rcp = 1.0f / det;
    float t = T * rcp;
    if (!(t >= p.tmin && t <= tbest)) return false;
    *t_out = t;
    *u_out = V * rcp;
    *v_out = W * rcp;
    return true;
}

struct Best {
    float t, u, v;
    uint32_t prim;  // 0xFFFFFFFF = none
};

// Closest-hit acceptance: smaller t wins, equal t goes to the smaller prim id,
// which makes the result independent of the order triangles are visited in.
inline void consider(const RayPre& p, const float* tri, Best& b) {
    float t, u, v;
    if (!tri_test(p, tri, tri + 4, tri + 8, b.t, &t, &u, &v)) return;
    uint32_t prim = w_of(tri[3]);
    if (t < b.t || prim < b.prim) {
        b.t = t; b.u = u; b.v = v; b.prim = prim;
    }
}

void trace_one(const uint32_t* nodes, const float* tris, uint32_t root, const float* ray, int any, float* hit,
               uint32_t* st) {
    RayPre p;
    prepare(ray, p);
    Best b{p.tmax, 0.0f, 0.0f, 0xFFFFFFFFu};
    uint32_t visits = 0, tests = 0;
    struct Entry { int32_t node; float tn; };
    Entry stack[128];
    int sp = 0;
    int32_t node = (int32_t)root;
    bool done = (root == 0xFFFFFFFFu);
    while (!done) {
        const uint32_t* w = nodes + 16ull * (uint32_t)node;
        const float* f = reinterpret_cast<const float*>(w);
        ++visits;
        float tn0, tn1;
        bool h0 = slab(p, f[0], f[1], f[2], f[3], f[8], f[9], b.t, &tn0);
        bool h1 = slab(p, f[4], f[5], f[6], f[7], f[10], f[11], b.t, &tn1);
        int32_t c[2] = {(int32_t)w[12], (int32_t)w[13]};
        float tn[2] = {tn0, tn1};
        bool h[2] = {h0, h1};
        int first = (h0 && h1 && tn1 < tn0) ? 1 : 0;
        int32_t next = -1;
        bool have_next = false;
        for (int s = 0; s < 2 && !done; ++s) {
            int k = s == 0 ? first : 1 - first;
            if (!h[k]) continue;
            if (c[k] < 0) {
                const float* tri = tris + 12ull * (uint32_t)(~c[k]);
                ++tests;
                if (any) {
                    float t, u, v;
                    if (tri_test(p, tri, tri + 4, tri + 8, b.t, &t, &u, &v)) {
                        b.t = t; b.u = u; b.v = v; b.prim = w_of(tri[3]);
                        done = true;
                    }
                } else {
                    consider(p, tri, b);
                }
            } else if (!have_next) {
                next = c[k];
                have_next = true;
            } else {
                stack[sp].node = c[k];
                stack[sp].tn = tn[k];
                ++sp;
            }
        }
        if (done) break;
        if (!have_next) {
            for (;;) {
                if (sp == 0) { done = true; break; }
                --sp;
                if (any || stack[sp].tn <= b.t * kCullSlack) { next = stack[sp].node; have_next = true; break; }
            }
        }
        node = next;
    }
    if (b.prim == 0xFFFFFFFFu) {
        hit[0] = p.tmax;  // t of a miss is left at tMax; prim -1; u = v = 0
        uint32_t m = 0xFFFFFFFFu;
        std::memcpy(hit + 1, &m, 4);
        hit[2] = 0.0f; hit[3] = 0.0f;
    } else {
        hit[0] = b.t;
        std::memcpy(hit + 1, &b.prim, 4);
        hit[2] = b.u; hit[3] = b.v;
    }
    if (st) { st[0] = visits; st[1] = tests; }
}

// ---------------------------------------------------------------------------
// 4-wide layouts (product specification): every binary node at even depth
// becomes a 4-wide node at its own index; slots are its children, an inner
// child replaced by its two children. Boxes are copied (FP32) or quantised
// outward to 8 bits against origin + q * 2^e (one fma).
// ---------------------------------------------------------------------------
struct CB { float lo[3], hi[3]; };

inline CB child_box(const uint32_t* w, int slot) {
    const float* f = reinterpret_cast<const float*>(w);
    CB b;
    const float* xy = f + (slot == 0 ? 0 : 4);
    b.lo[0] = xy[0]; b.hi[0] = xy[1]; b.lo[1] = xy[2]; b.hi[1] = xy[3];
    b.lo[2] = f[slot == 0 ? 8 : 10];
    b.hi[2] = f[slot == 0 ? 9 : 11];
    return b;
}

inline float pow2(int e) { return f_of((uint32_t)(e + 127) << 23); }
inline float qdecode(int q, float scale, float origin) { return std::fmaf((float)q, scale, origin); }

inline int pick_exponent(float lo, float hi) {
    const float extent = hi - lo;
    int e = -126;
    if (extent > 0.0f) {
        int ex;
        std::frexp(extent / 255.0f, &ex);
        e = std::max(-126, std::min(127, ex));
    }
    while (e < 127 && qdecode(255, pow2(e), lo) < hi) ++e;
    return e;
}

inline uint32_t quant_lo(float v, float scale, float origin) {
    int q = (int)std::fmin(std::fmax(std::floor((v - origin) / scale), 0.0f), 255.0f);
    while (q > 0 && qdecode(q, scale, origin) > v) --q;
    while (q < 255 && qdecode(q + 1, scale, origin) <= v) ++q;
    return (uint32_t)q;
}

inline uint32_t quant_hi(float v, float scale, float origin) {
    int q = (int)std::fmin(std::fmax(std::ceil((v - origin) / scale), 0.0f), 255.0f);
    while (q < 255 && qdecode(q, scale, origin) < v) ++q;
    while (q > 0 && qdecode(q - 1, scale, origin) >= v) --q;
    return (uint32_t)q;
}

void build4(const uint32_t* nodes, uint32_t n, int quant, uint32_t* out) {
    const uint32_t count = n > 1 ? n - 1 : 1;
    const size_t words = quant ? 16 : 32;
    std::memset(out, 0, 4ull * words * count);
    for (uint32_t G = 0; G < count; ++G) {
        uint32_t depth = 0, x = G;
        while (nodes[16ull * x + 14] != 0xFFFFFFFFu) {
            x = nodes[16ull * x + 14];
            ++depth;
        }
        if (depth & 1u) continue;
        const uint32_t* nd = nodes + 16ull * G;
        CB box[4];
        int32_t ref[4] = {0, 0, 0, 0};
        int ns = 0;
        for (int k = 0; k < 2; ++k) {
            const int32_t c = (int32_t)nd[12 + k];
            if (c < 0) {
                box[ns] = child_box(nd, k);
                ref[ns++] = c;
            } else {
                const uint32_t* cn = nodes + 16ull * (uint32_t)c;
                box[ns] = child_box(cn, 0);
                ref[ns++] = (int32_t)cn[12];
                box[ns] = child_box(cn, 1);
                ref[ns++] = (int32_t)cn[13];
            }
        }
        const uint32_t mask = (1u << ns) - 1u;
        uint32_t* o = out + words * G;
        if (!quant) {  // lo.x[4] hi.x[4] lo.y[4] hi.y[4] lo.z[4] hi.z[4] child[4] meta[4]
            float* f = reinterpret_cast<float*>(o);
            for (int k = 0; k < ns; ++k)
                for (int a = 0; a < 3; ++a) {
                    f[8 * a + k] = box[k].lo[a];
                    f[8 * a + 4 + k] = box[k].hi[a];
                }
            for (int k = 0; k < 4; ++k) o[24 + k] = (uint32_t)ref[k];
            o[28] = mask;
        } else {
            float org[3], scale[3];
            uint32_t be[3];
            for (int a = 0; a < 3; ++a) {
                float lo = box[0].lo[a], hi = box[0].hi[a];
                for (int k = 1; k < ns; ++k) {
                    lo = std::fmin(lo, box[k].lo[a]);
                    hi = std::fmax(hi, box[k].hi[a]);
                }
                const int e = pick_exponent(lo, hi);
                org[a] = lo;
                be[a] = (uint32_t)(e + 127);
                scale[a] = pow2(e);
            }
            uint32_t wq[6] = {0, 0, 0, 0, 0, 0};
            for (int k = 0; k < ns; ++k)
                for (int a = 0; a < 3; ++a) {
                    wq[2 * a] |= quant_lo(box[k].lo[a], scale[a], org[a]) << (8 * k);
                    wq[2 * a + 1] |= quant_hi(box[k].hi[a], scale[a], org[a]) << (8 * k);
                }
            std::memcpy(o, org, 12);
            o[3] = be[0] | (be[1] << 8) | (be[2] << 16) | (mask << 24);
            for (int k = 0; k < 6; ++k) o[4 + k] = wq[k];
            for (int k = 0; k < 4; ++k) o[12 + k] = (uint32_t)ref[k];
        }
    }
}

void trace4_one(const uint32_t* nodes, int quant, const float* tris, uint32_t root, const float* ray, int any,
                float* hit, uint32_t* st) {
    RayPre p;
    prepare(ray, p);
    Best b{p.tmax, 0.0f, 0.0f, 0xFFFFFFFFu};
    uint32_t visits = 0, tests = 0;
    struct Entry { int32_t node; float tn; };
    Entry stack[256];
    int sp = 0;
    int32_t node = (int32_t)root;
    bool done = root == 0xFFFFFFFFu;
    const size_t words = quant ? 16 : 32;
    while (!done) {
        const uint32_t* o = nodes + words * (uint32_t)node;
        ++visits;
        float tn[4] = {0, 0, 0, 0};
        bool h[4] = {false, false, false, false};
        int32_t c[4];
        if (quant) {
            const float* org = reinterpret_cast<const float*>(o);
            const uint32_t meta = o[3];
            const float sc[3] = {f_of((meta & 0xFFu) << 23), f_of(((meta >> 8) & 0xFFu) << 23),
                                 f_of(((meta >> 16) & 0xFFu) << 23)};
            const uint32_t mask = meta >> 24;
            for (int k = 0; k < 4; ++k) {
                c[k] = (int32_t)o[12 + k];
                if (!(mask & (1u << k))) continue;
                float pl[6];
                for (int a = 0; a < 3; ++a) {
                    pl[2 * a] = qdecode((int)((o[4 + 2 * a] >> (8 * k)) & 0xFFu), sc[a], org[a]);
                    pl[2 * a + 1] = qdecode((int)((o[5 + 2 * a] >> (8 * k)) & 0xFFu), sc[a], org[a]);
                }
                h[k] = slab(p, pl[0], pl[1], pl[2], pl[3], pl[4], pl[5], b.t, &tn[k]);
            }
        } else {
            const float* f = reinterpret_cast<const float*>(o);
            const uint32_t mask = o[28];
            for (int k = 0; k < 4; ++k) {
                c[k] = (int32_t)o[24 + k];
                if (!(mask & (1u << k))) continue;
                h[k] = slab(p, f[k], f[4 + k], f[8 + k], f[12 + k], f[16 + k], f[20 + k], b.t, &tn[k]);
            }
        }
        int rank[4];
        for (int k = 0; k < 4; ++k) {
            int r = 0;
            for (int j = 0; j < 4; ++j)
                if (j != k && h[j] && (tn[j] < tn[k] || (tn[j] == tn[k] && j < k))) ++r;
            rank[k] = r;
        }
        int32_t next = -1;
        bool have = false;
        int np = 0;
        int32_t pc[3];
        float pt[3];
        for (int r = 0; r < 4 && !done; ++r) {
            int k = -1;
            for (int j = 0; j < 4; ++j)
                if (h[j] && rank[j] == r) k = j;
            if (k < 0) continue;
            if (c[k] < 0) {
                const float* tri = tris + 12ull * (uint32_t)(~c[k]);
                ++tests;
                if (any) {
                    float t, u, v;
                    if (tri_test(p, tri, tri + 4, tri + 8, b.t, &t, &u, &v)) {
                        b.t = t; b.u = u; b.v = v; b.prim = w_of(tri[3]);
                        done = true;
                    }
                } else {
                    consider(p, tri, b);
                }
            } else if (!have) {
                next = c[k];
                have = true;
            } else {
                pc[np] = c[k];
                pt[np] = tn[k];
                ++np;
            }
        }
        if (done) break;
        for (int k = np - 1; k >= 0; --k) stack[sp++] = {pc[k], pt[k]};
        if (!have) {
            for (;;) {
                if (sp == 0) { done = true; break; }
                --sp;
                if (any || stack[sp].tn <= b.t * kCullSlack) { next = stack[sp].node; have = true; break; }
            }
        }
        node = next;
    }
    if (b.prim == 0xFFFFFFFFu) {
        hit[0] = p.tmax;
        uint32_t m = 0xFFFFFFFFu;
        std::memcpy(hit + 1, &m, 4);
        hit[2] = 0.0f; hit[3] = 0.0f;
    } else {
        hit[0] = b.t;
        std::memcpy(hit + 1, &b.prim, 4);
        hit[2] = b.u; hit[3] = b.v;
    }
    if (st) { st[0] = visits; st[1] = tests; }
}

// ---------------------------------------------------------------------------
// 8-wide quantised layout: the level-by-level collapse and its traversal,
// restated sequentially in the same order (nodes breadth first, a level's
// children in node order then slot order) so nodes, triangles and any-hit
// results compare word for word.
// ---------------------------------------------------------------------------
inline float half_area(const CB& b) {
    const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    return (dx * dy + dy * dz) + dz * dx;
}

constexpr int32_t kEmpty8 = std::numeric_limits<int32_t>::min();
constexpr int kMaxExp8 = 119;

// 8-wide planes: plane(q) = q * 2^e + lo taken exactly. q * 2^e is a float,
// so a plane compares with a coordinate exactly through the rounded sum and
// its two-sum error.
inline int cmp_sum(float a, float b, float v) {
    const float s = a + b;
    if (s != v) return s < v ? -1 : 1;
    const float bp = s - a;
    const float e = (a - (s - bp)) + (b - bp);
    return e < 0.0f ? -1 : (e > 0.0f ? 1 : 0);
}

inline int cmp_plane(int q, float scale, float lo, float v) { return cmp_sum((float)q * scale, lo, v); }

inline int pick_exponent8(float lo, float hi) {
    const float extent = hi - lo;
    int e = -126;
    if (extent > 0.0f) {
        int ex;
        std::frexp(extent / 255.0f, &ex);
        e = std::max(-126, std::min(kMaxExp8, ex - 1));
    }
    while (cmp_plane(255, pow2(e), lo, hi) < 0) {
        if (e >= kMaxExp8) break;
        ++e;
    }
    return e;
}

inline uint32_t quant_lo8(float v, float scale, float lo) {
    int q = 0;
    for (int step = 128; step > 0; step >>= 1)
        if (q + step <= 255 && cmp_plane(q + step, scale, lo, v) <= 0) q += step;
    return (uint32_t)q;
}

inline uint32_t quant_hi8(float v, float scale, float lo) {
    int q = 255;
    for (int step = 128; step > 0; step >>= 1)
        if (q - step >= 0 && cmp_plane(q - step, scale, lo, v) >= 0) q -= step;
    return (uint32_t)q;
}

void build8(const uint32_t* nodes, const float* tris, uint32_t root, std::vector<uint32_t>& out,
            std::vector<float>& out_tris) {
    std::vector<uint32_t> frontier{root};
    uint32_t out_base = 0, tri_cursor = 0;
    while (!frontier.empty()) {
        const uint32_t level_n = (uint32_t)frontier.size();
        const uint32_t next_base = out_base + level_n;
        std::vector<uint32_t> next;
        out.resize(24ull * (out_base + level_n), 0u);
        uint32_t inner_acc = 0, leaf_acc = 0;
        for (uint32_t i = 0; i < level_n; ++i) {
            const uint32_t* rw = nodes + 16ull * frontier[i];
            CB box[8];
            int32_t ref[8];
            int cnt = 2;
            ref[0] = (int32_t)rw[12];
            box[0] = child_box(rw, 0);
            ref[1] = (int32_t)rw[13];
            box[1] = child_box(rw, 1);
            while (cnt < 8) {
                int best = -1;
                float best_a = 0.0f;
                for (int k = 0; k < cnt; ++k)
                    if (ref[k] >= 0) {
                        const float a = half_area(box[k]);
                        if (best < 0 || a > best_a) { best = k; best_a = a; }
                    }
                if (best < 0) break;
                const uint32_t* cw = nodes + 16ull * (uint32_t)ref[best];
                ref[best] = (int32_t)cw[12];
                box[best] = child_box(cw, 0);
                ref[cnt] = (int32_t)cw[13];
                box[cnt] = child_box(cw, 1);
                ++cnt;
            }
            float lo[3], hi[3], nc[3];
            for (int a = 0; a < 3; ++a) {
                lo[a] = box[0].lo[a];
                hi[a] = box[0].hi[a];
                for (int k = 1; k < cnt; ++k) {
                    lo[a] = std::fmin(lo[a], box[k].lo[a]);
                    hi[a] = std::fmax(hi[a], box[k].hi[a]);
                }
                nc[a] = lo[a] + hi[a];
            }
            int slot_of[8];
            uint32_t used = 0;
            for (int k = 0; k < 8; ++k) slot_of[k] = -1;
            for (int it = 0; it < cnt; ++it) {
                int bk = -1, bs = -1;
                float bsc = 0.0f;
                for (int k = 0; k < cnt; ++k) {
                    if (slot_of[k] >= 0) continue;
                    const float dx = (box[k].lo[0] + box[k].hi[0]) - nc[0];
                    const float dy = (box[k].lo[1] + box[k].hi[1]) - nc[1];
                    const float dz = (box[k].lo[2] + box[k].hi[2]) - nc[2];
                    for (int s2 = 0; s2 < 8; ++s2) {
                        if (used & (1u << s2)) continue;
                        const float sc = (((s2 & 1) ? dx : -dx) + ((s2 & 2) ? dy : -dy)) + ((s2 & 4) ? dz : -dz);
                        if (bk < 0 || sc > bsc) { bk = k; bs = s2; bsc = sc; }
                    }
                }
                slot_of[bk] = bs;
                used |= 1u << bs;
            }
            float scale[3];
            uint32_t be[3];
            for (int a = 0; a < 3; ++a) {
                const int e = pick_exponent8(lo[a], hi[a]);
                be[a] = (uint32_t)(e + 127);
                scale[a] = f_of(be[a] << 23);
            }
            uint32_t* o = out.data() + 24ull * (out_base + i);
            o[0] = w_of(lo[0]);
            o[1] = w_of(lo[1]);
            o[2] = w_of(lo[2]);
            int32_t sref[8];
            for (int s2 = 0; s2 < 8; ++s2) sref[s2] = kEmpty8;
            uint32_t imask = 0, ni = 0, nl = 0;
            for (int k = 0; k < cnt; ++k) {
                const int s2 = slot_of[k];
                sref[s2] = ref[k];
                if (ref[k] >= 0) { imask |= 1u << s2; ++ni; } else { ++nl; }
                for (int a = 0; a < 3; ++a) {
                    o[8 + 4 * a + (s2 >> 2)] |= quant_lo8(box[k].lo[a], scale[a], lo[a]) << (8 * (s2 & 3));
                    o[8 + 4 * a + 2 + (s2 >> 2)] |= quant_hi8(box[k].hi[a], scale[a], lo[a]) << (8 * (s2 & 3));
                }
            }
            o[3] = be[0] | (be[1] << 8) | (be[2] << 16) | (imask << 24);
            o[4] = next_base + inner_acc;
            o[5] = tri_cursor + leaf_acc;
            o[6] = used;
            uint32_t rl = 0;
            for (int s2 = 0; s2 < 8; ++s2) {
                const int32_t r = sref[s2];
                if (r == kEmpty8) continue;
                if (r >= 0) {
                    next.push_back((uint32_t)r);
                } else {
                    const size_t dst = 12ull * (tri_cursor + leaf_acc + rl++);
                    if (out_tris.size() < dst + 12) out_tris.resize(dst + 12);
                    std::memcpy(out_tris.data() + dst, tris + 12ull * (uint32_t)(~r), 48);
                }
            }
            inner_acc += ni;
            leaf_acc += nl;
        }
        out_base += level_n;
        tri_cursor += leaf_acc;
        frontier.swap(next);
    }
}

inline uint32_t byte_of(uint32_t w, int k) { return (w >> (8 * k)) & 0xFFu; }
inline int ctz32(uint32_t x) { int k = 0; while (!(x & 1u)) { x >>= 1; ++k; } return k; }
inline uint32_t popc32(uint32_t x) { uint32_t c = 0; while (x) { x &= x - 1u; ++c; } return c; }

void trace8_one(const uint32_t* nodes, const float* tris, uint32_t root, const float* ray, int any, float* hit,
                uint32_t* st) {
    RayPre p;
    prepare(ray, p);
    Best b{p.tmax, 0.0f, 0.0f, 0xFFFFFFFFu};
    uint32_t visits = 0, tests = 0;
    struct Group { uint32_t base, word; };
    Group stack[256];
    int sp = 0;
    uint32_t node = 0;
    bool done = root == 0xFFFFFFFFu;
    const uint32_t sg[3] = {w_of(p.idir[0]) >> 31, w_of(p.idir[1]) >> 31, w_of(p.idir[2]) >> 31};
    const uint32_t oct = sg[0] | (sg[1] << 1) | (sg[2] << 2);
    while (!done) {
        const uint32_t* o = nodes + 24ull * node;
        ++visits;
        const uint32_t meta = o[3], child_base = o[4], tri_base = o[5], valid = o[6], imask = meta >> 24;
        float S[3], cn[3], cf[3];
        uint32_t nw[3][2], fw[3][2];
        const float bound = b.t * kCullSlack;
        for (int a = 0; a < 3; ++a) {
            // plane distance q * S + C measured as fma(1 + q * 2^-15, S', C' -+ m)
            // with S' = 2^15 S, C' = C - S' and m = |C| 2^-20 + |S| 2^-7
            const float Sa = f_of(((meta >> (8 * a)) & 0xFFu) << 23) * p.idir[a];
            const float C = (f_of(o[a]) - p.o[a]) * p.idir[a];
            S[a] = Sa * 32768.0f;
            const float Cp = C - S[a];
            const float m = std::fmaf(std::fabs(C), 0x1p-20f, std::fabs(Sa) * 0x1p-7f);
            cn[a] = Cp - m;
            cf[a] = Cp + m;
            for (int h = 0; h < 2; ++h) {
                const uint32_t lo = o[8 + 4 * a + h], hi = o[8 + 4 * a + 2 + h];
                nw[a][h] = sg[a] ? hi : lo;
                fw[a][h] = sg[a] ? lo : hi;
            }
        }
        uint32_t ihits = 0, thits = 0;
        for (int k = 0; k < 8; ++k) {
            float tn[3], tf[3];
            for (int a = 0; a < 3; ++a) {
                tn[a] = std::fmaf(f_of(0x3F800000u | (byte_of(nw[a][k >> 2], k & 3) << 8)), S[a], cn[a]);
                tf[a] = std::fmaf(f_of(0x3F800000u | (byte_of(fw[a][k >> 2], k & 3) << 8)), S[a], cf[a]);
            }
            const float tnear = std::fmax(std::fmax(std::fmax(tn[0], tn[1]), tn[2]), p.tmin);
            const float tfar = std::fmin(std::fmin(std::fmin(tf[0], tf[1]), tf[2]), bound);
            if (((valid >> k) & 1u) && tnear <= tfar) {
                if ((imask >> k) & 1u) ihits |= 1u << (k ^ (int)oct);
                else thits |= 1u << k;
            }
        }
        const uint32_t leafmask = valid & ~imask;
        while (thits && !done) {
            const int k = ctz32(thits);
            thits &= thits - 1u;
            const float* tri = tris + 12ull * (tri_base + popc32(leafmask & ((1u << k) - 1u)));
            ++tests;
            if (any) {
                float t, u, v;
                if (tri_test(p, tri, tri + 4, tri + 8, b.t, &t, &u, &v)) {
                    b.t = t; b.u = u; b.v = v; b.prim = w_of(tri[3]);
                    done = true;
                }
            } else {
                consider(p, tri, b);
            }
        }
        if (done) break;
        uint32_t gbase = child_base, gmask = imask, hits = ihits;
        if (hits) {
            if (hits & (hits - 1u)) stack[sp++] = {child_base, imask | ((hits & (hits - 1u)) << 8)};
        } else {
            if (sp == 0) break;
            Group& g = stack[sp - 1];
            gbase = g.base;
            gmask = g.word & 0xFFu;
            hits = g.word >> 8;
            const uint32_t rest = hits & (hits - 1u);
            if (rest) g.word = gmask | (rest << 8); else --sp;
        }
        const uint32_t slot = (uint32_t)ctz32(hits) ^ oct;
        node = gbase + popc32(gmask & ((1u << slot) - 1u));
    }
    if (b.prim == 0xFFFFFFFFu) {
        hit[0] = p.tmax;
        uint32_t m = 0xFFFFFFFFu;
        std::memcpy(hit + 1, &m, 4);
        hit[2] = 0.0f; hit[3] = 0.0f;
    } else {
        hit[0] = b.t;
        std::memcpy(hit + 1, &b.prim, 4);
        hit[2] = b.u; hit[3] = b.v;
    }
    if (st) { st[0] = visits; st[1] = tests; }
}

// ---------------------------------------------------------------------------
// Reference traversal (pathtracer_kernel.h)
// ---------------------------------------------------------------------------
struct V3 { float x, y, z; };
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// triangle_intersect (:119-152): float cross/dot, double determinant chain,
// inclusive edges and inclusive [tMin, tMax]
inline bool ref_tri(const float* tv, V3 o, V3 D, float tmin, float tmax, float* th, float* uh, float* vh) {
    V3 p0{tv[0], tv[1], tv[2]}, p1{tv[3], tv[4], tv[5]}, p2{tv[6], tv[7], tv[8]};
    V3 E1 = sub(p1, p0), E2 = sub(p2, p0);
    V3 P = cross(D, E2);
    double det = dot(P, E1);
    if (det == 0) return false;
    double invDet = 1.0 / det;
    V3 T = sub(o, p0);
    double u = dot(P, T) * invDet;
    if (u < 0.0 || u > 1.0) return false;
    V3 Q = cross(T, E1);
    double v = dot(Q, D) * invDet;
    if (v < 0.0 || u + v > 1.0) return false;
    double t = dot(Q, E2) * invDet;
    if (t < tmin || t > tmax) return false;
    *th = (float)t; *uh = (float)u; *vh = (float)v;
    return true;
}

// aabb_intersect (:154-173); device min/max on floats are fminf/fmaxf
inline bool ref_box(const float* lo, const float* hi, V3 o, V3 inv, const int neg[3], float rtmin, float rtmax) {
    const float* sel[2] = {lo, hi};
    float tMin = (sel[neg[0]][0] - o.x) * inv.x;
    float tMax = (sel[1 - neg[0]][0] - o.x) * inv.x;
    float tyMin = (sel[neg[1]][1] - o.y) * inv.y;
    float tyMax = (sel[1 - neg[1]][1] - o.y) * inv.y;
    if (tMin > tyMax || tyMin > tMax) return false;
    tMin = std::fmax(tMin, tyMin);
    tMax = std::fmin(tMax, tyMax);
    float tzMin = (sel[neg[2]][2] - o.z) * inv.z;
    float tzMax = (sel[1 - neg[2]][2] - o.z) * inv.z;
    if (tMin > tzMax || tzMin > tMax) return false;
    tMin = std::fmax(tMin, tzMin);
    tMax = std::fmin(tMax, tzMax);
    return (tMin < rtmax) && (tMax > rtmin);
}

void trace_ref_one(const uint32_t* nodes, const float* verts, const float* ray, int any, float* hit, uint32_t* st) {
    V3 o{ray[0], ray[1], ray[2]}, d{ray[3], ray[4], ray[5]};
    float tmin = ray[6], tmax = ray[7];
    V3 inv{1 / d.x, 1 / d.y, 1 / d.z};
    int neg[3] = {inv.x < 0, inv.y < 0, inv.z < 0};
    float ht = 0, hu = 0, hv = 0;
    int32_t hid = -1;
    int cur = 0, sp = 0;
    int stack[64];
    uint32_t visits = 0, tests = 0;
    for (;;) {
        const uint32_t* w = nodes + 8ull * cur;
        const float* f = reinterpret_cast<const float*>(w);
        ++visits;
        if (ref_box(f, f + 3, o, inv, neg, tmin, tmax)) {
            if (w[7]) {
                ++tests;
                float t, u, v;
                if (ref_tri(verts + 9ull * w[6], o, d, tmin, tmax, &t, &u, &v)) {
                    ht = t; hu = u; hv = v;
                    tmax = t;
                    hid = (int32_t)w[6];
                    if (any) break;
                }
                if (sp == 0) break;
                cur = stack[--sp];
            } else {
                if (sp >= 64) break;  // the reference's stack holds 64 entries
                stack[sp++] = cur + 1;
                cur = (int)w[6];
            }
        } else {
            if (sp == 0) break;
            cur = stack[--sp];
        }
    }
    // the reference leaves t/u/v unset on a miss; the oracle reports zeros
    hit[0] = hid < 0 ? 0.0f : ht;
    std::memcpy(hit + 1, &hid, 4);
    hit[2] = hid < 0 ? 0.0f : hu;
    hit[3] = hid < 0 ? 0.0f : hv;
    if (st) { st[0] = visits; st[1] = tests; }
}

// ---------------------------------------------------------------------------
// FP64 oracle
// ---------------------------------------------------------------------------
struct D3 { double x, y, z; };
inline D3 dsub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 dcross(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double ddot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// Double-precision Moller-Trumbore. Accepts a near miss whose smallest
// barycentric coordinate is at least -tol, or whose hit point lies at most
// edge_tol (world units) outside the nearest edge. Returns t, the smallest
// barycentric coordinate and the signed distance of the hit point from the
// nearest edge line (each barycentric times its vertex's height over the
// opposite edge).
inline bool tri64(const float* tv, D3 o, D3 d, double tol, double edge_tol, double* t, double* minbary,
                  double* edge_dist) {
    D3 p0{tv[0], tv[1], tv[2]}, p1{tv[3], tv[4], tv[5]}, p2{tv[6], tv[7], tv[8]};
    D3 e1 = dsub(p1, p0), e2 = dsub(p2, p0);
    D3 P = dcross(d, e2);
    double det = ddot(P, e1);
    if (det == 0) return false;
    double inv = 1.0 / det;
    D3 T = dsub(o, p0);
    double u = ddot(P, T) * inv;
    D3 Q = dcross(T, e1);
    double v = ddot(Q, d) * inv;
    double w = 1.0 - u - v;
    double mb = std::fmin(u, std::fmin(v, w));
    D3 nrm = dcross(e1, e2), e12 = dsub(p2, p1);
    const double twice_area = std::sqrt(ddot(nrm, nrm));
    const double l0 = std::sqrt(ddot(e12, e12)), l1 = std::sqrt(ddot(e2, e2)), l2 = std::sqrt(ddot(e1, e1));
    double dist = 0.0;
    if (l0 > 0 && l1 > 0 && l2 > 0)
        dist = std::fmin(w * twice_area / l0, std::fmin(u * twice_area / l1, v * twice_area / l2));
    if (mb < -tol && dist < -edge_tol) return false;
    *t = ddot(Q, e2) * inv;
    *minbary = mb;
    *edge_dist = dist;
    return true;
}

// Largest coordinate magnitude among the ray origin and the triangle's
// vertices: the scale of the FP32 rounding in either traversal's arithmetic.
inline double coord_scale(const float* tv, D3 o) {
    double s = std::fmax(std::fabs(o.x), std::fmax(std::fabs(o.y), std::fabs(o.z)));
    for (int k = 0; k < 9; ++k) s = std::fmax(s, std::fabs((double)tv[k]));
    return s;
}

}  // namespace

extern "C" void or_trace(const uint32_t* nodes, const float* tris, uint32_t root, const float* rays, uint64_t nrays,
                         int any_hit, float* hits, uint32_t* stats, int threads) {
    parallel_rays(nrays, threads, [&](uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; ++i)
            trace_one(nodes, tris, root, rays + 8 * i, any_hit, hits + 4 * i, stats ? stats + 2 * i : nullptr);
    });
}

extern "C" void or_trace_brute(const float* verts, uint32_t n, const float* rays, uint64_t nrays, int any_hit,
                               float* hits, int threads) {
    parallel_rays(nrays, threads, [&](uint64_t b, uint64_t e) {
        float tri[12];
        for (uint64_t i = b; i < e; ++i) {
            RayPre p;
            prepare(rays + 8 * i, p);
            Best best{p.tmax, 0.0f, 0.0f, 0xFFFFFFFFu};
            for (uint32_t j = 0; j < n; ++j) {
                const float* v = verts + 9ull * j;
                tri[0] = v[0]; tri[1] = v[1]; tri[2] = v[2]; std::memcpy(tri + 3, &j, 4);
                tri[4] = v[3]; tri[5] = v[4]; tri[6] = v[5];
                tri[8] = v[6]; tri[9] = v[7]; tri[10] = v[8];
                if (any_hit) {
                    float t, u, vv;
                    if (tri_test(p, tri, tri + 4, tri + 8, p.tmax, &t, &u, &vv)) {
                        best = {t, u, vv, j};
                        break;
                    }
                } else {
                    consider(p, tri, best);
                }
            }
            float* h = hits + 4 * i;
            if (best.prim == 0xFFFFFFFFu) {
                h[0] = p.tmax; uint32_t m = 0xFFFFFFFFu; std::memcpy(h + 1, &m, 4); h[2] = h[3] = 0.0f;
            } else {
                h[0] = best.t; std::memcpy(h + 1, &best.prim, 4); h[2] = best.u; h[3] = best.v;
            }
        }
    });
}

extern "C" void or_trace_ref(const uint32_t* ref_nodes, const float* verts, uint32_t n, const float* rays,
                             uint64_t nrays, int any_hit, float* hits, uint32_t* stats, int threads) {
    if (n == 0) {
        for (uint64_t i = 0; i < nrays; ++i) {
            int32_t m = -1;
            hits[4 * i] = 0.0f; std::memcpy(hits + 4 * i + 1, &m, 4); hits[4 * i + 2] = hits[4 * i + 3] = 0.0f;
            if (stats) stats[2 * i] = stats[2 * i + 1] = 0;
        }
        return;
    }
    parallel_rays(nrays, threads, [&](uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; ++i)
            trace_ref_one(ref_nodes, verts, rays + 8 * i, any_hit, hits + 4 * i, stats ? stats + 2 * i : nullptr);
    });
}

extern "C" void or_fp64_check(const uint32_t* ref_nodes, const float* verts, uint32_t n, const float* rays,
                              uint64_t nrays, const int32_t* prim, double* t64, uint8_t* ambiguous, double rel_gap,
                              double bary_margin, double edge_rel, int threads) {
    parallel_rays(nrays, threads, [&](uint64_t b, uint64_t e) {
        std::vector<int> stack;
        stack.reserve(128);
        for (uint64_t i = b; i < e; ++i) {
            const float* r = rays + 8 * i;
            D3 o{r[0], r[1], r[2]}, d{r[3], r[4], r[5]};
            double tmin = r[6], tmax = r[7];
            // distance to the reported triangle
            double tp = std::numeric_limits<double>::quiet_NaN();
            if (prim[i] >= 0 && (uint32_t)prim[i] < n) {
                double t, mb, ed;
                if (tri64(verts + 9ull * prim[i], o, d, 1e30, 1e30, &t, &mb, &ed)) tp = t;
            }
            t64[i] = tp;
            // all candidates within tolerance: closest and runner-up distances
            double best = std::numeric_limits<double>::infinity(), second = best, best_mb = 1.0;
            double best_ed = 1.0, best_tol = 0.0;
            if (n > 0) {
                stack.clear();
                stack.push_back(0);
                while (!stack.empty()) {
                    int cur = stack.back();
                    stack.pop_back();
                    const uint32_t* w = ref_nodes + 8ull * cur;
                    const float* f = reinterpret_cast<const float*>(w);
                    // padded FP64 slab test (conservative)
                    double t0 = -std::numeric_limits<double>::infinity(), t1 = -t0;
                    const double pad = 1e-6;
                    double dd[3] = {d.x, d.y, d.z}, oo[3] = {o.x, o.y, o.z};
                    bool in = true;
                    for (int k = 0; k < 3 && in; ++k) {
                        double lo = f[k], hi = f[3 + k];
                        double ext = pad * (1.0 + std::fabs(lo) + std::fabs(hi));
                        lo -= ext; hi += ext;
                        if (dd[k] == 0.0) {
                            if (oo[k] < lo || oo[k] > hi) in = false;
                            continue;
                        }
                        double a = (lo - oo[k]) / dd[k], c = (hi - oo[k]) / dd[k];
                        if (a > c) std::swap(a, c);
                        t0 = std::fmax(t0, a);
                        t1 = std::fmin(t1, c);
                    }
                    if (!in || t0 > t1 || t1 < tmin * (1 - 1e-6) - 1e-9 || t0 > tmax * (1 + 1e-6) + 1e-9) continue;
                    if (t0 > second * (1 + 1e-6) + 1e-9) continue;
                    if (w[7]) {
                        double t, mb, ed;
                        const float* tv = verts + 9ull * w[6];
                        const double etol = edge_rel * coord_scale(tv, o);
                        if (tri64(tv, o, d, bary_margin, etol, &t, &mb, &ed)) {
                            if (t < tmin * (1 - 1e-7) - 1e-12 || t > tmax * (1 + 1e-7) + 1e-12) continue;
                            if (t < best) { second = best; best = t; best_mb = mb; best_ed = ed; best_tol = etol; }
                            else if (t < second) second = t;
                        }
                    } else {
                        stack.push_back(cur + 1);
                        stack.push_back((int)w[6]);
                    }
                }
            }
            bool amb = false;
            if (best < std::numeric_limits<double>::infinity()) {
                if (best_mb < bary_margin || best_ed < best_tol) amb = true;
                if (second - best <= rel_gap * std::fmax(std::fabs(best), 1e-30)) amb = true;
                if (std::fabs(best - tmin) <= rel_gap * std::fmax(std::fabs(best), 1e-30)) amb = true;
                if (std::fabs(best - tmax) <= rel_gap * std::fmax(std::fabs(best), 1e-30)) amb = true;
            }
            ambiguous[i] = amb ? 1 : 0;
        }
    });
}

extern "C" void or_bvh4_build(const uint32_t* bvh2_nodes, uint32_t n, int quant, uint32_t* out) {
    if (n == 0) return;
    build4(bvh2_nodes, n, quant, out);
}

extern "C" void or_trace4(const uint32_t* nodes4, int quant, const float* tris, uint32_t root, const float* rays,
                          uint64_t nrays, int any_hit, float* hits, uint32_t* stats, int threads) {
    parallel_rays(nrays, threads, [&](uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; ++i)
            trace4_one(nodes4, quant, tris, root, rays + 8 * i, any_hit, hits + 4 * i, stats ? stats + 2 * i : nullptr);
    });
}

extern "C" uint32_t or_bvh8_build(const uint32_t* bvh2_nodes, const float* tri_sorted, uint32_t n, uint32_t root,
                                  uint32_t* out_nodes, uint32_t max_nodes, float* out_tris, uint32_t max_tris,
                                  uint32_t* n_tris) {
    if (n == 0) { if (n_tris) *n_tris = 0; return 0; }
    std::vector<uint32_t> nodes;
    std::vector<float> tris;
    build8(bvh2_nodes, tri_sorted, root, nodes, tris);
    const uint32_t count = (uint32_t)(nodes.size() / 24), nt = (uint32_t)(tris.size() / 12);
    if (out_nodes) std::memcpy(out_nodes, nodes.data(), 96ull * std::min(count, max_nodes));
    if (out_tris) std::memcpy(out_tris, tris.data(), 48ull * std::min(nt, max_tris));
    if (n_tris) *n_tris = nt;
    return count;
}

extern "C" void or_trace8(const uint32_t* nodes8, const float* tris8, uint32_t root, const float* rays,
                          uint64_t nrays, int any_hit, float* hits, uint32_t* stats, int threads) {
    parallel_rays(nrays, threads, [&](uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; ++i)
            trace8_one(nodes8, tris8, root, rays + 8 * i, any_hit, hits + 4 * i, stats ? stats + 2 * i : nullptr);
    });
}
