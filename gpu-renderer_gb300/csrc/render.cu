// Wavefront path tracer: camera rays, closest-hit queue traversal, shading
// with next-event estimation + MIS, shadow any-hit with fused accumulation,
// Russian roulette, and the per-pixel resolve.
//
// Replaces PathTracer::render(uint32*) and its kernels (slongle/GPU-Renderer
// src/renderer/pathtracer.cu:41-150, pathtracer_kernel.h:59-821). The
// reference runs one 1-spp frame per call with 9 device syncs and 4 host reads
// of queue counters per bounce. Here every count stays on the device: a wave
// of paths (several samples per pixel at once) runs a fixed kernel sequence
// whose sizes are read on the device, with no host synchronisation inside a
// render call.
//
// Path state is indexed by a stable path id (pid = s * npix + pixel) and the
// queues hold path ids, so a path keeps its RNG stream and its radiance
// accumulator wherever it is queued. Each path accumulates its own radiance;
// the resolve adds paths to their pixel in sample order, so the image does not
// depend on queue order, wave size, or what else is rendered alongside.
#include <algorithm>

#include "render.h"
#include "shading.cuh"
#include "traverse.cuh"

namespace gr {
namespace {

using namespace sh;

constexpr uint32_t kFlagSpecular = 1u;
constexpr int kShadeThreads = 256;
constexpr int kShadowBase = kMaxDepth + 1;  // shadow queue counters start here
constexpr int kErrWord = 2 * kMaxDepth + 4;

__device__ __forceinline__ uint32_t lane_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Warp-aggregated append: one atomic per warp, slots in lane order. Every lane
// of the warp must call it (pred false for lanes with nothing to append).
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool pred) {
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, pred);
    uint32_t base = 0;
    const int lane = threadIdx.x & 31;
    if (lane == 0 && m) base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    return base + __popc(m & lane_lt());
}

__device__ __forceinline__ V3 load3(const float* p) { return v3(p[0], p[1], p[2]); }

// ---- BSDF over one material (bsdf.h:16-184 for a single lobe) ------------------
struct Bsdf {
    Frame fr;
    const DevMaterial* m;
    bool compat;
};

__device__ __forceinline__ V3 mcolor(const DevMaterial* m) { return v3(m->cr, m->cg, m->cb); }

// GGX reflection f*cos (MicrofacetReflectEval, microfacet.h:159-181)
__device__ __forceinline__ V3 mf_eval(const DevMaterial* m, V3 wo, V3 wi) {
    const float co = fabsf(wo.z), ci = fabsf(wi.z);
    V3 wh = wi + wo;
    if (ci == 0.0f || co == 0.0f) return vs(0.0f);
    if (wh.x == 0.0f && wh.y == 0.0f && wh.z == 0.0f) return vs(0.0f);
    wh = normalize(wh);
    const V3 F = fr_conductor(fabsf(dot(wi, wh)), v3(m->eir, m->eig, m->eib), v3(m->etr, m->etg, m->etb),
                              v3(m->kr, m->kg, m->kb));
    return mcolor(m) * ggx_d(wh, m->ax, m->ay) * ggx_g(wo, wi, m->ax, m->ay) * F / (4.0f * co);
}

// GGX pdf of reflecting wo about wh. The reference's form D|cos h|/(4 wo.h)
// (microfacet.h:224) does not match its visible-normal sampling; the corrected
// form is the visible-normal density G1(wo) D(h) / (4 |cos o|).
__device__ __forceinline__ float mf_pdf_wh(const DevMaterial* m, V3 wo, V3 wh, bool compat) {
    if (compat) return ggx_d(wh, m->ax, m->ay) * fabsf(wh.z) / (4.0f * dot(wo, wh));
    return ggx_g1(wo, m->ax, m->ay) * ggx_d(wh, m->ax, m->ay) / (4.0f * fabsf(wo.z));
}

__device__ __forceinline__ V3 bsdf_eval(const Bsdf& b, V3 wo_w, V3 wi_w) {
    const V3 wo = to_local(b.fr, wo_w), wi = to_local(b.fr, wi_w);
    if (wo.z == 0.0f) return vs(0.0f);
    const bool refl = wo.z * wi.z > 0.0f;
    if (!refl) return vs(0.0f);
    if (b.m->type == GR_MAT_DIFFUSE) return mcolor(b.m) * kInvPi * fabsf(wi.z);
    if (b.m->type == GR_MAT_CONDUCTOR) return mf_eval(b.m, wo, wi);
    return vs(0.0f);
}

__device__ __forceinline__ float bsdf_pdf(const Bsdf& b, V3 wo_w, V3 wi_w) {
    const V3 wo = to_local(b.fr, wo_w), wi = to_local(b.fr, wi_w);
    if (wo.z == 0.0f) return 0.0f;
    if (!(wo.z * wi.z > 0.0f)) return 0.0f;
    if (b.m->type == GR_MAT_DIFFUSE) return fabsf(wi.z) * kInvPi;
    if (b.m->type == GR_MAT_CONDUCTOR) return mf_pdf_wh(b.m, wo, normalize(wo + wi), b.compat);
    return 0.0f;
}

struct Sample {
    V3 wi, f;
    float pdf;
    bool specular;
};

__device__ __forceinline__ Sample bsdf_sample(const Bsdf& b, V3 wo_w, float u0, float u1) {
    Sample s;
    s.f = vs(0.0f);
    s.pdf = 0.0f;
    s.wi = vs(0.0f);
    s.specular = b.m->type == GR_MAT_DIELECTRIC;
    const V3 wo = to_local(b.fr, wo_w);
    if (wo.z == 0.0f) return s;
    V3 wi = vs(0.0f);
    if (b.m->type == GR_MAT_DIFFUSE) {
        wi = cosine_hemisphere(u0, u1);
        if (wo.z < 0.0f) wi.z = -wi.z;
        s.f = mcolor(b.m) * kInvPi * fabsf(wi.z);
        s.pdf = fabsf(wi.z) * kInvPi;
    } else if (b.m->type == GR_MAT_CONDUCTOR) {
        const V3 wh = ggx_sample_wh(wo, u0, u1, b.m->ax, b.m->ay);
        wi = reflect(wo, wh);
        if (!(wo.z * wi.z > 0.0f)) return s;
        s.pdf = mf_pdf_wh(b.m, wo, wh, b.compat);
        s.f = mf_eval(b.m, wo, wi);
    } else {
        const float F = fr_dielectric(wo.z, 1.0f, b.m->ior);
        if (u0 < F) {
            wi = v3(-wo.x, -wo.y, wo.z);
            s.pdf = F;
            s.f = mcolor(b.m) * F;
        } else {
            const bool entering = wo.z > 0.0f;
            const float ei = entering ? 1.0f : b.m->ior, et = entering ? b.m->ior : 1.0f;
            const V3 n = wo.z < 0.0f ? v3(0.0f, 0.0f, -1.0f) : v3(0.0f, 0.0f, 1.0f);
            if (!refract(wo, n, ei / et, wi)) return s;
            s.f = mcolor(b.m) * (1.0f - F) * ((ei * ei) / (et * et));
            s.pdf = 1.0f - F;
        }
    }
    if (s.pdf == 0.0f) return s;
    s.wi = to_world(b.fr, wi);
    if (!s.specular) {
        const bool refl = wo.z * wi.z > 0.0f;
        if (!refl) {
            s.f = vs(0.0f);
        } else if (b.m->type == GR_MAT_DIFFUSE) {
            s.f = mcolor(b.m) * kInvPi * fabsf(wi.z);
        } else {
            s.f = mf_eval(b.m, wo, wi);
        }
    }
    return s;
}

// Surface point on triangle `prim` at barycentrics (u, v) (Triangle::setupDifferential, triangle.h:103-138).
struct Surf {
    V3 p, ng, ns;
};
__device__ __forceinline__ Surf surface(const SceneDev& sc, uint32_t prim, float u, float v) {
    const float* t = sc.verts + 9ull * prim;
    const V3 p0 = load3(t), p1 = load3(t + 3), p2 = load3(t + 6);
    const float w = 1.0f - u - v;
    Surf s;
    s.p = p0 * w + p1 * u + p2 * v;
    s.ng = normalize(cross(p0 - p2, p1 - p2));
    if (sc.tri_mat[prim] & 0x80000000u) {
        const float4 a = sc.normals[3ull * prim], b = sc.normals[3ull * prim + 1], c = sc.normals[3ull * prim + 2];
        s.ns = normalize(v3(a.x, a.y, a.z) * w + v3(b.x, b.y, b.z) * u + v3(c.x, c.y, c.z) * v);
    } else {
        s.ns = s.ng;
    }
    return s;
}

__device__ __forceinline__ float tri_area(const SceneDev& sc, uint32_t prim) {
    const float* t = sc.verts + 9ull * prim;
    const V3 p0 = load3(t), p1 = load3(t + 3), p2 = load3(t + 6);
    const V3 c = cross(p1 - p0, p2 - p0);
    return sqrtf(dot(c, c)) * 0.5f;
}

__device__ __forceinline__ void add_acc(Paths& ps, uint32_t pid, V3 L) {
    float4 a = ps.acc[pid];
    a.x += L.x;
    a.y += L.y;
    a.z += L.z;
    ps.acc[pid] = a;
}

// ---- camera rays (generate_primary_rays_kernel, pathtracer_kernel.h:59-104) ------
__global__ void __launch_bounds__(kShadeThreads) k_camera(SceneDev sc, Paths ps, RenderParams rp) {
    const WaveHeader h = *ps.hdr;
    const uint32_t P = h.wave_samples * rp.npix;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t pid = blockIdx.x * blockDim.x + threadIdx.x; pid < P; pid += stride) {
        const uint32_t pixel = pid % rp.npix;
        const uint32_t s = h.sample_base + pid / rp.npix;
        const uint64_t inc = pcg_inc(pixel);
        uint64_t st = pcg_seed(rp.seed + (uint64_t)s * 0x9E3779B97F4A7C15ull, inc);
        const float j0 = pcg_float(st, inc), j1 = pcg_float(st, inc);
        const DevCamera& c = sc.cam;
        const float rx = (float)(pixel % c.width) + j0;
        const float ry = (float)(pixel / c.width) + j1;
        const V3 dc = normalize(v3((1.0f - 2.0f * rx / (float)c.width) * c.tan_half,
                                   (2.0f * ry / (float)c.height - 1.0f) * c.tan_half / c.aspect, 1.0f));
        const V3 d = normalize(v3(c.m[0] * dc.x + c.m[1] * dc.y + c.m[2] * dc.z,
                                  c.m[4] * dc.x + c.m[5] * dc.y + c.m[6] * dc.z,
                                  c.m[8] * dc.x + c.m[9] * dc.y + c.m[10] * dc.z));
        ps.ray[2ull * pid] = make_float4(c.m[3], c.m[7], c.m[11], d.x);
        ps.ray[2ull * pid + 1] = make_float4(d.y, d.z, 0.0f, 1e34f);
        ps.thr[pid] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
        ps.acc[pid] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        ps.flags[pid] = 0;
        ps.rng[pid] = st;
        ps.qa[pid] = pid;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) ps.cnt[0] = P;
}

// ---- traversal over queues ----------------------------------------------------------
struct QueueSrc {
    const uint32_t* __restrict__ q;
    const float4* __restrict__ ray;
    float4* __restrict__ hit;
    uint64_t n;
    __device__ __forceinline__ void load(uint64_t i, float4& r0, float4& r1) const {
        const uint32_t pid = q[i];
        r0 = ray[2ull * pid];
        r1 = ray[2ull * pid + 1];
    }
    __device__ __forceinline__ void finish(uint64_t i, const trav::Lane& L) const {
        const uint32_t pid = q[i];
        hit[pid] = L.best_prim == 0xFFFFFFFFu ? make_float4(L.p.tmax, __int_as_float(-1), 0.0f, 0.0f)
                                              : make_float4(L.best_t, __uint_as_float(L.best_prim), L.bu, L.bv);
    }
};

__global__ void __launch_bounds__(trav::kTraceThreads) k_trace_queue(SceneDev sc, Paths ps, int b) {
    __shared__ int2 s_stack[trav::kShortStack][trav::kTraceThreads];
    QueueSrc src{(b & 1) ? ps.qb : ps.qa, ps.ray, ps.hit, ps.cnt[b]};
    trav::traverse_loop<false>(sc.nodes, sc.tris, sc.meta->root, src, ps.work + b, ps.cnt + kErrWord, s_stack);
}

// Shadow rays: an unoccluded ray adds its contribution to its path
// (accumulate_light_sampling_contribution_kernel, pathtracer_kernel.h:642-664).
struct ShadowSrc {
    const float4* __restrict__ sray;
    const float4* __restrict__ scon;
    float4* acc;
    uint64_t n;
    __device__ __forceinline__ void load(uint64_t i, float4& r0, float4& r1) const {
        r0 = sray[2 * i];
        r1 = sray[2 * i + 1];
    }
    __device__ __forceinline__ void finish(uint64_t i, const trav::Lane& L) const {
        if (L.best_prim != 0xFFFFFFFFu) return;
        const float4 c = scon[i];
        const uint32_t pid = __float_as_uint(c.w);
        float4 a = acc[pid];
        a.x += c.x;
        a.y += c.y;
        a.z += c.z;
        acc[pid] = a;
    }
};

__global__ void __launch_bounds__(trav::kTraceThreads) k_trace_shadow(SceneDev sc, Paths ps, int b) {
    __shared__ int2 s_stack[trav::kShortStack][trav::kTraceThreads];
    ShadowSrc src{ps.sray, ps.scon, ps.acc, ps.cnt[kShadowBase + b]};
    trav::traverse_loop<true>(sc.nodes, sc.tris, sc.meta->root, src, ps.work + kShadowBase + b, ps.cnt + kErrWord,
                              s_stack);
}

// ---- shading --------------------------------------------------------------------------
// Step b first finishes the rays that shading step b-1 scattered (MIS-weighted
// emission of a BSDF-sampled light hit, then Russian roulette:
// accumulate_BSDF_sampling_contribution_kernel, pathtracer_kernel.h:684-749),
// then shades the surviving hits (shade_hit_with_MIS_kernel, :488-628).
// Step b == max_depth only finishes.
__global__ void __launch_bounds__(kShadeThreads) k_shade(SceneDev sc, Paths ps, RenderParams rp, int b) {
    const uint32_t n = ps.cnt[b];
    const uint32_t* q = (b & 1) ? ps.qb : ps.qa;
    uint32_t* qn = (b & 1) ? ps.qa : ps.qb;
    const bool compat = (rp.flags & GR_RENDER_REFERENCE_COMPAT) != 0;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t i = base + threadIdx.x;
        bool scatter = false, shadow = false;
        uint32_t pid = 0;
        float4 new_r0, new_r1, sh_r0, sh_r1, sh_c;
        float4 new_thr;
        uint32_t new_flags = 0;
        if (i < n) {
            pid = q[i];
            const uint32_t pixel = pid % rp.npix;
            const uint64_t inc = pcg_inc(pixel);
            uint64_t st = ps.rng[pid];
            const float4 r0 = ps.ray[2ull * pid], r1 = ps.ray[2ull * pid + 1];
            const float4 hv = ps.hit[pid];
            float4 th = ps.thr[pid];
            const uint32_t flags = ps.flags[pid];
            V3 thr = v3(th.x, th.y, th.z);
            const V3 rd = v3(r0.w, r1.x, r1.y);
            const int32_t prim = __float_as_int(hv.y);
            bool alive = true;
            bool as_miss = false;
            if (b > 0) {
                const float rr = pcg_float(st, inc);
                if (prim >= 0 && !(flags & kFlagSpecular)) {
                    const DevMaterial* lm = sc.mats + (sc.tri_mat[prim] & 0x7FFFFFFFu);
                    if (lm->emissive) {
                        const Surf ls = surface(sc, (uint32_t)prim, hv.z, hv.w);
                        float lpdf = (1.0f / tri_area(sc, (uint32_t)prim)) / (float)sc.num_lights;
                        lpdf *= hv.x * hv.x / fabsf(dot(rd, ls.ns));
                        const V3 Le = dot(-rd, ls.ns) > 0.0f ? v3(lm->er, lm->eg, lm->eb) : vs(0.0f);
                        const float bp = th.w;
                        const float w = (bp * bp) / (bp * bp + lpdf * lpdf);
                        add_acc(ps, pid, thr * Le * w);
                    }
                }
                if (rp.rr_depth >= 0 && (int)(b - 1) > rp.rr_depth && maxc(thr) < 1.0f) {
                    const float qk = fmaxf(0.05f, 1.0f - maxc(thr));
                    if (rr < qk) {
                        if (compat) as_miss = true; else alive = false;
                    } else if (!compat) {
                        thr = thr / (1.0f - qk);
                    }
                }
            }
            if (alive && b < (int)rp.max_depth) {
                float s[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) s[k] = pcg_float(st, inc);
                if (prim < 0 || as_miss) {
                    if (sc.has_env) add_acc(ps, pid, thr * v3(sc.env_r, sc.env_g, sc.env_b));
                } else {
                    const uint32_t tm = sc.tri_mat[prim];
                    const DevMaterial* m = sc.mats + (tm & 0x7FFFFFFFu);
                    const Surf sf = surface(sc, (uint32_t)prim, hv.z, hv.w);
                    const V3 wo = -normalize(rd);
                    if ((b == 0 || (flags & kFlagSpecular)) && m->emissive && dot(wo, sf.ns) > 0.0f)
                        add_acc(ps, pid, thr * v3(m->er, m->eg, m->eb));
                    Bsdf bs;
                    bs.fr = make_frame(sf.ns);
                    bs.m = m;
                    bs.compat = compat;
                    // next-event estimation with MIS
                    if (m->type != GR_MAT_DIELECTRIC && sc.num_lights > 0) {
                        const uint32_t lid = min((uint32_t)(s[0] * (float)sc.num_lights), sc.num_lights - 1);
                        const uint32_t lt = sc.lights[lid];
                        const float a = sqrtf(s[1]);
                        const Surf ls = surface(sc, lt, 1.0f - a, s[2] * a);
                        float lpdf = (1.0f / tri_area(sc, lt)) / (float)sc.num_lights;
                        V3 wi = ls.p - sf.p;
                        const float d2 = dot(wi, wi);
                        wi = wi / sqrtf(d2);
                        lpdf *= d2 / fabsf(dot(wi, ls.ns));
                        if (isinf(lpdf)) lpdf = 0.0f;
                        const DevMaterial* lm = sc.mats + (sc.tri_mat[lt] & 0x7FFFFFFFu);
                        const V3 Le = dot(-wi, ls.ns) > 0.0f ? v3(lm->er, lm->eg, lm->eb) : vs(0.0f);
                        const V3 f = bsdf_eval(bs, wo, wi);
                        const float bp = bsdf_pdf(bs, wo, wi);
                        const float w = (lpdf * lpdf) / (lpdf * lpdf + bp * bp);
                        if (lpdf > 0.0f) {
                            const V3 c = thr * Le * f * w / lpdf;
                            if (!black(c)) {
                                const V3 so = sf.p - rd * 1.0e-4f;
                                const V3 sd = ls.p - so;
                                sh_r0 = make_float4(so.x, so.y, so.z, sd.x);
                                sh_r1 = make_float4(sd.y, sd.z, 0.0f, 0.9999f);
                                sh_c = make_float4(c.x, c.y, c.z, __uint_as_float(pid));
                                shadow = true;
                            }
                        }
                    }
                    // BSDF sampling and scatter
                    const Sample smp = bsdf_sample(bs, wo, s[5], s[6]);
                    const V3 wgt = smp.pdf == 0.0f ? vs(0.0f) : thr * smp.f / smp.pdf;
                    if (!black(wgt)) {
                        new_r0 = make_float4(sf.p.x, sf.p.y, sf.p.z, smp.wi.x);
                        new_r1 = make_float4(smp.wi.y, smp.wi.z, 1e-4f, 1e38f);
                        new_thr = make_float4(wgt.x, wgt.y, wgt.z, smp.pdf);
                        new_flags = smp.specular ? kFlagSpecular : 0u;
                        scatter = true;
                    }
                }
            }
            ps.rng[pid] = st;
        }
        const uint32_t sslot = warp_append(ps.cnt + kShadowBase + b, shadow);
        const uint32_t nslot = warp_append(ps.cnt + b + 1, scatter);
        if (shadow) {
            ps.sray[2ull * sslot] = sh_r0;
            ps.sray[2ull * sslot + 1] = sh_r1;
            ps.scon[sslot] = sh_c;
        }
        if (scatter) {
            ps.ray[2ull * pid] = new_r0;
            ps.ray[2ull * pid + 1] = new_r1;
            ps.thr[pid] = new_thr;
            ps.flags[pid] = new_flags;
            qn[nslot] = pid;
        }
    }
}

// ---- resolve: paths -> pixels in sample order ------------------------------------------
__global__ void __launch_bounds__(kShadeThreads) k_resolve(Paths ps, RenderParams rp, double* fb, uint32_t* fbc) {
    const WaveHeader h = *ps.hdr;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t px = blockIdx.x * blockDim.x + threadIdx.x; px < rp.npix; px += stride) {
        double r = fb[3ull * px], g = fb[3ull * px + 1], bl = fb[3ull * px + 2];
        for (uint32_t s = 0; s < h.wave_samples; ++s) {
            const float4 a = ps.acc[(size_t)s * rp.npix + px];
            r += (double)a.x;
            g += (double)a.y;
            bl += (double)a.z;
        }
        fb[3ull * px] = r;
        fb[3ull * px + 1] = g;
        fb[3ull * px + 2] = bl;
        fbc[px] += h.wave_samples;
    }
}

__global__ void k_wave_end(Paths ps, RenderParams rp) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    WaveHeader* h = ps.hdr;
    unsigned long long c = 0, sh = 0;
    for (uint32_t b = 0; b <= rp.max_depth; ++b) c += ps.cnt[b];
    for (uint32_t b = 0; b < rp.max_depth; ++b) sh += ps.cnt[kShadowBase + b];
    h->closest_rays += c;
    h->shadow_rays += sh;
    h->sample_base += h->wave_samples;
    h->remaining -= h->wave_samples;
    h->wave_samples = min(h->max_wave, h->remaining);
}

}  // namespace

cudaError_t render_waves(const SceneDev& sc, Paths& ps, const RenderParams& rp, double* fb, uint32_t* fb_count,
                         uint32_t waves, int num_sms, cudaStream_t s) {
    static int occ = 0;
    cudaError_t e;
    if (occ == 0) {
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_trace_queue, trav::kTraceThreads, 0)) !=
            cudaSuccess)
            return e;
        occ = std::max(occ, 1);
    }
    const int tgrid = num_sms * occ;
    const int sgrid = num_sms * 4;
    const size_t cnt_bytes = sizeof(uint32_t) * (2 * kMaxDepth + 8);
    const size_t work_bytes = sizeof(unsigned long long) * (2 * kMaxDepth + 4);
    for (uint32_t w = 0; w < waves; ++w) {
        if ((e = cudaMemsetAsync(ps.cnt, 0, cnt_bytes, s)) != cudaSuccess) return e;
        if ((e = cudaMemsetAsync(ps.work, 0, work_bytes, s)) != cudaSuccess) return e;
        k_camera<<<sgrid, kShadeThreads, 0, s>>>(sc, ps, rp);
        for (int b = 0; b <= (int)rp.max_depth; ++b) {
            k_trace_queue<<<tgrid, trav::kTraceThreads, 0, s>>>(sc, ps, b);
            k_shade<<<sgrid, kShadeThreads, 0, s>>>(sc, ps, rp, b);
            if (b < (int)rp.max_depth) k_trace_shadow<<<tgrid, trav::kTraceThreads, 0, s>>>(sc, ps, b);
        }
        k_resolve<<<sgrid, kShadeThreads, 0, s>>>(ps, rp, fb, fb_count);
        k_wave_end<<<1, 32, 0, s>>>(ps, rp);
    }
    return cudaGetLastError();
}

}  // namespace gr
