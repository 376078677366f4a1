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
#include <cstddef>
#include <cstring>

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
constexpr int kBinBase = 2 * kMaxDepth + 8;  // kShadeBins counters per bounce start here
constexpr int kCntWords = kBinBase + kShadeBins * (kMaxDepth + 1);

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
    V3 color;  // the material's color at the shading point (constant or texture lookup)
    bool compat;
};

// GGX reflection f*cos (MicrofacetReflectEval, microfacet.h:159-181); conductor
// Fresnel, or for rough plastic dielectric Fresnel of the red indices
// (Fresnel::eval, optical.h:127-137).
__device__ __forceinline__ V3 mf_eval(const DevMaterial* m, V3 color, V3 wo, V3 wi) {
    const float co = fabsf(wo.z), ci = fabsf(wi.z);
    V3 wh = wi + wo;
    if (ci == 0.0f || co == 0.0f) return vs(0.0f);
    if (wh.x == 0.0f && wh.y == 0.0f && wh.z == 0.0f) return vs(0.0f);
    wh = normalize(wh);
    const V3 F = m->type == GR_MAT_PLASTIC
                     ? vs(fr_dielectric(dot(wi, wh), m->eir, m->etr))
                     : fr_conductor(fabsf(dot(wi, wh)), v3(m->eir, m->eig, m->eib), v3(m->etr, m->etg, m->etb),
                                    v3(m->kr, m->kg, m->kb));
    return color * ggx_d(wh, m->ax, m->ay) * ggx_g(wo, wi, m->ax, m->ay) * F / (4.0f * co);
}

// GGX pdf of reflecting wo about wh. The reference's form D|cos h|/(4 wo.h)
// (microfacet.h:224) does not match its visible-normal sampling; the corrected
// form is the visible-normal density G1(wo) D(h) / (4 |cos o|).
__device__ __forceinline__ float mf_pdf_wh(const DevMaterial* m, V3 wo, V3 wh, bool compat) {
    if (compat) return ggx_d(wh, m->ax, m->ay) * fabsf(wh.z) / (4.0f * dot(wo, wh));
    return ggx_g1(wo, m->ax, m->ay) * ggx_d(wh, m->ax, m->ay) / (4.0f * fabsf(wo.z));
}

// Rough plastic, both lobes (BSDF::eval over its two BxDFs, bsdf.h:57-78); local directions, same side.
__device__ __forceinline__ V3 plastic_eval(const Bsdf& b, V3 wo, V3 wi) {
    return b.color * kInvPi * fabsf(wi.z) + mf_eval(b.m, v3(b.m->sr, b.m->sg, b.m->sb), wo, wi);
}

// Rough plastic pdf: each lobe is picked with probability 1/2, so the density
// is the mean of the lobes' densities. The reference sums them (its division
// by the lobe count is a discarded expression, bsdf.h:98, :142); compat keeps it.
__device__ __forceinline__ float plastic_pdf(const Bsdf& b, V3 wo, V3 wi) {
    const float p = fabsf(wi.z) * kInvPi + mf_pdf_wh(b.m, wo, normalize(wo + wi), b.compat);
    return b.compat ? p : 0.5f * p;
}

__device__ __forceinline__ V3 bsdf_eval(const Bsdf& b, V3 wo_w, V3 wi_w) {
    const V3 wo = to_local(b.fr, wo_w), wi = to_local(b.fr, wi_w);
    if (wo.z == 0.0f) return vs(0.0f);
    const bool refl = wo.z * wi.z > 0.0f;
    if (!refl) return vs(0.0f);
    if (b.m->type == GR_MAT_DIFFUSE) return b.color * kInvPi * fabsf(wi.z);
    if (b.m->type == GR_MAT_CONDUCTOR) return mf_eval(b.m, b.color, wo, wi);
    if (b.m->type == GR_MAT_PLASTIC) return plastic_eval(b, wo, wi);
    return vs(0.0f);
}

__device__ __forceinline__ float bsdf_pdf(const Bsdf& b, V3 wo_w, V3 wi_w) {
    const V3 wo = to_local(b.fr, wo_w), wi = to_local(b.fr, wi_w);
    if (wo.z == 0.0f) return 0.0f;
    if (!(wo.z * wi.z > 0.0f)) return 0.0f;
    if (b.m->type == GR_MAT_DIFFUSE) return fabsf(wi.z) * kInvPi;
    if (b.m->type == GR_MAT_CONDUCTOR) return mf_pdf_wh(b.m, wo, normalize(wo + wi), b.compat);
    if (b.m->type == GR_MAT_PLASTIC) return plastic_pdf(b, wo, wi);
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
        s.f = b.color * kInvPi * fabsf(wi.z);
        s.pdf = fabsf(wi.z) * kInvPi;
    } else if (b.m->type == GR_MAT_CONDUCTOR) {
        const V3 wh = ggx_sample_wh(wo, u0, u1, b.m->ax, b.m->ay);
        wi = reflect(wo, wh);
        if (!(wo.z * wi.z > 0.0f)) return s;
        s.pdf = mf_pdf_wh(b.m, wo, wh, b.compat);
        s.f = mf_eval(b.m, b.color, wo, wi);
    } else if (b.m->type == GR_MAT_PLASTIC) {
        // pick a lobe with the first number and reuse its remainder (BSDF::sample, bsdf.h:109-120)
        const int lobe = min((int)floorf(u0 * 2.0f), 1);
        const float v0 = u0 * 2.0f - (float)lobe;
        if (lobe == 0) {
            wi = cosine_hemisphere(v0, u1);
            if (wo.z < 0.0f) wi.z = -wi.z;
        } else {
            wi = reflect(wo, ggx_sample_wh(wo, v0, u1, b.m->ax, b.m->ay));
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
        const bool refl = wo.z * wi.z > 0.0f;
        if (!refl) {
            s.f = vs(0.0f);
        } else if (b.m->type == GR_MAT_DIFFUSE) {
            s.f = b.color * kInvPi * fabsf(wi.z);
        } else if (b.m->type == GR_MAT_PLASTIC) {
            s.f = plastic_eval(b, wo, wi);
        } else {
            s.f = mf_eval(b.m, b.color, wo, wi);
        }
    }
    return s;
}

// Surface point on triangle `prim` at barycentrics (u, v) (Triangle::setupDifferential, triangle.h:103-138).
struct Surf {
    V3 p, ng, ns;
    float tu, tv;  // texture coordinates (Triangle::setupDifferential, triangle.h:103-135)
};
__device__ __forceinline__ Surf surface(const SceneDev& sc, uint32_t prim, float u, float v) {
    const float* t = sc.verts + 9ull * prim;
    const V3 p0 = load3(t), p1 = load3(t + 3), p2 = load3(t + 6);
    const float w = 1.0f - u - v;
    Surf s;
    s.p = p0 * w + p1 * u + p2 * v;
    s.ng = normalize(cross(p0 - p2, p1 - p2));
    const uint32_t tm = sc.tri_mat[prim];
    if (tm & 0x80000000u) {
        const float4 a = sc.normals[3ull * prim], b = sc.normals[3ull * prim + 1], c = sc.normals[3ull * prim + 2];
        s.ns = normalize(v3(a.x, a.y, a.z) * w + v3(b.x, b.y, b.z) * u + v3(c.x, c.y, c.z) * v);
    } else {
        s.ns = s.ng;
    }
    if (tm & 0x40000000u) {
        const float* q = sc.uvs + 6ull * prim;
        s.tu = q[0] * w + q[2] * u + q[4] * v;
        s.tv = q[1] * w + q[3] * u + q[5] * v;
    } else {  // without texcoords the barycentrics are the uv
        s.tu = u;
        s.tv = v;
    }
    return s;
}

// Nearest texel at uv * scale + offset (TextureView::evalSpectrum, texture.h:37-44:
// truncation toward zero, then the index wrapped into [0, size)).
__device__ __forceinline__ int wrap_texel(float x, uint32_t size) {
    const float f = fminf(fmaxf(x * (float)size, -1073741824.0f), 1073741824.0f);
    const int i = (int)f % (int)size;
    return i < 0 ? i + (int)size : i;
}

__device__ __forceinline__ V3 color_at(const SceneDev& sc, const DevMaterial* m, float tu, float tv) {
    if (m->tex_w == 0) return v3(m->cr, m->cg, m->cb);
    const int x = wrap_texel(tu * m->tus + m->tuo, m->tex_w);
    const int y = wrap_texel(tv * m->tvs + m->tvo, m->tex_h);
    const float4 c = sc.texels[m->tex_off + (uint32_t)y * m->tex_w + (uint32_t)x];
    return v3(c.x, c.y, c.z);
}

// Radiance of a ray leaving the scene (EnvironmentLightView::Le, environment.h:15-27).
__device__ __forceinline__ V3 env_radiance(const SceneDev& sc, V3 o, V3 d) {
    if (sc.env_w == 0) return v3(sc.env_r, sc.env_g, sc.env_b);
    V3 w = normalize(o + d * 100000.0f - v3(sc.env_c[0], sc.env_c[1], sc.env_c[2]));
    const float* M = sc.env_m;
    w = normalize(v3(M[0] * w.x + M[1] * w.y + M[2] * w.z, M[3] * w.x + M[4] * w.y + M[5] * w.z,
                     M[6] * w.x + M[7] * w.y + M[8] * w.z));
    const float theta = acosf(fminf(fmaxf(w.z, -1.0f), 1.0f));
    float phi = atan2f(w.y, w.x);
    if (phi < 0.0f) phi += 6.28318530717958647692f;
    const float u = phi * 0.15915494309189533577f, v = theta * 0.31830988618379067154f;
    const uint32_t x = min(sc.env_w - 1, (uint32_t)(int)(u * (float)sc.env_w));
    const uint32_t y = min(sc.env_h - 1, (uint32_t)(int)(v * (float)sc.env_h));
    const float4 c = sc.env_map[y * sc.env_w + x];
    return v3(c.x, c.y, c.z);
}

__device__ __forceinline__ float tri_area(const SceneDev& sc, uint32_t prim) {
    const float* t = sc.verts + 9ull * prim;
    const V3 p0 = load3(t), p1 = load3(t + 3), p2 = load3(t + 6);
    const V3 c = cross(p1 - p0, p2 - p0);
    return sqrtf(dot(c, c)) * 0.5f;
}

__device__ __forceinline__ void add_acc(const Paths& ps, uint32_t pid, V3 L) {
    float4 a = ps.acc[pid];
    a.x += L.x;
    a.y += L.y;
    a.z += L.z;
    ps.acc[pid] = a;
}

// ---- job lookup ---------------------------------------------------------------------
// Jobs are packed in path-id order; the job of a path id is found by binary
// search over the per-job path bases staged in shared memory.
__device__ __forceinline__ uint32_t find_job(const uint32_t* s_base, uint32_t njobs, uint32_t x) {
    uint32_t lo = 0, hi = njobs;  // s_base[lo] <= x < s_base[hi] (s_base[njobs] = total)
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (s_base[mid] <= x) lo = mid; else hi = mid;
    }
    return lo;
}

// ---- camera rays (generate_primary_rays_kernel, pathtracer_kernel.h:59-104) ------
__global__ void __launch_bounds__(kShadeThreads) k_camera(Paths ps) {
    __shared__ uint32_t s_base[kMaxJobs + 1];
    const WaveHeader h = *ps.hdr;
    for (uint32_t j = threadIdx.x; j < h.njobs; j += blockDim.x) s_base[j] = ps.jobs[j].path_base;
    if (threadIdx.x == 0) s_base[h.njobs] = h.total_paths;
    __syncthreads();
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t pid = blockIdx.x * blockDim.x + threadIdx.x; pid < h.total_paths; pid += stride) {
        const uint32_t j = find_job(s_base, h.njobs, pid);
        const JobDev& J = ps.jobs[j];
        const uint32_t local = pid - J.path_base;
        const uint32_t pixel = local % J.npix;
        const uint32_t s = J.sample_base + local / J.npix;
        const uint64_t inc = pcg_inc(pixel);
        uint64_t st = pcg_seed(J.seed + (uint64_t)s * 0x9E3779B97F4A7C15ull, inc);
        const float j0 = pcg_float(st, inc), j1 = pcg_float(st, inc);
        const DevCamera& c = J.sc.cam;
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
        ps.job[pid] = j;
        ps.rng[pid] = st;
        ps.qa[pid] = pid;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) ps.cnt[0] = h.total_paths;
}

// ---- traversal over queues ----------------------------------------------------------
struct QueueSrc {
    const uint32_t* __restrict__ q;
    const Paths* ps;
    uint64_t n;
    __device__ __forceinline__ uint32_t load(uint64_t i, float4& r0, float4& r1, const void*& nd, const Tri*& tr) const {
        const uint32_t pid = q[i];
        r0 = ps->ray[2ull * pid];
        r1 = ps->ray[2ull * pid + 1];
        const SceneDev& sc = ps->jobs[ps->job[pid]].sc;
        nd = sc.nodes;
        tr = sc.tris;
        return sc.meta->root;
    }
    __device__ __forceinline__ void finish(uint64_t i, const trav::Lane& L) const {
        const uint32_t pid = q[i];
        ps->hit[pid] = L.best_prim == 0xFFFFFFFFu ? make_float4(L.p.tmax, __int_as_float(-1), 0.0f, 0.0f)
                                                  : make_float4(L.best_t, __uint_as_float(L.best_prim), L.bu, L.bv);
    }
};

template <int LAYOUT, int SSTACK>
__global__ void __launch_bounds__(trav::kMaxTraceThreads, 4) k_trace_queue(Paths ps, int b) {
    extern __shared__ int2 s_stack[];
    if (b > (int)ps.hdr->max_depth) return;
    QueueSrc src{(b & 1) ? ps.qb : ps.qa, &ps, ps.cnt[b]};
    trav::traverse_loop<false, LAYOUT, SSTACK, trav::kRefillQueue>(src, ps.work + b, ps.cnt + kErrWord, s_stack);
}

// Shadow rays: an unoccluded ray adds its contribution to its path
// (accumulate_light_sampling_contribution_kernel, pathtracer_kernel.h:642-664).
struct ShadowSrc {
    const Paths* ps;
    uint64_t n;
    __device__ __forceinline__ uint32_t load(uint64_t i, float4& r0, float4& r1, const void*& nd, const Tri*& tr) const {
        r0 = ps->sray[2 * i];
        r1 = ps->sray[2 * i + 1];
        const uint32_t pid = __float_as_uint(ps->scon[i].w);
        const SceneDev& sc = ps->jobs[ps->job[pid]].sc;
        nd = sc.nodes;
        tr = sc.tris;
        return sc.meta->root;
    }
    __device__ __forceinline__ void finish(uint64_t i, const trav::Lane& L) const {
        if (L.best_prim != 0xFFFFFFFFu) return;
        const float4 c = ps->scon[i];
        const uint32_t pid = __float_as_uint(c.w);
        float4 a = ps->acc[pid];
        a.x += c.x;
        a.y += c.y;
        a.z += c.z;
        ps->acc[pid] = a;
    }
};

template <int LAYOUT, int SSTACK>
__global__ void __launch_bounds__(trav::kMaxTraceThreads, 4) k_trace_shadow(Paths ps, int b) {
    extern __shared__ int2 s_stack[];
    if (b >= (int)ps.hdr->max_depth) return;
    ShadowSrc src{&ps, ps.cnt[kShadowBase + b]};
    trav::traverse_loop<true, LAYOUT, SSTACK, trav::kRefillQueue>(src, ps.work + kShadowBase + b, ps.cnt + kErrWord,
                                                                   s_stack);
}

// ---- shading groups -----------------------------------------------------------------
// Regroups the paths of bounce b by what their ray hit (group 0: a miss; 1 + t:
// a surface of material type t), appending each path id to its group with one
// atomic per warp and group. The order inside a group is arbitrary; shading
// depends on nothing but the path's own state, so images do not change.
// (Filing the paths in the closest-hit kernel's epilogue instead measured
// slower: the extra gathers lengthened that kernel by as much as this one takes.)
__global__ void __launch_bounds__(kShadeThreads) k_bin(Paths ps, int b) {
    if (b > (int)ps.hdr->max_depth) return;
    const uint32_t n = ps.cnt[b];
    const uint32_t* q = (b & 1) ? ps.qb : ps.qa;
    uint32_t* cnt = ps.cnt + kBinBase + kShadeBins * b;
    const uint32_t stride = gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t i = base + threadIdx.x;
        int bin = -1;
        uint32_t pid = 0;
        if (i < n) {
            pid = q[i];
            const int32_t prim = __float_as_int(ps.hit[pid].y);
            bin = 0;
            if (prim >= 0) {
                const SceneDev& sc = ps.jobs[ps.job[pid]].sc;
                bin = 1 + min((int)sc.mats[sc.tri_mat[prim] & 0x3FFFFFFFu].type, kShadeBins - 2);
            }
        }
#pragma unroll
        for (int k = 0; k < kShadeBins; ++k) {
            const uint32_t m = __ballot_sync(0xFFFFFFFFu, bin == k);
            if (!m) continue;
            const int leader = __ffs(m) - 1;
            uint32_t at = 0;
            if (lane == leader) at = atomicAdd(cnt + k, (uint32_t)__popc(m));
            at = __shfl_sync(0xFFFFFFFFu, at, leader);
            if (bin == k) ps.bins[(size_t)k * ps.capacity + at + __popc(m & lane_lt())] = pid;
        }
    }
}

// ---- shading --------------------------------------------------------------------------
// Step b first finishes the rays that shading step b-1 scattered (MIS-weighted
// emission of a BSDF-sampled light hit, then Russian roulette:
// accumulate_BSDF_sampling_contribution_kernel, pathtracer_kernel.h:684-749),
// then shades the surviving hits (shade_hit_with_MIS_kernel, :488-628).
// Step b == the job's max_depth only finishes.
// Register cap of 64 (4 blocks of 256 per SM): measured 8 % faster renders than
// the uncapped 118 registers (2 blocks per SM), whose few warps could not hide
// instruction-fetch stalls of this large, divergent kernel; the spills are small.
// BINNED: read the bounce's paths in k_bin's groups, as one array; else the
// queue itself (waves whose scenes use one material type).
template <bool BINNED>
__global__ void __launch_bounds__(kShadeThreads, 4) k_shade(Paths ps, int b) {
    if (b > (int)ps.hdr->max_depth) return;
    __shared__ uint32_t s_first[kShadeBins + 1];
    if (BINNED) {
        if (threadIdx.x == 0) {
            uint32_t a = 0;
            for (int k = 0; k < kShadeBins; ++k) {
                s_first[k] = a;
                a += ps.cnt[kBinBase + kShadeBins * b + k];
            }
            s_first[kShadeBins] = a;
        }
        __syncthreads();
    }
    const uint32_t n = BINNED ? s_first[kShadeBins] : ps.cnt[b];
    const uint32_t* q = (b & 1) ? ps.qb : ps.qa;
    uint32_t* qn = (b & 1) ? ps.qa : ps.qb;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t i = base + threadIdx.x;
        bool scatter = false, shadow = false;
        uint32_t pid = 0;
        float4 new_r0, new_r1, sh_r0, sh_r1, sh_c;
        float4 new_thr;
        uint32_t new_flags = 0;
        if (i < n) {
            if (BINNED) {
                int k = 0;
                while (k + 1 < kShadeBins && i >= s_first[k + 1]) ++k;
                pid = ps.bins[(size_t)k * ps.capacity + (i - s_first[k])];
            } else {
                pid = q[i];
            }
            const JobDev& J = ps.jobs[ps.job[pid]];
            const SceneDev& sc = J.sc;
            const bool compat = (J.flags & GR_RENDER_REFERENCE_COMPAT) != 0;
            const uint32_t pixel = (pid - J.path_base) % J.npix;
            const uint64_t inc = pcg_inc(pixel);
            uint64_t st = ps.rng[pid];
            const float4 r0 = ps.ray[2ull * pid], r1 = ps.ray[2ull * pid + 1];
            const float4 hv = ps.hit[pid];
            float4 th = ps.thr[pid];
            const uint32_t flags = ps.flags[pid];
            V3 thr = v3(th.x, th.y, th.z);
            const V3 rd = v3(r0.w, r1.x, r1.y);
            const int32_t prim = __float_as_int(hv.y);
            bool alive = b <= (int)J.max_depth;
            bool as_miss = false;
            if (alive && b > 0) {
                const float rr = pcg_float(st, inc);
                if (prim >= 0 && !(flags & kFlagSpecular)) {
                    const DevMaterial* lm = sc.mats + (sc.tri_mat[prim] & 0x3FFFFFFFu);
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
                if (J.rr_depth >= 0 && (int)(b - 1) > J.rr_depth && maxc(thr) < 1.0f) {
                    const float qk = fmaxf(0.05f, 1.0f - maxc(thr));
                    if (rr < qk) {
                        if (compat) as_miss = true; else alive = false;
                    } else if (!compat) {
                        thr = thr / (1.0f - qk);
                    }
                }
            }
            if (alive && b < (int)J.max_depth) {
                float s[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) s[k] = pcg_float(st, inc);
                if (prim < 0 || as_miss) {
                    if (sc.has_env) add_acc(ps, pid, thr * env_radiance(sc, v3(r0.x, r0.y, r0.z), rd));
                } else {
                    const uint32_t tm = sc.tri_mat[prim];
                    const DevMaterial* m = sc.mats + (tm & 0x3FFFFFFFu);
                    const Surf sf = surface(sc, (uint32_t)prim, hv.z, hv.w);
                    const V3 wo = -normalize(rd);
                    if ((b == 0 || (flags & kFlagSpecular)) && m->emissive && dot(wo, sf.ns) > 0.0f)
                        add_acc(ps, pid, thr * v3(m->er, m->eg, m->eb));
                    Bsdf bs;
                    bs.fr = make_frame(sf.ns);
                    bs.m = m;
                    bs.color = color_at(sc, m, sf.tu, sf.tv);
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
                        const DevMaterial* lm = sc.mats + (sc.tri_mat[lt] & 0x3FFFFFFFu);
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
__global__ void __launch_bounds__(kShadeThreads) k_resolve(Paths ps) {
    __shared__ uint32_t s_base[kMaxJobs + 1];
    const WaveHeader h = *ps.hdr;
    for (uint32_t j = threadIdx.x; j < h.njobs; j += blockDim.x) s_base[j] = ps.jobs[j].pix_base;
    if (threadIdx.x == 0) s_base[h.njobs] = h.total_pix;
    __syncthreads();
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < h.total_pix; r += stride) {
        const JobDev& J = ps.jobs[find_job(s_base, h.njobs, r)];
        const uint32_t px = r - J.pix_base;
        double* f = J.fb + 3ull * px;
        double cr = f[0], cg = f[1], cb = f[2];
        for (uint32_t s = 0; s < J.wave_samples; ++s) {
            const float4 a = ps.acc[J.path_base + (size_t)s * J.npix + px];
            cr += (double)a.x;
            cg += (double)a.y;
            cb += (double)a.z;
        }
        f[0] = cr;
        f[1] = cg;
        f[2] = cb;
        J.fbc[px] += J.wave_samples;
    }
}

// ---- 8-bit output (filter_kernel, pathtracer_kernel.h:792-810) -----------------------
// sRGB transfer curve (spectrum.h:63-72): 12.92 v below 0.0031308, else
// 1.055 v^(1/2.4) - 0.055; then 255 v + 0.5 clamped to [0, 255] and truncated.
__device__ __forceinline__ uint32_t srgb8(float v) {
    const float g = v <= 0.0031308f ? 12.92f * v : 1.055f * powf(v, 1.0f / 2.4f) - 0.055f;
    return (uint32_t)fminf(fmaxf(255.0f * g + 0.5f, 0.0f), 255.0f);
}

__global__ void __launch_bounds__(kShadeThreads) k_filter(const double* __restrict__ fb, const uint32_t* __restrict__ fbc,
                                                          uint32_t npix, uint32_t* __restrict__ out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += gridDim.x * blockDim.x) {
        const uint32_t n = fbc[i];
        uint32_t px = 0xFF000000u;
        if (n) {
            const double inv = 1.0 / (double)n;
            px |= srgb8((float)(fb[3ull * i] * inv)) | (srgb8((float)(fb[3ull * i + 1] * inv)) << 8) |
                  (srgb8((float)(fb[3ull * i + 2] * inv)) << 16);
        }
        out[i] = px;
    }
}

// Mean linear radiance per pixel (3 floats), the same arithmetic as the host
// read-back of gr_render: sum * (1 / count) in double, rounded to float.
__global__ void __launch_bounds__(kShadeThreads) k_mean_rgb(const double* __restrict__ fb,
                                                            const uint32_t* __restrict__ fbc, uint32_t npix,
                                                            float* __restrict__ out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += gridDim.x * blockDim.x) {
        const uint32_t n = fbc[i];
        const double inv = n ? 1.0 / (double)n : 0.0;
#pragma unroll
        for (int c = 0; c < 3; ++c) out[3ull * i + c] = (float)(fb[3ull * i + c] * inv);
    }
}

__global__ void k_wave_end(Paths ps) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    WaveHeader* h = ps.hdr;
    unsigned long long c = 0, sh = 0;
    for (uint32_t b = 0; b <= h->max_depth; ++b) c += ps.cnt[b];
    for (uint32_t b = 0; b < h->max_depth; ++b) sh += ps.cnt[kShadowBase + b];
    h->closest_rays += c;
    h->shadow_rays += sh;
}

// One wave: clear counters, camera rays, depth_steps x (trace, shade, shadow)
// (steps past the wave's max_depth return at once), resolve, ray counts.
template <int LAYOUT, int SSTACK>
cudaError_t issue_wave_l(const Paths& ps, uint32_t depth_steps, int tgrid, int tblock, int sgrid, bool bin,
                         cudaStream_t s) {
    const size_t smem = trav::traverse_smem(LAYOUT, SSTACK, tblock);
    cudaError_t e;
    const size_t cnt_bytes = sizeof(uint32_t) * (2 * kMaxDepth + 4);
    const size_t bin_bytes = sizeof(uint32_t) * (kCntWords - kBinBase);
    const size_t work_bytes = sizeof(unsigned long long) * (2 * kMaxDepth + 4);
    if ((e = cudaMemsetAsync(ps.cnt, 0, cnt_bytes, s)) != cudaSuccess) return e;
    if (bin && (e = cudaMemsetAsync(ps.cnt + kBinBase, 0, bin_bytes, s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(ps.work, 0, work_bytes, s)) != cudaSuccess) return e;
    k_camera<<<sgrid, kShadeThreads, 0, s>>>(ps);
    for (int b = 0; b <= (int)depth_steps; ++b) {
        k_trace_queue<LAYOUT, SSTACK><<<tgrid, tblock, smem, s>>>(ps, b);
        if (bin) {
            k_bin<<<sgrid, kShadeThreads, 0, s>>>(ps, b);
            k_shade<true><<<sgrid, kShadeThreads, 0, s>>>(ps, b);
        } else {
            k_shade<false><<<sgrid, kShadeThreads, 0, s>>>(ps, b);
        }
        if (b < (int)depth_steps) k_trace_shadow<LAYOUT, SSTACK><<<tgrid, tblock, smem, s>>>(ps, b);
    }
    k_resolve<<<sgrid, kShadeThreads, 0, s>>>(ps);
    k_wave_end<<<1, 32, 0, s>>>(ps);
    return cudaGetLastError();
}

template <int LAYOUT>
cudaError_t issue_wave_s(const Paths& ps, uint32_t steps, int tgrid, const TraceTuning& t, int sgrid, bool bin,
                         cudaStream_t s) {
    if (t.sstack == 8) return issue_wave_l<LAYOUT, 8>(ps, steps, tgrid, t.block, sgrid, bin, s);
    if (t.sstack == 16) return issue_wave_l<LAYOUT, 16>(ps, steps, tgrid, t.block, sgrid, bin, s);
    return issue_wave_l<LAYOUT, 12>(ps, steps, tgrid, t.block, sgrid, bin, s);
}

// bin: group the paths by material before shading (waves whose scenes mix
// material types).
cudaError_t issue_wave(const Paths& ps, uint32_t steps, int tgrid, int sgrid, bool bin, cudaStream_t s,
                       const TraceTuning& t) {
    if (t.layout == kLayoutBvh4) return issue_wave_s<kLayoutBvh4>(ps, steps, tgrid, t, sgrid, bin, s);
    if (t.layout == kLayoutBvh4Q8) return issue_wave_s<kLayoutBvh4Q8>(ps, steps, tgrid, t, sgrid, bin, s);
    if (t.layout == kLayoutBvh8Q8) return issue_wave_s<kLayoutBvh8Q8>(ps, steps, tgrid, t, sgrid, bin, s);
    return issue_wave_s<kLayoutBvh2>(ps, steps, tgrid, t, sgrid, bin, s);
}

// Resident blocks per SM of the closest-hit queue kernel for a configuration.
cudaError_t trace_occupancy(const TraceTuning& t, int* occ) {
    const size_t smem = trav::traverse_smem(t.layout, t.sstack, t.block);
    const void* fn = nullptr;
#define GR_PICK(L, S) \
    if (t.layout == L && t.sstack == S) fn = (const void*)k_trace_queue<L, S>;
    GR_PICK(kLayoutBvh2, 8) GR_PICK(kLayoutBvh2, 12) GR_PICK(kLayoutBvh2, 16)
    GR_PICK(kLayoutBvh4, 8) GR_PICK(kLayoutBvh4, 12) GR_PICK(kLayoutBvh4, 16)
    GR_PICK(kLayoutBvh4Q8, 8) GR_PICK(kLayoutBvh4Q8, 12) GR_PICK(kLayoutBvh4Q8, 16)
    GR_PICK(kLayoutBvh8Q8, 8) GR_PICK(kLayoutBvh8Q8, 12) GR_PICK(kLayoutBvh8Q8, 16)
#undef GR_PICK
    if (!fn) return cudaErrorInvalidValue;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, fn, t.block, smem);
    if (*occ < 1) *occ = 1;
    return e;
}

uint64_t mix64(uint64_t h, uint64_t v) {
    h ^= v + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
    return h;
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

size_t path_layout(uint32_t cap, char* base, Paths* ps) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char* p = base ? base + off : nullptr;
        off += align256(bytes);
        return p;
    };
    const size_t c = cap;
    ps->ray = (float4*)take(32 * c);
    ps->hit = (float4*)take(16 * c);
    ps->thr = (float4*)take(16 * c);
    ps->acc = (float4*)take(16 * c);
    ps->flags = (uint32_t*)take(4 * c);
    ps->job = (uint32_t*)take(4 * c);
    ps->rng = (unsigned long long*)take(8 * c);
    ps->qa = (uint32_t*)take(4 * c);
    ps->qb = (uint32_t*)take(4 * c);
    ps->bins = (uint32_t*)take(4 * kShadeBins * c);
    ps->sray = (float4*)take(32 * c);
    ps->scon = (float4*)take(16 * c);
    ps->cnt = (uint32_t*)take(sizeof(uint32_t) * kCntWords);
    ps->work = (unsigned long long*)take(sizeof(unsigned long long) * (2 * kMaxDepth + 4));
    ps->hdr = (WaveHeader*)take(sizeof(WaveHeader));
    ps->jobs = (JobDev*)take(sizeof(JobDev) * kMaxJobs);
    ps->capacity = cap;
    return off;
}



}  // namespace

void WaveGraph::release() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    key = 0;
}

void WavePool::release_graphs() {
    for (WaveGraph& g : graphs) g.release();
}

void WavePool::release() {
    release_graphs();
    for (int i = 0; i < kSlots; ++i)
        if (ev[i]) {
            cudaEventSynchronize(ev[i]);
            cudaEventDestroy(ev[i]);
            ev[i] = nullptr;
        }
    if (h_jobs) cudaFreeHost(h_jobs);
    if (h_hdr) cudaFreeHost(h_hdr);
    h_jobs = nullptr;
    h_hdr = nullptr;
    mem.release();
    capacity = 0;
}

cudaError_t WavePool::ensure(uint32_t paths) {
    cudaError_t e;
    if (!h_jobs) {
        if ((e = cudaMallocHost((void**)&h_jobs, sizeof(JobDev) * kMaxJobs * kSlots)) != cudaSuccess) return e;
        if ((e = cudaMallocHost((void**)&h_hdr, sizeof(WaveHeader) * kSlots)) != cudaSuccess) return e;
        for (int i = 0; i < kSlots; ++i)
            if ((e = cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming)) != cudaSuccess) return e;
    }
    if (paths <= capacity && mem.p) return cudaSuccess;
    release_graphs();  // a captured wave points into the old path memory
    Paths p;
    const size_t bytes = path_layout(paths, nullptr, &p);
    e = mem.ensure(bytes);
    if (e != cudaSuccess) {
        capacity = 0;
        return e;
    }
    path_layout(paths, (char*)mem.p, &ps);
    capacity = paths;
    if ((e = cudaMemset(ps.hdr, 0, sizeof(WaveHeader))) != cudaSuccess) return e;
    return cudaMemset(ps.cnt + kErrWord, 0, 4);
}

cudaError_t WavePool::clear_errors(cudaStream_t s) {
    return mem.p ? cudaMemsetAsync(ps.cnt + kErrWord, 0, 4, s) : cudaSuccess;
}

const uint32_t* WavePool::error_word() const { return ps.cnt + kErrWord; }

uint32_t pack_wave(std::vector<HostJob*>& jobs, uint32_t capacity, std::vector<JobDev>& out, uint32_t* total_paths,
                   uint32_t* total_pix, uint32_t* max_depth) {
    out.clear();
    uint32_t paths = 0, pix = 0, depth = 0;
    for (HostJob* j : jobs) {
        if (out.size() >= kMaxJobs) break;
        if (j->spp_done >= j->spp_total) continue;
        const uint32_t free_paths = capacity - paths;
        uint32_t take = std::min(j->spp_total - j->spp_done, free_paths / j->npix);
        if (take == 0) continue;
        JobDev d;
        d.sc = j->sc;
        d.fb = j->fb;
        d.fbc = j->fbc;
        d.path_base = paths;
        d.npix = j->npix;
        d.pix_base = pix;
        d.wave_samples = take;
        d.sample_base = j->sample_offset + j->spp_done;
        d.max_depth = j->max_depth;
        d.rr_depth = j->rr_depth;
        d.flags = j->flags;
        d.seed = j->seed;
        out.push_back(d);
        paths += take * j->npix;
        pix += j->npix;
        depth = std::max(depth, j->max_depth);
        j->spp_done += take;
    }
    *total_paths = paths;
    *total_pix = pix;
    *max_depth = depth;
    return (uint32_t)out.size();
}

cudaError_t filter_rgba8(const double* fb, const uint32_t* fbc, uint32_t npix, uint32_t* out, cudaStream_t s) {
    if (npix == 0) return cudaSuccess;
    const int grid = (int)std::min<uint32_t>((npix + kShadeThreads - 1) / kShadeThreads, 4096u);
    k_filter<<<grid, kShadeThreads, 0, s>>>(fb, fbc, npix, out);
    return cudaGetLastError();
}

cudaError_t mean_rgb(const double* fb, const uint32_t* fbc, uint32_t npix, float* out, cudaStream_t s) {
    if (npix == 0) return cudaSuccess;
    const int grid = (int)std::min<uint32_t>((npix + kShadeThreads - 1) / kShadeThreads, 4096u);
    k_mean_rgb<<<grid, kShadeThreads, 0, s>>>(fb, fbc, npix, out);
    return cudaGetLastError();
}

cudaError_t run_wave(WavePool& pool, const JobDev* h_jobs, uint32_t njobs, uint32_t total_paths, uint32_t total_pix,
                     uint32_t max_depth, int num_sms, cudaStream_t s, bool use_graph, const TraceTuning& tune) {
    cudaError_t e;
    if (!tuning_valid(tune)) return cudaErrorInvalidValue;
    static int occ_cache[kNumLayouts][3][3] = {};
    const int bi = tune.block == 64 ? 0 : (tune.block == 128 ? 1 : 2);
    const int si = tune.sstack == 8 ? 0 : (tune.sstack == 12 ? 1 : 2);
    int& occ = occ_cache[tune.layout][bi][si];
    if (occ == 0 && (e = trace_occupancy(tune, &occ)) != cudaSuccess) return e;
    if (njobs == 0 || njobs > kMaxJobs || total_paths > pool.capacity || max_depth > (uint32_t)kMaxDepth)
        return cudaErrorInvalidValue;
    for (uint32_t j = 0; j < njobs; ++j)  // traversal reads nodes with 32-byte loads
        if (reinterpret_cast<uintptr_t>(h_jobs[j].sc.nodes) & 31) return cudaErrorMisalignedAddress;
    const Paths& ps = pool.ps;
    const int slot = pool.slot;
    pool.slot = (pool.slot + 1) % WavePool::kSlots;
    if ((e = cudaEventSynchronize(pool.ev[slot])) != cudaSuccess) return e;
    JobDev* stage = pool.h_jobs + (size_t)slot * kMaxJobs;
    std::memcpy(stage, h_jobs, sizeof(JobDev) * njobs);
    WaveHeader& h = pool.h_hdr[slot];
    h = WaveHeader{};
    h.njobs = njobs;
    h.total_paths = total_paths;
    h.total_pix = total_pix;
    h.max_depth = max_depth;
    if ((e = cudaMemcpyAsync(ps.jobs, stage, sizeof(JobDev) * njobs, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return e;
    // the header's running ray totals stay on the device; only the wave fields are written
    if ((e = cudaMemcpyAsync(ps.hdr, &h, offsetof(WaveHeader, closest_rays), cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return e;
    if ((e = cudaEventRecord(pool.ev[slot], s)) != cudaSuccess) return e;
    const int tgrid = num_sms * occ;
    const int sgrid = num_sms * 4;
    // the captured sequence runs exactly the wave's bounce steps (an empty step
    // still costs three launches)
    const uint32_t steps = max_depth;
    // shade in material groups when the wave's scenes mix material types
    uint32_t types = 0;
    for (uint32_t j = 0; j < njobs; ++j) types |= h_jobs[j].sc.mat_types;
    const bool bin = __builtin_popcount(types) >= 2;
    if (!use_graph) return issue_wave(ps, max_depth, tgrid, sgrid, bin, s, tune);
    uint64_t key = 0x51ED270B27A3C1F5ull;
    const uint64_t words[] = {(uint64_t)(uintptr_t)ps.ray, ps.capacity, steps, (uint64_t)tgrid, (uint64_t)sgrid,
                              (uint64_t)tune.layout, (uint64_t)tune.block, (uint64_t)tune.sstack, (uint64_t)bin};
    for (uint64_t w : words) key = mix64(key, w);
    int hit = -1;
    for (int i = 0; i < WavePool::kGraphs; ++i)
        if (pool.graphs[i].exec && pool.graphs[i].key == key) hit = i;
    if (hit < 0) {
        // evict the least recently used (the last), then capture into the front
        pool.graphs[WavePool::kGraphs - 1].release();
        hit = WavePool::kGraphs - 1;
    }
    for (int i = hit; i > 0; --i) {  // the handles move, not the owning objects
        std::swap(pool.graphs[i].exec, pool.graphs[i - 1].exec);
        std::swap(pool.graphs[i].key, pool.graphs[i - 1].key);
    }
    WaveGraph& g = pool.graphs[0];
    if (!g.exec) {
        cudaGraph_t graph = nullptr;
        if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
        const cudaError_t ei = issue_wave(ps, steps, tgrid, sgrid, bin, s, tune);
        e = cudaStreamEndCapture(s, &graph);
        if (ei != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return ei;
        }
        if (e != cudaSuccess) return e;
        e = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            g.exec = nullptr;
            return e;
        }
        g.key = key;
    }
    return cudaGraphLaunch(g.exec, s);
}

}  // namespace gr
