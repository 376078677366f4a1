// Scene records and the render entry points of the C ABI (include/gr.h).
//
// gr_scene_create replaces Scene::Scene + Scene::createDeviceData
// (slongle/GPU-Renderer src/renderer/scene.cpp:4-51): meshes are flattened to
// one triangle list, emissive triangles become the light list, and the LBVH is
// built on the GPU instead of on the host. The reference stores a 408-byte
// Triangle record per triangle (embedding its mesh view and material); here
// the device holds the flat vertex soup, optional per-corner normals, and a
// 4-byte material index per triangle.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "render.h"

namespace gr {

DevCamera make_camera(const gr_camera& camera) {
    // Camera::setup (camera.h:21-38); degToRad (fwd.h:28-31)
    DevCamera c{};
    const float* M = camera.to_world;
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 4; ++k) c.m[4 * r + k] = M[4 * r + k];
    const float fov = camera.fov_deg / 180.0f * 3.14159265358979323846f;
    c.tan_half = std::tan(fov * 0.5f);
    c.aspect = (float)camera.width / (float)camera.height;
    c.width = camera.width;
    c.height = camera.height;
    return c;
}

}  // namespace gr

namespace {

gr_status fail(gr_ctx* ctx, gr_status st, const std::string& what) {
    if (ctx) ctx->last_error = what;
    return st;
}

gr_status cuda_fail(gr_ctx* ctx, cudaError_t e, const char* where) {
    cudaGetLastError();
    if (ctx) ctx->last_error = std::string(where) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? GR_ERR_OOM_BUDGET : GR_ERR_CUDA;
}

#define SC_CUDA(ctx, call)                                                \
    do {                                                                  \
        cudaError_t e__ = (call);                                         \
        if (e__ != cudaSuccess) return cuda_fail(ctx, e__, #call);        \
    } while (0)

bool emissive(const gr_material& m) { return m.emission[0] != 0.0f || m.emission[1] != 0.0f || m.emission[2] != 0.0f; }

}  // namespace

gr::TraceTuning scene_tuning(const gr_scene* sc) {
    gr::TraceTuning t;
    t.layout = sc->bvh->layout;
    t.block = sc->bvh->block;
    t.sstack = sc->bvh->sstack;
    return t;
}

gr::SceneDev gr::scene_view(gr_scene* sc, int layout) {
    gr::SceneDev d{};
    d.verts = (const float*)sc->verts.p;
    d.normals = (const float4*)sc->normals.p;
    d.tri_mat = (const uint32_t*)sc->tri_mat.p;
    d.uvs = (const float*)sc->uvs.p;
    d.texels = (const float4*)sc->texels.p;
    d.env_map = (const float4*)sc->env_map.p;
    d.env_w = sc->env_w;
    d.env_h = sc->env_h;
    std::memcpy(d.env_m, sc->env_m, sizeof(d.env_m));
    std::memcpy(d.env_c, sc->env_c, sizeof(d.env_c));
    d.mats = (const gr::DevMaterial*)sc->mats.p;
    d.lights = (const uint32_t*)sc->lights.p;
    d.num_lights = sc->num_lights;
    d.num_tris = sc->num_tris;
    d.nodes = gr::layout_nodes(sc->bvh, layout);
    d.tris = gr::layout_tris(sc->bvh, layout);
    d.meta = (const gr::BvhMeta*)sc->bvh->buf.meta.p;
    d.cam = sc->cam;
    d.env_r = sc->env[0];
    d.env_g = sc->env[1];
    d.env_b = sc->env[2];
    d.has_env = sc->has_env;
    d.mat_types = sc->mat_types;
    return d;
}

extern "C" {

gr_status gr_scene_set_layout(gr_scene* sc, int layout) {
    if (!sc) return GR_ERR_INVALID;
    gr_status st = gr_bvh_set_layout(sc->bvh, layout, sc->ctx->stream);
    if (st != GR_OK) return st;
    SC_CUDA(sc->ctx, cudaStreamSynchronize(sc->ctx->stream));
    return GR_OK;
}

int gr_scene_layout(const gr_scene* sc) { return sc && sc->bvh ? sc->bvh->layout : -1; }

gr_status gr_scene_create(gr_ctx* ctx, const gr_mesh* meshes, uint32_t num_meshes, const gr_material* materials,
                          uint32_t num_materials, const gr_camera* camera, const gr_environment* env,
                          gr_scene** out) {
    if (!ctx || !out || !camera || (num_meshes && !meshes) || (num_materials && !materials))
        return fail(ctx, GR_ERR_INVALID, "gr_scene_create: null argument");
    *out = nullptr;
    if (!gr::pixels_ok(camera->width, camera->height) || !(camera->fov_deg > 0.0f && camera->fov_deg < 180.0f))
        return fail(ctx, GR_ERR_INVALID, "gr_scene_create: bad camera");
    uint64_t ntri = 0;
    bool any_normals = false, any_uvs = false;
    for (uint32_t i = 0; i < num_meshes; ++i) {
        const gr_mesh& m = meshes[i];
        if (m.num_triangles && (!m.positions || !m.indices))
            return fail(ctx, GR_ERR_INVALID, "gr_scene_create: mesh without positions or indices");
        if (m.material >= num_materials) return fail(ctx, GR_ERR_INVALID, "gr_scene_create: material out of range");
        for (uint64_t k = 0; k < 3ull * m.num_triangles; ++k)
            if (m.indices[k] >= m.num_vertices) return fail(ctx, GR_ERR_INVALID, "gr_scene_create: index out of range");
        ntri += m.num_triangles;
        any_normals |= m.normals != nullptr;
        any_uvs |= m.texcoords != nullptr;
    }
    if (ntri > gr::kMaxTriangles) return fail(ctx, GR_ERR_INVALID, "gr_scene_create: too many triangles");
    for (uint32_t i = 0; i < num_materials; ++i) {
        const int t = materials[i].type;
        if (t != GR_MAT_DIFFUSE && t != GR_MAT_DIELECTRIC && t != GR_MAT_CONDUCTOR && t != GR_MAT_PLASTIC)
            return fail(ctx, GR_ERR_INVALID, "gr_scene_create: unknown material type");
        if (materials[i].color_map &&
            (materials[i].color_map_width == 0 || materials[i].color_map_height == 0 ||
             (uint64_t)materials[i].color_map_width * materials[i].color_map_height > (1ull << 28)))
            return fail(ctx, GR_ERR_INVALID, "gr_scene_create: bad color_map size");
    }
    if (env && env->enabled && env->map &&
        (env->map_width == 0 || env->map_height == 0 || (uint64_t)env->map_width * env->map_height > (1ull << 28)))
        return fail(ctx, GR_ERR_INVALID, "gr_scene_create: bad environment map size");

    std::vector<float> soup(9 * ntri);
    std::vector<float> nrm(any_normals ? 12 * ntri : 0, 0.0f);
    std::vector<float> uvs(any_uvs ? 6 * ntri : 0, 0.0f);
    std::vector<uint32_t> tmat(ntri);
    std::vector<uint32_t> lights;
    uint64_t t = 0;
    for (uint32_t i = 0; i < num_meshes; ++i) {
        const gr_mesh& m = meshes[i];
        const bool light = emissive(materials[m.material]);
        for (uint32_t j = 0; j < m.num_triangles; ++j, ++t) {
            for (int c = 0; c < 3; ++c) {
                const uint32_t vi = m.indices[3ull * j + c];
                std::memcpy(&soup[9 * t + 3 * c], m.positions + 3ull * vi, 12);
                if (m.normals) std::memcpy(&nrm[12 * t + 4 * c], m.normals + 3ull * vi, 12);
                if (m.texcoords) std::memcpy(&uvs[6 * t + 2 * c], m.texcoords + 2ull * vi, 8);
            }
            tmat[t] = m.material | (m.normals ? 0x80000000u : 0u) | (m.texcoords ? 0x40000000u : 0u);
            if (light) lights.push_back((uint32_t)t);
        }
    }
    std::vector<gr::DevMaterial> dm(num_materials ? num_materials : 1);
    std::vector<float> texels;  // 4 floats per texel (rgb, 0)
    for (uint32_t i = 0; i < num_materials; ++i) {
        const gr_material& s = materials[i];
        gr::DevMaterial& d = dm[i];
        d.type = s.type;
        d.cr = s.color[0]; d.cg = s.color[1]; d.cb = s.color[2];
        d.er = s.emission[0]; d.eg = s.emission[1]; d.eb = s.emission[2];
        d.ax = s.alpha_u; d.ay = s.alpha_v;
        d.eir = s.eta_i[0]; d.eig = s.eta_i[1]; d.eib = s.eta_i[2];
        d.etr = s.eta_t[0]; d.etg = s.eta_t[1]; d.etb = s.eta_t[2];
        d.kr = s.k[0]; d.kg = s.k[1]; d.kb = s.k[2];
        d.ior = s.ior;
        d.emissive = emissive(s) ? 1u : 0u;
        d.tex_off = d.tex_w = d.tex_h = 0;
        d.sr = s.specular[0]; d.sg = s.specular[1]; d.sb = s.specular[2];
        d.tuo = s.uv_offset[0]; d.tvo = s.uv_offset[1];
        d.tus = s.uv_scale[0]; d.tvs = s.uv_scale[1];
        if (s.color_map) {
            const size_t nt = (size_t)s.color_map_width * s.color_map_height;
            d.tex_off = (uint32_t)(texels.size() / 4);
            d.tex_w = s.color_map_width;
            d.tex_h = s.color_map_height;
            for (size_t k = 0; k < nt; ++k) {
                texels.push_back(s.color_map[3 * k]);
                texels.push_back(s.color_map[3 * k + 1]);
                texels.push_back(s.color_map[3 * k + 2]);
                texels.push_back(0.0f);
            }
        }
    }
    // environment map: texels, world-to-map rotation, scene bounding-box centre (scene.cpp:27)
    std::vector<float> env_texels;
    float env_m[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, env_c[3] = {0, 0, 0};
    if (env && env->enabled && env->map) {
        const size_t nt = (size_t)env->map_width * env->map_height;
        env_texels.resize(4 * nt);
        for (size_t k = 0; k < nt; ++k) {
            env_texels[4 * k] = env->map[3 * k];
            env_texels[4 * k + 1] = env->map[3 * k + 1];
            env_texels[4 * k + 2] = env->map[3 * k + 2];
            env_texels[4 * k + 3] = 0.0f;
        }
        // inverse of the upper 3x3 of to_world (directions ignore the translation)
        const float* M = env->to_world;
        const double a = M[0], b = M[1], c = M[2], d = M[4], e = M[5], f = M[6], g = M[8], h = M[9], i = M[10];
        const double det = a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
        if (!(std::fabs(det) > 0.0)) return fail(ctx, GR_ERR_INVALID, "gr_scene_create: singular environment to_world");
        const double inv[9] = {(e * i - f * h) / det, (c * h - b * i) / det, (b * f - c * e) / det,
                               (f * g - d * i) / det, (a * i - c * g) / det, (c * d - a * f) / det,
                               (d * h - e * g) / det, (b * g - a * h) / det, (a * e - b * d) / det};
        for (int k = 0; k < 9; ++k) env_m[k] = (float)inv[k];
        if (ntri) {
            float lo[3] = {soup[0], soup[1], soup[2]}, hi[3] = {soup[0], soup[1], soup[2]};
            for (size_t k = 0; k < 3 * ntri; ++k)
                for (int ax = 0; ax < 3; ++ax) {
                    lo[ax] = std::min(lo[ax], soup[3 * k + ax]);
                    hi[ax] = std::max(hi[ax], soup[3 * k + ax]);
                }
            for (int ax = 0; ax < 3; ++ax) env_c[ax] = (lo[ax] + hi[ax]) * 0.5f;
        }
    }

    gr_scene* sc = new (std::nothrow) gr_scene();
    if (!sc) return fail(ctx, GR_ERR_OOM_BUDGET, "host allocation failed");
    sc->ctx = ctx;
    gr::ctx_retain(ctx);
    auto cleanup = [&](gr_status st) {
        gr_scene_destroy(sc);
        return st;
    };
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cleanup(cuda_fail(ctx, e, "cudaSetDevice"));
    sc->num_tris = (uint32_t)ntri;
    if (!env_texels.empty()) {
        sc->env_w = env->map_width;
        sc->env_h = env->map_height;
        std::memcpy(sc->env_m, env_m, sizeof(env_m));
        std::memcpy(sc->env_c, env_c, sizeof(env_c));
    }
    sc->num_lights = (uint32_t)lights.size();
    for (uint32_t i = 0; i < num_meshes; ++i)
        if (meshes[i].num_triangles) sc->mat_types |= 1u << (uint32_t)materials[meshes[i].material].type;
    struct Up {
        gr::DevBuf* buf;
        const void* src;
        size_t bytes;
    } ups[] = {
        {&sc->verts, soup.data(), soup.size() * 4},
        {&sc->normals, nrm.data(), nrm.size() * 4},
        {&sc->tri_mat, tmat.data(), tmat.size() * 4},
        {&sc->mats, dm.data(), dm.size() * sizeof(gr::DevMaterial)},
        {&sc->lights, lights.data(), lights.size() * 4},
        {&sc->uvs, uvs.data(), uvs.size() * 4},
        {&sc->texels, texels.data(), texels.size() * 4},
        {&sc->env_map, env_texels.data(), env_texels.size() * 4},
    };
    for (auto& u : ups) {
        if (u.bytes == 0) continue;
        if ((e = u.buf->ensure(u.bytes)) != cudaSuccess) return cleanup(cuda_fail(ctx, e, "scene upload alloc"));
        if ((e = cudaMemcpy(u.buf->p, u.src, u.bytes, cudaMemcpyHostToDevice)) != cudaSuccess)
            return cleanup(cuda_fail(ctx, e, "scene upload"));
    }
    gr_status st = gr_bvh_create(ctx, &sc->bvh);
    if (st != GR_OK) return cleanup(st);
    st = gr_bvh_build(sc->bvh, (const float*)sc->verts.p, (uint32_t)ntri, ctx->stream);
    if (st != GR_OK) return cleanup(st);
    if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return cleanup(cuda_fail(ctx, e, "bvh build"));

    sc->cam = gr::make_camera(*camera);
    sc->cam_rec = *camera;
    if (env && env->enabled) {
        sc->has_env = 1;
        std::memcpy(sc->env, env->radiance, 12);
    }
    const size_t npix = (size_t)camera->width * camera->height;
    if ((e = sc->fb.ensure(24 * npix)) != cudaSuccess) return cleanup(cuda_fail(ctx, e, "framebuffer"));
    if ((e = sc->fb_count.ensure(4 * npix)) != cudaSuccess) return cleanup(cuda_fail(ctx, e, "framebuffer"));
    if ((e = cudaMemset(sc->fb.p, 0, 24 * npix)) != cudaSuccess) return cleanup(cuda_fail(ctx, e, "framebuffer"));
    if ((e = cudaMemset(sc->fb_count.p, 0, 4 * npix)) != cudaSuccess) return cleanup(cuda_fail(ctx, e, "framebuffer"));
    *out = sc;
    return GR_OK;
}

gr_status gr_scene_destroy(gr_scene* sc) {
    if (!sc) return GR_ERR_INVALID;
    gr_ctx* ctx = sc->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (sc->bvh) gr_bvh_destroy(sc->bvh);
    delete sc;
    gr::ctx_release(ctx);
    return GR_OK;
}

gr_status gr_scene_info(const gr_scene* sc, uint32_t* width, uint32_t* height, uint32_t* triangles, uint32_t* lights) {
    if (!sc) return GR_ERR_INVALID;
    if (width) *width = sc->cam.width;
    if (height) *height = sc->cam.height;
    if (triangles) *triangles = sc->num_tris;
    if (lights) *lights = sc->num_lights;
    return GR_OK;
}

gr_status gr_render(gr_scene* sc, const gr_render_opts* opts, float* rgb, gr_render_stats* stats) {
    if (!sc || !opts) return GR_ERR_INVALID;
    gr_ctx* ctx = sc->ctx;
    if (opts->max_depth > (uint32_t)gr::kMaxDepth)
        return fail(ctx, GR_ERR_INVALID, "gr_render: max_depth above " + std::to_string(gr::kMaxDepth));
    const auto t0 = std::chrono::steady_clock::now();
    SC_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const uint32_t npix = sc->cam.width * sc->cam.height;
    const bool asked = opts->wave_paths || sc->default_wave_paths;
    const uint64_t want_paths = opts->wave_paths ? opts->wave_paths
                                : (sc->default_wave_paths ? sc->default_wave_paths : ctx->default_wave_paths);
    uint32_t per_wave = (uint32_t)std::max<uint64_t>(1, want_paths / npix);
    if (opts->spp) per_wave = std::min(per_wave, opts->spp);
    uint64_t cap64 = (uint64_t)per_wave * npix;
    if (cap64 > 0xFFFFFFFFull / 2) return fail(ctx, GR_ERR_INVALID, "gr_render: wave too large");
    gr::WavePool* pool = gr::context_pool(ctx);
    if (!pool) return fail(ctx, GR_ERR_OOM_BUDGET, "gr_render: host allocation failed");
    // a wave size nobody asked for halves until the device has room for it
    cudaError_t pe;
    while ((pe = pool->ensure((uint32_t)cap64)) != cudaSuccess && !asked && per_wave > 1) {
        cudaGetLastError();
        per_wave /= 2;
        cap64 = (uint64_t)per_wave * npix;
    }
    SC_CUDA(ctx, pe);
    SC_CUDA(ctx, pool->clear_errors(s));
    gr::WaveHeader before{};
    SC_CUDA(ctx, cudaMemcpyAsync(&before, pool->ps.hdr, sizeof(before), cudaMemcpyDeviceToHost, s));
    gr::HostJob job;
    const int layout = sc->bvh->layout;
    job.sc = gr::scene_view(sc, layout);
    job.fb = (double*)sc->fb.p;
    job.fbc = (uint32_t*)sc->fb_count.p;
    job.npix = npix;
    job.spp_total = opts->spp;
    job.spp_done = 0;
    job.sample_offset = sc->samples_done;
    job.max_depth = opts->max_depth;
    job.rr_depth = opts->rr_depth;
    job.flags = opts->flags;
    job.seed = opts->seed;
    std::vector<gr::HostJob*> jobs{&job};
    std::vector<gr::JobDev> table;
    uint32_t waves = 0;
    for (;;) {
        uint32_t paths = 0, pix = 0, depth = 0;
        const uint32_t nj = gr::pack_wave(jobs, (uint32_t)cap64, table, &paths, &pix, &depth);
        if (nj == 0) break;
        SC_CUDA(ctx, gr::run_wave(*pool, table.data(), nj, paths, pix, depth, ctx->num_sms, s,
                                  (opts->flags & GR_RENDER_NO_GRAPH) == 0, scene_tuning(sc)));
        ++waves;
    }
    gr::WaveHeader after{};
    uint32_t err = 0;
    SC_CUDA(ctx, cudaMemcpyAsync(&after, pool->ps.hdr, sizeof(after), cudaMemcpyDeviceToHost, s));
    SC_CUDA(ctx, cudaMemcpyAsync(&err, pool->error_word(), 4, cudaMemcpyDeviceToHost, s));
    // the image goes to device memory by a kernel, or to host memory below
    bool on_device = false;
    if (rgb) {
        cudaPointerAttributes pa{};
        SC_CUDA(ctx, cudaPointerGetAttributes(&pa, rgb));
        on_device = pa.type == cudaMemoryTypeDevice || pa.type == cudaMemoryTypeManaged;
        if (on_device && pa.device != ctx->device)
            return fail(ctx, GR_ERR_INVALID, "gr_render: output buffer on another device");
        if (on_device) SC_CUDA(ctx, gr::mean_rgb((const double*)sc->fb.p, (const uint32_t*)sc->fb_count.p, npix, rgb, s));
    }
    SC_CUDA(ctx, cudaStreamSynchronize(s));
    sc->samples_done += opts->spp;
    if (rgb && !on_device) {
        float* h_rgb = rgb;
        std::vector<double> sum(3ull * npix);
        std::vector<uint32_t> cnt(npix);
        SC_CUDA(ctx, cudaMemcpy(sum.data(), sc->fb.p, 24ull * npix, cudaMemcpyDeviceToHost));
        SC_CUDA(ctx, cudaMemcpy(cnt.data(), sc->fb_count.p, 4ull * npix, cudaMemcpyDeviceToHost));
        for (uint32_t p = 0; p < npix; ++p) {
            const double inv = cnt[p] ? 1.0 / cnt[p] : 0.0;
            for (int c = 0; c < 3; ++c) h_rgb[3ull * p + c] = (float)(sum[3ull * p + c] * inv);
        }
    }
    if (stats) {
        stats->ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        stats->closest_rays = after.closest_rays - before.closest_rays;
        stats->shadow_rays = after.shadow_rays - before.shadow_rays;
        stats->samples = (uint64_t)opts->spp * npix;
        stats->waves = waves;
        stats->device_errors = err;
    }
    if (err & gr::ERR_STACK) return fail(ctx, GR_ERR_OVERFLOW, "gr_render: traversal stack overflow");
    if (err) return fail(ctx, GR_ERR_CUDA, "gr_render: device error bits set");
    return GR_OK;
}

gr_status gr_scene_accumulation(gr_scene* sc, double* h_sum_rgb, uint32_t* h_count) {
    if (!sc) return GR_ERR_INVALID;
    gr_ctx* ctx = sc->ctx;
    SC_CUDA(ctx, cudaSetDevice(ctx->device));
    SC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const size_t npix = (size_t)sc->cam.width * sc->cam.height;
    if (h_sum_rgb) SC_CUDA(ctx, cudaMemcpy(h_sum_rgb, sc->fb.p, 24 * npix, cudaMemcpyDeviceToHost));
    if (h_count) SC_CUDA(ctx, cudaMemcpy(h_count, sc->fb_count.p, 4 * npix, cudaMemcpyDeviceToHost));
    return GR_OK;
}

gr_status gr_scene_reset(gr_scene* sc) {
    if (!sc) return GR_ERR_INVALID;
    gr_ctx* ctx = sc->ctx;
    SC_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t npix = (size_t)sc->cam.width * sc->cam.height;
    SC_CUDA(ctx, cudaMemsetAsync(sc->fb.p, 0, 24 * npix, ctx->stream));
    SC_CUDA(ctx, cudaMemsetAsync(sc->fb_count.p, 0, 4 * npix, ctx->stream));
    SC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    sc->samples_done = 0;
    return GR_OK;
}

}  // extern "C"

extern "C" gr_status gr_scene_autotune(gr_scene* sc, const gr_render_opts* probe, gr_trace_tuning* best_out,
                                       uint32_t* best_wave_paths) {
    if (!sc || !probe) return GR_ERR_INVALID;
    gr_ctx* ctx = sc->ctx;
    gr_render_opts o = *probe;
    o.flags &= ~GR_RENDER_NO_GRAPH;
    auto timed = [&](double* ms) -> gr_status {
        gr_render_stats st{};
        // the first call captures the wave's graph; time the second
        gr_status r = gr_render(sc, &o, nullptr, &st);
        if (r != GR_OK) return r;
        r = gr_render(sc, &o, nullptr, &st);
        *ms = st.ms;
        return r;
    };
    const int layouts[] = {0, 1, 2, 3}, blocks[] = {64, 128, 256}, stacks[] = {8, 12, 16};
    gr_trace_tuning best{sc->bvh->layout, sc->bvh->block, sc->bvh->sstack};
    double best_ms = 1e300;
    for (int lay : layouts)
        for (int blk : blocks)
            for (int ss : stacks) {
                gr_trace_tuning t{lay, blk, ss};
                gr_status r = gr_bvh_set_tuning(sc->bvh, &t);
                if (r == GR_OK) {
                    SC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
                    double ms = 0;
                    r = timed(&ms);
                    if (r == GR_OK && ms < best_ms) {
                        best_ms = ms;
                        best = t;
                    }
                }
                if (r != GR_OK) return r;
            }
    gr_status r = gr_bvh_set_tuning(sc->bvh, &best);
    if (r != GR_OK) return r;
    SC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    // wave size (queue capacity): the probe must fill the largest candidate
    const uint32_t npix = sc->cam.width * sc->cam.height;
    uint32_t best_wave = gr::kDefaultWavePaths;
    double best_wms = 1e300;
    const uint32_t waves[] = {1u << 22, 1u << 23, 1u << 24, 1u << 25, gr::kDefaultWavePaths};
    const uint32_t fill_spp = (uint32_t)std::max<uint64_t>(probe->spp, ((uint64_t)waves[4] + npix - 1) / npix);
    for (uint32_t w : waves) {
        o = *probe;
        o.flags &= ~GR_RENDER_NO_GRAPH;
        o.spp = fill_spp;
        o.wave_paths = w;
        double ms = 0;
        r = timed(&ms);
        if (r != GR_OK) return r;
        const double per_sample = ms / ((double)o.spp * npix);
        if (per_sample < best_wms) {
            best_wms = per_sample;
            best_wave = w;
        }
    }
    sc->default_wave_paths = best_wave;
    gr_scene_reset(sc);
    if (best_out) *best_out = best;
    if (best_wave_paths) *best_wave_paths = best_wave;
    return GR_OK;
}

extern "C" gr_status gr_scene_set_tuning(gr_scene* sc, const gr_trace_tuning* t, uint32_t wave_paths) {
    if (!sc || !t) return GR_ERR_INVALID;
    gr_status st = gr_bvh_set_tuning(sc->bvh, t);
    if (st != GR_OK) return st;
    SC_CUDA(sc->ctx, cudaStreamSynchronize(sc->ctx->stream));
    sc->default_wave_paths = wave_paths;
    return GR_OK;
}

extern "C" gr_status gr_scene_get_tuning(const gr_scene* sc, gr_trace_tuning* t, uint32_t* wave_paths) {
    if (!sc) return GR_ERR_INVALID;
    if (t) gr_bvh_get_tuning(sc->bvh, t);
    if (wave_paths) *wave_paths = sc->default_wave_paths;
    return GR_OK;
}
