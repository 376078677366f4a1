// Internal scene and wavefront-integrator declarations (host + device).
#pragma once

#include <vector>

#include "gr_internal.h"

namespace gr {

struct DevMaterial {
    int32_t type;
    float cr, cg, cb;     // color
    float er, eg, eb;     // emission
    float ax, ay;         // GGX roughness
    float eir, eig, eib;  // eta_i
    float etr, etg, etb;  // eta_t
    float kr, kg, kb;     // k
    float ior;
    uint32_t emissive;
};

// Camera in the reference's non-free mode: camera-space direction
// ((1 - 2 rx/W) tan(fov/2), (2 ry/H - 1) tan(fov/2) / aspect, 1), rotated by
// the upper 3x3 of to_world; origin = to_world translation.
struct DevCamera {
    float m[12];  // row-major 3x4 of to_world
    float tan_half;
    float aspect;
    uint32_t width, height;
};

// Everything a shading or traversal kernel needs about one scene.
struct SceneDev {
    const float* verts;       // 9 floats per triangle, scene order
    const float4* normals;    // 3 per triangle (w unused) or nullptr
    const uint32_t* tri_mat;  // material index | 0x80000000 when the triangle has normals
    const DevMaterial* mats;
    const uint32_t* lights;   // emissive triangle ids
    uint32_t num_lights;
    uint32_t num_tris;
    const Node* nodes;
    const Tri* tris;
    const BvhMeta* meta;
    DevCamera cam;
    float env_r, env_g, env_b;
    int32_t has_env;
};

// Per-wave header in device memory, updated on the device between waves so a
// wave's launch sequence is identical every time (graph friendly).
struct WaveHeader {
    uint32_t sample_base;   // first sample index of this wave
    uint32_t wave_samples;  // samples per pixel in this wave
    uint32_t remaining;     // samples per pixel still to do, this wave included
    uint32_t max_wave;      // samples per pixel per full wave
    unsigned long long closest_rays, shadow_rays;
};

constexpr int kMaxDepth = 64;

// Path state for one wave, indexed by path id pid = s * npix + pixel.
struct Paths {
    float4* ray;    // 2 per path: (o.xyz, d.x), (d.y, d.z, tmin, tmax)
    float4* hit;    // (t, prim bits, u, v)
    float4* thr;    // (throughput rgb, pdf of the last BSDF sample)
    float4* acc;    // (radiance rgb, 0)
    uint32_t* flags;
    unsigned long long* rng;
    uint32_t* qa;   // path-id queues, ping-pong by bounce
    uint32_t* qb;
    float4* sray;   // shadow rays, 2 per entry
    float4* scon;   // shadow contribution (rgb, pid bits)
    uint32_t* cnt;  // [0, kMaxDepth]: closest queue sizes; [kMaxDepth+1, ...]: shadow queue sizes
    unsigned long long* work;  // dynamic-fetch counters, one per trace launch of a wave
    WaveHeader* hdr;
    uint32_t capacity;
};

struct RenderParams {
    uint32_t max_depth;
    int32_t rr_depth;
    uint32_t flags;
    uint64_t seed;
    uint32_t npix;
};

cudaError_t render_waves(const SceneDev& sc, Paths& ps, const RenderParams& rp, double* fb, uint32_t* fb_count,
                         uint32_t waves, int num_sms, cudaStream_t s);

}  // namespace gr

struct gr_scene {
    gr_ctx* ctx = nullptr;
    gr_bvh* bvh = nullptr;
    uint32_t num_tris = 0, num_lights = 0;
    gr::DevBuf verts, normals, tri_mat, mats, lights;
    gr::DevBuf fb, fb_count;
    gr::DevBuf path_mem;
    uint32_t path_capacity = 0;
    uint32_t samples_done = 0;
    gr::DevCamera cam{};
    float env[3] = {0, 0, 0};
    int has_env = 0;
};
