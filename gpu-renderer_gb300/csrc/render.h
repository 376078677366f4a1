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
    // color texture: tex_w == 0 for the constant color; else texels
    // [tex_off, tex_off + tex_w * tex_h) of the scene's texel pool
    uint32_t tex_off, tex_w, tex_h;
    float tuo, tvo, tus, tvs;  // uv offset and scale
    float sr, sg, sb;          // rough plastic: specular lobe reflectance
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

// Camera::setup (camera.h:21-38) from the C-ABI record.
DevCamera make_camera(const gr_camera& c);

// Everything a shading or traversal kernel needs about one scene.
struct SceneDev {
    const float* verts;       // 9 floats per triangle, scene order
    const float4* normals;    // 3 per triangle (w unused) or nullptr
    const uint32_t* tri_mat;  // material index | 0x80000000 with normals | 0x40000000 with texcoords
    const float* uvs;         // 6 floats per triangle (texcoords of its corners) or nullptr
    const float4* texels;     // texel pool of the material textures (rgb, unused)
    const DevMaterial* mats;
    const uint32_t* lights;   // emissive triangle ids
    uint32_t num_lights;
    uint32_t num_tris;
    const void* nodes;  // traversal nodes in the wave's layout
    const Tri* tris;
    const BvhMeta* meta;
    DevCamera cam;
    float env_r, env_g, env_b;
    int32_t has_env;
    // latitude-longitude environment map (env_w == 0: the constant radiance above)
    const float4* env_map;
    uint32_t env_w, env_h;
    float env_m[9];        // world-to-map rotation (row-major 3x3)
    float env_c[3];        // scene bounding-box centre
    uint32_t mat_types;    // bit t set when a triangle has a material of type t
};

constexpr int kMaxDepth = 64;
// Shading groups a bounce's paths by what they hit: a miss, or one of the four
// material types (GR_MAT_DIFFUSE .. GR_MAT_PLASTIC), so that the paths of a warp
// run one material's code.
constexpr int kShadeBins = 5;
constexpr uint32_t kMaxJobs = 1024;  // jobs in one wave

// One render job in a wave: a scene, its accumulation target, and the slice
// of the wave's path ids that render its samples. Paths of a job are
// pid = path_base + s * npix + pixel for s < wave_samples.
struct JobDev {
    SceneDev sc;
    double* fb;          // 3 doubles per pixel (running sums)
    uint32_t* fbc;       // samples per pixel
    uint32_t path_base;  // first path id of the job in this wave
    uint32_t npix;
    uint32_t pix_base;   // first resolve slot of the job in this wave
    uint32_t wave_samples;
    uint32_t sample_base;  // sample index of the job's first sample in this wave
    uint32_t max_depth;
    int32_t rr_depth;
    uint32_t flags;
    uint64_t seed;
};

// Device-resident description of the current wave (written by the host
// before each wave; the captured kernel sequence reads it).
struct WaveHeader {
    uint32_t njobs;
    uint32_t total_paths;
    uint32_t total_pix;
    uint32_t max_depth;  // bounces the wave runs (max over its jobs)
    unsigned long long closest_rays, shadow_rays;  // running totals
};

// Path state for one wave, indexed by path id.
struct Paths {
    float4* ray;    // 2 per path: (o.xyz, d.x), (d.y, d.z, tmin, tmax)
    float4* hit;    // (t, prim bits, u, v)
    float4* thr;    // (throughput rgb, pdf of the last BSDF sample)
    float4* acc;    // (radiance rgb, 0)
    uint32_t* flags;
    uint32_t* job;  // job of each path
    unsigned long long* rng;
    uint32_t* qa;   // path-id queues, ping-pong by bounce
    uint32_t* qb;
    uint32_t* bins; // the bounce's queue regrouped for shading: kShadeBins runs of capacity entries
    float4* sray;   // shadow rays, 2 per entry
    float4* scon;   // shadow contribution (rgb, pid bits)
    uint32_t* cnt;  // [0, kMaxDepth]: closest queue sizes; [kMaxDepth+1, ...]: shadow queue sizes
    unsigned long long* work;  // dynamic-fetch counters, one per trace launch of a wave
    WaveHeader* hdr;
    JobDev* jobs;   // kMaxJobs entries
    uint32_t capacity;
};

// A captured wave (CUDA graph), reused while its key (pointers, sizes) is
// unchanged. The wave's contents (jobs, counts) live in device memory.
struct WaveGraph {
    cudaGraphExec_t exec = nullptr;
    uint64_t key = 0;
    WaveGraph() = default;
    WaveGraph(const WaveGraph&) = delete;  // owns exec
    WaveGraph& operator=(const WaveGraph&) = delete;
    void release();
    ~WaveGraph() { release(); }
};

// Path memory, job staging and the captured wave of one renderer (a scene's
// own gr_render, or a server).
struct WavePool {
    static constexpr int kSlots = 4;
    DevBuf mem;
    Paths ps{};
    uint32_t capacity = 0;
    // captured waves, most recently used first (waves of different depth,
    // grouping or tuning each keep their own)
    static constexpr int kGraphs = 4;
    WaveGraph graphs[kGraphs];
    void release_graphs();
    // pinned staging for the per-wave job table and header, one slot per wave
    // in flight; a slot is rewritten only after its event has completed
    JobDev* h_jobs = nullptr;
    WaveHeader* h_hdr = nullptr;
    cudaEvent_t ev[kSlots] = {};
    int slot = 0;
    cudaError_t ensure(uint32_t paths);
    // clears the device error bits before a call, on stream s
    cudaError_t clear_errors(cudaStream_t s);
    // device address of the error bits (ERR_*), read back after a call
    const uint32_t* error_word() const;
    void release();
    ~WavePool() { release(); }
};

// Paths per wave when the caller and the scene leave it open: a whole render
// of up to 64 Mi paths (about 11.5 GB of path state) runs as one wave, which
// on the glossy 1024 x 768 x 64-spp render measured 80 ms against 108 ms in
// 8 Mi-path waves (per-wave costs: the tails of 17 bounce steps, the resolve).
constexpr uint32_t kDefaultWavePaths = 1u << 26;

// The path pool of a context's gr_render and gr_render_batch calls (created on
// first use, freed with the context); scenes share it, calls run one at a
// time on the context's stream.
WavePool* context_pool(gr_ctx* ctx);

// Host-side view of one job for the wave scheduler.
struct HostJob {
    SceneDev sc;
    double* fb;
    uint32_t* fbc;
    uint32_t npix;
    uint32_t spp_total;
    uint32_t spp_done;  // samples already scheduled
    uint32_t sample_offset;  // sample index of this job's sample 0
    uint32_t max_depth;
    int32_t rr_depth;
    uint32_t flags;
    uint64_t seed;
};

// Runs one wave over `jobs` (already packed by the caller: path_base, pix_base,
// wave_samples, sample_base filled in). Uses the pool's captured graph unless
// use_graph is false.
cudaError_t run_wave(WavePool& pool, const JobDev* h_jobs, uint32_t njobs, uint32_t total_paths, uint32_t total_pix,
                     uint32_t max_depth, int num_sms, cudaStream_t s, bool use_graph, const TraceTuning& tune);

// Scene view for a wave of the given node layout (the layout must be built).
SceneDev scene_view(gr_scene* sc, int layout);

}  // namespace gr

// The traversal configuration a scene renders with (its BVH's tuning).
gr::TraceTuning scene_tuning(const gr_scene* sc);

namespace gr {

// Packs as many samples of `jobs` (in order) as fit into `capacity` paths;
// returns the number of jobs in the wave (0 when nothing fits). Advances
// spp_done of the scheduled jobs.
uint32_t pack_wave(std::vector<HostJob*>& jobs, uint32_t capacity, std::vector<JobDev>& out, uint32_t* total_paths,
                   uint32_t* total_pix, uint32_t* max_depth);

// Mean radiance -> sRGB-encoded RGBA8 (R in the low byte), the reference's
// filter_kernel (pathtracer_kernel.h:792-810); pixels without samples are black.
cudaError_t filter_rgba8(const double* fb, const uint32_t* fbc, uint32_t npix, uint32_t* out, cudaStream_t s);
// Mean radiance of an accumulation into 3 floats per pixel in device memory.
cudaError_t mean_rgb(const double* fb, const uint32_t* fbc, uint32_t npix, float* out, cudaStream_t s);

}  // namespace gr

struct gr_scene {
    gr_ctx* ctx = nullptr;
    gr_bvh* bvh = nullptr;
    uint32_t num_tris = 0, num_lights = 0;
    gr::DevBuf verts, normals, tri_mat, mats, lights, uvs, texels, env_map;
    uint32_t env_w = 0, env_h = 0;
    float env_m[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    float env_c[3] = {0, 0, 0};
    gr::DevBuf fb, fb_count;
    uint32_t samples_done = 0;
    uint32_t default_wave_paths = 0;  // 0 = library default (autotuned by gr_scene_autotune)
    gr::DevCamera cam{};
    uint32_t mat_types = 0;  // material types its triangles use (bit per GR_MAT_*)
    gr_camera cam_rec{};  // the camera record cam was made from (view operations edit it)
    float env[3] = {0, 0, 0};
    int has_env = 0;
};
