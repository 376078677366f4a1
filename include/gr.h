/*
 * gr — GB300-native wavefront path tracer: the C ABI.
 *
 * This is the drop-in boundary for slongle/GPU-Renderer's render path. The
 * reference has no C ABI (everything links into one executable); each entry
 * point below names the in-process reference interface it replaces.
 *
 * Conventions
 *   - every call returns a gr_status; nothing here calls exit() or aborts
 *     (the reference's CUDA_CHECK exits, src/utility/buffer.h:3-12);
 *   - `stream` arguments are cudaStream_t passed as void* (NULL = legacy
 *     default stream); calls that take a stream are stream-ordered and do not
 *     synchronise the device;
 *   - pointers named d_* are device pointers, h_* are host pointers;
 *   - one gr_ctx per host thread; objects created from a context are used from
 *     that context's thread only.
 */
#ifndef GR_H_
#define GR_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gr_status {
    GR_OK = 0,
    GR_ERR_INVALID = 1,     /* bad argument or object state */
    GR_ERR_CUDA = 2,        /* a CUDA runtime call failed; see gr_last_error */
    GR_ERR_OOM_BUDGET = 3,  /* allocation failed or exceeds the memory budget */
    GR_ERR_PARSE = 4,       /* scene file could not be parsed */
    GR_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
    GR_ERR_OVERFLOW = 6,    /* a device-side capacity (stack, queue) was exceeded */
    GR_ERR_IO = 7,          /* a file could not be written */
    GR_ERR_BUSY = 8         /* the render server refused a job it could not start in time (load shedding) */
} gr_status;

/* Ray and hit records, byte-compatible with the reference's Ray and Hit
 * (src/renderer/ray.h:5-19). A miss has prim == -1. */
typedef struct gr_ray {
    float o[3];
    float d[3];
    float tmin, tmax;
} gr_ray;

typedef struct gr_hit {
    float t;      /* distance in units of |d|; tmax when prim == -1 */
    int32_t prim; /* triangle index in the input order, -1 on a miss */
    float u, v;   /* barycentric weights of vertex 1 and vertex 2 */
} gr_hit;

typedef struct gr_ctx gr_ctx;
typedef struct gr_bvh gr_bvh;

/* ---- context ------------------------------------------------------------ */

/* Context options (the reference has none: its frame size and queues follow
 * the scene, pathtracer.cu:41-150). */
typedef struct gr_opts {
    uint32_t default_wave_paths; /* paths in flight per render wave when neither the call nor its scene sets the
                                    wave size (0 = the whole call as one wave up to 64 Mi paths); the context's
                                    pool of path state, about 172 bytes per path, grows to the largest wave used */
    uint32_t flags;              /* reserved, 0 */
} gr_opts;

/* Binds `device` and creates a context (streams, memory pool); `opts` may be
 * NULL for the defaults. The context keeps the 8-wide layout build's scratch
 * (about 144 bytes per triangle of the largest BVH it has collapsed) between
 * builds, so building a layout neither allocates nor frees device memory once
 * it has grown; destroying the context frees it. Replaces the process-global
 * CUDA state the reference sets up implicitly. */
gr_status gr_context_create(int device, const gr_opts* opts, gr_ctx** out);
gr_status gr_context_destroy(gr_ctx* ctx);
/* Text of the last error recorded on `ctx` (never NULL). */
const char* gr_last_error(const gr_ctx* ctx);
/* Static description of a status code. */
const char* gr_status_string(int status);
/* Library version as an integer: major*10000 + minor*100 + patch. */
int gr_version(void);

/* ---- acceleration structure ----------------------------------------------
 * Replaces LBVH_build (src/renderer/bvh.h:186-221), which runs single-threaded
 * on the host. The GPU build computes 30-bit Morton codes of triangle
 * centroids, sorts them with a stable LSD radix sort, and builds the radix tree
 * over unique codes with midpoint splits inside equal-code runs (the
 * reference's rule, bvh.h:161-176) in one bottom-up pass that links the nodes
 * and fits their boxes. */

gr_status gr_bvh_create(gr_ctx* ctx, gr_bvh** out);
gr_status gr_bvh_destroy(gr_bvh* bvh);

/* Builds over `n` triangles given as 9 floats each (p0.xyz, p1.xyz, p2.xyz)
 * in device memory. The BVH keeps no pointer to d_verts. */
gr_status gr_bvh_build(gr_bvh* bvh, const float* d_verts, uint32_t n, void* stream);

/* Same, from host memory (copies in, builds, waits). */
gr_status gr_bvh_build_host(gr_bvh* bvh, const float* h_verts, uint32_t n);

/* Number of triangles the BVH was built over. */
uint32_t gr_bvh_size(const gr_bvh* bvh);

/* Build without any device allocation. This entry point has no counterpart in
 * the reference. It is for callers that cannot call cudaMalloc: plug-ins whose
 * host application owns all device memory and hands them only the buffers of
 * a call, and latency-critical loops where cudaMalloc / cudaFree would
 * synchronise the device.
 *
 * The caller passes the input soup and every output buffer (device memory):
 *   d_nodes        64 bytes x max(n-1, 1)  traversal nodes (layout of gr_bvh_export's h_nodes)
 *   d_tris         48 bytes x n            triangles in leaf order (gr_bvh_export's h_tris)
 *   d_sorted_prim  4 bytes x n             triangle ids in Morton order
 *   d_sorted_code  4 bytes x n             Morton codes in sorted order
 *   d_header       64 bytes                uint32 root index at byte 0, device error bits at byte 8
 * The build's scratch is one fixed device array inside the library, sized for
 * at most 131,072 triangles (about 4.5 MB, held on every GPU that loads the
 * library until the process exits); a larger n returns GR_ERR_INVALID. The
 * first call on a device looks up that array's device address, so make the
 * first call on each device before any stream capture. All calls share the
 * array: it is cleared where it must start at zero, and calls that overlap on
 * the GPU race on it. If the device's context is destroyed and created again
 * (cudaDeviceReset), the next call looks the array's address up again.
 * Stream-ordered; does not wait for the device. */
gr_status gr_bvh_build_noalloc(gr_ctx* ctx, const float* d_verts, uint32_t n, void* d_nodes, void* d_tris,
                               uint32_t* d_sorted_prim, uint32_t* d_sorted_code, void* d_header, void* stream);

/* Copies the build to host buffers for parity checks (waits for the device):
 *   h_sorted_prim, h_sorted_code : n words — triangle ids and Morton codes in
 *                                  sorted order (the reference's MortonInfo)
 *   h_ref_nodes                  : 8 words x (2n-1) — the reference's
 *                                  BVHLinearNode array in DFS preorder
 *                                  (box min.xyz, max.xyz, tri/right index, leaf)
 *   h_nodes                      : 16 words x max(n-1,1) — the traversal layout
 *   h_tris                       : 12 floats x n — triangles in leaf order
 *   h_root                       : root node index
 * Any pointer may be NULL. */
gr_status gr_bvh_export(gr_bvh* bvh, uint32_t* h_sorted_prim, uint32_t* h_sorted_code, uint32_t* h_ref_nodes,
                        uint32_t* h_nodes, float* h_tris, uint32_t* h_root);

/* Node layouts for traversal (no counterpart in the reference, whose nodes are
 * binary 32-byte records tested one at a time):
 *   GR_LAYOUT_BVH2     binary nodes with both child boxes in the parent (64 B)
 *   GR_LAYOUT_BVH4     4-wide nodes with FP32 child boxes (128 B), the binary
 *                      tree with every other level folded
 *   GR_LAYOUT_BVH4_Q8  the same 4-wide tree with 8-bit child boxes quantised
 *                      outward against a per-node origin and power-of-two
 *                      scale (64 B); the boxes contain the FP32 boxes, so the
 *                      closest hit is the same
 *   GR_LAYOUT_BVH8_Q8  8-wide nodes with 8-bit child boxes (96 B), collapsed
 *                      from the binary tree by opening the largest child
 *                      first, children placed so a ray's octant gives a
 *                      near-to-far order, nodes numbered breadth first, and
 *                      leaf triangles copied into node order
 * The binary tree is always built; another layout is derived from it on the
 * GPU when first requested and kept until the next build (the 8-wide build
 * waits for the stream once per tree level). */
#define GR_LAYOUT_BVH2 0
#define GR_LAYOUT_BVH4 1
#define GR_LAYOUT_BVH4_Q8 2
#define GR_LAYOUT_BVH8_Q8 3

/* Selects the layout gr_trace uses (building it if needed; stream-ordered). */
gr_status gr_bvh_set_layout(gr_bvh* bvh, int layout, void* stream);

/* Traversal launch configuration for gr_trace: node layout, threads per block
 * (64, 128, 256) and stack entries per thread kept in shared memory (8, 12,
 * 16; deeper entries spill to local memory). The reference launches 32-thread
 * blocks with a 64-entry local stack (pathtracer_kernel.h:192, :242). */
typedef struct gr_trace_tuning {
    int32_t layout;
    int32_t block;
    int32_t short_stack;
} gr_trace_tuning;

typedef struct gr_tuning_result {
    gr_trace_tuning tuning;
    float ms; /* best of two timed launches */
} gr_tuning_result;

gr_status gr_bvh_set_tuning(gr_bvh* bvh, const gr_trace_tuning* tuning);
gr_status gr_bvh_get_tuning(const gr_bvh* bvh, gr_trace_tuning* tuning);

/* Autotuner: times every configuration (3 layouts x 3 block sizes x 3 stack
 * depths) on the caller's rays (device memory; d_hits is overwritten), keeps
 * the fastest for this BVH, and reports up to max_results timings. All
 * configurations return the same closest hits. Waits for the device. */
gr_status gr_bvh_autotune(gr_bvh* bvh, const gr_ray* d_rays, uint64_t n, int any_hit, gr_hit* d_hits,
                          gr_tuning_result* h_table, uint32_t max_results, uint32_t* n_results);

/* Bytes of a layout's nodes and of the triangle array it traverses (the
 * 8-wide layout has its own, in node order; the others share the leaf-order
 * triangles of gr_bvh_export). Builds the layout if needed; waits. */
gr_status gr_bvh_layout_size(gr_bvh* bvh, int layout, uint64_t* node_bytes, uint64_t* tri_bytes);

/* Copies a derived layout's nodes to host memory (node_bytes of
 * gr_bvh_layout_size; for the 4-wide layouts only even-depth entries are
 * nodes, the others are zero). Waits for the device. */
gr_status gr_bvh_export_layout(gr_bvh* bvh, int layout, void* h_nodes);

/* Copies the triangles a layout traverses (tri_bytes of gr_bvh_layout_size,
 * 12 floats each: v0, prim-id bits, v1, 0, v2, 0). Waits for the device. */
gr_status gr_bvh_export_layout_tris(gr_bvh* bvh, int layout, float* h_tris);

/* ---- traversal -------------------------------------------------------------
 * Replaces trace / trace_shadow (src/renderer/pathtracer_kernel.h:235-246 and
 * :310-321) on a queue of rays: closest hit (any_hit = 0) or first hit found
 * (any_hit = 1). FP32 watertight triangle test; closest-hit ties at equal t go
 * to the smaller prim id. */

gr_status gr_trace(gr_bvh* bvh, const gr_ray* d_rays, uint64_t n, gr_hit* d_hits, int any_hit, void* stream);

/* Host-memory variant: rays in host memory, hits to host memory; waits. With
 * page-locked buffers (cudaHostAlloc / cudaHostRegister) the traversal reads
 * and writes them directly over the host link; other buffers are staged
 * through device memory in chunks of at least 1 Mi rays on two streams, so
 * the copies of one chunk overlap the traversal of another. */
gr_status gr_trace_host(gr_bvh* bvh, const gr_ray* h_rays, uint64_t n, gr_hit* h_hits, int any_hit);

/* ---- scene records ----------------------------------------------------------
 * Mirror the reference's TriangleMesh / Material / Camera / EnvironmentLight
 * (src/renderer/triangle.h:28-49, material.h:15-34, camera.h:7-132,
 * environment.h:30-53) as plain structs. Textures are constant (one value per
 * material), as the reference's 1x1 textures are. */

typedef enum gr_material_type {
    GR_MAT_DIFFUSE = 0,    /* Lambert (reference MATERIAL_DIFFUSE, "diffuse") */
    GR_MAT_DIELECTRIC = 1, /* smooth Fresnel dielectric (MATERIAL_SPECULAR: "dielectric", "glass", "mirror") */
    GR_MAT_CONDUCTOR = 2,  /* GGX rough conductor (MATERIAL_ROUGH_CONDUCTOR: "roughconductor", "conductor") */
    GR_MAT_PLASTIC = 3     /* rough plastic (MATERIAL_ROUGH_PLASTIC, "roughplastic", bsdf.h:33-39): a Lambert lobe
                              of color plus a GGX lobe of specular with dielectric Fresnel from eta_i[0] to
                              eta_t[0], each lobe sampled with probability 1/2 */
} gr_material_type;

typedef struct gr_material {
    int32_t type;       /* gr_material_type */
    float color[3];     /* reflectance (diffuse) or specular reflectance */
    float emission[3];  /* area-light radiance; non-zero makes the material's triangles lights */
    float alpha_u, alpha_v; /* GGX roughness (conductor) */
    float eta_i[3], eta_t[3], k[3]; /* conductor Fresnel terms */
    float ior;          /* dielectric index of refraction (interior / exterior) */
    /* Optional color texture (Texture / TextureView, texture.h:15-50): NULL for
     * the constant color above, else color_map_width x color_map_height RGB
     * floats, row 0 first, looked up nearest at uv * uv_scale + uv_offset
     * (uv: the triangle's interpolated texcoords, or its barycentrics when the
     * mesh has none; texel (int(u * width) mod width, int(v * height) mod
     * height)). A checkerboard is the 2 x 2 map (c0, c1; c1, c0). The color
     * scales the Lambert reflectance, the conductor's specular reflectance and
     * the dielectric's transmission and reflection, as color does. */
    const float* color_map;
    uint32_t color_map_width, color_map_height;
    float uv_offset[2], uv_scale[2];
    float specular[3];  /* rough plastic: the GGX lobe's reflectance */
} gr_material;

typedef struct gr_mesh {
    const float* positions;  /* 3 floats per vertex, world space */
    uint32_t num_vertices;
    const float* normals;    /* NULL, or 3 floats per vertex (shading normals) */
    const uint32_t* indices; /* 3 vertex indices per triangle */
    uint32_t num_triangles;
    uint32_t material;       /* index into the material table */
    const float* texcoords;  /* NULL, or 2 floats per vertex (texture coordinates) */
} gr_mesh;

/* Pinhole camera in the reference's Mitsuba convention (camera.h:21-38):
 * row-major camera-to-world matrix, horizontal field of view in degrees. */
typedef struct gr_camera {
    float to_world[16];
    float fov_deg;
    uint32_t width, height;
} gr_camera;

typedef struct gr_environment {
    float radiance[3]; /* constant environment radiance (reference "constant" emitter) */
    int32_t enabled;
    /* Optional latitude-longitude map (EnvironmentLight, environment.h:15-27):
     * NULL for the constant radiance, else map_width x map_height RGB floats,
     * row 0 first. A ray that leaves the scene sees the texel of the direction
     * from the scene's bounding-box centre to o + 1e5 d, turned into the map's
     * frame by the inverse of to_world (row-major 4x4): theta = acos(z) picks
     * the row, phi = atan2(y, x) in [0, 2 pi) the column. */
    const float* map;
    uint32_t map_width, map_height;
    float to_world[16];
} gr_environment;

/* Render options. The reference's PTOptions (pathtracer.h:7-14) fixes
 * max_path_length at 33 and draws one sample per render() call. */
typedef struct gr_render_opts {
    uint32_t spp;        /* samples per pixel added by this call */
    uint32_t max_depth;  /* shading steps per path (the reference's max_path_length) */
    uint64_t seed;       /* RNG seed; a path's stream is keyed by (seed, pixel, sample index) */
    int32_t rr_depth;    /* Russian roulette after this bounce (reference: 3); < 0 disables */
    uint32_t flags;      /* GR_RENDER_* */
    uint32_t wave_paths; /* paths in flight per wave (0 = the scene's default, else the library's: the
                            whole call as one wave up to 64 Mi paths, smaller when the device lacks room) */
} gr_render_opts;

/* Reproduce the reference's integrator quirks for comparison with its
 * images: the Russian-roulette rescale is not stored, roulette-killed paths
 * see the environment at the next bounce, and the GGX pdf is D|cos h|/(4 wo.h)
 * (pathtracer_kernel.h:738-748, microfacet.h:148-155). Default: corrected. */
#define GR_RENDER_REFERENCE_COMPAT 1u
/* Launch each wave's kernels directly instead of replaying the wave as a
 * captured CUDA graph (the default). The image is the same either way. */
#define GR_RENDER_NO_GRAPH 2u

typedef struct gr_render_stats {
    double ms;             /* host wall time of the call */
    uint64_t closest_rays; /* camera + scatter rays traced */
    uint64_t shadow_rays;  /* NEE shadow rays traced */
    uint64_t samples;      /* pixel samples added */
    uint32_t waves;        /* path waves launched */
    uint32_t device_errors;/* device error bits seen (0 = none) */
} gr_render_stats;

typedef struct gr_scene gr_scene;

/* Replaces Scene::Scene + createDeviceData (scene.cpp:4-51): flattens the
 * meshes into one triangle list (mesh order, then triangle order), collects
 * emissive triangles as lights, uploads, and builds the LBVH on the GPU. */
gr_status gr_scene_create(gr_ctx* ctx, const gr_mesh* meshes, uint32_t num_meshes, const gr_material* materials,
                          uint32_t num_materials, const gr_camera* camera, const gr_environment* env,
                          gr_scene** out);
gr_status gr_scene_destroy(gr_scene* scene);
gr_status gr_scene_info(const gr_scene* scene, uint32_t* width, uint32_t* height, uint32_t* triangles,
                        uint32_t* lights);

/* Replaces PathTracer::render(uint32 num) (pathtracer.cu:152-170): adds
 * opts->spp samples per pixel to the scene's accumulation buffer with the
 * wavefront integrator (camera rays, closest hit, NEE + MIS shading, shadow
 * any-hit, Russian roulette) and, when rgb is not NULL, writes the running
 * mean radiance (width x height x 3 floats, row 0 first) to it. rgb may be
 * host memory or device memory of the scene's device (told apart with
 * cudaPointerGetAttributes; a device buffer is written by a kernel, with the
 * same floats as the host read-back). Waits for the device. Successive calls
 * continue the sample sequence, as repeated render() calls do. */
gr_status gr_render(gr_scene* scene, const gr_render_opts* opts, float* rgb, gr_render_stats* stats);

/* The raw accumulation: per-pixel radiance sums (3 doubles) and sample counts.
 * Either pointer may be NULL. Replaces FrameBuffer's m_buffer / m_sample_num. */
gr_status gr_scene_accumulation(gr_scene* scene, double* h_sum_rgb, uint32_t* h_count);

/* Clears the accumulation and restarts the sample sequence (PathTracer::reset,
 * pathtracer.cu:195-200). */
gr_status gr_scene_reset(gr_scene* scene);

/* Device bytes the scene holds (geometry, BVH, accumulation). */
uint64_t gr_scene_device_bytes(const gr_scene* scene);

/* ---- view: camera operations and 8-bit output -------------------------------
 * The interactive operations of the reference's viewer (PathTracer::zoom /
 * translate / rotate / resize, pathtracer.cu:177-213, camera.h:40-83). Each
 * camera change clears the accumulation (the reference's m_reset). They act on
 * the scene's to_world matrix: zoom moves the eye by d along the view
 * direction; translate by x along normalize(cross(dir, world up)) and y along
 * the vertical axis normalize(cross(horizontal, dir)); rotate turns the camera
 * by yaw radians about the world up axis, then by pitch about its horizontal
 * axis; resize changes the resolution (the field of view stays horizontal). */
gr_status gr_scene_get_camera(const gr_scene* scene, gr_camera* out);
gr_status gr_scene_set_camera(gr_scene* scene, const gr_camera* camera);
gr_status gr_scene_zoom(gr_scene* scene, float d);
gr_status gr_scene_translate(gr_scene* scene, float x, float y);
gr_status gr_scene_rotate(gr_scene* scene, float yaw, float pitch);
gr_status gr_scene_resize(gr_scene* scene, uint32_t width, uint32_t height);

/* The mean radiance as sRGB-encoded 8-bit RGBA, one uint32 per pixel (R in
 * the low byte, alpha 255, row 0 first): the reference's filter_kernel
 * (pathtracer_kernel.h:792-810), which fills the viewer's display buffer after
 * each render(uint32*). Pixels without samples are black. The device variant
 * is ordered after the scene's renders and runs on `stream`; the host variant
 * waits. */
gr_status gr_scene_rgba8(gr_scene* scene, uint32_t* d_rgba, void* stream);
gr_status gr_scene_rgba8_host(gr_scene* scene, uint32_t* h_rgba);

/* ---- diagnostics -------------------------------------------------------------
 * Every device-side wait of the library is bounded: a wait that runs out sets an
 * error bit and returns, the call reports GR_ERR_TIMEOUT, and the context stays
 * usable. This runs the LBVH build's two kinds of wait, each for `polls` polls:
 * the sort's look-back on a status word nothing publishes, and the cooperative
 * sort's grid barrier in a one-block launch waiting for a second block; both run
 * out, so it returns GR_ERR_TIMEOUT with the device error bits (ERR_TIMEOUT = 1)
 * in *err_bits. */
gr_status gr_diag_bounded_wait(gr_ctx* ctx, uint32_t polls, uint32_t* err_bits);

/* ---- image files: FrameBuffer::output / WriteImage (framebuffer.cpp:11-26, imageio.cpp:59-82) ----
 * Writes a linear RGB image (width x height x 3 floats, row 0 = the first
 * framebuffer row) to `path`, chosen by extension:
 *   ".png": 8-bit sRGB (the reference's GammaCorrect curve, clamp(255 g + 0.5)),
 *           rows bottom-up as the reference writes them (vertical flip);
 *   ".pfm": linear 32-bit floats, little-endian, rows bottom-up (PFM order).
 * GR_ERR_INVALID for another extension or a bad size, GR_ERR_IO when the file
 * cannot be written. Host-only: no GPU work. */
gr_status gr_image_write(const char* path, const float* rgb, uint32_t width, uint32_t height);
/* The scene's accumulated mean radiance written as by gr_image_write
 * (PathTracer::output, pathtracer.cu:172-175). */
gr_status gr_scene_write_image(gr_scene* scene, const char* path);

/* Node layout the scene's renders traverse (GR_LAYOUT_*; default binary).
 * Builds the layout if needed and waits. All scenes of one gr_render_batch
 * must use the same layout. */
gr_status gr_scene_set_layout(gr_scene* scene, int layout);
int gr_scene_layout(const gr_scene* scene);

/* Autotuner for renders: times the probe render (e.g. a few samples per
 * pixel) for every traversal configuration (layout x block x short-stack
 * depth), then for wave sizes (queue capacity) of 4, 8, 16, 32 and 64 Mi
 * paths, and keeps the fastest as the scene's configuration and default wave
 * size. Images do not depend on any of these. Clears the scene's
 * accumulation. gr_render and gr_render_batch keep their path state in one
 * pool per context, sized by the largest wave asked of it (about 172 bytes
 * per path). */
gr_status gr_scene_autotune(gr_scene* scene, const gr_render_opts* probe, gr_trace_tuning* best,
                            uint32_t* best_wave_paths);

/* Sets / reads a scene's traversal configuration and default wave size
 * (0 = library default), e.g. to reuse one autotuning result for many scenes. */
gr_status gr_scene_set_tuning(gr_scene* scene, const gr_trace_tuning* tuning, uint32_t wave_paths);
gr_status gr_scene_get_tuning(const gr_scene* scene, gr_trace_tuning* tuning, uint32_t* wave_paths);

/* ---- scene files ---------------------------------------------------------------
 * Replaces load_scene / load_mitsuba_file / load_obj_file (src/renderer/loaders/
 * loader.h:11-29, mitsubaloader.cpp, objloader.cpp). The Mitsuba-XML subset
 * the reference reads: sensor (fov, toWorld), film (width, height), bsdf
 * (diffuse, mirror, glass, dielectric, roughdielectric, conductor,
 * roughconductor; roughplastic is read as Lambert; twosided; named ids and
 * ref), emitter (area, constant), shape (obj, sphere, rectangle, cube),
 * transform (lookat, translate, scale, rotate, matrix). A parsed description
 * can be inspected without a GPU. */
typedef struct gr_scene_desc gr_scene_desc;

/* Parses an XML scene and the OBJ files it names. On GR_ERR_PARSE the
 * description still exists and gr_scene_desc_error tells why. */
gr_status gr_scene_desc_load_xml(const char* path, gr_scene_desc** out);
gr_status gr_scene_desc_destroy(gr_scene_desc* desc);
const char* gr_scene_desc_error(const gr_scene_desc* desc);
/* Features read approximately (one per line), e.g. a roughplastic bsdf. */
const char* gr_scene_desc_warnings(const gr_scene_desc* desc);
gr_status gr_scene_desc_info(const gr_scene_desc* desc, uint32_t* meshes, uint32_t* triangles, uint32_t* lights,
                             gr_camera* camera, gr_environment* env);
/* Flattened triangles (9 floats each, world space), the mesh of each triangle,
 * and one material per mesh. Any pointer may be NULL. */
gr_status gr_scene_desc_triangles(const gr_scene_desc* desc, float* h_verts, uint32_t* h_mesh, gr_material* h_mats);
/* Mesh i as parsed (world space): vertex and triangle counts, whether it has
 * per-vertex normals, and with non-NULL buffers its positions (3 floats per
 * vertex), normals (3 per vertex, when it has them) and indices (3 per
 * triangle). Its material is h_mats[i] of gr_scene_desc_triangles. */
gr_status gr_scene_desc_mesh(const gr_scene_desc* desc, uint32_t i, uint32_t* num_vertices, uint32_t* num_triangles,
                             int* has_normals, float* h_positions, float* h_normals, uint32_t* h_indices);
/* Mesh i's texture coordinates as parsed (2 floats per vertex of
 * gr_scene_desc_mesh), when it has them (Triangle::getTexcoords,
 * triangle.h:71-76: OBJ "vt", and the rectangle and cube shapes). */
gr_status gr_scene_desc_mesh_texcoords(const gr_scene_desc* desc, uint32_t i, int* has_texcoords,
                                       float* h_texcoords);
gr_status gr_scene_create_from_desc(gr_ctx* ctx, const gr_scene_desc* desc, gr_scene** out);
/* Parse + create: the drop-in for PathTracer(filename) (pathtracer.cu:8-11). */
gr_status gr_scene_load_xml(gr_ctx* ctx, const char* path, gr_scene** out);

/* ---- batched rendering (no counterpart in the reference) --------------------
 * Renders n jobs to completion with their samples packed into shared waves:
 * each wave's kernels cover every job in it (rays of all scenes share the
 * queues; each ray traverses its own scene's BVH). Job i adds opts[i].spp
 * samples to scenes[i]'s accumulation exactly as gr_render would, bit for bit:
 * a pixel's value does not depend on which jobs share its waves. A scene may
 * appear at most once. wave_paths = 0 picks the library default. */
gr_status gr_render_batch(gr_ctx* ctx, gr_scene* const* scenes, const gr_render_opts* opts, uint32_t n,
                          uint32_t wave_paths, gr_render_stats* stats);

/* ---- serving (no counterpart in the reference) --------------------------------
 * A render server with its own worker thread and stream. Submitted jobs wait
 * until they fit the device-memory budget (path pool + per-job accumulation +
 * the scenes they reference, each scene counted once while any job uses it),
 * then join the running waves at the next wave boundary (continuous
 * batching); finished jobs leave and free their budget. Scenes stay resident
 * as long as the caller keeps them. */
typedef struct gr_server gr_server;

typedef struct gr_server_opts {
    uint64_t budget_bytes; /* device-memory budget for admission (0 = no limit) */
    uint32_t wave_paths;   /* paths per wave (0 = 4 Mi) */
    uint32_t max_active;   /* jobs in flight at most (0 = 1024) */
    int32_t layout;        /* node layout of every job (GR_LAYOUT_*); set on the scenes at submit */
    int32_t block;         /* traversal threads per block (0 = 128; see gr_trace_tuning) */
    int32_t short_stack;   /* shared-memory stack entries per thread (0 = 12) */
    int32_t policy;        /* order in which jobs are admitted and packed into waves (GR_SERVER_*) */
    double age_cap_s;      /* GR_SERVER_SHORTEST_FIRST: a job submitted longer ago than this goes ahead of
                              shorter ones, oldest first (0 = no cap) */
    double max_wait_s;     /* load shedding: gr_server_submit refuses a job with GR_ERR_BUSY when the work
                              queued ahead of it plus its own, at the throughput measured so far, would take
                              longer than this (0 = accept everything) */
} gr_server_opts;

/* Job order of a server: first come first served, or the job with the least
 * remaining work (pixels x samples left) first, with the age cap above. */
#define GR_SERVER_FIFO 0
#define GR_SERVER_SHORTEST_FIRST 1

typedef struct gr_job_stats {
    double submit_s, admit_s, done_s; /* seconds on the server's clock */
    uint64_t samples;
    int32_t status;                   /* gr_status of the job */
    uint32_t waves;                   /* waves the job's samples ran in */
    uint64_t first_wave, last_wave;   /* the server's wave numbers (1, 2, ...) of its first and last wave */
} gr_job_stats;

typedef struct gr_server_stats {
    uint64_t submitted, admitted, completed, waves;
    uint64_t closest_rays, shadow_rays;
    uint64_t bytes_in_use, peak_bytes;
    double busy_s;      /* time with at least one job in flight */
    uint64_t rejected;  /* jobs refused with GR_ERR_BUSY */
} gr_server_stats;

gr_status gr_server_create(gr_ctx* ctx, const gr_server_opts* opts, gr_server** out);
/* Stops the worker after the jobs in flight finish; pending jobs are dropped. */
gr_status gr_server_destroy(gr_server* server);
/* Queues a job; returns at once with a ticket. The scene must outlive the job.
 * `camera` (may be NULL) overrides the scene's camera and resolution for this
 * job only, so one resident scene and BVH serve requests of any resolution.
 * The job's samples start at sample index 0. */
gr_status gr_server_submit(gr_server* server, gr_scene* scene, const gr_camera* camera, const gr_render_opts* opts,
                           uint64_t* ticket);
/* Waits up to timeout_s (< 0: forever) for a job; *done is 1 when finished.
 * When finished and h_rgb is not NULL, writes its mean radiance image
 * (width x height x 3 floats). A finished job is reported once: its ticket is
 * forgotten after the call that sees it done. */
gr_status gr_server_wait(gr_server* server, uint64_t ticket, double timeout_s, int* done, float* h_rgb,
                         gr_job_stats* stats);
/* gr_server_wait without waiting: *done tells whether the job has finished
 * (and then the image and stats are written as by gr_server_wait). */
gr_status gr_server_poll(gr_server* server, uint64_t ticket, int* done, float* h_rgb, gr_job_stats* stats);
/* Seconds on the server's clock (the clock of gr_job_stats). */
double gr_server_now(const gr_server* server);
gr_status gr_server_stats_get(gr_server* server, gr_server_stats* out);

/* Host-side fault injection for the render server (no counterpart in the
 * reference): the server's next `count` waves report a failed launch instead
 * of running (nothing reaches the GPU). Every job in flight then ends with
 * GR_ERR_CUDA, as after a real launch failure; later jobs run normally. This
 * exercises the server's error path: waiters and gr_server_destroy return. */
gr_status gr_diag_server_fail_waves(gr_server* server, uint32_t count);

#ifdef __cplusplus
}
#endif

#endif /* GR_H_ */
