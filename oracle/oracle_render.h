/*
 * CPU oracle for the wavefront integrator — TEST INFRASTRUCTURE ONLY (see
 * oracle.h). Restates, one path at a time, the integrator of
 * slongle/GPU-Renderer (pathtracer_kernel.h:59-117 camera rays, :488-628
 * shading with NEE + MIS, :642-749 light/BSDF accumulation and Russian
 * roulette; bsdf.h, the BSDF headers, sampling.h, triangle.h) with the product's
 * per-path PCG32 stream and per-path accumulation, so images can be compared
 * sample for sample.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Material record: same field order as the product's device material. */
typedef struct or_material {
    int32_t type; /* 0 diffuse, 1 smooth dielectric, 2 GGX conductor, 3 rough plastic */
    float color[3];
    float emission[3];
    float ax, ay;
    float eta_i[3], eta_t[3], k[3];
    float ior;
    uint32_t emissive;
    /* color texture: tex_w == 0 for the constant color, else texels
     * [tex_off, tex_off + tex_w * tex_h) of the texel pool, looked up nearest at
     * uv * (tus, tvs) + (tuo, tvo) */
    uint32_t tex_off, tex_w, tex_h;
    float tuo, tvo, tus, tvs;
    float spec[3]; /* rough plastic: specular lobe reflectance */
} or_material;

/* Latitude-longitude environment map (w == 0: the constant radiance). */
typedef struct or_envmap {
    const float* texels; /* 3 floats per texel, row 0 first */
    uint32_t w, h;
    float m[9];          /* world-to-map rotation, row-major */
    float c[3];          /* scene bounding-box centre */
} or_envmap;

typedef struct or_camera {
    float m[12];   /* row-major 3x4 camera-to-world */
    float fov_deg; /* horizontal field of view */
    uint32_t width, height;
} or_camera;

/* Renders `spp` samples per pixel starting at sample index `sample_base` and
 * adds each path's radiance to fb (3 doubles per pixel) in sample order.
 *   verts    9 floats per triangle;  normals 12 floats per triangle or NULL
 *   tri_mat  material index | 0x80000000 with normals | 0x40000000 with texcoords
 *   uvs      6 floats per triangle or NULL;  texels 3 floats per texel (material textures) or NULL
 *   envmap   NULL or a map that replaces the constant env radiance
 *   flags    1 = reference-compatibility quirks
 * Returns 0 on success. */
int or_render(const float* verts, const float* normals, const uint32_t* tri_mat, uint32_t ntri,
              const or_material* mats, uint32_t nmat, const or_camera* cam, const float* env, int has_env,
              uint32_t spp, uint32_t sample_base, uint32_t max_depth, uint64_t seed, int32_t rr_depth,
              uint32_t flags, double* fb, int threads, const float* uvs, const float* texels,
              const or_envmap* envmap);

#ifdef __cplusplus
}
#endif
