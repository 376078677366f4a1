// Harness around the reference's own scene loading (built by build_ref.sh into
// oracle/_ref/libref_loader.so, here, where the reference sources are): runs
// Scene::Scene(filename) (src/renderer/scene.cpp:4-27) — load_scene /
// load_mitsuba_file / load_obj_file and the flattening of the meshes into
// m_cpu_triangles — and copies out what the loader produced, for pinning this
// library's own XML / OBJ loader against it:
//   per triangle (m_cpu_triangles order): the three positions
//     (Triangle::getVertices, triangle.h:87-93), the three shading normals and
//     texture coordinates when the mesh has them (hasNormal / hasTexcoords),
//     and the index of the mesh it came from;
//   per mesh: its material record (type, the texel of each constant texture,
//     texture sizes, emission);
//   the camera (cameraToWorld matrix, fov in radians, resolution) and the
//   environment light (constant radiance, or the size of its map).
// Nothing here changes the reference's arithmetic; its stdout is silenced.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <sstream>
#include <string>
#include <vector>
#include "renderer/scene.h"

namespace {

struct Loaded {
    std::unique_ptr<Scene> scene;
    std::vector<uint32_t> tri_mesh;
};

// First texel of a texture view and its size (constant textures are 1 x 1).
void texel(const TextureView& t, float* rgb, float* wh) {
    if (t.m_buffer && t.m_width && t.m_height) {
        rgb[0] = t.m_buffer[0].r;
        rgb[1] = t.m_buffer[0].g;
        rgb[2] = t.m_buffer[0].b;
    } else {
        rgb[0] = rgb[1] = rgb[2] = NAN;
    }
    wh[0] = (float)t.m_width;
    wh[1] = (float)t.m_height;
}

}  // namespace

extern "C" {

// Number of floats ref_materials writes per mesh.
int ref_material_floats(void) { return 48; }

// Loads `path` with the reference's Scene constructor. Returns the triangle
// count (>= 0) and the mesh count in *num_meshes, or -1.
int ref_load(const char* path, void** handle, uint32_t* num_meshes) {
    std::stringstream sink;
    std::streambuf* old = std::cout.rdbuf(sink.rdbuf());
    Loaded* L = new Loaded();
    L->scene.reset(new Scene(std::string(path)));
    std::cout.rdbuf(old);
    for (uint32_t i = 0; i < L->scene->m_meshes.size(); ++i)
        for (uint32_t j = 0; j < L->scene->m_meshes[i].m_triangle_num; ++j) L->tri_mesh.push_back(i);
    if (L->tri_mesh.size() != L->scene->m_cpu_triangles.size()) {
        delete L;
        return -1;
    }
    *handle = L;
    *num_meshes = (uint32_t)L->scene->m_meshes.size();
    return (int)L->scene->m_cpu_triangles.size();
}

// verts: 9 floats per triangle; normals: 9 (NaN without normals); uvs: 6 (NaN
// without texture coordinates); mesh: 1 word. Any pointer may be NULL.
void ref_triangles(void* handle, float* verts, float* normals, float* uvs, uint32_t* mesh) {
    Loaded* L = static_cast<Loaded*>(handle);
    const std::vector<Triangle>& tris = L->scene->m_cpu_triangles;
    for (size_t i = 0; i < tris.size(); ++i) {
        const Triangle& t = tris[i];
        float3 p[3];
        t.getVertices(p[0], p[1], p[2]);
        if (verts)
            for (int k = 0; k < 3; ++k) {
                verts[9 * i + 3 * k + 0] = p[k].x;
                verts[9 * i + 3 * k + 1] = p[k].y;
                verts[9 * i + 3 * k + 2] = p[k].z;
            }
        if (normals) {
            if (t.hasNormal()) {
                float3 n[3];
                t.getNormals(n[0], n[1], n[2]);
                for (int k = 0; k < 3; ++k) {
                    normals[9 * i + 3 * k + 0] = n[k].x;
                    normals[9 * i + 3 * k + 1] = n[k].y;
                    normals[9 * i + 3 * k + 2] = n[k].z;
                }
            } else {
                for (int k = 0; k < 9; ++k) normals[9 * i + k] = NAN;
            }
        }
        if (uvs) {
            if (t.hasTexcoords()) {
                float2 u[3];
                t.getTexcoords(u[0], u[1], u[2]);
                for (int k = 0; k < 3; ++k) {
                    uvs[6 * i + 2 * k + 0] = u[k].x;
                    uvs[6 * i + 2 * k + 1] = u[k].y;
                }
            } else {
                for (int k = 0; k < 6; ++k) uvs[6 * i + k] = NAN;
            }
        }
        if (mesh) mesh[i] = L->tri_mesh[i];
    }
}

// Per mesh, ref_material_floats() floats:
//   [0] type (MaterialType), [1..3] emission,
//   then for m_color, m_color1, m_etaI, m_etaT, m_k, m_ior, m_alpha_x,
//   m_alpha_y in that order: first texel rgb and width, height (5 each).
void ref_materials(void* handle, float* out) {
    Loaded* L = static_cast<Loaded*>(handle);
    const int nf = ref_material_floats();
    for (size_t i = 0; i < L->scene->m_meshes.size(); ++i) {
        const Material& m = L->scene->m_meshes[i].m_material;
        float* o = out + nf * i;
        for (int k = 0; k < nf; ++k) o[k] = 0.0f;
        o[0] = (float)m.m_type;
        o[1] = m.m_emission.r;
        o[2] = m.m_emission.g;
        o[3] = m.m_emission.b;
        const TextureView* tv[8] = {&m.m_color, &m.m_color1, &m.m_etaI, &m.m_etaT,
                                    &m.m_k,     &m.m_ior,    &m.m_alpha_x, &m.m_alpha_y};
        for (int k = 0; k < 8; ++k) texel(*tv[k], o + 4 + 5 * k, o + 7 + 5 * k);
    }
}

// cam: the 16 entries of cameraToWorld (row-major), fov (radians, as the
// camera stores it), width, height. env: has, first texel rgb, width, height.
void ref_camera_env(void* handle, float* cam, float* env) {
    Loaded* L = static_cast<Loaded*>(handle);
    const Camera& c = L->scene->m_camera;
    // Transform keeps its matrix (then its inverse) as private members; read
    // the object's bytes (a standard-layout class of two Matrix4x4)
    static_assert(sizeof(Transform) == 2 * sizeof(Matrix4x4), "Transform layout");
    float tm[32];
    std::memcpy(tm, &c.m_cameraToWorld, sizeof(tm));
    for (int k = 0; k < 16; ++k) cam[k] = tm[k];
    cam[16] = c.m_fov.x;
    cam[17] = (float)c.m_resolution_x;
    cam[18] = (float)c.m_resolution_y;
    const EnvironmentLight& e = L->scene->m_environment_light;
    env[0] = e.m_has ? 1.0f : 0.0f;
    if (e.m_has && !e.m_cpu_buffer.empty()) {
        env[1] = e.m_cpu_buffer[0].r;
        env[2] = e.m_cpu_buffer[0].g;
        env[3] = e.m_cpu_buffer[0].b;
    } else {
        env[1] = env[2] = env[3] = 0.0f;
    }
    env[4] = (float)(e.m_has ? e.m_width : 0);
    env[5] = (float)(e.m_has ? e.m_height : 0);
}

void ref_free(void* handle) { delete static_cast<Loaded*>(handle); }

}  // extern "C"
