// Host probe run by build_ref.sh (here, where the reference sources are): prints
// as JSON the byte layout of the reference records its device kernels read —
// SceneView (scene.h:15-30), Camera (camera.h:7-132) and Transform
// (transform.h:87-148), Triangle / TriangleMeshView (triangle.h:10-60), Material
// (material.h:15-36), TextureView (texture.h:14-20), EnvironmentLightView
// (environment.h:10-35), FrameBufferView (framebuffer.h:8-35), RayQueue
// (rayqueue.h:6-17), PTContext (pathtracer_kernel.h:15-22), Ray / Hit (ray.h)
// and BVHLinearNode (bvh.h:34-43) — so that ref_gpu.py can lay out the
// kernels' argument and scene records without the reference headers. Host and
// device share these layouts, and so do x86-64 and AArch64 (LP64).
#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <device_launch_parameters.h>
#include "renderer/pathtracer_kernel.h"

TextureView::TextureView() : m_width(0), m_height(0), m_buffer(nullptr) {}

namespace {
bool first_field = true;
bool first_type = true;

void begin(const char* type, size_t size, size_t align) {
    std::printf("%s\n  \"%s\": {\"size\": %zu, \"align\": %zu", first_type ? "" : ",", type, size, align);
    first_type = false;
    first_field = false;
}
void field(const char* name, size_t off) { std::printf(", \"%s\": %zu", name, off); }
void end() { std::printf("}"); }
}  // namespace

#define TYPE(T) begin(#T, sizeof(T), alignof(T))
#define FIELD(T, f) field(#f, offsetof(T, f))

int main() {
    std::printf("{");
    TYPE(SceneView);
    FIELD(SceneView, m_camera); FIELD(SceneView, m_triangles); FIELD(SceneView, m_triangles_num);
    FIELD(SceneView, m_lights); FIELD(SceneView, m_lights_num); FIELD(SceneView, m_environment_light);
    FIELD(SceneView, m_bvh);
    end();
    TYPE(Camera);
    FIELD(Camera, m_eye); FIELD(Camera, m_dir); FIELD(Camera, m_up); FIELD(Camera, m_yaw); FIELD(Camera, m_pitch);
    FIELD(Camera, m_fov); FIELD(Camera, m_resolution_x); FIELD(Camera, m_resolution_y);
    FIELD(Camera, m_aspect_ratio); FIELD(Camera, m_rasterToCamera); FIELD(Camera, m_cameraToWorld);
    FIELD(Camera, m_free);
    end();
    {
        // Transform's matrices are private: locate them from a known matrix
        // (diag(2, 4, 8, 1) and its inverse) in the object's bytes.
        const Transform t(Matrix4x4(2, 0, 0, 0, 0, 4, 0, 0, 0, 0, 8, 0, 0, 0, 0, 1));
        float w[sizeof(Transform) / sizeof(float)];
        std::memcpy(w, &t, sizeof(Transform));
        const bool m_first = sizeof(Transform) == 2 * sizeof(Matrix4x4) && w[0] == 2.0f && w[5] == 4.0f &&
                             w[10] == 8.0f && w[16] == 0.5f && w[21] == 0.25f && w[26] == 0.125f;
        if (!m_first) {
            std::fprintf(stderr, "unexpected Transform layout\n");
            return 1;
        }
        TYPE(Transform);
        field("m", 0);
        field("mInv", sizeof(Matrix4x4));
        end();
    }
    TYPE(Matrix4x4);
    FIELD(Matrix4x4, m);
    end();
    TYPE(Triangle);
    FIELD(Triangle, m_mesh); FIELD(Triangle, m_index);
    end();
    TYPE(TriangleMeshView);
    FIELD(TriangleMeshView, m_triangle_num); FIELD(TriangleMeshView, m_p_num); FIELD(TriangleMeshView, m_n_num);
    FIELD(TriangleMeshView, m_uv_num); FIELD(TriangleMeshView, m_index_num); FIELD(TriangleMeshView, m_p);
    FIELD(TriangleMeshView, m_n); FIELD(TriangleMeshView, m_uv); FIELD(TriangleMeshView, m_index);
    FIELD(TriangleMeshView, m_material);
    end();
    TYPE(Material);
    FIELD(Material, m_emission); FIELD(Material, m_color); FIELD(Material, m_color1); FIELD(Material, m_etaI);
    FIELD(Material, m_etaT); FIELD(Material, m_k); FIELD(Material, m_ior); FIELD(Material, m_alpha_x);
    FIELD(Material, m_alpha_y); FIELD(Material, m_type);
    end();
    TYPE(TextureView);
    FIELD(TextureView, m_uvoffset); FIELD(TextureView, m_uvscale); FIELD(TextureView, m_width);
    FIELD(TextureView, m_height); FIELD(TextureView, m_buffer); FIELD(TextureView, m_type);
    end();
    TYPE(EnvironmentLightView);
    FIELD(EnvironmentLightView, m_has); FIELD(EnvironmentLightView, m_buffer); FIELD(EnvironmentLightView, m_width);
    FIELD(EnvironmentLightView, m_height); FIELD(EnvironmentLightView, m_o2w); FIELD(EnvironmentLightView, m_w2o);
    FIELD(EnvironmentLightView, m_world_center);
    end();
    TYPE(FrameBufferView);
    FIELD(FrameBufferView, m_resolution_x); FIELD(FrameBufferView, m_resolution_y);
    FIELD(FrameBufferView, m_buffer); FIELD(FrameBufferView, m_sample_num);
    end();
    TYPE(RayQueue);
    FIELD(RayQueue, m_rays); FIELD(RayQueue, m_hits); FIELD(RayQueue, m_weight); FIELD(RayQueue, m_pdf);
    FIELD(RayQueue, m_specular); FIELD(RayQueue, m_idx); FIELD(RayQueue, m_seed); FIELD(RayQueue, m_size);
    end();
    TYPE(PTContext);
    FIELD(PTContext, m_bounce); FIELD(PTContext, m_sample_num); FIELD(PTContext, m_in_queue);
    FIELD(PTContext, m_shadow_queue); FIELD(PTContext, m_scatter_queue);
    end();
    TYPE(Ray);
    FIELD(Ray, o); FIELD(Ray, d); FIELD(Ray, tMin); FIELD(Ray, tMax);
    end();
    TYPE(Hit);
    FIELD(Hit, t); FIELD(Hit, triangle_id); FIELD(Hit, u); FIELD(Hit, v);
    end();
    TYPE(BVHLinearNode);
    end();
    TYPE(Spectrum);
    end();
    std::printf(",\n  \"enums\": {\"MATERIAL_DIFFUSE\": %d, \"MATERIAL_SPECULAR\": %d, \"MATERIAL_ROUGH_CONDUCTOR\": %d, "
                "\"MATERIAL_ROUGH_DIELECTRIC\": %d, \"MATERIAL_ROUGH_PLASTIC\": %d, \"TEXTURE_SPECTRUM\": %d, "
                "\"TEXTURE_FLOAT\": %d}\n}\n",
                (int)MATERIAL_DIFFUSE, (int)MATERIAL_SPECULAR, (int)MATERIAL_ROUGH_CONDUCTOR,
                (int)MATERIAL_ROUGH_DIELECTRIC, (int)MATERIAL_ROUGH_PLASTIC, (int)TEXTURE_SPECTRUM,
                (int)TEXTURE_FLOAT);
    (void)first_field;
    return 0;
}
