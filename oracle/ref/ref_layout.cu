// Host probe run by build_ref.sh (here, where the reference sources are): prints
// as JSON the byte layout of the reference records that trace_kernel reads —
// SceneView (scene.h:15-30), Triangle and TriangleMeshView (triangle.h:10-60),
// Ray / Hit (ray.h) and BVHLinearNode (bvh.h:34-43) — so that ref_gpu.py can lay
// out the kernel's argument and triangle records without the reference headers.
// Host and device share these layouts, and so do x86-64 and AArch64 (LP64).
#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <device_launch_parameters.h>
#include "renderer/pathtracer_kernel.h"

TextureView::TextureView() : m_width(0), m_height(0), m_buffer(nullptr) {}

int main() {
    std::printf("{\"scene_view_size\": %zu, \"scene_view_align\": %zu, \"sv_triangles\": %zu, "
                "\"sv_triangles_num\": %zu, \"sv_bvh\": %zu, ",
                sizeof(SceneView), alignof(SceneView), offsetof(SceneView, m_triangles),
                offsetof(SceneView, m_triangles_num), offsetof(SceneView, m_bvh));
    std::printf("\"triangle_size\": %zu, \"tri_index\": %zu, \"tri_mesh\": %zu, \"mesh_triangle_num\": %zu, "
                "\"mesh_p\": %zu, \"mesh_n\": %zu, \"mesh_uv\": %zu, \"mesh_index\": %zu, ",
                sizeof(Triangle), offsetof(Triangle, m_index), offsetof(Triangle, m_mesh),
                offsetof(TriangleMeshView, m_triangle_num), offsetof(TriangleMeshView, m_p),
                offsetof(TriangleMeshView, m_n), offsetof(TriangleMeshView, m_uv), offsetof(TriangleMeshView, m_index));
    std::printf("\"ray_size\": %zu, \"hit_size\": %zu, \"hit_id\": %zu, \"node_size\": %zu}\n", sizeof(Ray),
                sizeof(Hit), offsetof(Hit, triangle_id), sizeof(BVHLinearNode));
    return 0;
}
