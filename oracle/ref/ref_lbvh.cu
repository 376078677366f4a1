// Harness that runs the reference's own host LBVH (src/renderer/bvh.h:186-221)
// on a triangle soup, for pinning the oracle. Compiled by build_ref.sh against
// the reference sources where they lie; the output library goes to oracle/_ref/.
//
// bvh.h sorts with std::sort (unstable, :207). The harness pre-includes every
// header bvh.h depends on and then maps the token `sort` to `stable_sort` for
// bvh.h's own text only, so ties keep their original order and the result is
// comparable bit for bit with the oracle and the GPU build.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <iostream>
#include <sstream>
#include <vector>
#include <device_launch_parameters.h>
#include <thrust/device_ptr.h>
#include <thrust/reduce.h>
#include "renderer/aabb.h"
#include "renderer/triangle.h"
#define sort stable_sort
#include "renderer/bvh.h"
#undef sort

// texture.cpp is not compiled here; Material's TextureView members only need
// a default constructor to exist.
TextureView::TextureView() : m_width(0), m_height(0), m_buffer(nullptr) {}

// Builds the reference BVH over `n` triangles (9 floats each). Writes the
// reference nodes as 8 words each (box min.xyz, max.xyz, idx, leaf) into
// `nodes` (2n-1 entries) and the Morton code of every triangle (original
// order) into `codes`, computed with the reference's own EncodeMorton3.
extern "C" int ref_lbvh_build(const float* verts, uint32_t n, uint32_t* nodes, uint32_t* codes) {
    if (n == 0) return 0;
    std::vector<float3> p(3ull * n);
    std::vector<int3> idx(3ull * n);
    for (uint64_t i = 0; i < 3ull * n; ++i) {
        p[i] = make_float3(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
        idx[i] = make_int3((int)i, -1, -1);
    }
    TriangleMeshView view;
    view.m_triangle_num = n;
    view.m_p = p.data();
    view.m_index = idx.data();
    view.m_n = nullptr;
    view.m_uv = nullptr;
    std::vector<Triangle> tris(n);
    for (uint32_t j = 0; j < n; ++j) {
        tris[j].m_mesh = view;
        tris[j].m_index = 3 * j;
    }
    // LBVH_build prints progress on std::cout; keep the caller's stdout clean
    std::stringstream sink;
    std::streambuf* old = std::cout.rdbuf(sink.rdbuf());
    std::vector<BVHLinearNode> bvh = LBVH_build(tris);
    std::cout.rdbuf(old);
    for (size_t k = 0; k < bvh.size(); ++k) {
        uint32_t* w = nodes + 8 * k;
        std::memcpy(w, &bvh[k].m_box.m_min, 12);
        std::memcpy(w + 3, &bvh[k].m_box.m_max, 12);
        w[6] = bvh[k].m_tri_idx;
        w[7] = bvh[k].m_leaf;
    }
    if (codes) {
        // the same expression LBVH_build evaluates (bvh.h:193-204)
        AABB box;
        for (uint32_t i = 0; i < n; i++) box = Union(box, tris[i].worldBound().centroid());
        for (uint32_t i = 0; i < n; i++)
            codes[i] = EncodeMorton3((tris[i].worldBound().centroid() - box.m_min) / (box.m_max - box.m_min) * 1024);
    }
    return (int)bvh.size();
}
