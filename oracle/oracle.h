/*
 * CPU oracle for the wavefront render path — TEST INFRASTRUCTURE ONLY.
 *
 * This library restates, on the host, the algorithms of slongle/GPU-Renderer's
 * render path so that the CUDA implementation can be checked against it:
 *   - LBVH build:        src/renderer/bvh.h:12-32 (Morton), :143-184 (split rule),
 *                        :121-141 (DFS flatten), :186-221 (driver)
 *   - reference traversal: src/renderer/pathtracer_kernel.h:119-173 (intersectors),
 *                        :175-308 (closest-hit / any-hit loops)
 *   - the product's own FP32 watertight traversal, restated independently for
 *     bit-exact hit-id parity.
 *   - the wavefront integrator (render.cpp).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this library, and only as the checker or the timed CPU baseline. The product
 * path (libgr.so) never links or calls it.
 *
 * Data formats (shared with include/gr.h):
 *   triangle soup : 9 floats per triangle (p0.xyz, p1.xyz, p2.xyz)
 *   ray           : 8 floats (o.xyz, d.xyz, tMin, tMax) — reference Ray layout
 *   hit           : 4 words (float t, int32 prim, float u, float v) — reference Hit
 *   ref node      : 8 words (box min.xyz, box max.xyz, idx, leaf) — BVHLinearNode
 *   bvh2 node     : 16 words, see or_lbvh_build
 *   sorted tri    : 12 floats (v0.xyz, prim bits, v1.xyz, 0, v2.xyz, 0)
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Morton codes exactly as bvh.h:193-204 computes them (centroid box, scale by
 * 1024, truncating float->uint conversion, 1024 clamped to 1023). */
void or_morton(const float* verts, uint32_t n, uint32_t* codes, float* centroid_box6);

/* Full LBVH restatement with a stable sort on the Morton code.
 *   sorted_prim/sorted_code : n entries each (the sorted MortonInfo array)
 *   ref_nodes               : 8 words x (2n-1) in the reference DFS-preorder layout
 *   bvh2_nodes              : 16 words x max(n-1,1), gap-indexed binary BVH with
 *                             child boxes stored in the parent (product layout)
 *   tri_sorted              : 12 floats x n, triangles in leaf order
 *   root                    : index of the root bvh2 node (0xFFFFFFFF if n == 0)
 * Any output pointer may be NULL. Returns 0 on success. */
int or_lbvh_build(const float* verts, uint32_t n, uint32_t* sorted_prim, uint32_t* sorted_code,
                  uint32_t* ref_nodes, uint32_t* bvh2_nodes, float* tri_sorted, uint32_t* root);

/* Product traversal restated (watertight FP32, near-first, (t, prim) tie rule).
 * stats (nullable): 2 words per ray (node visits, triangle tests). */
void or_trace(const uint32_t* bvh2_nodes, const float* tri_sorted, uint32_t root, const float* rays,
              uint64_t nrays, int any_hit, float* hits, uint32_t* stats, int threads);

/* 4-wide layouts restated: collapse (quant = 0: 32 words per node, FP32 boxes;
 * quant = 1: 16 words per node, 8-bit outward-quantised boxes) and traversal
 * in the product's child order. out holds max(n-1,1) nodes. */
void or_bvh4_build(const uint32_t* bvh2_nodes, uint32_t n, int quant, uint32_t* out);

/* 8-wide quantised layout (24 words per node) collapsed from the binary nodes
 * with the product's rules and numbering; returns the node count (copies at
 * most max_nodes nodes and max_tris node-order triangles, 12 floats each). */
uint32_t or_bvh8_build(const uint32_t* bvh2_nodes, const float* tri_sorted, uint32_t n, uint32_t root,
                       uint32_t* out_nodes, uint32_t max_nodes, float* out_tris, uint32_t max_tris, uint32_t* n_tris);
void or_trace8(const uint32_t* nodes8, const float* tris8, uint32_t root, const float* rays, uint64_t nrays,
               int any_hit, float* hits, uint32_t* stats, int threads);
void or_trace4(const uint32_t* nodes4, int quant, const float* tri_sorted, uint32_t root, const float* rays,
               uint64_t nrays, int any_hit, float* hits, uint32_t* stats, int threads);

/* Brute force over all triangles with the same watertight FP32 test and the
 * (t, prim) lexicographic rule. any_hit returns the lowest-index hit. */
void or_trace_brute(const float* verts, uint32_t n, const float* rays, uint64_t nrays, int any_hit,
                    float* hits, int threads);

/* Reference traversal restated: pathtracer_kernel.h:175-308 over the reference
 * layout with the mixed-precision Moller-Trumbore of :119-152.
 * stats (nullable): 2 words per ray (node visits, triangle tests). */
void or_trace_ref(const uint32_t* ref_nodes, const float* verts, uint32_t n, const float* rays,
                  uint64_t nrays, int any_hit, float* hits, uint32_t* stats, int threads);

/* FP64 distance oracle. For each ray: the FP64 distance to triangle prim[i]
 * (NaN if prim < 0), and an ambiguity flag that is 1 when another triangle is
 * hit within rel_gap of the closest distance, or the closest hit lies within
 * bary_margin (barycentric) or within edge_rel times the largest coordinate
 * magnitude (world units: FP32 rounding of the coordinates) of an edge.
 * Near misses within the same margins count as hits. */
void or_fp64_check(const uint32_t* ref_nodes, const float* verts, uint32_t n, const float* rays,
                   uint64_t nrays, const int32_t* prim, double* t64, uint8_t* ambiguous,
                   double rel_gap, double bary_margin, double edge_rel, int threads);

#ifdef __cplusplus
}
#endif
