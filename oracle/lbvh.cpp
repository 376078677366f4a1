// CPU oracle: LBVH build restated from slongle/GPU-Renderer src/renderer/bvh.h.
// Test infrastructure only (see oracle.h); never linked into the product.
//
// Compiled with -ffp-contract=off so every float operation rounds exactly as
// written, like the reference's host build (which runs on the CPU).
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>

namespace {

// helper_math.h host min/max used by AABB / Union (aabb.h:5-48)
inline float hmin(float a, float b) { return a < b ? a : b; }
inline float hmax(float a, float b) { return a > b ? a : b; }

struct Box {
    float lo[3], hi[3];
};

// Triangle::worldBound (triangle.h:95-101): Union(AABB(p0, p1), p2)
inline Box tri_box(const float* v) {
    Box b;
    for (int k = 0; k < 3; ++k) {
        b.lo[k] = hmin(hmin(v[k], v[3 + k]), v[6 + k]);
        b.hi[k] = hmax(hmax(v[k], v[3 + k]), v[6 + k]);
    }
    return b;
}

inline Box box_union(const Box& a, const Box& b) {
    Box r;
    for (int k = 0; k < 3; ++k) {
        r.lo[k] = hmin(a.lo[k], b.lo[k]);
        r.hi[k] = hmax(a.hi[k], b.hi[k]);
    }
    return r;
}

// The reference converts the scaled coordinate (a float in [0, 1024]) to
// uint32 by truncation (LeftShift3's implicit conversion, bvh.h:13,31).
// A NaN coordinate (a flat centroid box) converts to 0, as it does on the
// reference's x86 host build and on the GPU.
inline uint32_t to_cell(float v) {
    if (!(v >= 0.0f)) return 0u;
    uint32_t x = (uint32_t)v;
    if (x >= 1024u) x = 1023u;  // bvh.h:15 clamps exactly 1024 to 1023
    return x;
}

// Interleave: bit i of x goes to bit 3i (bit-by-bit loop, deliberately not the
// magic-constant form the GPU kernel uses, so the two cross-check each other).
inline uint32_t spread3(uint32_t x) {
    uint32_t r = 0;
    for (int i = 0; i < 10; ++i) r |= ((x >> i) & 1u) << (3 * i);
    return r;
}

void centroid_box(const float* verts, uint32_t n, Box& cb) {
    for (int k = 0; k < 3; ++k) {
        cb.lo[k] = std::numeric_limits<float>::infinity();
        cb.hi[k] = -std::numeric_limits<float>::infinity();
    }
    for (uint32_t i = 0; i < n; ++i) {
        Box b = tri_box(verts + 9ull * i);
        for (int k = 0; k < 3; ++k) {
            float c = (b.lo[k] + b.hi[k]) * 0.5f;  // AABB::centroid
            cb.lo[k] = hmin(cb.lo[k], c);
            cb.hi[k] = hmax(cb.hi[k], c);
        }
    }
}

uint32_t morton_of(const float* v, const Box& cb) {
    Box b = tri_box(v);
    uint32_t cell[3];
    for (int k = 0; k < 3; ++k) {
        float c = (b.lo[k] + b.hi[k]) * 0.5f;
        float q = (c - cb.lo[k]) / (cb.hi[k] - cb.lo[k]) * 1024.0f;  // bvh.h:203
        cell[k] = to_cell(q);
    }
    // EncodeMorton3 (bvh.h:28-32): z in the highest of each bit triple, x lowest
    return (spread3(cell[2]) << 2) | (spread3(cell[1]) << 1) | spread3(cell[0]);
}

struct Built {
    int32_t code;  // bvh2 child code: ~p for a leaf, gap index for an internal node
    uint32_t pre;  // DFS preorder index in the reference layout
    Box box;
};

struct Builder {
    const float* verts;
    const std::vector<uint32_t>& prim;
    const std::vector<uint32_t>& code;
    uint32_t* ref_nodes;
    uint32_t* bvh2;
    uint32_t counter = 0;

    Builder(const float* v, const std::vector<uint32_t>& p, const std::vector<uint32_t>& c, uint32_t* rn,
            uint32_t* b2)
        : verts(v), prim(p), code(c), ref_nodes(rn), bvh2(b2) {}

    void write_ref(uint32_t idx, const Box& b, uint32_t word, uint32_t leaf) {
        if (!ref_nodes) return;
        uint32_t* w = ref_nodes + 8ull * idx;
        std::memcpy(w + 0, b.lo, 12);
        std::memcpy(w + 3, b.hi, 12);
        w[6] = word;
        w[7] = leaf;
    }

    // recursive_build (bvh.h:143-184) fused with flatten_nodes (:121-141):
    // preorder numbering is assigned on entry, left subtree first.
    Built build(uint32_t l, uint32_t r) {
        Built out;
        out.pre = counter++;
        if (l + 1 == r) {
            out.box = tri_box(verts + 9ull * prim[l]);
            out.code = ~(int32_t)l;
            write_ref(out.pre, out.box, prim[l], 1);
            return out;
        }
        uint32_t split = l;
        if (code[l] == code[r - 1]) {
            split = ((l + r) >> 1) - 1;  // equal-code run: midpoint split (bvh.h:162-165)
        } else {
            // first adjacent pair with the largest xor (bvh.h:168-175)
            for (uint32_t i = l; i + 1 < r; ++i) {
                uint32_t now = code[i] ^ code[i + 1];
                uint32_t best = code[split] ^ code[split + 1];
                if (now > best) split = i;
            }
        }
        Built a = build(l, split + 1);
        Built b = build(split + 1, r);
        out.box = box_union(a.box, b.box);
        out.code = (int32_t)split;
        write_ref(out.pre, out.box, b.pre, 0);
        if (bvh2) {
            uint32_t* w = bvh2 + 16ull * split;
            float* f = reinterpret_cast<float*>(w);
            f[0] = a.box.lo[0]; f[1] = a.box.hi[0]; f[2] = a.box.lo[1]; f[3] = a.box.hi[1];
            f[4] = b.box.lo[0]; f[5] = b.box.hi[0]; f[6] = b.box.lo[1]; f[7] = b.box.hi[1];
            f[8] = a.box.lo[2]; f[9] = a.box.hi[2]; f[10] = b.box.lo[2]; f[11] = b.box.hi[2];
            w[12] = (uint32_t)a.code;
            w[13] = (uint32_t)b.code;
            if (a.code >= 0) bvh2[16ull * a.code + 14] = split;
            if (b.code >= 0) bvh2[16ull * b.code + 14] = split;
        }
        return out;
    }
};

}  // namespace

extern "C" void or_morton(const float* verts, uint32_t n, uint32_t* codes, float* cbox6) {
    Box cb;
    centroid_box(verts, n, cb);
    for (uint32_t i = 0; i < n; ++i) codes[i] = morton_of(verts + 9ull * i, cb);
    if (cbox6) {
        std::memcpy(cbox6, cb.lo, 12);
        std::memcpy(cbox6 + 3, cb.hi, 12);
    }
}

extern "C" int or_lbvh_build(const float* verts, uint32_t n, uint32_t* sorted_prim, uint32_t* sorted_code,
                             uint32_t* ref_nodes, uint32_t* bvh2_nodes, float* tri_sorted, uint32_t* root) {
    if (n == 0) {
        if (root) *root = 0xFFFFFFFFu;
        return 0;
    }
    Box cb;
    centroid_box(verts, n, cb);
    std::vector<uint32_t> code(n), prim(n);
    for (uint32_t i = 0; i < n; ++i) code[i] = morton_of(verts + 9ull * i, cb);
    std::iota(prim.begin(), prim.end(), 0u);
    // bvh.h:207 sorts with an unstable std::sort; the oracle fixes ties by
    // original index (a stable sort), which the GPU radix sort also yields.
    std::stable_sort(prim.begin(), prim.end(), [&](uint32_t a, uint32_t b) { return code[a] < code[b]; });
    std::vector<uint32_t> scode(n);
    for (uint32_t i = 0; i < n; ++i) scode[i] = code[prim[i]];
    if (sorted_prim) std::memcpy(sorted_prim, prim.data(), 4ull * n);
    if (sorted_code) std::memcpy(sorted_code, scode.data(), 4ull * n);

    if (bvh2_nodes) std::memset(bvh2_nodes, 0, 64ull * (n > 1 ? n - 1 : 1));
    Builder b(verts, prim, scode, ref_nodes, bvh2_nodes);
    Built top = b.build(0, n);
    if (n == 1) {
        // a lone leaf: the product layout still needs one internal node; both
        // children name the same triangle (testing it twice changes nothing)
        if (bvh2_nodes) {
            float* f = reinterpret_cast<float*>(bvh2_nodes);
            const Box& x = top.box;
            f[0] = x.lo[0]; f[1] = x.hi[0]; f[2] = x.lo[1]; f[3] = x.hi[1];
            f[4] = x.lo[0]; f[5] = x.hi[0]; f[6] = x.lo[1]; f[7] = x.hi[1];
            f[8] = x.lo[2]; f[9] = x.hi[2]; f[10] = x.lo[2]; f[11] = x.hi[2];
            bvh2_nodes[12] = bvh2_nodes[13] = (uint32_t)~0;
        }
        if (root) *root = 0;
    } else {
        if (root) *root = (uint32_t)top.code;
    }
    if (bvh2_nodes && n > 1) bvh2_nodes[16ull * top.code + 14] = 0xFFFFFFFFu;
    if (bvh2_nodes && n == 1) bvh2_nodes[14] = 0xFFFFFFFFu;
    if (tri_sorted) {
        for (uint32_t p = 0; p < n; ++p) {
            const float* v = verts + 9ull * prim[p];
            float* o = tri_sorted + 12ull * p;
            o[0] = v[0]; o[1] = v[1]; o[2] = v[2];
            std::memcpy(o + 3, &prim[p], 4);
            o[4] = v[3]; o[5] = v[4]; o[6] = v[5]; o[7] = 0.0f;
            o[8] = v[6]; o[9] = v[7]; o[10] = v[8]; o[11] = 0.0f;
        }
    }
    return 0;
}
