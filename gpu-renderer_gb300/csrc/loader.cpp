// Scene loading: the Mitsuba-XML subset and Wavefront OBJ files the reference
// reads (slongle/GPU-Renderer src/renderer/loaders/mitsubaloader.cpp,
// objloader.cpp), written from scratch (no XML or OBJ library).
//
// Interpretation follows the reference's loader:
//   - children are handled before their parent (ParseTag/HandleTag,
//     mitsubaloader.cpp:600-805), so a shape's <bsdf> and <emitter> children set
//     the "current" material and light before the shape is created;
//   - the current material is not reset between shapes; the current light is
//     (createShape, :481-522);
//   - <transform> starts from identity and each child multiplies on the right
//     (m_transform *= X);
//   - material types, parameter names and defaults as in createMaterial
//     (:289-441), including its quirks: "dielectric"/"roughdielectric" take the
//     index from the "ior" property only (intIOR/extIOR are read but not used),
//     and a rough conductor's alphaV is taken from "alphaU";
//   - shapes: obj, sphere (lat-long, subdiv), rectangle, cube (:53-221).
//   - textures: "checkerboard" (color0 / color1, the reference's 2 x 2 map) and
//     "bitmap", with uoffset / voffset / uscale / vscale (createTexture,
//     :530-555); OBJ texture coordinates ("vt"); "envmap" emitters with their
//     toWorld (:472-478). Float images are read as stb_image's stbi_loadf with
//     vertical flip does for the reference (ReadImage, imageio.cpp:45-57): an
//     8-bit channel c becomes (c / 255)^2.2 and row 0 is the image's bottom row.
// Differences: only binary PPM (P6, 8-bit) and PFM images are read (another
// image format leaves a texture at its 0.5 grey, an envmap skipped; recorded
// as a warning); only the colour slots (reflectance, specularReflectance,
// diffuseReflectance) take textures.
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <fstream>
#include <map>
#include <memory>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "gr_internal.h"

namespace {

// ---- minimal XML ----------------------------------------------------------------
struct XNode {
    std::string name;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<std::unique_ptr<XNode>> kids;
    size_t line = 0;
    const char* attr(const char* k) const {
        for (auto& a : attrs)
            if (a.first == k) return a.second.c_str();
        return nullptr;
    }
};

struct XmlParser {
    const std::string& s;
    size_t i = 0;
    std::string err;
    explicit XmlParser(const std::string& src) : s(src) {}
    size_t line_at(size_t pos) const {
        size_t l = 1;
        for (size_t k = 0; k < pos && k < s.size(); ++k) l += s[k] == '\n';
        return l;
    }
    void ws() {
        while (i < s.size() && isspace((unsigned char)s[i])) ++i;
    }
    bool starts(const char* p) const { return s.compare(i, strlen(p), p) == 0; }
    bool fail(const std::string& m) {
        if (err.empty()) err = m + " (line " + std::to_string(line_at(i)) + ")";
        return false;
    }
    // skips comments, declarations, processing instructions and text
    void skip_misc() {
        for (;;) {
            ws();
            if (starts("<!--")) {
                const size_t e = s.find("-->", i + 4);
                i = e == std::string::npos ? s.size() : e + 3;
            } else if (starts("<?")) {
                const size_t e = s.find("?>", i + 2);
                i = e == std::string::npos ? s.size() : e + 2;
            } else if (starts("<!")) {
                const size_t e = s.find('>', i + 2);
                i = e == std::string::npos ? s.size() : e + 1;
            } else if (i < s.size() && s[i] != '<') {
                while (i < s.size() && s[i] != '<') ++i;  // character data (ignored)
            } else {
                return;
            }
        }
    }
    std::string name() {
        const size_t b = i;
        while (i < s.size() && (isalnum((unsigned char)s[i]) || s[i] == '_' || s[i] == '-' || s[i] == ':' || s[i] == '.'))
            ++i;
        return s.substr(b, i - b);
    }
    bool element(std::unique_ptr<XNode>& out) {
        if (i >= s.size() || s[i] != '<') return fail("expected '<'");
        out.reset(new XNode());
        out->line = line_at(i);
        ++i;
        out->name = name();
        if (out->name.empty()) return fail("empty element name");
        for (;;) {
            ws();
            if (i >= s.size()) return fail("unterminated element <" + out->name + ">");
            if (starts("/>")) {
                i += 2;
                return true;
            }
            if (s[i] == '>') {
                ++i;
                break;
            }
            std::string k = name();
            if (k.empty()) return fail("bad attribute in <" + out->name + ">");
            ws();
            if (i >= s.size() || s[i] != '=') return fail("expected '=' after attribute " + k);
            ++i;
            ws();
            if (i >= s.size() || (s[i] != '"' && s[i] != '\'')) return fail("expected quoted value for " + k);
            const char q = s[i++];
            const size_t e = s.find(q, i);
            if (e == std::string::npos) return fail("unterminated attribute value");
            out->attrs.emplace_back(k, s.substr(i, e - i));
            i = e + 1;
        }
        for (;;) {
            skip_misc();
            if (i >= s.size()) return fail("missing </" + out->name + ">");
            if (starts("</")) {
                i += 2;
                const std::string n = name();
                ws();
                if (n != out->name || i >= s.size() || s[i] != '>')
                    return fail("mismatched </" + n + "> for <" + out->name + ">");
                ++i;
                return true;
            }
            std::unique_ptr<XNode> kid;
            if (!element(kid)) return false;
            out->kids.push_back(std::move(kid));
        }
    }
    bool document(std::unique_ptr<XNode>& root) {
        skip_misc();
        if (!element(root)) return false;
        skip_misc();
        return true;
    }
};

// ---- small math -------------------------------------------------------------------------
struct F3 {
    float x, y, z;
};
F3 f3(float x, float y, float z) { return {x, y, z}; }
F3 operator-(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
F3 cross(F3 a, F3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
F3 normalize(F3 v) {
    const float l = 1.0f / std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
    return {v.x * l, v.y * l, v.z * l};
}

struct M4 {
    float m[4][4];
    static M4 identity() {
        M4 r{};
        for (int k = 0; k < 4; ++k) r.m[k][k] = 1.0f;
        return r;
    }
    M4 operator*(const M4& b) const {
        M4 r{};
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j)
                r.m[i][j] = m[i][0] * b.m[0][j] + m[i][1] * b.m[1][j] + m[i][2] * b.m[2][j] + m[i][3] * b.m[3][j];
        return r;
    }
};

// 4x4 inverse by Gauss-Jordan elimination with full pivoting in FP32, in the
// operation order of the Numerical Recipes / pbrt routine the reference uses
// (transform.cpp:30-90), so inverses (and the normals transformed by them) are
// the same floats. False for a singular matrix.
bool invert(const M4& a, M4& out) {
    int indxc[4], indxr[4];
    int ipiv[4] = {0, 0, 0, 0};
    float minv[4][4];
    std::memcpy(minv, a.m, sizeof(minv));
    for (int i = 0; i < 4; ++i) {
        int irow = 0, icol = 0;
        float big = 0.0f;
        for (int j = 0; j < 4; ++j) {
            if (ipiv[j] == 1) continue;
            for (int k = 0; k < 4; ++k) {
                if (ipiv[k] == 0) {
                    if (std::fabs(minv[j][k]) >= big) {
                        big = std::fabs(minv[j][k]);
                        irow = j;
                        icol = k;
                    }
                } else if (ipiv[k] > 1) {
                    return false;
                }
            }
        }
        ++ipiv[icol];
        if (irow != icol)
            for (int k = 0; k < 4; ++k) std::swap(minv[irow][k], minv[icol][k]);
        indxr[i] = irow;
        indxc[i] = icol;
        if (minv[icol][icol] == 0.0f) return false;
        const float pivinv = 1.0f / minv[icol][icol];
        minv[icol][icol] = 1.0f;
        for (int j = 0; j < 4; ++j) minv[icol][j] *= pivinv;
        for (int j = 0; j < 4; ++j) {
            if (j == icol) continue;
            const float save = minv[j][icol];
            minv[j][icol] = 0.0f;
            for (int k = 0; k < 4; ++k) minv[j][k] -= minv[icol][k] * save;
        }
    }
    for (int j = 3; j >= 0; --j)
        if (indxr[j] != indxc[j])
            for (int k = 0; k < 4; ++k) std::swap(minv[k][indxr[j]], minv[k][indxc[j]]);
    std::memcpy(out.m, minv, sizeof(minv));
    return true;
}

M4 transpose(const M4& a) {
    M4 r;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) r.m[i][j] = a.m[j][i];
    return r;
}

// A transform and its inverse, composed as the reference's Transform is
// (transform.h:89-113): (A * B).inv = B.inv * A.inv, each elementary transform
// carrying its own exact or computed inverse, so a normal is mapped by the same
// inverse matrix the reference maps it by.
struct XF {
    M4 m = M4::identity(), inv = M4::identity();
};
XF compose(const XF& a, const XF& b) { return {a.m * b.m, b.inv * a.inv}; }

float deg2rad(float d) { return d / 180.0f * 3.14159265358979323846f; }

XF translate(F3 d) {
    XF r;
    r.m.m[0][3] = d.x; r.m.m[1][3] = d.y; r.m.m[2][3] = d.z;
    r.inv.m[0][3] = -d.x; r.inv.m[1][3] = -d.y; r.inv.m[2][3] = -d.z;
    return r;
}
XF scale(F3 s) {
    XF r;
    r.m.m[0][0] = s.x; r.m.m[1][1] = s.y; r.m.m[2][2] = s.z;
    // reciprocals taken in double and rounded to float, as the reference's do
    r.inv.m[0][0] = (float)(1.0 / (double)s.x);
    r.inv.m[1][1] = (float)(1.0 / (double)s.y);
    r.inv.m[2][2] = (float)(1.0 / (double)s.z);
    return r;
}
XF rotate(float deg, F3 axis) {  // rotation about an axis (Rodrigues); its inverse is the transpose
    const F3 a = normalize(axis);
    const float s = std::sin(deg2rad(deg)), c = std::cos(deg2rad(deg));
    XF r;
    r.m.m[0][0] = a.x * a.x + (1 - a.x * a.x) * c;
    r.m.m[0][1] = a.x * a.y * (1 - c) - a.z * s;
    r.m.m[0][2] = a.x * a.z * (1 - c) + a.y * s;
    r.m.m[1][0] = a.x * a.y * (1 - c) + a.z * s;
    r.m.m[1][1] = a.y * a.y + (1 - a.y * a.y) * c;
    r.m.m[1][2] = a.y * a.z * (1 - c) - a.x * s;
    r.m.m[2][0] = a.x * a.z * (1 - c) - a.y * s;
    r.m.m[2][1] = a.y * a.z * (1 - c) + a.x * s;
    r.m.m[2][2] = a.z * a.z + (1 - a.z * a.z) * c;
    r.inv = transpose(r.m);
    return r;
}
// camera-to-world with columns (left, up, forward, origin) (transform.cpp:220-249)
bool look_at(F3 target, F3 origin, F3 up, XF& out) {
    const F3 f = normalize(target - origin);
    const F3 l = normalize(cross(up, f));
    const F3 u = cross(f, l);
    M4 r = M4::identity();
    r.m[0][0] = l.x; r.m[1][0] = l.y; r.m[2][0] = l.z;
    r.m[0][1] = u.x; r.m[1][1] = u.y; r.m[2][1] = u.z;
    r.m[0][2] = f.x; r.m[1][2] = f.y; r.m[2][2] = f.z;
    r.m[0][3] = origin.x; r.m[1][3] = origin.y; r.m[2][3] = origin.z;
    out.m = r;
    return invert(r, out.inv);
}

bool parse_floats(const char* s, float* out, int n) {
    if (!s) return false;
    const char* p = s;
    for (int k = 0; k < n; ++k) {
        while (*p && (isspace((unsigned char)*p) || *p == ',')) ++p;
        char* e = nullptr;
        out[k] = strtof(p, &e);
        if (e == p) return false;
        p = e;
    }
    return true;
}

// ---- property values ---------------------------------------------------------------------
struct Prop {
    enum Kind { Bool, Int, Float, String, Vector, Color, Transform, Texture } kind = Float;
    bool b = false;
    int i = 0;
    float f = 0.0f;
    std::string s;
    F3 v{0, 0, 0};
    M4 t = M4::identity(), tinv = M4::identity();  // transform and its inverse
    // texture: map index into the description's maps (-1: constant v), size, uv offset and scale
    int tex = -1;
    uint32_t tw = 0, th = 0;
    float uo = 0.0f, vo = 0.0f, us = 1.0f, vs = 1.0f;
};
using Props = std::map<std::string, Prop>;

float get_float(const Props& p, const char* k, float def) {
    auto it = p.find(k);
    if (it == p.end()) return def;
    if (it->second.kind == Prop::Float) return it->second.f;
    if (it->second.kind == Prop::Int) return (float)it->second.i;
    if (it->second.kind == Prop::Texture || it->second.kind == Prop::Color) return it->second.v.x;
    return def;
}
int get_int(const Props& p, const char* k, int def) {
    auto it = p.find(k);
    return it != p.end() && it->second.kind == Prop::Int ? it->second.i : def;
}
F3 get_color(const Props& p, const char* k, F3 def) {
    auto it = p.find(k);
    if (it == p.end()) return def;
    if (it->second.kind == Prop::Color || it->second.kind == Prop::Texture) return it->second.v;
    if (it->second.kind == Prop::Float) return f3(it->second.f, it->second.f, it->second.f);
    return def;
}
bool has(const Props& p, const char* k, Prop::Kind kind) {
    auto it = p.find(k);
    return it != p.end() && it->second.kind == kind;
}

struct Mat {
    gr_material m{};
};

struct MeshData {
    std::vector<float> pos, nrm, uv;
    std::vector<uint32_t> idx;
    bool has_normals = false, has_uvs = false;
};

}  // namespace

// A parsed scene, ready for gr_scene_create.
struct gr_scene_desc {
    std::vector<MeshData> meshes;
    std::vector<uint32_t> mesh_mat;
    std::vector<gr_material> mats;
    std::deque<std::vector<float>> maps;  // texture and environment texels (stable addresses)
    gr_camera cam{};
    gr_environment env{};
    std::string warnings;
    std::string error;
};

namespace {

// ---- OBJ (objloader.cpp:12-121) -------------------------------------------------------------
bool load_obj(const std::string& path, MeshData& out, std::string& err) {
    std::ifstream f(path);
    if (!f) {
        err = "cannot open " + path;
        return false;
    }
    std::vector<float> P, N, T;
    std::map<std::pair<std::pair<int, int>, int>, uint32_t> remap;  // ((position, texcoord), normal) -> vertex
    std::string line;
    size_t ln = 0;
    auto resolve = [](int i, size_t n) -> int {
        if (i > 0) return i - 1;
        if (i < 0) return (int)n + i;
        return -1;
    };
    while (std::getline(f, line)) {
        ++ln;
        const char* s = line.c_str();
        while (*s == ' ' || *s == '\t') ++s;
        if (s[0] == 'v' && (s[1] == ' ' || s[1] == '\t')) {
            float v[3];
            if (!parse_floats(s + 2, v, 3)) { err = path + ": bad vertex at line " + std::to_string(ln); return false; }
            P.insert(P.end(), v, v + 3);
        } else if (s[0] == 'v' && s[1] == 't') {
            float v[2];
            if (!parse_floats(s + 3, v, 2)) { err = path + ": bad texcoord at line " + std::to_string(ln); return false; }
            T.insert(T.end(), v, v + 2);
        } else if (s[0] == 'v' && s[1] == 'n') {
            float v[3];
            if (!parse_floats(s + 3, v, 3)) { err = path + ": bad normal at line " + std::to_string(ln); return false; }
            N.insert(N.end(), v, v + 3);
        } else if (s[0] == 'f' && (s[1] == ' ' || s[1] == '\t')) {
            std::istringstream is(s + 2);
            std::string tok;
            std::vector<uint32_t> face;
            while (is >> tok) {
                int vi = 0, ti = 0, ni = 0;
                const char* t = tok.c_str();
                vi = (int)strtol(t, (char**)&t, 10);
                if (*t == '/') {
                    ++t;
                    if (*t != '/') ti = (int)strtol(t, (char**)&t, 10);
                    if (*t == '/') {
                        ++t;
                        ni = (int)strtol(t, (char**)&t, 10);
                    }
                }
                const int p = resolve(vi, P.size() / 3);
                const int n = ni ? resolve(ni, N.size() / 3) : -1;
                const int tc = ti ? resolve(ti, T.size() / 2) : -1;
                if (p < 0 || (size_t)p >= P.size() / 3 || (ni && (n < 0 || (size_t)n >= N.size() / 3)) ||
                    (ti && (tc < 0 || (size_t)tc >= T.size() / 2))) {
                    err = path + ": face index out of range at line " + std::to_string(ln);
                    return false;
                }
                const auto key = std::make_pair(std::make_pair(p, tc), n);
                auto it = remap.find(key);
                uint32_t v;
                if (it == remap.end()) {
                    v = (uint32_t)(out.pos.size() / 3);
                    out.pos.insert(out.pos.end(), P.begin() + 3 * p, P.begin() + 3 * p + 3);
                    if (n >= 0) {
                        out.nrm.insert(out.nrm.end(), N.begin() + 3 * n, N.begin() + 3 * n + 3);
                        out.has_normals = true;
                    } else {
                        out.nrm.insert(out.nrm.end(), {0.0f, 0.0f, 0.0f});
                    }
                    if (tc >= 0) {
                        out.uv.insert(out.uv.end(), T.begin() + 2 * tc, T.begin() + 2 * tc + 2);
                        out.has_uvs = true;
                    } else {
                        out.uv.insert(out.uv.end(), {0.0f, 0.0f});
                    }
                    remap.emplace(key, v);
                } else {
                    v = it->second;
                }
                face.push_back(v);
            }
            if (face.size() < 3) {
                err = path + ": face with fewer than 3 vertices at line " + std::to_string(ln);
                return false;
            }
            for (size_t k = 1; k + 1 < face.size(); ++k) {  // fan (the reference accepts triangles only)
                out.idx.push_back(face[0]);
                out.idx.push_back(face[k]);
                out.idx.push_back(face[k + 1]);
            }
        }
    }
    if (out.has_normals) {
        // vertices without a normal in a mesh that has normals keep a zero normal; the
        // reference would index garbage there, a zero normal normalises to NaN, so drop them
        for (size_t v = 0; v < out.nrm.size() / 3; ++v)
            if (out.nrm[3 * v] == 0 && out.nrm[3 * v + 1] == 0 && out.nrm[3 * v + 2] == 0) {
                out.has_normals = false;
                break;
            }
    }
    return true;
}

// ---- procedural shapes (mitsubaloader.cpp:53-221) --------------------------------------------
void make_rectangle(MeshData& m) {
    // the unit square in z = 0 with texture coordinates at its corners and the
    // +z normal; triangles (0, 1, 2) and (2, 3, 0) (mitsubaloader.cpp:119-151)
    const float p[] = {-1, -1, 0, 1, -1, 0, 1, 1, 0, -1, 1, 0};
    m.pos.assign(p, p + 12);
    m.nrm = {0, 0, 1, 0, 0, 1, 0, 0, 1, 0, 0, 1};
    m.uv = {0, 0, 1, 0, 1, 1, 0, 1};
    m.has_normals = true;
    m.has_uvs = true;
    m.idx = {0, 1, 2, 2, 3, 0};
}

void make_cube(MeshData& m) {
    // [-1, 1]^3 as the reference builds it (mitsubaloader.cpp:53-116): eight
    // corners, six face normals and fourteen texture coordinates, each face a
    // quad of (corner, texcoord, normal) triples split into (q0, q1, q2) and
    // (q0, q2, q3). The triangle order (and so every hit's primitive id) and
    // the corner order within each triangle are the reference's. A vertex here
    // is one distinct triple, numbered in order of first use.
    static const float corner[8][3] = {{1, 1, -1}, {1, -1, -1}, {1, 1, 1},   {1, -1, 1},
                                       {-1, 1, -1}, {-1, -1, -1}, {-1, 1, 1}, {-1, -1, 1}};
    static const float normal[6][3] = {{0, 1, 0}, {0, 0, 1}, {-1, 0, 0}, {0, -1, 0}, {1, 0, 0}, {0, 0, -1}};
    static const float tex[14][2] = {{0.625f, 0.5f},  {0.875f, 0.5f},  {0.875f, 0.75f}, {0.625f, 0.75f},
                                     {0.375f, 0.75f}, {0.625f, 1.0f},  {0.375f, 1.0f},  {0.375f, 0.0f},
                                     {0.625f, 0.0f},  {0.625f, 0.25f}, {0.375f, 0.25f}, {0.125f, 0.5f},
                                     {0.375f, 0.5f},  {0.125f, 0.75f}};
    // per face: the quad's four (corner, texcoord) pairs; the face's normal is its index
    static const int quad[6][4][2] = {{{0, 0}, {4, 1}, {6, 2}, {2, 3}},   {{3, 4}, {2, 3}, {6, 5}, {7, 6}},
                                      {{7, 7}, {6, 8}, {4, 9}, {5, 10}},  {{5, 11}, {1, 12}, {3, 4}, {7, 13}},
                                      {{1, 12}, {0, 0}, {2, 3}, {3, 4}},  {{5, 10}, {4, 9}, {0, 0}, {1, 12}}};
    std::map<std::array<int, 3>, uint32_t> vertex_of;
    auto vertex = [&](int c, int t, int n) {
        const std::array<int, 3> key{c, t, n};
        auto it = vertex_of.find(key);
        if (it != vertex_of.end()) return it->second;
        const uint32_t v = (uint32_t)vertex_of.size();
        vertex_of.emplace(key, v);
        m.pos.insert(m.pos.end(), {corner[c][0], corner[c][1], corner[c][2]});
        m.nrm.insert(m.nrm.end(), {normal[n][0], normal[n][1], normal[n][2]});
        m.uv.insert(m.uv.end(), {tex[t][0], tex[t][1]});
        return v;
    };
    for (int f = 0; f < 6; ++f) {
        uint32_t q[4];
        for (int k = 0; k < 4; ++k) q[k] = vertex(quad[f][k][0], quad[f][k][1], f);
        m.idx.insert(m.idx.end(), {q[0], q[1], q[2], q[0], q[2], q[3]});
    }
    m.has_normals = true;
    m.has_uvs = true;
}

void make_sphere(MeshData& m, float radius, int subdiv) {
    const int nlat = subdiv, nlon = 2 * subdiv;
    const float dlat = 3.14159265358979323846f / nlat, dlon = 2 * 3.14159265358979323846f / nlon;
    auto push = [&](float x, float y, float z) {
        m.pos.insert(m.pos.end(), {x * radius, y * radius, z * radius});
        m.nrm.insert(m.nrm.end(), {x, y, z});
    };
    push(0, 0, 1);
    for (int i = 1; i < nlat; ++i) {
        const float th = i * dlat;
        for (int j = 0; j < nlon; ++j) {
            const float ph = j * dlon;
            push(std::sin(th) * std::cos(ph), std::sin(th) * std::sin(ph), std::cos(th));
        }
    }
    push(0, 0, -1);
    for (int i = 0; i < nlon; ++i) {
        const uint32_t a = i + 1, b = (i == nlon - 1) ? 1 : a + 1;
        m.idx.insert(m.idx.end(), {a, b, 0});
    }
    for (int i = 2; i < nlat; ++i)
        for (int j = 0; j < nlon; ++j) {
            uint32_t a = (i - 1) * nlon + j + 1, b = a + 1, c = a - nlon, d = c + 1;
            if (j == nlon - 1) {
                b = (i - 1) * nlon + 1;
                d = b - nlon;
            }
            m.idx.insert(m.idx.end(), {a, b, c, c, b, d});
        }
    const uint32_t bottom = nlon * (nlat - 1) + 1;
    for (int i = 0; i < nlon; ++i) {
        const uint32_t a = (nlat - 2) * nlon + i + 1, b = (i == nlon - 1) ? (nlat - 2) * nlon + 1 : a + 1;
        m.idx.insert(m.idx.end(), {a, bottom, b});
    }
    m.has_normals = true;
}

// ---- float images (ReadImage, imageio.cpp:45-57) -------------------------------------------------
// Binary PPM (P6, maxval <= 255: each channel (c / maxval)^2.2, as stbi_loadf
// linearises 8-bit data) and PFM (linear floats); rows returned bottom first,
// as the reference's loader flips them.
bool ppm_token(std::istream& f, std::string& tok) {
    tok.clear();
    int c;
    while ((c = f.get()) != EOF) {
        if (c == '#') {
            while ((c = f.get()) != EOF && c != '\n') {}
            continue;
        }
        if (isspace(c)) {
            if (!tok.empty()) return true;
            continue;
        }
        tok.push_back((char)c);
    }
    return !tok.empty();
}

bool read_float_image(const std::string& path, std::vector<float>& rgb, uint32_t& w, uint32_t& h, std::string& why) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        why = "cannot open " + path;
        return false;
    }
    std::string magic, sw, sh, sm;
    if (!ppm_token(f, magic) || (magic != "P6" && magic != "PF")) {
        why = path + ": only binary PPM (P6) and colour PFM (PF) images are read";
        return false;
    }
    if (!ppm_token(f, sw) || !ppm_token(f, sh) || !ppm_token(f, sm)) {
        why = path + ": bad header";
        return false;
    }
    const long W = strtol(sw.c_str(), nullptr, 10), H = strtol(sh.c_str(), nullptr, 10);
    if (W <= 0 || H <= 0 || (uint64_t)W * (uint64_t)H > (1ull << 28)) {
        why = path + ": bad size";
        return false;
    }
    w = (uint32_t)W;
    h = (uint32_t)H;
    const size_t n = (size_t)W * (size_t)H * 3;
    rgb.assign(n, 0.0f);
    if (magic == "P6") {
        const long maxval = strtol(sm.c_str(), nullptr, 10);
        if (maxval <= 0 || maxval > 255) {
            why = path + ": only 8-bit PPM is read";
            return false;
        }
        std::vector<unsigned char> px(n);
        if (!f.read((char*)px.data(), (std::streamsize)n)) {
            why = path + ": truncated";
            return false;
        }
        for (long y = 0; y < H; ++y)  // file rows run top to bottom
            for (long k = 0; k < 3 * W; ++k)
                rgb[(size_t)(H - 1 - y) * 3 * W + k] =
                    std::pow((float)px[(size_t)y * 3 * W + k] / (float)maxval, 2.2f);
    } else {
        const float scale = strtof(sm.c_str(), nullptr);
        std::vector<unsigned char> raw(4 * n);
        if (!f.read((char*)raw.data(), (std::streamsize)raw.size())) {
            why = path + ": truncated";
            return false;
        }
        const bool little = scale < 0.0f;
        for (size_t k = 0; k < n; ++k) {  // file rows already run bottom to top
            const unsigned char* b = &raw[4 * k];
            const uint32_t u = little ? (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) |
                                            ((uint32_t)b[3] << 24)
                                      : (uint32_t)b[3] | ((uint32_t)b[2] << 8) | ((uint32_t)b[1] << 16) |
                                            ((uint32_t)b[0] << 24);
            float v;
            std::memcpy(&v, &u, 4);
            rgb[k] = v;
        }
    }
    return true;
}

// ---- the Mitsuba interpreter --------------------------------------------------------------------
struct Interp {
    gr_scene_desc* out;
    std::string dir;
    XF xf;
    gr_material cur{};
    bool have_cur = false;
    F3 cur_light{0, 0, 0};
    std::map<std::string, gr_material> named;
    uint32_t film_w = 256, film_h = 256;
    bool ok = true;

    void warn(const std::string& w) { out->warnings += w + "\n"; }
    bool fail(const std::string& e, const XNode& n) {
        if (ok) out->error = e + " (line " + std::to_string(n.line) + ")";
        ok = false;
        return false;
    }

    gr_material diffuse(F3 c) {
        gr_material m{};
        m.type = GR_MAT_DIFFUSE;
        m.color[0] = c.x; m.color[1] = c.y; m.color[2] = c.z;
        return m;
    }

    // The color slot `key` of a material: a texture property fills color_map.
    void color_texture(gr_material& m, const Props& L, const char* key) {
        auto it = L.find(key);
        if (it == L.end() || it->second.kind != Prop::Texture || it->second.tex < 0) return;
        const Prop& t = it->second;
        m.color_map = out->maps[(size_t)t.tex].data();
        m.color_map_width = t.tw;
        m.color_map_height = t.th;
        m.uv_offset[0] = t.uo;
        m.uv_offset[1] = t.vo;
        m.uv_scale[0] = t.us;
        m.uv_scale[1] = t.vs;
    }

    void create_material(const std::string& type, const Props& L) {
        gr_material m{};
        if (type == "diffuse") {
            m = diffuse(get_color(L, "reflectance", f3(0.3f, 0.3f, 0.3f)));
            color_texture(m, L, "reflectance");
        } else if (type == "mirror" || type == "glass" || type == "dielectric" || type == "roughdielectric") {
            const F3 c = get_color(L, "reflectance", f3(1, 1, 1));
            m.type = GR_MAT_DIELECTRIC;
            m.color[0] = c.x; m.color[1] = c.y; m.color[2] = c.z;
            m.ior = get_float(L, "ior", type == "mirror" ? 100.0f : 1.5f);
            color_texture(m, L, "reflectance");
        } else if (type == "roughconductor" || type == "conductor") {
            const F3 c = get_color(L, "specularReflectance", f3(0.3f, 0.3f, 0.3f));
            F3 ei, et;
            if (has(L, "etaI", Prop::Color)) {
                ei = get_color(L, "etaI", f3(1, 1, 1));
                et = get_color(L, "etaT", f3(0.200438f, 0.924033f, 1.10221f));
            } else {
                ei = get_color(L, "etaI", f3(1, 1, 1));
                et = get_color(L, "eta", f3(0.200438f, 0.924033f, 1.10221f));
            }
            const F3 k = get_color(L, "k", f3(3.91295f, 2.45285f, 2.14219f));
            float au, av;
            if (has(L, "alphaU", Prop::Float)) {
                au = get_float(L, "alphaU", 0.1f);
                av = get_float(L, "alphaV", 0.1f);
            } else {
                au = av = get_float(L, "alpha", 0.1f);
            }
            av = has(L, "alphaU", Prop::Float) ? get_float(L, "alphaU", av) : av;  // alphaV read from "alphaU"
            m.type = GR_MAT_CONDUCTOR;
            m.color[0] = c.x; m.color[1] = c.y; m.color[2] = c.z;
            m.eta_i[0] = ei.x; m.eta_i[1] = ei.y; m.eta_i[2] = ei.z;
            m.eta_t[0] = et.x; m.eta_t[1] = et.y; m.eta_t[2] = et.z;
            m.k[0] = k.x; m.k[1] = k.y; m.k[2] = k.z;
            m.alpha_u = au;
            m.alpha_v = av;
            color_texture(m, L, "specularReflectance");
        } else if (type == "roughplastic") {
            // createMaterial's roughplastic (mitsubaloader.cpp:386-428): with an "etaI" colour the
            // indices are etaI / etaT, else "eta" / "etaI"; alphaV is read from "alphaU"
            F3 ei, et;
            if (has(L, "etaI", Prop::Color)) {
                ei = get_color(L, "etaI", f3(1.5f, 1.5f, 1.5f));
                et = get_color(L, "etaT", f3(1, 1, 1));
            } else {
                ei = get_color(L, "eta", f3(1.5f, 1.5f, 1.5f));
                et = get_color(L, "etaI", f3(1, 1, 1));
            }
            float au = has(L, "alphaU", Prop::Float) ? get_float(L, "alphaU", 0.1f) : get_float(L, "alpha", 0.1f);
            const float av = au;
            const F3 dc = get_color(L, "diffuseReflectance", f3(0.5f, 0.5f, 0.5f));
            const F3 sp = get_color(L, "specularReflectance", f3(1, 1, 1));
            m.type = GR_MAT_PLASTIC;
            m.color[0] = dc.x; m.color[1] = dc.y; m.color[2] = dc.z;
            m.specular[0] = sp.x; m.specular[1] = sp.y; m.specular[2] = sp.z;
            m.eta_i[0] = ei.x; m.eta_i[1] = ei.y; m.eta_i[2] = ei.z;
            m.eta_t[0] = et.x; m.eta_t[1] = et.y; m.eta_t[2] = et.z;
            m.alpha_u = au;
            m.alpha_v = av;
            color_texture(m, L, "diffuseReflectance");
        } else if (type == "disney") {
            return;  // the reference ignores it and keeps the current material
        } else {
            warn("unknown bsdf '" + type + "' loaded as 0.2 Lambert");
            m = diffuse(f3(0.2f, 0.2f, 0.2f));
        }
        cur = m;
        have_cur = true;
    }

    bool create_shape(const std::string& type, const Props& L, const XNode& n) {
        MeshData mesh;
        if (type == "obj") {
            auto it = L.find("filename");
            if (it == L.end()) return fail("obj shape without filename", n);
            std::string err;
            if (!load_obj(dir + it->second.s, mesh, err)) return fail(err, n);
        } else if (type == "sphere") {
            make_sphere(mesh, get_float(L, "radius", 1.0f), get_int(L, "subdiv", 30));
        } else if (type == "rectangle") {
            make_rectangle(mesh);
        } else if (type == "cube") {
            make_cube(mesh);
        } else {
            return fail("unsupported shape type '" + type + "'", n);
        }
        M4 o2w = M4::identity(), inv = M4::identity();
        auto it = L.find("toWorld");
        if (it != L.end() && it->second.kind == Prop::Transform) {
            o2w = it->second.t;
            inv = it->second.tinv;
        }
        for (size_t v = 0; v < mesh.pos.size() / 3; ++v) {
            const float x = mesh.pos[3 * v], y = mesh.pos[3 * v + 1], z = mesh.pos[3 * v + 2];
            float r[4];
            for (int k = 0; k < 4; ++k) r[k] = o2w.m[k][0] * x + o2w.m[k][1] * y + o2w.m[k][2] * z + o2w.m[k][3];
            const float w = r[3] == 1.0f ? 1.0f : r[3];
            mesh.pos[3 * v] = r[0] / w;
            mesh.pos[3 * v + 1] = r[1] / w;
            mesh.pos[3 * v + 2] = r[2] / w;
            if (mesh.has_normals) {  // normals by the inverse transpose
                const float a = mesh.nrm[3 * v], b = mesh.nrm[3 * v + 1], c = mesh.nrm[3 * v + 2];
                const F3 t = normalize(f3(inv.m[0][0] * a + inv.m[1][0] * b + inv.m[2][0] * c,
                                          inv.m[0][1] * a + inv.m[1][1] * b + inv.m[2][1] * c,
                                          inv.m[0][2] * a + inv.m[1][2] * b + inv.m[2][2] * c));
                mesh.nrm[3 * v] = t.x;
                mesh.nrm[3 * v + 1] = t.y;
                mesh.nrm[3 * v + 2] = t.z;
            }
        }
        gr_material m = have_cur ? cur : diffuse(f3(0.3f, 0.3f, 0.3f));
        m.emission[0] = cur_light.x;
        m.emission[1] = cur_light.y;
        m.emission[2] = cur_light.z;
        out->mats.push_back(m);
        out->mesh_mat.push_back((uint32_t)out->mats.size() - 1);
        out->meshes.push_back(std::move(mesh));
        cur_light = f3(0, 0, 0);
        return true;
    }

    // Post-order walk (ParseTag, mitsubaloader.cpp:774-805).
    bool visit(const XNode& n, Props& parent) {
        const std::string& tag = n.name;
        if (tag == "transform") xf = XF();
        Props mine;
        for (auto& k : n.kids)
            if (!visit(*k, mine)) return false;
        const char* nm = n.attr("name");
        const std::string name = nm ? nm : "";
        const std::string type = n.attr("type") ? n.attr("type") : "";
        const std::string id = n.attr("id") ? n.attr("id") : "";
        const char* value = n.attr("value");
        if (tag == "scene" || tag == "mode" || tag == "integrator" || tag == "sampler" || tag == "rfilter" ||
            tag == "medium" || tag == "volume" || tag == "hide")
            return true;
        if (tag == "sensor" || tag == "camera") {
            M4 c2w = M4::identity();
            auto it = mine.find("toWorld");
            if (it != mine.end() && it->second.kind == Prop::Transform) c2w = it->second.t;
            for (int r = 0; r < 4; ++r)
                for (int c = 0; c < 4; ++c) out->cam.to_world[4 * r + c] = c2w.m[r][c];
            out->cam.fov_deg = get_float(mine, "fov", 30.0f);
            out->cam.width = film_w;
            out->cam.height = film_h;
            return true;
        }
        if (tag == "film") {
            film_w = (uint32_t)get_int(mine, "width", 256);
            film_h = (uint32_t)get_int(mine, "height", 256);
            return true;
        }
        if (tag == "bsdf") {
            if (type == "twosided") {
                if (!id.empty()) named[id] = cur;
            } else {
                create_material(type, mine);
                if (!id.empty()) named[id] = cur;
            }
            return true;
        }
        if (tag == "ref") {
            auto it = named.find(id);
            if (it == named.end()) return fail("ref to unknown id '" + id + "'", n);
            cur = it->second;
            have_cur = true;
            return true;
        }
        if (tag == "emitter") {
            if (type == "area") {
                const F3 r = get_color(mine, "radiance", f3(1, 1, 1));
                const float s = get_float(mine, "scale", 1.0f);
                cur_light = f3(r.x * s, r.y * s, r.z * s);
            } else if (type == "constant") {
                const F3 r = get_color(mine, "radiance", f3(1, 1, 1));
                out->env.radiance[0] = r.x;
                out->env.radiance[1] = r.y;
                out->env.radiance[2] = r.z;
                out->env.enabled = 1;
            } else if (type == "envmap") {
                auto fn = mine.find("filename");
                std::vector<float> rgb;
                uint32_t w = 0, h = 0;
                std::string why;
                if (fn == mine.end() || !read_float_image(dir + fn->second.s, rgb, w, h, why)) {
                    warn("envmap emitter skipped: " + (fn == mine.end() ? std::string("no filename") : why));
                    return true;
                }
                out->maps.push_back(std::move(rgb));
                M4 o2w = M4::identity();
                auto tw = mine.find("toWorld");
                if (tw != mine.end() && tw->second.kind == Prop::Transform) o2w = tw->second.t;
                out->env = gr_environment{};
                out->env.enabled = 1;
                out->env.map = out->maps.back().data();
                out->env.map_width = w;
                out->env.map_height = h;
                for (int r = 0; r < 4; ++r)
                    for (int c = 0; c < 4; ++c) out->env.to_world[4 * r + c] = o2w.m[r][c];
            } else {
                return fail("unsupported emitter type '" + type + "'", n);
            }
            return true;
        }
        if (tag == "shape") return create_shape(type, mine, n);
        if (tag == "texture") {
            Prop p;
            p.kind = Prop::Texture;
            p.uo = get_float(mine, "uoffset", 0.0f);
            p.vo = get_float(mine, "voffset", 0.0f);
            p.us = get_float(mine, "uscale", 1.0f);
            p.vs = get_float(mine, "vscale", 1.0f);
            if (type == "checkerboard") {  // the 2 x 2 map (c0, c1; c1, c0) of texture.cpp:45-56
                const F3 a = get_color(mine, "color0", f3(0.4f, 0.4f, 0.4f));
                const F3 b = get_color(mine, "color1", f3(0.2f, 0.2f, 0.2f));
                p.v = f3((a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f);
                out->maps.push_back({a.x, a.y, a.z, b.x, b.y, b.z, b.x, b.y, b.z, a.x, a.y, a.z});
                p.tex = (int)out->maps.size() - 1;
                p.tw = p.th = 2;
            } else if (type == "bitmap") {
                auto fn = mine.find("filename");
                std::vector<float> rgb;
                uint32_t w = 0, h = 0;
                std::string why;
                if (fn != mine.end() && read_float_image(dir + fn->second.s, rgb, w, h, why)) {
                    double sum[3] = {0, 0, 0};
                    for (size_t k = 0; k < rgb.size(); ++k) sum[k % 3] += rgb[k];
                    const double np = (double)w * h;
                    p.v = f3((float)(sum[0] / np), (float)(sum[1] / np), (float)(sum[2] / np));
                    out->maps.push_back(std::move(rgb));
                    p.tex = (int)out->maps.size() - 1;
                    p.tw = w;
                    p.th = h;
                } else {
                    p.v = f3(0.5f, 0.5f, 0.5f);
                    warn("bitmap texture '" + name + "' loaded as 0.5 grey: " +
                         (fn == mine.end() ? std::string("no filename") : why));
                }
            } else {
                p.v = f3(0.5f, 0.5f, 0.5f);
                warn("texture '" + name + "' of type '" + type + "' loaded as 0.5 grey");
            }
            parent[name] = p;
            return true;
        }
        // values
        Prop p;
        if (tag == "boolean" || tag == "bool") {
            p.kind = Prop::Bool;
            p.b = value && std::string(value) == "true";
        } else if (tag == "integer") {
            p.kind = Prop::Int;
            p.i = value ? (int)strtol(value, nullptr, 10) : 0;
        } else if (tag == "float") {
            p.kind = Prop::Float;
            if (!parse_floats(value, &p.f, 1)) return fail("bad float '" + name + "'", n);
        } else if (tag == "string") {
            p.kind = Prop::String;
            p.s = value ? value : "";
        } else if (tag == "vector" || tag == "point") {
            p.kind = Prop::Vector;
            if (!parse_floats(value, &p.v.x, 3)) return fail("bad vector '" + name + "'", n);
        } else if (tag == "rgb" || tag == "color") {
            p.kind = Prop::Color;
            float c[3];
            if (!value) return fail("colour without value", n);
            int cnt = 0;
            for (const char* q = value; *q;) {
                while (*q && (isspace((unsigned char)*q) || *q == ',')) ++q;
                if (!*q) break;
                char* e = nullptr;
                const float f = strtof(q, &e);
                if (e == q) return fail("bad colour '" + name + "'", n);
                if (cnt < 3) c[cnt] = f;
                ++cnt;
                q = e;
            }
            if (cnt == 1) c[1] = c[2] = c[0];
            else if (cnt != 3) return fail("bad colour '" + name + "'", n);
            p.v = f3(c[0], c[1], c[2]);
        } else if (tag == "spectrum") {
            return fail("spectrum values are not supported", n);
        } else if (tag == "transform") {
            p.kind = Prop::Transform;
            p.t = xf.m;
            p.tinv = xf.inv;
        } else if (tag == "lookat" || tag == "lookAt") {
            F3 t, o, u;
            if (!parse_floats(n.attr("target"), &t.x, 3) || !parse_floats(n.attr("origin"), &o.x, 3) ||
                !parse_floats(n.attr("up"), &u.x, 3))
                return fail("bad lookat", n);
            XF la;
            if (!look_at(t, o, u, la)) return fail("singular lookat", n);
            xf = compose(xf, la);
            return true;
        } else if (tag == "translate") {
            F3 d;
            if (value) {
                if (!parse_floats(value, &d.x, 3)) return fail("bad translate", n);
            } else {
                d = f3(n.attr("x") ? strtof(n.attr("x"), nullptr) : 0.0f, n.attr("y") ? strtof(n.attr("y"), nullptr) : 0.0f,
                       n.attr("z") ? strtof(n.attr("z"), nullptr) : 0.0f);
            }
            xf = compose(xf, translate(d));
            return true;
        } else if (tag == "scale") {
            F3 d;
            if (value) {
                if (!parse_floats(value, &d.x, 3)) return fail("bad scale", n);
            } else {
                d = f3(n.attr("x") ? strtof(n.attr("x"), nullptr) : 1.0f, n.attr("y") ? strtof(n.attr("y"), nullptr) : 1.0f,
                       n.attr("z") ? strtof(n.attr("z"), nullptr) : 1.0f);
            }
            xf = compose(xf, scale(d));
            return true;
        } else if (tag == "rotate") {
            const F3 a = f3(n.attr("x") ? strtof(n.attr("x"), nullptr) : 0.0f, n.attr("y") ? strtof(n.attr("y"), nullptr) : 0.0f,
                            n.attr("z") ? strtof(n.attr("z"), nullptr) : 0.0f);
            const float ang = n.attr("angle") ? strtof(n.attr("angle"), nullptr) : 0.0f;
            xf = compose(xf, rotate(ang, a));
            return true;
        } else if (tag == "matrix") {
            XF m;
            if (!parse_floats(value, &m.m.m[0][0], 16)) return fail("bad matrix", n);
            if (!invert(m.m, m.inv)) return fail("singular matrix", n);
            xf = compose(xf, m);
            return true;
        } else {
            return fail("unexpected tag <" + tag + ">", n);
        }
        parent[name] = p;
        return true;
    }
};

gr_scene_desc* parse_file(const char* path) {
    gr_scene_desc* d = new (std::nothrow) gr_scene_desc();
    if (!d) return nullptr;
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        d->error = std::string("cannot open ") + path;
        return d;
    }
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string src = ss.str();
    XmlParser xp(src);
    std::unique_ptr<XNode> root;
    if (!xp.document(root)) {
        d->error = std::string(path) + ": " + xp.err;
        return d;
    }
    Interp in;
    in.out = d;
    const std::string p(path);
    const size_t slash = p.find_last_of('/');
    in.dir = slash == std::string::npos ? "" : p.substr(0, slash + 1);
    in.out->cam.fov_deg = 30.0f;
    in.out->cam.width = 256;
    in.out->cam.height = 256;
    for (int k = 0; k < 4; ++k) in.out->cam.to_world[5 * k] = 1.0f;
    Props top;
    in.visit(*root, top);
    return d;
}

}  // namespace

extern "C" {

gr_status gr_scene_desc_load_xml(const char* path, gr_scene_desc** out) {
    if (!path || !out) return GR_ERR_INVALID;
    *out = parse_file(path);
    if (!*out) return GR_ERR_OOM_BUDGET;
    return (*out)->error.empty() ? GR_OK : GR_ERR_PARSE;
}

gr_status gr_scene_desc_destroy(gr_scene_desc* d) {
    delete d;
    return GR_OK;
}

const char* gr_scene_desc_error(const gr_scene_desc* d) { return d ? d->error.c_str() : "no description"; }
const char* gr_scene_desc_warnings(const gr_scene_desc* d) { return d ? d->warnings.c_str() : ""; }

gr_status gr_scene_desc_info(const gr_scene_desc* d, uint32_t* meshes, uint32_t* triangles, uint32_t* lights,
                             gr_camera* camera, gr_environment* env) {
    if (!d) return GR_ERR_INVALID;
    uint32_t tris = 0, lt = 0;
    for (size_t i = 0; i < d->meshes.size(); ++i) {
        const uint32_t t = (uint32_t)(d->meshes[i].idx.size() / 3);
        tris += t;
        const gr_material& m = d->mats[d->mesh_mat[i]];
        if (m.emission[0] != 0 || m.emission[1] != 0 || m.emission[2] != 0) lt += t;
    }
    if (meshes) *meshes = (uint32_t)d->meshes.size();
    if (triangles) *triangles = tris;
    if (lights) *lights = lt;
    if (camera) *camera = d->cam;
    if (env) *env = d->env;
    return GR_OK;
}

gr_status gr_scene_desc_triangles(const gr_scene_desc* d, float* h_verts, uint32_t* h_material, gr_material* h_mats) {
    if (!d) return GR_ERR_INVALID;
    size_t t = 0;
    for (size_t i = 0; i < d->meshes.size(); ++i) {
        const MeshData& m = d->meshes[i];
        for (size_t k = 0; k < m.idx.size(); k += 3, ++t) {
            if (h_verts)
                for (int c = 0; c < 3; ++c) std::memcpy(h_verts + 9 * t + 3 * c, &m.pos[3ull * m.idx[k + c]], 12);
            if (h_material) h_material[t] = (uint32_t)i;
        }
    }
    if (h_mats)
        for (size_t i = 0; i < d->meshes.size(); ++i) h_mats[i] = d->mats[d->mesh_mat[i]];
    return GR_OK;
}

gr_status gr_scene_desc_mesh(const gr_scene_desc* d, uint32_t i, uint32_t* num_vertices, uint32_t* num_triangles,
                             int* has_normals, float* h_positions, float* h_normals, uint32_t* h_indices) {
    if (!d || i >= d->meshes.size()) return GR_ERR_INVALID;
    const MeshData& m = d->meshes[i];
    if (num_vertices) *num_vertices = (uint32_t)(m.pos.size() / 3);
    if (num_triangles) *num_triangles = (uint32_t)(m.idx.size() / 3);
    if (has_normals) *has_normals = m.has_normals ? 1 : 0;
    if (h_positions && !m.pos.empty()) std::memcpy(h_positions, m.pos.data(), m.pos.size() * 4);
    if (h_normals && m.has_normals) std::memcpy(h_normals, m.nrm.data(), m.nrm.size() * 4);
    if (h_indices && !m.idx.empty()) std::memcpy(h_indices, m.idx.data(), m.idx.size() * 4);
    return GR_OK;
}

gr_status gr_scene_desc_mesh_texcoords(const gr_scene_desc* d, uint32_t i, int* has_texcoords, float* h_texcoords) {
    if (!d || i >= d->meshes.size()) return GR_ERR_INVALID;
    const MeshData& m = d->meshes[i];
    if (has_texcoords) *has_texcoords = m.has_uvs ? 1 : 0;
    if (h_texcoords && m.has_uvs && !m.uv.empty()) std::memcpy(h_texcoords, m.uv.data(), m.uv.size() * 4);
    return GR_OK;
}

gr_status gr_scene_create_from_desc(gr_ctx* ctx, const gr_scene_desc* d, gr_scene** out) {
    if (!ctx || !d || !out) return GR_ERR_INVALID;
    if (!d->error.empty()) {
        ctx->last_error = d->error;
        return GR_ERR_PARSE;
    }
    std::vector<gr_mesh> meshes(d->meshes.size());
    for (size_t i = 0; i < d->meshes.size(); ++i) {
        const MeshData& m = d->meshes[i];
        meshes[i].positions = m.pos.data();
        meshes[i].num_vertices = (uint32_t)(m.pos.size() / 3);
        meshes[i].normals = m.has_normals ? m.nrm.data() : nullptr;
        meshes[i].indices = m.idx.data();
        meshes[i].num_triangles = (uint32_t)(m.idx.size() / 3);
        meshes[i].material = d->mesh_mat[i];
        meshes[i].texcoords = m.has_uvs ? m.uv.data() : nullptr;
    }
    return gr_scene_create(ctx, meshes.data(), (uint32_t)meshes.size(), d->mats.data(), (uint32_t)d->mats.size(),
                           &d->cam, &d->env, out);
}

gr_status gr_scene_load_xml(gr_ctx* ctx, const char* path, gr_scene** out) {
    if (!ctx || !path || !out) return GR_ERR_INVALID;
    gr_scene_desc* d = nullptr;
    gr_status st = gr_scene_desc_load_xml(path, &d);
    if (st != GR_OK) {
        ctx->last_error = d ? d->error : "out of memory";
        gr_scene_desc_destroy(d);
        return st;
    }
    st = gr_scene_create_from_desc(ctx, d, out);
    gr_scene_desc_destroy(d);
    return st;
}

}  // extern "C"
