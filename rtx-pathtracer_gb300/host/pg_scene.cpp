// pg_scene.cpp - procedural scenes, OBJ / Mitsuba-XML subset loading and the
// binned-SAH BVH builder (host side of the tracer).
#include "pg_scene.h"
#include "pg_exr.h"
#include "pg_jpeg.h"
#include "pg_png.h"

#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <fstream>
#include <iterator>
#include <map>
#include <sstream>

namespace pg {

namespace {

struct V3 {
    float x, y, z;
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline V3 normalize(V3 a) { return a * (1.0f / sqrtf(dot(a, a))); }

uint32_t add_material(SceneData &s, int type, V3 albedo, V3 emission, float roughness, float ior) {
    pg_material m;
    memset(&m, 0, sizeof m);
    m.type = type;
    m.albedo[0] = albedo.x;
    m.albedo[1] = albedo.y;
    m.albedo[2] = albedo.z;
    m.emission[0] = emission.x;
    m.emission[1] = emission.y;
    m.emission[2] = emission.z;
    m.roughness = roughness;
    m.ior = ior;
    s.mats.push_back(m);
    return (uint32_t)s.mats.size() - 1;
}

uint32_t add_vertex(SceneData &s, V3 p) {
    s.pos.push_back(p.x);
    s.pos.push_back(p.y);
    s.pos.push_back(p.z);
    return (uint32_t)(s.pos.size() / 3 - 1);
}

void add_tri(SceneData &s, uint32_t a, uint32_t b, uint32_t c, uint32_t m) {
    s.idx.push_back(a);
    s.idx.push_back(b);
    s.idx.push_back(c);
    s.tri_mat.push_back(m);
    s.tri_uv.insert(s.tri_uv.end(), 6, 0.0f);
}

}  // namespace

void add_quad(SceneData &s, const float p0[3], const float p1[3], const float p2[3], const float p3[3],
              uint32_t material) {
    const uint32_t a = add_vertex(s, v3(p0[0], p0[1], p0[2]));
    const uint32_t b = add_vertex(s, v3(p1[0], p1[1], p1[2]));
    const uint32_t c = add_vertex(s, v3(p2[0], p2[1], p2[2]));
    const uint32_t d = add_vertex(s, v3(p3[0], p3[1], p3[2]));
    add_tri(s, a, b, c, material);
    add_tri(s, a, c, d, material);
}

void add_icosphere(SceneData &s, const float center[3], float radius, int level, uint32_t material) {
    const float t = (1.0f + sqrtf(5.0f)) * 0.5f;
    std::vector<V3> v = {v3(-1, t, 0), v3(1, t, 0),  v3(-1, -t, 0), v3(1, -t, 0), v3(0, -1, t),  v3(0, 1, t),
                         v3(0, -1, -t), v3(0, 1, -t), v3(t, 0, -1),  v3(t, 0, 1),  v3(-t, 0, -1), v3(-t, 0, 1)};
    for (auto &p : v) p = normalize(p);
    std::vector<std::array<uint32_t, 3>> f = {{0, 11, 5}, {0, 5, 1},  {0, 1, 7},   {0, 7, 10}, {0, 10, 11},
                                              {1, 5, 9},  {5, 11, 4}, {11, 10, 2}, {10, 7, 6}, {7, 1, 8},
                                              {3, 9, 4},  {3, 4, 2},  {3, 2, 6},   {3, 6, 8},  {3, 8, 9},
                                              {4, 9, 5},  {2, 4, 11}, {6, 2, 10},  {8, 6, 7},  {9, 8, 1}};
    for (int l = 0; l < level; ++l) {
        std::map<std::pair<uint32_t, uint32_t>, uint32_t> mid;
        auto midpoint = [&](uint32_t a, uint32_t b) {
            auto key = std::make_pair(std::min(a, b), std::max(a, b));
            auto it = mid.find(key);
            if (it != mid.end()) return it->second;
            v.push_back(normalize((v[a] + v[b]) * 0.5f));
            const uint32_t id = (uint32_t)v.size() - 1;
            mid[key] = id;
            return id;
        };
        std::vector<std::array<uint32_t, 3>> g;
        g.reserve(f.size() * 4);
        for (auto &tri : f) {
            const uint32_t a = midpoint(tri[0], tri[1]), b = midpoint(tri[1], tri[2]), c = midpoint(tri[2], tri[0]);
            g.push_back({tri[0], a, c});
            g.push_back({tri[1], b, a});
            g.push_back({tri[2], c, b});
            g.push_back({a, b, c});
        }
        f.swap(g);
    }
    const uint32_t base = (uint32_t)(s.pos.size() / 3);
    for (auto &p : v) add_vertex(s, v3(center[0] + radius * p.x, center[1] + radius * p.y, center[2] + radius * p.z));
    for (auto &tri : f) add_tri(s, base + tri[0], base + tri[1], base + tri[2], material);
}

void make_cornell(SceneData &s, const pg_cornell_params &p) {
    const uint32_t white = add_material(s, PG_MAT_DIFFUSE, v3(0.7f, 0.7f, 0.7f), v3(0, 0, 0), 0, 1);
    const uint32_t red = add_material(s, PG_MAT_DIFFUSE, v3(0.7f, 0.12f, 0.1f), v3(0, 0, 0), 0, 1);
    const uint32_t green = add_material(s, PG_MAT_DIFFUSE, v3(0.12f, 0.7f, 0.15f), v3(0, 0, 0), 0, 1);
    const float L = p.light_radiance > 0 ? p.light_radiance : 15.0f;
    const uint32_t light = add_material(s, PG_MAT_LIGHT, v3(0, 0, 0), v3(L, L, L), 0, 1);
    const uint32_t glass = add_material(s, PG_MAT_DIELECTRIC, v3(1, 1, 1), v3(0, 0, 0), 0, p.ior > 0 ? p.ior : 1.5f);
    // unit box, open at z = 1 (towards the camera)
    const float f0[3] = {0, 0, 0}, f1[3] = {1, 0, 0}, f2[3] = {1, 0, 1}, f3[3] = {0, 0, 1};
    add_quad(s, f0, f3, f2, f1, white);  // floor (normal +y)
    const float c0[3] = {0, 1, 0}, c1[3] = {1, 1, 0}, c2[3] = {1, 1, 1}, c3[3] = {0, 1, 1};
    add_quad(s, c0, c1, c2, c3, white);  // ceiling (normal -y)
    const float b0[3] = {0, 0, 0}, b1[3] = {1, 0, 0}, b2[3] = {1, 1, 0}, b3[3] = {0, 1, 0};
    add_quad(s, b0, b1, b2, b3, white);  // back wall (normal +z)
    const float l0[3] = {0, 0, 0}, l1[3] = {0, 1, 0}, l2[3] = {0, 1, 1}, l3[3] = {0, 0, 1};
    add_quad(s, l0, l1, l2, l3, red);  // left wall (normal +x)
    const float r0[3] = {1, 0, 0}, r1[3] = {1, 0, 1}, r2[3] = {1, 1, 1}, r3[3] = {1, 1, 0};
    add_quad(s, r0, r1, r2, r3, green);  // right wall (normal -x)
    const float y = 0.999f, a = 0.375f, b = 0.625f;
    const float q0[3] = {a, y, a}, q1[3] = {b, y, a}, q2[3] = {b, y, b}, q3[3] = {a, y, b};
    add_quad(s, q0, q1, q2, q3, light);  // 0.25 x 0.25 area light facing down
    const float cen[3] = {0.5f, 0.28f, 0.52f};
    add_icosphere(s, cen, 0.25f, p.ico_level, glass);
    s.camera.origin[0] = 0.5f;
    s.camera.origin[1] = 0.5f;
    s.camera.origin[2] = 2.35f;
    s.camera.target[0] = 0.5f;
    s.camera.target[1] = 0.5f;
    s.camera.target[2] = 0.0f;
    s.camera.up[0] = 0.0f;
    s.camera.up[1] = 1.0f;
    s.camera.up[2] = 0.0f;
    s.camera.vfov_deg = 36.0f;
    s.camera.width = p.width;
    s.camera.height = p.height;
}

namespace {
// small deterministic hash noise for the displaced plane
inline uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
inline float lattice(int i, int j, uint32_t seed) {
    return (float)(hash32((uint32_t)i * 73856093u ^ (uint32_t)j * 19349663u ^ seed) & 0xFFFFFF) / 16777216.0f;
}
float value_noise(float x, float y, uint32_t seed) {
    const int i = (int)floorf(x), j = (int)floorf(y);
    const float fx = x - i, fy = y - j;
    const float sx = fx * fx * (3 - 2 * fx), sy = fy * fy * (3 - 2 * fy);
    const float a = lattice(i, j, seed), b = lattice(i + 1, j, seed), c = lattice(i, j + 1, seed),
                d = lattice(i + 1, j + 1, seed);
    return (a + (b - a) * sx) + ((c + (d - c) * sx) - (a + (b - a) * sx)) * sy;
}
}  // namespace

void make_glossy_plates(SceneData &s, const pg_plates_params &p) {
    const V3 cam = v3(0.0f, 2.0f, 15.0f), look = v3(0.0f, 1.2f, 1.0f);
    const float radii[4] = {0.03f, 0.1f, 0.3f, 1.0f};
    const float rough[4] = {0.005f, 0.02f, 0.07f, 0.2f};
    const float lx[4] = {-3.75f, -1.25f, 1.25f, 3.75f};
    const V3 light_c = v3(0.0f, 6.5f, -2.0f);
    // equal power: radiance proportional to 1 / r^2
    for (int i = 0; i < 4; ++i) {
        const float L = 0.8f / (radii[i] * radii[i]);
        const uint32_t m = add_material(s, PG_MAT_LIGHT, v3(0, 0, 0), v3(L, L, L), 0, 1);
        pg_sphere sp;
        memset(&sp, 0, sizeof sp);
        sp.center[0] = lx[i];
        sp.center[1] = light_c.y;
        sp.center[2] = light_c.z;
        sp.radius = radii[i];
        sp.material = m;
        s.spheres.push_back(sp);
    }
    for (int i = 0; i < 4; ++i) {
        const uint32_t m = add_material(s, PG_MAT_GGX, v3(0.9f, 0.9f, 0.9f), v3(0, 0, 0), rough[i], 1);
        const V3 c = v3(0.0f, 3.2f - 0.85f * i, 0.9f * i);
        const V3 n = normalize(normalize(cam - c) + normalize(light_c - c));
        const V3 xa = v3(1, 0, 0);
        const V3 ya = normalize(cross(n, xa));  // in-plate direction perpendicular to x
        const float hw = 4.0f, hd = 0.38f;
        const V3 q0 = c - xa * hw - ya * hd, q1 = c + xa * hw - ya * hd, q2 = c + xa * hw + ya * hd,
                 q3 = c - xa * hw + ya * hd;
        // winding so the geometric normal faces +n
        const float a0[3] = {q0.x, q0.y, q0.z}, a1[3] = {q1.x, q1.y, q1.z}, a2[3] = {q2.x, q2.y, q2.z},
                    a3[3] = {q3.x, q3.y, q3.z};
        if (dot(cross(q1 - q0, q2 - q0), n) > 0)
            add_quad(s, a0, a1, a2, a3, m);
        else
            add_quad(s, a0, a3, a2, a1, m);
    }
    // seeded displaced plane (heightfield) under the plates: 2 * grid^2 triangles
    const uint32_t floor_m = add_material(s, PG_MAT_DIFFUSE, v3(0.55f, 0.55f, 0.5f), v3(0, 0, 0), 0, 1);
    const uint32_t g = p.occluder_grid > 0 ? p.occluder_grid : 64;
    const float x0 = -7.0f, x1 = 7.0f, z0 = -4.0f, z1 = 7.0f, y0 = -0.6f;
    const uint32_t base = (uint32_t)(s.pos.size() / 3);
    for (uint32_t j = 0; j <= g; ++j)
        for (uint32_t i = 0; i <= g; ++i) {
            const float u = (float)i / g, w = (float)j / g;
            const float x = x0 + (x1 - x0) * u, z = z0 + (z1 - z0) * w;
            const float h = 0.35f * value_noise(x * 1.3f, z * 1.3f, p.seed) + 0.08f * value_noise(x * 7.0f, z * 7.0f, p.seed + 1);
            add_vertex(s, v3(x, y0 + h, z));
        }
    for (uint32_t j = 0; j < g; ++j)
        for (uint32_t i = 0; i < g; ++i) {
            const uint32_t a = base + j * (g + 1) + i, b = a + 1, c = a + (g + 1), d = c + 1;
            add_tri(s, a, c, b, floor_m);
            add_tri(s, b, c, d, floor_m);
        }
    s.camera.origin[0] = cam.x;
    s.camera.origin[1] = cam.y;
    s.camera.origin[2] = cam.z;
    s.camera.target[0] = look.x;
    s.camera.target[1] = look.y;
    s.camera.target[2] = look.z;
    s.camera.up[0] = 0.0f;
    s.camera.up[1] = 1.0f;
    s.camera.up[2] = 0.0f;
    s.camera.vfov_deg = 38.0f;
    s.camera.width = p.width;
    s.camera.height = p.height;
}

// ---------------------------------------------------------------------------
// BVH
// ---------------------------------------------------------------------------

namespace {

struct Box {
    float lo[3] = {INFINITY, INFINITY, INFINITY};
    float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    void grow(const float *p) {
        for (int i = 0; i < 3; ++i) {
            lo[i] = std::min(lo[i], p[i]);
            hi[i] = std::max(hi[i], p[i]);
        }
    }
    void grow(const Box &b) {
        for (int i = 0; i < 3; ++i) {
            lo[i] = std::min(lo[i], b.lo[i]);
            hi[i] = std::max(hi[i], b.hi[i]);
        }
    }
    float area() const {
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        if (!(dx >= 0 && dy >= 0 && dz >= 0)) return 0.0f;
        return 2.0f * (dx * dy + dy * dz + dz * dx);
    }
};

// Binary node of the SAH build, before the collapse into four-wide nodes.
struct BinNode {
    float lo0[3], hi0[3];
    float lo1[3], hi1[3];
    int32_t child[2];
    int32_t count[2];
};

struct Builder {
    SceneData &s;
    int max_leaf;
    std::vector<Box> tri_box;
    std::vector<float> cen;  // 3 per triangle
    std::vector<uint32_t> prims;

    struct Ref {
        bool leaf;
        int32_t index;  // node index or first prim
        int32_t count;
        Box box;
    };

    std::vector<BinNode> bin;  // the binary tree, pre-order

    Ref build(uint32_t begin, uint32_t end, int depth) {
        Box bounds, cb;
        for (uint32_t i = begin; i < end; ++i) {
            bounds.grow(tri_box[prims[i]]);
            cb.grow(&cen[3 * prims[i]]);
        }
        const uint32_t n = end - begin;
        if (n <= (uint32_t)max_leaf || depth >= 60) return Ref{true, (int32_t)begin, (int32_t)n, bounds};
        constexpr int NB = 32;
        float best_cost = INFINITY;
        int best_axis = -1, best_split = 0;
        for (int ax = 0; ax < 3; ++ax) {
            const float ext = cb.hi[ax] - cb.lo[ax];
            if (!(ext > 0.0f)) continue;
            Box bb[NB];
            uint32_t bc[NB] = {0};
            const float scale = NB / ext;
            for (uint32_t i = begin; i < end; ++i) {
                const uint32_t p = prims[i];
                int b = (int)((cen[3 * p + ax] - cb.lo[ax]) * scale);
                b = std::min(std::max(b, 0), NB - 1);
                bb[b].grow(tri_box[p]);
                bc[b]++;
            }
            Box left[NB];
            uint32_t lc[NB];
            Box acc;
            uint32_t cnt = 0;
            for (int b = 0; b < NB; ++b) {
                acc.grow(bb[b]);
                cnt += bc[b];
                left[b] = acc;
                lc[b] = cnt;
            }
            Box racc;
            uint32_t rcnt = 0;
            for (int b = NB - 1; b >= 1; --b) {
                racc.grow(bb[b]);
                rcnt += bc[b];
                const uint32_t l = lc[b - 1];
                if (l == 0 || rcnt == 0) continue;
                const float cost = left[b - 1].area() * l + racc.area() * rcnt;
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = ax;
                    best_split = b;
                }
            }
        }
        uint32_t mid;
        if (best_axis < 0) {
            mid = begin + n / 2;  // all centroids coincide: split by position in the list
        } else {
            const float ext = cb.hi[best_axis] - cb.lo[best_axis];
            const float scale = NB / ext;
            auto it = std::partition(prims.begin() + begin, prims.begin() + end, [&](uint32_t p) {
                int b = (int)((cen[3 * p + best_axis] - cb.lo[best_axis]) * scale);
                b = std::min(std::max(b, 0), NB - 1);
                return b < best_split;
            });
            mid = (uint32_t)(it - prims.begin());
            if (mid == begin || mid == end) mid = begin + n / 2;
        }
        const int32_t node = (int32_t)bin.size();
        bin.push_back(BinNode{});
        const Ref l = build(begin, mid, depth + 1);
        const Ref r = build(mid, end, depth + 1);
        BinNode &nd = bin[node];
        for (int i = 0; i < 3; ++i) {
            nd.lo0[i] = l.box.lo[i];
            nd.hi0[i] = l.box.hi[i];
            nd.lo1[i] = r.box.lo[i];
            nd.hi1[i] = r.box.hi[i];
        }
        nd.child[0] = l.index;
        nd.count[0] = l.leaf ? l.count : 0;
        nd.child[1] = r.index;
        nd.count[1] = r.leaf ? r.count : 0;
        return Ref{false, node, 0, bounds};
    }
};

}  // namespace

// One child reference of a binary node (empty when child < 0 and count == 0).
struct ChildRef {
    int32_t child, count;
    float lo[3], hi[3];
};

static float box_area(const float lo[3], const float hi[3]) {
    const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    if (!(dx >= 0 && dy >= 0 && dz >= 0)) return 0.0f;
    return 2.0f * (dx * dy + dy * dz + dz * dx);
}

static void bin_children(const BinNode &n, std::vector<ChildRef> &out) {
    for (int c = 0; c < 2; ++c) {
        if (n.child[c] < 0 && n.count[c] == 0) continue;
        ChildRef r;
        r.child = n.child[c];
        r.count = n.count[c];
        for (int i = 0; i < 3; ++i) {
            r.lo[i] = c == 0 ? n.lo0[i] : n.lo1[i];
            r.hi[i] = c == 0 ? n.hi0[i] : n.hi1[i];
        }
        out.push_back(r);
    }
}

// Four-wide node for binary node b, appended in pre-order; returns its index.
static int32_t collapse(const std::vector<BinNode> &bin, int32_t b, std::vector<BvhNode> &out) {
    std::vector<ChildRef> ch;
    bin_children(bin[b], ch);
    while (ch.size() < 4) {
        int best = -1;
        float best_a = -1.0f;
        for (size_t i = 0; i < ch.size(); ++i)
            if (ch[i].count == 0 && ch[i].child >= 0) {
                const float a = box_area(ch[i].lo, ch[i].hi);
                if (a > best_a) {
                    best_a = a;
                    best = (int)i;
                }
            }
        if (best < 0) break;
        std::vector<ChildRef> kids;
        bin_children(bin[ch[best].child], kids);
        if (ch.size() - 1 + kids.size() > 4) break;
        ch.erase(ch.begin() + best);
        ch.insert(ch.begin() + best, kids.begin(), kids.end());
    }
    const int32_t me = (int32_t)out.size();
    out.push_back(BvhNode{});
    int32_t child_idx[4] = {-1, -1, -1, -1};
    for (size_t i = 0; i < ch.size(); ++i)
        child_idx[i] = ch[i].count > 0 ? ch[i].child : collapse(bin, ch[i].child, out);
    BvhNode &n = out[me];
    for (int slot = 0; slot < 4; ++slot) {
        if (slot < (int)ch.size()) {
            for (int a = 0; a < 3; ++a) {
                n.lo[a][slot] = ch[slot].lo[a];
                n.hi[a][slot] = ch[slot].hi[a];
            }
            n.child[slot] = child_idx[slot];
            n.count[slot] = ch[slot].count;
        } else {
            for (int a = 0; a < 3; ++a) {
                n.lo[a][slot] = INFINITY;
                n.hi[a][slot] = -INFINITY;
            }
            n.child[slot] = -1;
            n.count[slot] = 0;
        }
    }
    return me;
}

void build_bvh(SceneData &s, int max_leaf) {
    const uint32_t T = (uint32_t)(s.idx.size() / 3);
    Builder b{s, max_leaf, {}, {}, {}, {}};
    b.tri_box.resize(T);
    b.cen.resize(3 * (size_t)T);
    b.prims.resize(T);
    for (uint32_t t = 0; t < T; ++t) {
        Box bx;
        for (int k = 0; k < 3; ++k) bx.grow(&s.pos[3 * (size_t)s.idx[3 * (size_t)t + k]]);
        b.tri_box[t] = bx;
        for (int i = 0; i < 3; ++i) b.cen[3 * (size_t)t + i] = 0.5f * (bx.lo[i] + bx.hi[i]);
        b.prims[t] = t;
    }
    s.nodes.clear();
    // binary nodes are numbered in pre-order, so an interior root is node 0;
    // a leaf root becomes a node with one leaf child
    BinNode root{};
    for (int i = 0; i < 3; ++i) {
        root.lo0[i] = root.lo1[i] = INFINITY;
        root.hi0[i] = root.hi1[i] = -INFINITY;
    }
    root.child[0] = root.child[1] = -1;
    if (T == 0) {
        b.bin.push_back(root);
    } else {
        const Builder::Ref top = b.build(0, T, 0);
        if (top.leaf) {
            for (int i = 0; i < 3; ++i) {
                root.lo0[i] = top.box.lo[i];
                root.hi0[i] = top.box.hi[i];
            }
            root.child[0] = top.index;
            root.count[0] = top.count;
            b.bin.push_back(root);
        }
    }
    s.nodes.reserve(b.bin.size() / 2 + 1);
    collapse(b.bin, 0, s.nodes);
    s.tri_order = b.prims;
    s.tri_verts.assign(12 * (size_t)T, 0.0f);
    for (uint32_t i = 0; i < T; ++i) {
        const uint32_t t = b.prims[i];
        for (int k = 0; k < 3; ++k) {
            const float *v = &s.pos[3 * (size_t)s.idx[3 * (size_t)t + k]];
            float *o = &s.tri_verts[12 * (size_t)i + 4 * k];
            o[0] = v[0];
            o[1] = v[1];
            o[2] = v[2];
            o[3] = 0.0f;
        }
        uint32_t id = t;
        memcpy(&s.tri_verts[12 * (size_t)i + 3], &id, 4);
        // v1.w: the material's texture (0 none), so traversal knows which hits to alpha-test
        // without another load
        const uint32_t m = s.tri_mat[t];
        const int32_t tex = m < s.mats.size() ? s.mats[m].texture : 0;
        memcpy(&s.tri_verts[12 * (size_t)i + 7], &tex, 4);
    }
}

// ---------------------------------------------------------------------------
// OBJ and Mitsuba-XML subset
// ---------------------------------------------------------------------------

namespace {
void xform_point(const float *m, const float *p, float *o) {
    for (int r = 0; r < 3; ++r) o[r] = m[4 * r] * p[0] + m[4 * r + 1] * p[1] + m[4 * r + 2] * p[2] + m[4 * r + 3];
}
void mat_identity(float *m) {
    for (int i = 0; i < 16; ++i) m[i] = (i % 5 == 0) ? 1.0f : 0.0f;
}
void mat_mul(const float *a, const float *b, float *o) {
    float t[16];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            float acc = 0;
            for (int k = 0; k < 4; ++k) acc += a[4 * r + k] * b[4 * k + c];
            t[4 * r + c] = acc;
        }
    memcpy(o, t, sizeof t);
}
}  // namespace

bool load_obj(SceneData &s, const std::string &path, const float *to_world, uint32_t material) {
    std::ifstream in(path);
    if (!in) {
        s.error = "cannot open OBJ file " + path;
        return false;
    }
    std::vector<float> vt;  // u, 1 - v (src/SceneLoader.cpp:288-291)
    std::string line;
    const uint32_t base_tri = (uint32_t)s.tri_mat.size();
    std::vector<uint32_t> local_to_global;
    while (std::getline(in, line)) {
        std::istringstream ls(line);
        std::string tag;
        ls >> tag;
        if (tag == "v") {
            float p[3] = {0, 0, 0}, o[3];
            ls >> p[0] >> p[1] >> p[2];
            if (to_world)
                xform_point(to_world, p, o);
            else
                memcpy(o, p, sizeof o);
            local_to_global.push_back(add_vertex(s, v3(o[0], o[1], o[2])));
        } else if (tag == "vt") {
            float u = 0.0f, v = 0.0f;
            ls >> u >> v;
            vt.push_back(u);
            vt.push_back(1.0f - v);
        } else if (tag == "f") {
            std::vector<uint32_t> ids;
            std::vector<long> tex;  // texture coordinate index per corner, -1 without one
            std::string tok;
            while (ls >> tok) {
                char *endp = nullptr;
                long v = strtol(tok.c_str(), &endp, 10);
                if (v < 0) v = (long)local_to_global.size() + v + 1;
                if (v < 1 || (size_t)v > local_to_global.size()) {
                    s.error = "OBJ face index out of range in " + path;
                    return false;
                }
                ids.push_back(local_to_global[(size_t)v - 1]);
                long t = -1;
                if (endp && *endp == '/' && endp[1] != '/' && endp[1] != 0) {
                    t = strtol(endp + 1, nullptr, 10);
                    if (t < 0) t = (long)(vt.size() / 2) + t + 1;
                    if (t < 1 || (size_t)t > vt.size() / 2) {
                        s.error = "OBJ texture coordinate index out of range in " + path;
                        return false;
                    }
                    --t;
                }
                tex.push_back(t);
            }
            for (size_t k = 2; k < ids.size(); ++k) {
                add_tri(s, ids[0], ids[k - 1], ids[k], material);
                const long c[3] = {tex[0], tex[k - 1], tex[k]};
                float *uv = &s.tri_uv[s.tri_uv.size() - 6];
                for (int q = 0; q < 3; ++q)
                    if (c[q] >= 0) {
                        uv[2 * q] = vt[2 * (size_t)c[q]];
                        uv[2 * q + 1] = vt[2 * (size_t)c[q] + 1];
                    }
            }
        }
    }
    if (s.tri_mat.size() == base_tri) {
        s.error = "OBJ file has no faces: " + path;
        return false;
    }
    return true;
}

namespace {

// Minimal XML DOM: elements with attributes and children (no text nodes).
struct XNode {
    std::string name;
    std::map<std::string, std::string> attr;
    std::vector<XNode> kids;
    const XNode *child(const std::string &n, const std::string &name_attr = "") const {
        for (auto &k : kids)
            if (k.name == n && (name_attr.empty() || (k.attr.count("name") && k.attr.at("name") == name_attr)))
                return &k;
        return nullptr;
    }
};

bool parse_xml(const std::string &text, XNode &root, std::string &err) {
    std::vector<XNode *> stack;
    root.name = "#root";
    stack.push_back(&root);
    size_t i = 0;
    while (i < text.size()) {
        const size_t lt = text.find('<', i);
        if (lt == std::string::npos) break;
        if (text.compare(lt, 4, "<!--") == 0) {
            const size_t e = text.find("-->", lt);
            if (e == std::string::npos) {
                err = "unterminated comment";
                return false;
            }
            i = e + 3;
            continue;
        }
        if (text.compare(lt, 2, "<?") == 0) {
            const size_t e = text.find("?>", lt);
            if (e == std::string::npos) {
                err = "unterminated declaration";
                return false;
            }
            i = e + 2;
            continue;
        }
        const size_t gt = text.find('>', lt);
        if (gt == std::string::npos) {
            err = "unterminated tag";
            return false;
        }
        std::string tag = text.substr(lt + 1, gt - lt - 1);
        i = gt + 1;
        if (!tag.empty() && tag[0] == '/') {
            if (stack.size() <= 1) {
                err = "unbalanced closing tag";
                return false;
            }
            const std::string nm = tag.substr(1);
            if (stack.back()->name != nm) {
                err = "mismatched closing tag </" + nm + ">";
                return false;
            }
            stack.pop_back();
            continue;
        }
        bool self_close = !tag.empty() && tag.back() == '/';
        if (self_close) tag.pop_back();
        XNode node;
        size_t p = 0;
        while (p < tag.size() && !isspace((unsigned char)tag[p])) ++p;
        node.name = tag.substr(0, p);
        while (p < tag.size()) {
            while (p < tag.size() && isspace((unsigned char)tag[p])) ++p;
            const size_t eq = tag.find('=', p);
            if (eq == std::string::npos) break;
            std::string key = tag.substr(p, eq - p);
            while (!key.empty() && isspace((unsigned char)key.back())) key.pop_back();
            size_t q = eq + 1;
            while (q < tag.size() && isspace((unsigned char)tag[q])) ++q;
            if (q >= tag.size() || (tag[q] != '"' && tag[q] != '\'')) {
                err = "malformed attribute in <" + node.name + ">";
                return false;
            }
            const char quote = tag[q];
            const size_t qe = tag.find(quote, q + 1);
            if (qe == std::string::npos) {
                err = "unterminated attribute in <" + node.name + ">";
                return false;
            }
            node.attr[key] = tag.substr(q + 1, qe - q - 1);
            p = qe + 1;
        }
        stack.back()->kids.push_back(node);
        if (!self_close) stack.push_back(&stack.back()->kids.back());
    }
    if (stack.size() != 1) {
        err = "unclosed element <" + stack.back()->name + ">";
        return false;
    }
    return true;
}

bool parse_floats(const std::string &s, float *out, int n) {
    std::string t = s;
    for (auto &c : t)
        if (c == ',') c = ' ';
    std::istringstream in(t);
    for (int i = 0; i < n; ++i)
        if (!(in >> out[i])) return false;
    return true;
}

void read_transform(const XNode *t, float *m) {
    mat_identity(m);
    if (!t) return;
    for (auto &op : t->kids) {
        float o[16];
        mat_identity(o);
        if (op.name == "translate") {
            o[3] = op.attr.count("x") ? strtof(op.attr.at("x").c_str(), nullptr) : 0.0f;
            o[7] = op.attr.count("y") ? strtof(op.attr.at("y").c_str(), nullptr) : 0.0f;
            o[11] = op.attr.count("z") ? strtof(op.attr.at("z").c_str(), nullptr) : 0.0f;
        } else if (op.name == "scale") {
            if (op.attr.count("value")) {
                const float v = strtof(op.attr.at("value").c_str(), nullptr);
                o[0] = o[5] = o[10] = v;
            } else {
                o[0] = op.attr.count("x") ? strtof(op.attr.at("x").c_str(), nullptr) : 1.0f;
                o[5] = op.attr.count("y") ? strtof(op.attr.at("y").c_str(), nullptr) : 1.0f;
                o[10] = op.attr.count("z") ? strtof(op.attr.at("z").c_str(), nullptr) : 1.0f;
            }
        } else if (op.name == "matrix" && op.attr.count("value")) {
            parse_floats(op.attr.at("value"), o, 16);
        } else if (op.name == "rotate") {
            float ax[3] = {0, 0, 0};
            ax[0] = op.attr.count("x") ? strtof(op.attr.at("x").c_str(), nullptr) : 0.0f;
            ax[1] = op.attr.count("y") ? strtof(op.attr.at("y").c_str(), nullptr) : 0.0f;
            ax[2] = op.attr.count("z") ? strtof(op.attr.at("z").c_str(), nullptr) : 0.0f;
            const float ang = (op.attr.count("angle") ? strtof(op.attr.at("angle").c_str(), nullptr) : 0.0f) *
                              3.14159265f / 180.0f;
            const float l = sqrtf(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
            if (l > 0) {
                const float x = ax[0] / l, y = ax[1] / l, z = ax[2] / l, c = cosf(ang), s = sinf(ang), C = 1 - c;
                const float r[16] = {x * x * C + c,     x * y * C - z * s, x * z * C + y * s, 0,
                                     y * x * C + z * s, y * y * C + c,     y * z * C - x * s, 0,
                                     z * x * C - y * s, z * y * C + x * s, z * z * C + c,     0,
                                     0,                 0,                 0,                 1};
                memcpy(o, r, sizeof o);
            }
        } else {
            continue;
        }
        mat_mul(o, m, m);  // later operations apply after earlier ones
    }
}

V3 read_rgb(const XNode &n, const std::string &name, V3 def) {
    for (auto &k : n.kids)
        if ((k.name == "rgb" || k.name == "spectrum" || k.name == "color") && k.attr.count("name") &&
            k.attr.at("name") == name && k.attr.count("value")) {
            float v[3];
            if (parse_floats(k.attr.at("value"), v, 3)) return v3(v[0], v[1], v[2]);
            if (parse_floats(k.attr.at("value"), v, 1)) return v3(v[0], v[0], v[0]);
        }
    return def;
}

float read_float(const XNode &n, const std::string &name, float def) {
    for (auto &k : n.kids)
        if (k.name == "float" && k.attr.count("name") && k.attr.at("name") == name && k.attr.count("value"))
            return strtof(k.attr.at("value").c_str(), nullptr);
    return def;
}

std::string read_string(const XNode &n, const std::string &name) {
    for (auto &k : n.kids)
        if (k.name == "string" && k.attr.count("name") && k.attr.at("name") == name && k.attr.count("value"))
            return k.attr.at("value");
    return "";
}

// A texture file (stbi_load with 4 channels, src/SceneLoader.cpp:200): PNG or
// baseline JPEG by signature, as RGBA8.
bool read_texture(const std::string &path, uint32_t &w, uint32_t &h, std::vector<uint8_t> &rgba, std::string &err) {
    std::ifstream in(path, std::ios::binary);
    if (!in) {
        err = "cannot open " + path;
        return false;
    }
    const std::vector<uint8_t> data((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    bool ok;
    if (data.size() >= 2 && data[0] == 0xFF && data[1] == 0xD8)
        ok = decode_jpeg(data.data(), data.size(), w, h, rgba, err);
    else
        ok = decode_png(data.data(), data.size(), w, h, rgba, err);
    if (!ok) err = path + ": " + err;
    return ok;
}

// parseXmlBSDF (src/SceneLoader.cpp:558-611): diffuse, phong, dielectric,
// conductor (a mirror when its material is "none"), roughconductor (Beckmann);
// roughplastic as GGX, anything else diffuse.
uint32_t bsdf_material(SceneData &s, const XNode &b, const std::map<std::string, int32_t> &textures) {
    const XNode *bb = &b;
    if (b.attr.count("type") && b.attr.at("type") == "twosided" && !b.kids.empty()) {
        for (auto &k : b.kids)
            if (k.name == "bsdf") bb = &k;
    }
    const std::string type = bb->attr.count("type") ? bb->attr.at("type") : "diffuse";
    if (type == "dielectric" || type == "thindielectric")
        // refractionIndex = intIOR / extIOR (src/SceneLoader.cpp:590)
        return add_material(s, PG_MAT_DIELECTRIC, v3(1, 1, 1), v3(0, 0, 0), 0,
                            read_float(*bb, "intIOR", 1.5f) / read_float(*bb, "extIOR", 1.0f));
    if (type == "phong") {
        const uint32_t id = add_material(s, PG_MAT_PHONG, read_rgb(*bb, "diffuseReflectance", v3(0.5f, 0.5f, 0.5f)),
                                         v3(0, 0, 0), 0, 1);
        const V3 sp = read_rgb(*bb, "specularReflectance", v3(0.2f, 0.2f, 0.2f));
        pg_material &m = s.mats[id];
        m.specular[0] = sp.x, m.specular[1] = sp.y, m.specular[2] = sp.z;
        m.exponent = read_float(*bb, "exponent", 30.0f);
        return id;
    }
    if (type == "conductor") {
        if (read_string(*bb, "material") == "none")
            return add_material(s, PG_MAT_SPECULAR, v3(1, 1, 1), v3(0, 0, 0), 0, 1);
        const uint32_t id = add_material(s, PG_MAT_CONDUCTOR, v3(1, 1, 1), v3(0, 0, 0), 0, 1);
        s.mats[id].eta = read_rgb(*bb, "eta", v3(0.2f, 0.2f, 0.2f)).x;
        s.mats[id].k = read_rgb(*bb, "k", v3(3.9f, 3.9f, 3.9f)).x;
        return id;
    }
    if (type == "roughconductor") {
        const uint32_t id = add_material(s, PG_MAT_BECKMANN, v3(1, 1, 1), v3(0, 0, 0), read_float(*bb, "alpha", 0.1f), 1);
        s.mats[id].eta = read_rgb(*bb, "eta", v3(0.2f, 0.2f, 0.2f)).x;
        s.mats[id].k = read_rgb(*bb, "k", v3(3.9f, 3.9f, 3.9f)).x;
        return id;
    }
    if (type == "roughplastic")
        return add_material(s, PG_MAT_GGX, read_rgb(*bb, "specularReflectance", v3(1, 1, 1)), v3(0, 0, 0),
                            read_float(*bb, "alpha", 0.1f), 1);
    // a diffuse reflectance given by a texture reference: white, scaled by the
    // texture (src/SceneLoader.cpp:574-587)
    for (auto &k : bb->kids)
        if (k.name == "ref" && k.attr.count("name") && k.attr.at("name") == "reflectance" && k.attr.count("id") &&
            textures.count(k.attr.at("id"))) {
            const uint32_t id = add_material(s, PG_MAT_DIFFUSE, v3(1, 1, 1), v3(0, 0, 0), 0, 1);
            s.mats[id].texture = textures.at(k.attr.at("id")) + 1;
            return id;
        }
    return add_material(s, PG_MAT_DIFFUSE, read_rgb(*bb, "reflectance", v3(0.5f, 0.5f, 0.5f)), v3(0, 0, 0), 0, 1);
}

}  // namespace

bool load_mitsuba(SceneData &s, const std::string &path, uint32_t width, uint32_t height) {
    std::ifstream in(path);
    if (!in) {
        s.error = "cannot open scene file " + path;
        return false;
    }
    std::stringstream ss;
    ss << in.rdbuf();
    XNode root;
    std::string err;
    if (!parse_xml(ss.str(), root, err)) {
        s.error = "malformed scene file " + path + ": " + err;
        return false;
    }
    const XNode *scene = root.child("scene");
    if (!scene) {
        s.error = "no <scene> element in " + path;
        return false;
    }
    const std::string dir = path.find('/') != std::string::npos ? path.substr(0, path.rfind('/') + 1) : "";
    std::map<std::string, uint32_t> named;
    // camera (parseCameraSettings, src/SceneLoader.cpp:613-648)
    s.camera.width = width;
    s.camera.height = height;
    s.camera.vfov_deg = 45.0f;
    s.camera.up[1] = 1.0f;
    s.camera.target[2] = -1.0f;
    if (const XNode *sensor = scene->child("sensor")) {
        s.camera.vfov_deg = read_float(*sensor, "fov", 45.0f);
        if (const XNode *tw = sensor->child("transform")) {
            // both spellings, as src/SceneLoader.cpp:620-622 accepts
            const XNode *la = tw->child("lookAt") ? tw->child("lookAt") : tw->child("lookat");
            if (la) {
                float o[3], t[3], u[3];
                if (la->attr.count("origin") && parse_floats(la->attr.at("origin"), o, 3) && la->attr.count("target") &&
                    parse_floats(la->attr.at("target"), t, 3)) {
                    memcpy(s.camera.origin, o, sizeof o);
                    memcpy(s.camera.target, t, sizeof t);
                }
                if (la->attr.count("up") && parse_floats(la->attr.at("up"), u, 3)) memcpy(s.camera.up, u, sizeof u);
            }
        }
    }
    // bitmap textures (SceneLoader::parseXmlTextures, src/SceneLoader.cpp:515-533)
    std::map<std::string, int32_t> textures;
    for (auto &k : scene->kids) {
        if (k.name != "texture" || !k.attr.count("id")) continue;
        if (textures.count(k.attr.at("id"))) {
            s.error = "duplicate texture id " + k.attr.at("id") + " in " + path;
            return false;
        }
        const std::string file = read_string(k, "filename");
        const std::string full = (!file.empty() && file[0] == '/') ? file : dir + file;
        SceneData::Texture tex;
        std::string terr;
        if (!read_texture(full, tex.w, tex.h, tex.rgba, terr)) {
            s.error = "texture " + k.attr.at("id") + ": " + terr;
            return false;
        }
        textures[k.attr.at("id")] = (int32_t)s.textures.size();
        s.textures.push_back(std::move(tex));
    }
    for (auto &k : scene->kids)
        if (k.name == "bsdf" && k.attr.count("id")) named[k.attr.at("id")] = bsdf_material(s, k, textures);
    // SceneLoader::parseEnvMap (src/SceneLoader.cpp:370-401): an envmap emitter's EXR image
    for (auto &k : scene->kids) {
        if (k.name != "emitter" || !k.attr.count("type") || k.attr.at("type") != "envmap") continue;
        const std::string file = read_string(k, "filename");
        if (file.empty()) {
            s.error = "envmap emitter without a filename";
            return false;
        }
        ExrImage img;
        std::string err;
        if (!read_exr(file[0] == '/' ? file : dir + file, img, err)) {
            s.error = err.rfind("cannot open", 0) == 0 ? err : "envmap: " + err;
            return false;
        }
        s.env_w = img.width;
        s.env_h = img.height;
        s.env.swap(img.rgb);
        break;
    }
    for (auto &sh : scene->kids) {
        if (sh.name != "shape") continue;
        const std::string type = sh.attr.count("type") ? sh.attr.at("type") : "";
        uint32_t mat = UINT32_MAX;
        for (auto &k : sh.kids) {
            if (k.name == "ref" && k.attr.count("id")) {
                if (!named.count(k.attr.at("id"))) {
                    s.error = "unknown bsdf reference " + k.attr.at("id");
                    return false;
                }
                mat = named.at(k.attr.at("id"));
            } else if (k.name == "bsdf") {
                mat = bsdf_material(s, k, textures);
            }
        }
        if (const XNode *em = sh.child("emitter")) {
            const V3 L = read_rgb(*em, "radiance", v3(1, 1, 1));
            mat = add_material(s, PG_MAT_LIGHT, v3(0, 0, 0), L, 0, 1);
        }
        if (mat == UINT32_MAX) mat = add_material(s, PG_MAT_DIFFUSE, v3(0.5f, 0.5f, 0.5f), v3(0, 0, 0), 0, 1);
        float m[16];
        read_transform(sh.child("transform", "toWorld") ? sh.child("transform", "toWorld") : sh.child("transform"), m);
        if (type == "obj") {
            const std::string fn = read_string(sh, "filename");
            if (fn.empty()) {
                s.error = "obj shape without filename";
                return false;
            }
            if (!load_obj(s, dir + fn, m, mat)) return false;
        } else if (type == "sphere") {
            pg_sphere sp;
            memset(&sp, 0, sizeof sp);
            float c[3] = {0, 0, 0};
            if (const XNode *pt = sh.child("point", "center")) {
                c[0] = pt->attr.count("x") ? strtof(pt->attr.at("x").c_str(), nullptr) : 0.0f;
                c[1] = pt->attr.count("y") ? strtof(pt->attr.at("y").c_str(), nullptr) : 0.0f;
                c[2] = pt->attr.count("z") ? strtof(pt->attr.at("z").c_str(), nullptr) : 0.0f;
            }
            float wc[3];
            xform_point(m, c, wc);
            memcpy(sp.center, wc, sizeof wc);
            sp.radius = read_float(sh, "radius", 1.0f) * sqrtf(m[0] * m[0] + m[4] * m[4] + m[8] * m[8]);
            sp.material = mat;
            s.spheres.push_back(sp);
        } else if (type == "rectangle" || type == "cube") {
            const float q[4][3] = {{-1, -1, 0}, {1, -1, 0}, {1, 1, 0}, {-1, 1, 0}};
            if (type == "rectangle") {
                float w[4][3];
                for (int i = 0; i < 4; ++i) xform_point(m, q[i], w[i]);
                add_quad(s, w[0], w[1], w[2], w[3], mat);
            } else {
                const float c8[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                        {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
                const int f[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4}, {2, 3, 7, 6}, {1, 2, 6, 5}, {0, 4, 7, 3}};
                float w[8][3];
                for (int i = 0; i < 8; ++i) xform_point(m, c8[i], w[i]);
                for (int i = 0; i < 6; ++i) add_quad(s, w[f[i][0]], w[f[i][1]], w[f[i][2]], w[f[i][3]], mat);
            }
        } else {
            s.error = "unsupported shape type '" + type + "'";
            return false;
        }
    }
    if (s.tri_mat.empty() && s.spheres.empty()) {
        s.error = "scene has no shapes: " + path;
        return false;
    }
    return true;
}

}  // namespace pg
