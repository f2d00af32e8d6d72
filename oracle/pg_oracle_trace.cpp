// pg_oracle_trace.cpp - TEST INFRASTRUCTURE (see pg_oracle_trace.h).
// Compiled with -ffp-contract=off: every FP32 operation of the traversal twin
// rounds exactly where the device code's explicit _rn intrinsics round (fmaf
// where the device uses __fmaf_rn).
#include "pg_oracle_trace.h"
#include "pg_oracle.h"

#include <math.h>
#include <pthread.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <vector>

namespace {

// four-wide node: child boxes slot-major per coordinate (the library's BvhNode)
struct Node {
    float lo[3][4];
    float hi[3][4];
    int32_t child[4];
    int32_t count[4];
};
static_assert(sizeof(Node) == 128, "node layout");
constexpr int kStack = 128;  // the device's stack depth; a full stack drops the push there too

// ---------------------------------------------------------------------------
// FP32 twin of the device traversal (pg_traverse.cuh), same operation order
// ---------------------------------------------------------------------------
struct RayPre {
    float org[3], dir[3], inv[3];
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

RayPre ray_setup(const float o[3], const float d[3]) {
    RayPre r;
    for (int i = 0; i < 3; ++i) {
        r.org[i] = o[i];
        r.dir[i] = d[i];
        r.inv[i] = 1.0f / d[i];
    }
    const float ax = fabsf(d[0]), ay = fabsf(d[1]), az = fabsf(d[2]);
    int kz = 0;
    if (ay > ax) kz = 1;
    if (az > fmaxf(ax, ay)) kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (d[kz] < 0.0f) std::swap(kx, ky);
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.Sx = d[kx] / d[kz];
    r.Sy = d[ky] / d[kz];
    r.Sz = 1.0f / d[kz];
    return r;
}

bool tri_intersect(const RayPre &r, const float *v0, const float *v1, const float *v2, float tmin, float tmax,
                   float &t_out, float &u_out, float &v_out) {
    const float A[3] = {v0[0] - r.org[0], v0[1] - r.org[1], v0[2] - r.org[2]};
    const float B[3] = {v1[0] - r.org[0], v1[1] - r.org[1], v1[2] - r.org[2]};
    const float C[3] = {v2[0] - r.org[0], v2[1] - r.org[1], v2[2] - r.org[2]};
    const float Akz = A[r.kz], Bkz = B[r.kz], Ckz = C[r.kz];
    const float Ax = fmaf(-r.Sx, Akz, A[r.kx]);  // fused where the device fuses
    const float Ay = fmaf(-r.Sy, Akz, A[r.ky]);
    const float Bx = fmaf(-r.Sx, Bkz, B[r.kx]);
    const float By = fmaf(-r.Sy, Bkz, B[r.ky]);
    const float Cx = fmaf(-r.Sx, Ckz, C[r.kx]);
    const float Cy = fmaf(-r.Sy, Ckz, C[r.ky]);
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = (U + V) + W;
    if (det == 0.0f) return false;
    const float Az = r.Sz * Akz, Bz = r.Sz * Bkz, Cz = r.Sz * Ckz;
    const float T = fmaf(W, Cz, fmaf(V, Bz, U * Az));
    const float t = T / det;
    if (!(t > tmin && t < tmax)) return false;
    t_out = t;
    u_out = V / det;
    v_out = W / det;
    return true;
}

float box_enter(const RayPre &r, const float *lo, const float *hi, float tmin, float tmax) {
    const float tx0 = (lo[0] - r.org[0]) * r.inv[0], tx1 = (hi[0] - r.org[0]) * r.inv[0];
    const float ty0 = (lo[1] - r.org[1]) * r.inv[1], ty1 = (hi[1] - r.org[1]) * r.inv[1];
    const float tz0 = (lo[2] - r.org[2]) * r.inv[2], tz1 = (hi[2] - r.org[2]) * r.inv[2];
    const float te = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), tmin));
    float tx = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tmax));
    tx = tx * 1.0000004f;
    return te <= tx ? te : INFINITY;
}

bool sphere_intersect(const RayPre &r, const pg_sphere &s, float tmin, float tmax, float &t_out) {
    const float oc[3] = {r.org[0] - s.center[0], r.org[1] - s.center[1], r.org[2] - s.center[2]};
    const float a = (r.dir[0] * r.dir[0] + r.dir[1] * r.dir[1]) + r.dir[2] * r.dir[2];
    const float b = (r.dir[0] * oc[0] + r.dir[1] * oc[1]) + r.dir[2] * oc[2];
    const float c = ((oc[0] * oc[0] + oc[1] * oc[1]) + oc[2] * oc[2]) - s.radius * s.radius;
    const float disc = b * b - a * c;
    if (disc < 0.0f) return false;
    const float sq = sqrtf(disc);
    const float t1 = (-b - sq) / a;
    if (t1 > tmin && t1 < tmax) {
        t_out = t1;
        return true;
    }
    const float t2 = (-b + sq) / a;
    if (t2 > tmin && t2 < tmax) {
        t_out = t2;
        return true;
    }
    return false;
}

uint32_t fbits(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}
float bitsf(uint32_t u) {
    float f;
    memcpy(&f, &u, 4);
    return f;
}

// Alpha test of a textured hit (raytrace.rahit:21-46, device alpha_keep in
// pg_traverse.cuh): same operations in the same order, each rounded to FP32
// (the file is compiled without FMA contraction).
uint32_t tea16(uint32_t v0, uint32_t v1) {
    uint32_t s0 = 0;
    for (int n = 0; n < 16; ++n) {
        s0 += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}

float tex_alpha(const pgo_scene &S, uint32_t tex, float u, float v) {
    const uint32_t *ti = S.tex_info + 4 * (size_t)tex;
    const int w = (int)ti[1], h = (int)ti[2];
    u = u - floorf(u);
    v = v - floorf(v);
    const float x = u * (float)w - 0.5f, y = v * (float)h - 0.5f;
    const float x0 = floorf(x), y0 = floorf(y);
    const float fx = x - x0, fy = y - y0;
    int ix0 = (int)x0, iy0 = (int)y0;
    int ix1 = ix0 + 1, iy1 = iy0 + 1;
    ix0 = ix0 < 0 ? ix0 + w : ix0;
    iy0 = iy0 < 0 ? iy0 + h : iy0;
    ix1 = ix1 >= w ? ix1 - w : ix1;
    iy1 = iy1 >= h ? iy1 - h : iy1;
    const uint8_t *d = S.tex_data + 4 * (size_t)ti[0];
    const float k = 1.0f / 255.0f;
    const float a00 = (float)d[4 * (iy0 * w + ix0) + 3] * k, a10 = (float)d[4 * (iy0 * w + ix1) + 3] * k;
    const float a01 = (float)d[4 * (iy1 * w + ix0) + 3] * k, a11 = (float)d[4 * (iy1 * w + ix1) + 3] * k;
    const float gx = 1.0f - fx, gy = 1.0f - fy;
    const float top = a00 * gx + a10 * fx;
    const float bot = a01 * gx + a11 * fx;
    return top * gy + bot * fy;
}

bool alpha_keep(const pgo_scene &S, float org_x, uint32_t id, uint32_t tex, float bu, float bv, float t) {
    const float *uv = S.tri_uv + 6 * (size_t)id;
    const float w0 = (1.0f - bu) - bv;
    const float tu = (uv[0] * w0 + uv[2] * bu) + uv[4] * bv;
    const float tv = (uv[1] * w0 + uv[3] * bu) + uv[5] * bv;
    const float a = tex_alpha(S, tex - 1u, tu, tv);
    const float sx = fminf(fmaxf(tu * 100000000.0f + org_x * t, -4.0e18f), 4.0e18f);
    uint32_t seed = tea16((uint32_t)(long long)sx, S.alpha_salt);
    seed = 1664525u * seed + 1013904223u;
    const float r = (float)(seed & 0x00FFFFFFu) * (1.0f / 16777216.0f);
    return !(r > a);
}

uint32_t tri_tex(const float *tv) { return fbits(tv[7]); }

// One node step of the device traversal (trav_step in pg_traverse.cuh), same
// order: four box tests against the best t at the start of the step, leaves
// in slot order, inner children nearest first (closest: stable by entry
// distance; any: slot order).  Returns true when the traversal is over.
template <bool kAny>
bool node_step(const pgo_scene &S, const RayPre &r, float tmin, float &best_t, uint32_t &best_id, float &best_u,
               float &best_v, int &node, int *stack, int &sp, uint32_t &n_nodes, uint32_t &n_tris) {
    const Node &n = ((const Node *)S.nodes)[node];
    ++n_nodes;
    float e[4];
    for (int j = 0; j < 4; ++j) {
        const float lo[3] = {n.lo[0][j], n.lo[1][j], n.lo[2][j]}, hi[3] = {n.hi[0][j], n.hi[1][j], n.hi[2][j]};
        e[j] = box_enter(r, lo, hi, tmin, best_t);
    }
    for (int j = 0; j < 4; ++j) {
        if (e[j] == INFINITY || n.count[j] <= 0) continue;
        for (int k = 0; k < n.count[j]; ++k) {
            const float *tv = S.tri_verts + 12 * (size_t)(n.child[j] + k);
            ++n_tris;
            float t, u, v;
            const uint32_t tex = tri_tex(tv);
            if (kAny) {
                if (tri_intersect(r, tv, tv + 4, tv + 8, tmin, best_t, t, u, v) &&
                    (tex == 0u || alpha_keep(S, r.org[0], fbits(tv[3]), tex, u, v, t))) {
                    best_id = fbits(tv[3]);
                    return true;
                }
            } else {
                const uint32_t id = fbits(tv[3]);
                const float lim = best_id == PG_NO_HIT ? best_t : bitsf(fbits(best_t) + 1u);
                if (tri_intersect(r, tv, tv + 4, tv + 8, tmin, lim, t, u, v) &&
                    (t < best_t || (t == best_t && id < best_id)) &&
                    (tex == 0u || alpha_keep(S, r.org[0], id, tex, u, v, t))) {
                    best_t = t;
                    best_id = id;
                    best_u = u;
                    best_v = v;
                }
            }
        }
    }
    int cand[4];
    float ce[4];
    int nn = 0;
    for (int j = 0; j < 4; ++j) {
        if (e[j] == INFINITY || n.count[j] > 0 || n.child[j] < 0) continue;
        int pos = nn;
        if (!kAny)
            while (pos > 0 && ce[pos - 1] > e[j]) {
                ce[pos] = ce[pos - 1];
                cand[pos] = cand[pos - 1];
                --pos;
            }
        ce[pos] = e[j];
        cand[pos] = n.child[j];
        ++nn;
    }
    if (nn > 0) {
        for (int q = nn - 1; q >= 1; --q)
            if (sp < kStack) stack[sp++] = cand[q];
        node = cand[0];
        return false;
    }
    if (sp == 0) return true;
    node = stack[--sp];
    return false;
}

// cnt (optional): [0] BVH nodes fetched, [1] triangles tested
void closest32(const pgo_scene &S, const pg_ray &ray, pg_hit &hit, uint32_t *cnt = nullptr) {
    uint32_t n_nodes = 0, n_tris = 0;
    const RayPre r = ray_setup(ray.org, ray.dir);
    float best_t = ray.tmax, best_u = 0, best_v = 0;
    uint32_t best_id = PG_NO_HIT;
    for (uint32_t i = 0; i < S.n_spheres; ++i) {
        float t;
        if (sphere_intersect(r, S.spheres[i], ray.tmin, best_t, t)) {
            best_t = t;
            best_id = PG_SPHERE_BIT | i;
        }
    }
    int stack[kStack];
    int sp = 0, node = 0;
    while (!node_step<false>(S, r, ray.tmin, best_t, best_id, best_u, best_v, node, stack, sp, n_nodes, n_tris)) {
    }
    hit.t = best_t;
    hit.u = best_u;
    hit.v = best_v;
    hit.prim = best_id;
    if (cnt) {
        cnt[0] = n_nodes;
        cnt[1] = n_tris;
    }
}

bool any32(const pgo_scene &S, const pg_ray &ray) {
    const RayPre r = ray_setup(ray.org, ray.dir);
    for (uint32_t i = 0; i < S.n_spheres; ++i) {
        float t;
        if (sphere_intersect(r, S.spheres[i], ray.tmin, ray.tmax, t)) return true;
    }
    float best_t = ray.tmax, best_u = 0, best_v = 0;
    uint32_t best_id = PG_NO_HIT, n_nodes = 0, n_tris = 0;
    int stack[kStack];
    int sp = 0, node = 0;
    while (!node_step<true>(S, r, ray.tmin, best_t, best_id, best_u, best_v, node, stack, sp, n_nodes, n_tris)) {
    }
    return best_id != PG_NO_HIT;
}

template <typename F>
void parallel_for(uint32_t n, int n_threads, F f) {
    if (n_threads <= 1 || n < 2) {
        for (uint32_t i = 0; i < n; ++i) f(i);
        return;
    }
    std::atomic<uint32_t> next{0};
    struct Ctx {
        std::atomic<uint32_t> *next;
        uint32_t n;
        F *f;
    } ctx{&next, n, &f};
    auto body = [](void *p) -> void * {
        Ctx *c = (Ctx *)p;
        for (;;) {
            const uint32_t i = c->next->fetch_add(1);
            if (i >= c->n) break;
            (*c->f)(i);
        }
        return nullptr;
    };
    std::vector<pthread_t> th(std::min(n_threads, 256));
    int started = 0;
    for (auto &t : th)
        if (pthread_create(&t, nullptr, body, &ctx) == 0) ++started;
    if (started == 0) body(&ctx);
    for (int i = 0; i < started; ++i) pthread_join(th[i], nullptr);
}

// ---------------------------------------------------------------------------
// FP64 renderer
// ---------------------------------------------------------------------------
struct D3 {
    double x, y, z;
};
inline D3 d3(double x, double y, double z) { return D3{x, y, z}; }
inline D3 operator+(D3 a, D3 b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline D3 operator-(D3 a, D3 b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline D3 operator*(D3 a, double s) { return d3(a.x * s, a.y * s, a.z * s); }
inline D3 hm(D3 a, D3 b) { return d3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 cross(D3 a, D3 b) { return d3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline D3 unit(D3 a) { return a * (1.0 / sqrt(dot(a, a))); }
inline double mx(D3 a) { return std::max(a.x, std::max(a.y, a.z)); }
inline D3 fv(const float *p) { return d3(p[0], p[1], p[2]); }
const double PI = 3.14159265358979323846;

uint32_t fmix32(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}
double rnd(uint32_t seed, uint32_t pixel, uint32_t sample, uint32_t dim) {
    const uint32_t h = fmix32(seed + fmix32(pixel + fmix32(sample * 1024u + dim)));
    return (double)(float)((float)(h >> 8) * (1.0f / 16777216.0f));
}
uint32_t dimb(int b, int d) { return 2u + 16u * (uint32_t)b + (uint32_t)d; }

struct Light {
    int type;
    std::vector<uint32_t> tris;
    std::vector<double> cdf;
    uint32_t sphere;
    double area;
    D3 emission;
};

struct Hit64 {
    double t;
    uint32_t prim;
    double u = 0.0, v = 0.0;  // barycentrics of the triangle's second and third corners
};

struct Scene64 {
    const pgo_scene *S;
    std::vector<Light> lights;
    std::vector<int> tri_light;
};

// double-precision closest hit (Moller-Trumbore over the same BVH)
bool tri64(D3 o, D3 d, D3 a, D3 b, D3 c, double tmin, double tmax, double &t, double &bu, double &bv) {
    const D3 e1 = b - a, e2 = c - a;
    const D3 p = cross(d, e2);
    const double det = dot(e1, p);
    if (det == 0.0) return false;
    const double inv = 1.0 / det;
    const D3 s = o - a;
    const double u = dot(s, p) * inv;
    if (u < 0.0 || u > 1.0) return false;
    const D3 q = cross(s, e1);
    const double v = dot(d, q) * inv;
    if (v < 0.0 || u + v > 1.0) return false;
    const double tt = dot(e2, q) * inv;
    if (!(tt > tmin && tt < tmax)) return false;
    t = tt;
    bu = u;
    bv = v;
    return true;
}

bool box64(D3 o, D3 inv, const float *lo, const float *hi, double tmin, double tmax) {
    double t0 = tmin, t1 = tmax;
    const double O[3] = {o.x, o.y, o.z}, I[3] = {inv.x, inv.y, inv.z};
    for (int i = 0; i < 3; ++i) {
        double a = ((double)lo[i] - 1e-7 * (1 + fabs(lo[i])) - O[i]) * I[i];
        double b = ((double)hi[i] + 1e-7 * (1 + fabs(hi[i])) - O[i]) * I[i];
        if (a > b) std::swap(a, b);
        if (std::isnan(a)) a = -INFINITY;
        if (std::isnan(b)) b = INFINITY;
        t0 = std::max(t0, a);
        t1 = std::min(t1, b);
    }
    return t0 <= t1;
}

bool sphere64(D3 o, D3 d, const pg_sphere &s, double tmin, double tmax, double &t) {
    const D3 oc = o - fv(s.center);
    const double a = dot(d, d), b = dot(d, oc), c = dot(oc, oc) - (double)s.radius * s.radius;
    const double disc = b * b - a * c;
    if (disc < 0) return false;
    const double sq = sqrt(disc);
    const double t1 = (-b - sq) / a;
    if (t1 > tmin && t1 < tmax) {
        t = t1;
        return true;
    }
    const double t2 = (-b + sq) / a;
    if (t2 > tmin && t2 < tmax) {
        t = t2;
        return true;
    }
    return false;
}

// sRGB byte to linear, and the bilinear linear-RGB texture colour at a hit
// (repeat addressing, texel centres at half-integers), in double.
double srgb64(uint8_t b) {
    const double c = b / 255.0;
    return c <= 0.04045 ? c / 12.92 : pow((c + 0.055) / 1.055, 2.4);
}
D3 tex_rgb64(const pgo_scene &S, uint32_t prim, uint32_t tex, double bu, double bv) {
    const float *uv = S.tri_uv + 6 * (size_t)prim;
    const double w0 = 1.0 - bu - bv;
    double u = uv[0] * w0 + uv[2] * bu + uv[4] * bv, v = uv[1] * w0 + uv[3] * bu + uv[5] * bv;
    const uint32_t *ti = S.tex_info + 4 * (size_t)tex;
    const int w = (int)ti[1], h = (int)ti[2];
    u -= floor(u);
    v -= floor(v);
    const double x = u * w - 0.5, y = v * h - 0.5, x0 = floor(x), y0 = floor(y), fx = x - x0, fy = y - y0;
    int ix0 = (int)x0, iy0 = (int)y0, ix1 = ix0 + 1, iy1 = iy0 + 1;
    ix0 = ix0 < 0 ? ix0 + w : ix0;
    iy0 = iy0 < 0 ? iy0 + h : iy0;
    ix1 = ix1 >= w ? ix1 - w : ix1;
    iy1 = iy1 >= h ? iy1 - h : iy1;
    const uint8_t *d = S.tex_data + 4 * (size_t)ti[0];
    double c[3];
    for (int k = 0; k < 3; ++k) {
        const double top = srgb64(d[4 * (iy0 * w + ix0) + k]) * (1 - fx) + srgb64(d[4 * (iy0 * w + ix1) + k]) * fx;
        const double bot = srgb64(d[4 * (iy1 * w + ix0) + k]) * (1 - fx) + srgb64(d[4 * (iy1 * w + ix1) + k]) * fx;
        c[k] = top * (1 - fy) + bot * fy;
    }
    return d3(c[0], c[1], c[2]);
}

Hit64 intersect64(const pgo_scene &S, D3 o, D3 d, double tmin, double tmax, bool any) {
    Hit64 h{tmax, PG_NO_HIT};
    for (uint32_t i = 0; i < S.n_spheres; ++i) {
        double t;
        if (sphere64(o, d, S.spheres[i], tmin, h.t, t)) {
            h.t = t;
            h.prim = PG_SPHERE_BIT | i;
            if (any) return h;
        }
    }
    const Node *nodes = (const Node *)S.nodes;
    const D3 inv = d3(1.0 / d.x, 1.0 / d.y, 1.0 / d.z);
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const Node &n = nodes[stack[--sp]];
        for (int c = 0; c < 4; ++c) {
            if (n.count[c] <= 0 && n.child[c] < 0) continue;  // empty slot
            const float lo[3] = {n.lo[0][c], n.lo[1][c], n.lo[2][c]}, hi[3] = {n.hi[0][c], n.hi[1][c], n.hi[2][c]};
            if (!box64(o, inv, lo, hi, tmin, h.t)) continue;
            if (n.count[c] > 0) {
                for (int k = 0; k < n.count[c]; ++k) {
                    const float *tv = S.tri_verts + 12 * (size_t)(n.child[c] + k);
                    double t, bu, bv;
                    if (tri64(o, d, fv(tv), fv(tv + 4), fv(tv + 8), tmin, h.t, t, bu, bv) &&
                        (tri_tex(tv) == 0u ||
                         alpha_keep(S, (float)o.x, fbits(tv[3]), tri_tex(tv), (float)bu, (float)bv, (float)t))) {
                        h.t = t;
                        h.prim = fbits(tv[3]);
                        h.u = bu;
                        h.v = bv;
                        if (any) return h;
                    }
                }
            } else if (n.child[c] >= 0 && sp < 128) {
                stack[sp++] = n.child[c];
            }
        }
    }
    return h;
}

void frame(D3 n, D3 &x, D3 &y) {
    if (fabs(n.x) > fabs(n.y)) {
        const double inv = 1.0 / sqrt(n.x * n.x + n.z * n.z);
        y = d3(n.z * inv, 0.0, -n.x * inv);
    } else {
        const double inv = 1.0 / sqrt(n.y * n.y + n.z * n.z);
        y = d3(0.0, n.z * inv, -n.y * inv);
    }
    x = cross(y, n);
}
D3 to_world(D3 l, D3 n) {
    D3 x, y;
    frame(n, x, y);
    return x * l.x + y * l.y + n * l.z;
}
D3 reflect(D3 i, D3 n) { return i - n * (2.0 * dot(n, i)); }

double fresnel(double eta, double ci) {
    const double s2 = eta * eta * (1.0 - ci * ci);
    if (s2 > 1.0) return 1.0;
    const double ct = sqrt(1.0 - s2);
    const double rs = (eta * ci - ct) / (eta * ci + ct), rp = (ci - eta * ct) / (ci + eta * ct);
    return 0.5 * (rs * rs + rp * rp);
}

// Fresnel of a conductor (raytrace.rgen:163-176), one spectrum value of eta and k
double fresnel_conductor(double ci, double eta, double k) {
    ci = fabs(ci);
    const double ek = eta * eta + k * k, c2 = ci * ci;
    const double rs2 = (ek * c2 - 2.0 * eta * ci + 1.0) / (ek * c2 + 2.0 * eta * ci + 1.0);
    const double rp2 = (ek - 2.0 * eta * ci + c2) / (ek + 2.0 * eta * ci + c2);
    return 0.5 * (rs2 + rp2);
}

// the reference's Beckmann D and G1 as written (raytrace.rgen:178-231): the
// tangent of the cosine dot(v, n), and 2.577 a in the denominator
double beckmann_D(double alpha, double c) {
    if (c <= 0.0) return 0.0;
    const double c2 = c * c, t2 = std::max(1.0 - c2, 0.0) / c2, a2 = alpha * alpha;
    return exp(-t2 / a2) / (PI * a2 * c2 * c2);
}
double beckmann_G1(double alpha, D3 n, D3 m, D3 v) {
    const double tv = dot(v, n);
    const double c = dot(v, m) / tv;
    if (c <= 0.0) return 0.0;
    const double a = 1.0 / (alpha * tan(tv));
    if (a >= 1.6) return 1.0;
    return (3.535 * a + 2.181 * a * a) / (1.0 + 2.276 * a + 2.577 * a);
}

struct Eval {
    D3 f;
    double pdf;
};
Eval bsdf(const pg_material &m, D3 n, D3 wi, D3 wo) {
    Eval r{d3(0, 0, 0), 0.0};
    const double co = dot(n, wo), ci = dot(n, wi);
    if (co <= 0 || ci <= 0) return r;
    if (m.type == PG_MAT_DIFFUSE) {
        r.f = fv(m.albedo) * (co / PI);
        r.pdf = co / PI;
    } else if (m.type == PG_MAT_GGX) {
        const D3 h = unit(wi + wo);
        const double a2 = std::max((double)m.roughness * m.roughness, 1e-12);
        const double ch = dot(n, h), hi = dot(wi, h);
        const double dd = ch * ch * (a2 - 1.0) + 1.0;
        const double D = a2 / (PI * dd * dd);
        auto G1 = [&](double c) {
            c = fabs(c);
            return 2.0 * c / (c + sqrt(a2 + (1.0 - a2) * c * c));
        };
        const double G = G1(ci) * G1(co);
        const double w = pow(1.0 - std::max(hi, 0.0), 5.0);
        const D3 F = d3(m.albedo[0] + (1 - m.albedo[0]) * w, m.albedo[1] + (1 - m.albedo[1]) * w,
                        m.albedo[2] + (1 - m.albedo[2]) * w);
        r.f = F * (D * G / (4.0 * ci));
        r.pdf = D * ch / (4.0 * fabs(hi));
    } else if (m.type == PG_MAT_BECKMANN) {
        const D3 h = unit(wi + wo);
        const double D = beckmann_D(m.roughness, dot(n, h));
        double G = beckmann_G1(m.roughness, n, h, wi) * beckmann_G1(m.roughness, n, h, wo);
        G = G < 0.0 ? 0.0 : G;
        const double v = fresnel_conductor(dot(wi, h), m.eta, m.k) * G * D / (4.0 * ci);
        r.f = std::isnan(v) ? d3(0, 0, 0) : d3(v, v, v);
        const double pm = D * fabs(dot(h, n)), oh = dot(wo, h);
        r.pdf = (pm <= 0.0 || oh <= 0.0) ? 0.0 : pm / (4.0 * fabs(oh));
    } else if (m.type == PG_MAT_PHONG) {
        const D3 kd = fv(m.albedo), ks = fv(m.specular);
        D3 res = kd * (1.0 / PI);
        const double rw = dot(reflect(wo * -1.0, n), wi);
        if (rw > 0.0) res = res + ks * ((m.exponent + 2.0) / (2.0 * PI) * pow(rw, (double)m.exponent));
        r.f = res * co;
        const double ld = sqrt(dot(kd, kd)), ls = sqrt(dot(ks, ks)), sum = ld + ls;
        if (sum > 0.0) {
            const double rr = dot(reflect(wi * -1.0, n), wo);
            const double pdf = rr > 0.0 ? (m.exponent + 1.0) * pow(rr, (double)m.exponent) / (2.0 * PI) * (ls / sum) : 0.0;
            r.pdf = pdf + co / PI * (ld / sum);
        }
    }
    return r;
}

bool is_delta(const pg_material &m) {
    return m.type == PG_MAT_DIELECTRIC || m.type == PG_MAT_SPECULAR || m.type == PG_MAT_CONDUCTOR;
}
bool almost_delta(const pg_material &m) {
    return ((m.type == PG_MAT_GGX || m.type == PG_MAT_BECKMANN) && m.roughness <= 0.3f) ||
           (m.type == PG_MAT_PHONG && m.exponent >= 250.0f);
}
// guiding follows the recording rule (not on discrete or almost-discrete
// lobes) unless PG_RENDER_GUIDE_ALMOST_DISCRETE asks for the reference's rule
bool guided_material(const pg_material &m, uint32_t flags) {
    return !is_delta(m) && ((flags & PG_RENDER_GUIDE_ALMOST_DISCRETE) || !almost_delta(m));
}

D3 sample_bsdf(const pg_material &m, D3 d, D3 n, double ul, double u1, double u2) {
    if (m.type == PG_MAT_PHONG) {
        const D3 kd = fv(m.albedo), ks = fv(m.specular);
        const double ld = sqrt(dot(kd, kd)), ls = sqrt(dot(ks, ks));
        if (ul * (ld + ls) > ld) {
            const double ct = pow(u1, 1.0 / (m.exponent + 1.0)), st = sqrt(std::max(0.0, 1.0 - ct * ct));
            const double ph = 2.0 * PI * u2;
            return to_world(d3(st * cos(ph), st * sin(ph), ct), reflect(d, n));
        }
    }
    if (m.type == PG_MAT_DIFFUSE || m.type == PG_MAT_PHONG) {
        const double sr = sqrt(u1), ph = 2.0 * PI * u2;
        return to_world(d3(sr * cos(ph), sr * sin(ph), sqrt(std::max(0.0, 1.0 - u1))), n);
    }
    if (m.type == PG_MAT_BECKMANN) {
        const double th = atan(sqrt(-(double)m.roughness * m.roughness * log(1.0 - u1))), ph = 2.0 * PI * u2;
        const D3 mh = to_world(d3(sin(th) * cos(ph), sin(th) * sin(ph), cos(th)), n);
        return reflect(d, mh);
    }
    const double a2 = std::max((double)m.roughness * m.roughness, 1e-12);
    const double t2 = a2 * u1 / std::max(1.0 - u1, 1e-12);
    const double cm = 1.0 / sqrt(1.0 + t2), sm = sqrt(std::max(0.0, 1.0 - cm * cm)), ph = 2.0 * PI * u2;
    return reflect(d, to_world(d3(sm * cos(ph), sm * sin(ph), cm), n));
}

uint32_t region_of(const pgo_guide &g, D3 p) {
    float lo[3] = {g.root[0], g.root[1], g.root[2]}, hi[3] = {g.root[3], g.root[4], g.root[5]};
    const float pp[3] = {(float)p.x, (float)p.y, (float)p.z};
    if (g.nodes) return pgo_region_of(g.root, g.nodes, pp);
    for (int i = 0; i < 3; ++i)
        if (!(pp[i] >= lo[i] && pp[i] <= hi[i])) return PG_INVALID_REGION;
    uint32_t id = 0;
    for (uint32_t l = 0; l < g.split_count; ++l) {
        float size[3];
        for (int i = 0; i < 3; ++i) size[i] = hi[i] - lo[i];
        const int ax = size[0] > size[1] ? (size[0] > size[2] ? 0 : 2) : (size[1] > size[2] ? 1 : 2);
        const float lhi = hi[ax] - 0.5f * size[ax];
        const float rlo = lo[ax] + 0.5f * size[ax];
        if (pp[ax] <= lhi) {
            hi[ax] = lhi;
            id = 2 * id;
        } else if (pp[ax] >= rlo) {
            lo[ax] = rlo;
            id = 2 * id + 1;
        } else {
            return PG_INVALID_REGION;
        }
    }
    return id;
}

D3 lobe_mu(const pg_vmf_theta &t, D3 x, int par) {
    D3 mu = fv(t.mu);
    if (par && t.distance > 0.0f) mu = unit(fv(t.target) - x);
    return mu;
}
double vmm_pdf(const pg_vmm_theta &v, D3 wo, D3 x, int par) {
    double res = 0.0;
    for (int i = 0; i < std::min(v.used_distributions, 16); ++i) {
        const pg_vmf_theta &t = v.thetas[i];
        const double f = t.k == 0.0f ? 1.0 / (4.0 * PI) : t.norm * exp(t.k * (dot(lobe_mu(t, x, par), wo) - 1.0));
        res += v.pi[i] * f;
    }
    return res;
}
D3 vmm_sample(const pg_vmm_theta &v, D3 x, int par, double ul, double u1, double u2) {
    const int K = std::min(v.used_distributions, 16);
    int i = 0;
    double acc = v.pi[0];
    while (acc < ul && i < K - 1) acc += v.pi[++i];
    const pg_vmf_theta &t = v.thetas[i];
    if (t.k > 0.0f) {
        const double ct = 1.0 + log(1.0 + t.e_min2k * u1 - u1) / t.k;
        const double st = 1.0 - ct * ct <= 0.0 ? 0.0 : sqrt(1.0 - ct * ct);
        const double ph = 2.0 * PI * u2;
        return to_world(d3(st * cos(ph), st * sin(ph), ct), lobe_mu(t, x, par));
    }
    const double z = 1.0 - 2.0 * u1, r = sqrt(std::max(0.0, 1.0 - z * z)), ph = 2.0 * PI * u2;
    return d3(r * cos(ph), r * sin(ph), z);
}

// The continuation of a path at a vertex: getNewDirection (raytrace.rgen:
// 923-960) and the throughput change evalBsdf / pdf (:1176), the estimator's
// choices as the device makes them (delta materials reflect or refract, a
// guided vertex without a region ends the path, draw_ua() supplies the lobe
// choice only when the guide is sampled).
struct Continuation {
    D3 wo;
    double pdf;
    D3 tc;
    bool delta;
};
template <typename DrawUa>
Continuation continue_path(const pg_material &m, D3 d, D3 n, bool front, D3 x, bool gm, const pg_vmm_theta *mix,
                           int par, double guiding_prob, double uch, double ul, double u1, double u2,
                           DrawUa draw_ua) {
    Continuation c{d3(0, 0, 1), 0.0, d3(0, 0, 0), false};
    const D3 wi = d * -1.0;
    if (m.type == PG_MAT_DIELECTRIC) {
        const double eta = front ? 1.0 / m.ior : m.ior;
        const double ci = dot(wi, n);
        const double F = fresnel(eta, ci);
        if (ul > F) {
            const double k = 1.0 - eta * eta * (1.0 - ci * ci);
            c.wo = k < 0.0 ? reflect(d, n) : unit(d * eta - n * (eta * (-ci) + sqrt(std::max(k, 0.0))));
        } else {
            c.wo = reflect(d, n);
        }
        c.pdf = 1.0;
        c.tc = fv(m.albedo);
        c.delta = true;
    } else if (m.type == PG_MAT_SPECULAR) {
        c.wo = reflect(d, n);
        c.pdf = 1.0;
        c.tc = fv(m.albedo);
        c.delta = true;
    } else if (m.type == PG_MAT_CONDUCTOR) {
        c.wo = reflect(d, n);
        c.pdf = 1.0;
        const double F = fresnel_conductor(dot(wi, n), m.eta, m.k);
        c.tc = d3(F, F, F);
        c.delta = true;
    } else {
        if (gm && !mix) return c;
        const bool use_guide = gm && uch < guiding_prob;
        D3 wo = use_guide ? vmm_sample(*mix, x, par, draw_ua(), u1, u2) : sample_bsdf(m, d, n, ul, u1, u2);
        Eval me = bsdf(m, n, wi, wo);
        double pdf = me.pdf;
        if (gm) {
            if (dot(wo, n) < 0.0 || me.pdf <= 0.0) {
                pdf = 0.0;
            } else {
                const double pg = vmm_pdf(*mix, wo, x, par);
                if (std::isnan(pg)) {
                    if (use_guide) {
                        wo = sample_bsdf(m, d, n, ul, u1, u2);
                        me = bsdf(m, n, wi, wo);
                    }
                    pdf = me.pdf;
                } else {
                    pdf = (1.0 - guiding_prob) * me.pdf + guiding_prob * pg;
                }
            }
        }
        c.wo = wo;
        if (dot(wo, n) > 0.0 && pdf > 0.0 && me.pdf > 0.0) {
            c.tc = me.f * (1.0 / pdf);
            c.pdf = pdf;
        }
    }
    return c;
}

// the lat-long environment along d (raytrace.rmiss), bilinear with wrap-around
D3 env_radiance(const pgo_scene &S, D3 d) {
    const double u = atan2(d.x, -d.z) / (2.0 * PI), v = acos(std::min(std::max(d.y, -1.0), 1.0)) / PI;
    const double sx = u * S.env_w - 0.5, sy = v * S.env_h - 0.5;
    const double fx0 = floor(sx), fy0 = floor(sy), fx = sx - fx0, fy = sy - fy0;
    const long W = S.env_w, H = S.env_h;
    long x0 = (long)fx0 % W, y0 = (long)fy0 % H;
    x0 += x0 < 0 ? W : 0;
    y0 += y0 < 0 ? H : 0;
    const long x1 = x0 + 1 == W ? 0 : x0 + 1, y1 = y0 + 1 == H ? 0 : y0 + 1;
    auto tx = [&](long x, long y) { return fv(S.env + 3 * (size_t)(y * W + x)); };
    return (tx(x0, y0) * (1.0 - fx) + tx(x1, y0) * fx) * (1.0 - fy) + (tx(x0, y1) * (1.0 - fx) + tx(x1, y1) * fx) * fy;
}

D3 render_pixel(const Scene64 &sc, const pg_render_params &rp, const pgo_guide *g, uint32_t pix, uint32_t smp) {
    const pgo_scene &S = *sc.S;
    const pg_camera &cam = S.camera;
    const uint32_t W = cam.width, H = cam.height, px = pix % W, py = pix / W;
    const D3 f = unit(fv(cam.target) - fv(cam.origin));
    const D3 r = unit(cross(f, fv(cam.up)));
    const D3 u = cross(r, f);
    const double th = tan(cam.vfov_deg * 0.5 * PI / 180.0), aspect = (double)W / H;
    const double jx = rnd(rp.seed, pix, smp, 0) - 0.5, jy = rnd(rp.seed, pix, smp, 1) - 0.5;
    const double sx = (2.0 * (px + 0.5 + jx) / W - 1.0) * th * aspect;
    const double sy = (1.0 - 2.0 * (py + 0.5 + jy) / H) * th;
    D3 o = fv(cam.origin), d = unit(f + r * sx + u * sy), thr = d3(1, 1, 1), L = d3(0, 0, 0);
    double prev_pdf = 0.0;
    const uint32_t nL = (uint32_t)sc.lights.size();
    const int par = g ? g->use_parallax : 0;
    for (int b = 0; b < (int)rp.max_depth; ++b) {
        const bool last = b + 1 == (int)rp.max_depth;
        const Hit64 h = intersect64(S, o, d, 0.001, 1e6, false);
        if (h.prim == PG_NO_HIT) {
            if (S.env && S.env_w) {
                double w = 1.0;
                if (rp.use_nee && prev_pdf > 0.0) {
                    const double pl = 1.0 / (2.0 * PI) / nL;
                    w = rp.use_mis ? prev_pdf * prev_pdf / (prev_pdf * prev_pdf + pl * pl) : 0.0;
                }
                L = L + hm(thr, env_radiance(S, d) * w);
            }
            break;
        }
        const D3 x = o + d * h.t;
        D3 ng;
        uint32_t mat_id;
        if (h.prim & PG_SPHERE_BIT) {
            const pg_sphere &sp = S.spheres[h.prim & ~PG_SPHERE_BIT];
            ng = (x - fv(sp.center)) * (1.0 / sp.radius);
            mat_id = sp.material;
        } else {
            const uint32_t t = h.prim;
            const D3 v0 = fv(S.pos + 3 * (size_t)S.idx[3 * t]), v1 = fv(S.pos + 3 * (size_t)S.idx[3 * t + 1]),
                     v2 = fv(S.pos + 3 * (size_t)S.idx[3 * t + 2]);
            ng = unit(cross(v1 - v0, v2 - v0));
            mat_id = S.tri_mat[t];
        }
        pg_material m = S.mats[mat_id];
        if (m.texture > 0 && !(h.prim & PG_SPHERE_BIT) && (m.type == PG_MAT_DIFFUSE || m.type == PG_MAT_PHONG)) {
            // diffuse reflectance times the texture (raytrace.rgen:233-249)
            const D3 tc = tex_rgb64(S, h.prim, (uint32_t)m.texture - 1u, h.u, h.v);
            m.albedo[0] = (float)(m.albedo[0] * tc.x);
            m.albedo[1] = (float)(m.albedo[1] * tc.y);
            m.albedo[2] = (float)(m.albedo[2] * tc.z);
        }
        const bool front = dot(d, ng) < 0.0;
        const D3 n = front ? ng : ng * -1.0;
        const D3 wi = d * -1.0;
        if (m.type == PG_MAT_LIGHT) {
            double w = 1.0;
            if (rp.use_nee && prev_pdf > 0.0) {
                if (!rp.use_mis) {
                    w = 0.0;
                } else {
                    int lid = -1;
                    if (h.prim & PG_SPHERE_BIT) {
                        for (uint32_t l = 0; l < nL; ++l)
                            if (sc.lights[l].type == 1 && sc.lights[l].sphere == (h.prim & ~PG_SPHERE_BIT)) lid = (int)l;
                    } else {
                        lid = sc.tri_light[h.prim];
                    }
                    if (lid >= 0) {
                        const double cl = fabs(dot(ng, d));
                        const double pl = h.t * h.t / (std::max(cl, 1e-12) * sc.lights[lid].area) / nL;
                        w = prev_pdf * prev_pdf / (prev_pdf * prev_pdf + pl * pl);
                    }
                }
            }
            if (front || (h.prim & PG_SPHERE_BIT) == 0) L = L + hm(thr, fv(m.emission) * w);
            break;
        }
        if (last) break;
        if (rp.use_nee && !is_delta(m) && nL > 0) {
            const uint32_t l = std::min((uint32_t)(rnd(rp.seed, pix, smp, dimb(b, 0)) * nL), nL - 1);
            const Light &Li = sc.lights[l];
            const double u1 = rnd(rp.seed, pix, smp, dimb(b, 1)), u2 = rnd(rp.seed, pix, smp, dimb(b, 2));
            D3 lp, ln;
            if (Li.type == 2) {
                const double ct = u1, st = sqrt(std::max(0.0, 1.0 - ct * ct)), ph = 2.0 * PI * u2;
                const D3 wl = to_world(d3(st * cos(ph), st * sin(ph), ct), n);
                const double pl = 1.0 / (2.0 * PI) / nL;
                const Eval me = bsdf(m, n, wi, wl);
                if (mx(me.f) > 0.0) {
                    double pb = me.pdf;
                    if (rp.use_guiding && g && guided_material(m, rp.flags)) {
                        const uint32_t reg = region_of(*g, x);
                        if (reg != PG_INVALID_REGION) {
                            const double pg = vmm_pdf(g->vmm[reg], wl, x, par);
                            if (!std::isnan(pg)) pb = (1.0 - rp.guiding_prob) * pb + rp.guiding_prob * pg;
                        }
                    }
                    const double w = rp.use_mis ? pl * pl / (pl * pl + pb * pb) : 1.0;
                    if (intersect64(S, x, wl, 0.001, 1e30, true).prim == PG_NO_HIT)
                        L = L + hm(thr, hm(me.f, env_radiance(S, wl)) * (w / pl));
                }
            } else {
            if (Li.type == 1) {
                const pg_sphere &sp = S.spheres[Li.sphere];
                const double z = 1.0 - 2.0 * u1, rr = sqrt(std::max(0.0, 1.0 - z * z)), ph = 2.0 * PI * u2;
                ln = d3(rr * cos(ph), rr * sin(ph), z);
                lp = fv(sp.center) + ln * sp.radius;
            } else {
                const size_t k = std::min<size_t>(std::lower_bound(Li.cdf.begin(), Li.cdf.end(), u1) - Li.cdf.begin(),
                                                  Li.cdf.size() - 1);
                const double c0 = k == 0 ? 0.0 : Li.cdf[k - 1], c1 = Li.cdf[k];
                const double ur = c1 > c0 ? std::min((u1 - c0) / (c1 - c0), 0.99999994) : 0.5;
                const uint32_t t = Li.tris[k];
                const D3 a = fv(S.pos + 3 * (size_t)S.idx[3 * t]), bb = fv(S.pos + 3 * (size_t)S.idx[3 * t + 1]),
                         c = fv(S.pos + 3 * (size_t)S.idx[3 * t + 2]);
                const double sx2 = sqrt(ur);
                lp = a * (1.0 - sx2) + bb * (sx2 * (1.0 - u2)) + c * (u2 * sx2);
                ln = unit(cross(bb - a, c - a));
            }
            const D3 tl = lp - x;
            const double dist2 = dot(tl, tl), dist = sqrt(dist2);
            const D3 wl = tl * (1.0 / dist);
            double cl = -dot(wl, ln);
            if (Li.type == 0) cl = fabs(cl);
            if (cl > 0.0 && dot(n, wl) > 0.0) {
                const double pl = dist2 / (cl * Li.area) / nL;
                const Eval me = bsdf(m, n, wi, wl);
                if (mx(me.f) > 0.0) {
                    double pb = me.pdf;
                    if (rp.use_guiding && g && guided_material(m, rp.flags)) {
                        const uint32_t reg = region_of(*g, x);
                        if (reg != PG_INVALID_REGION) {
                            const double pg = vmm_pdf(g->vmm[reg], wl, x, par);
                            if (!std::isnan(pg)) pb = (1.0 - rp.guiding_prob) * pb + rp.guiding_prob * pg;
                        }
                    }
                    const double w = rp.use_mis ? pl * pl / (pl * pl + pb * pb) : 1.0;
                    if (intersect64(S, x, wl, 0.001, dist * (1.0 - 0.0001), true).prim == PG_NO_HIT)
                        L = L + hm(thr, hm(me.f, Li.emission) * (w / pl));
                }
            }
            }
        }
        const double uch = rnd(rp.seed, pix, smp, dimb(b, 3)), ul = rnd(rp.seed, pix, smp, dimb(b, 4));
        const double u1 = rnd(rp.seed, pix, smp, dimb(b, 5)), u2 = rnd(rp.seed, pix, smp, dimb(b, 6));
        const bool gm = rp.use_guiding && g && guided_material(m, rp.flags);
        const pg_vmm_theta *mix = nullptr;
        if (gm) {
            const uint32_t reg = region_of(*g, x);
            if (reg != PG_INVALID_REGION) mix = &g->vmm[reg];
        }
        const Continuation cn = continue_path(m, d, n, front, x, gm, mix, par, rp.guiding_prob, uch, ul, u1, u2,
                                              [&] { return rnd(rp.seed, pix, smp, dimb(b, 7)); });
        const D3 wo = cn.wo, tc = cn.tc;
        const double pdf = cn.pdf;
        const bool delta = cn.delta;
        if (!(pdf > 0.0 && mx(tc) > 0.0)) break;
        thr = hm(thr, tc);
        o = x;
        d = wo;
        prev_pdf = delta ? 0.0 : pdf;
    }
    return L;
}

}  // namespace

extern "C" {

void pgo_probe_shading(const pg_material *mats, uint32_t n_mats, const pg_vmm_theta *vmms, uint32_t n_vmms,
                       const pg_shading_probe *P, uint32_t count, double *out) {
    for (uint32_t i = 0; i < count; ++i) {
        const pg_shading_probe &q = P[i];
        double *r = out + 8 * i;
        for (int k = 0; k < 8; ++k) r[k] = 0.0;
        const bool uses_mat = q.op == PG_PROBE_BSDF_EVAL || q.op == PG_PROBE_BSDF_SAMPLE || q.op == PG_PROBE_CONTINUE ||
                              q.op == PG_PROBE_APPROX_DIFFUSE;
        const bool uses_vmm = q.op == PG_PROBE_VMM_PDF || q.op == PG_PROBE_VMM_SAMPLE ||
                              (q.op == PG_PROBE_CONTINUE && (q.flags & 8u));
        if ((uses_mat && q.material >= n_mats) || (uses_vmm && q.vmm >= n_vmms)) {
            for (int k = 0; k < 8; ++k) r[k] = NAN;
            continue;
        }
        const D3 n = fv(q.n), wi = fv(q.wi), wo = fv(q.wo), x = fv(q.x);
        const bool front = (q.flags & 1u) != 0;
        const int par = (q.flags & 2u) ? 1 : 0;
        auto put = [&](int at, D3 v) {
            r[at] = v.x;
            r[at + 1] = v.y;
            r[at + 2] = v.z;
        };
        switch (q.op) {
            case PG_PROBE_FRESNEL:
                r[0] = fresnel(q.a, q.b);
                break;
            case PG_PROBE_FRESNEL_CONDUCTOR:
                r[0] = fresnel_conductor(q.a, q.b, q.c);
                break;
            case PG_PROBE_BSDF_EVAL: {
                const Eval e = bsdf(mats[q.material], n, wi, wo);
                put(0, e.f);
                r[3] = e.pdf;
                break;
            }
            case PG_PROBE_BSDF_SAMPLE: {
                const pg_material &m = mats[q.material];
                const D3 w = sample_bsdf(m, wi * -1.0, n, q.u[1], q.u[2], q.u[3]);
                put(0, w);
                r[3] = bsdf(m, n, wi, w).pdf;
                break;
            }
            case PG_PROBE_VMM_PDF:
                r[0] = vmm_pdf(vmms[q.vmm], wo, x, par);
                break;
            case PG_PROBE_VMM_SAMPLE:
                put(0, vmm_sample(vmms[q.vmm], x, par, q.u[4], q.u[2], q.u[3]));
                break;
            case PG_PROBE_CONTINUE: {
                const pg_material &m = mats[q.material];
                const uint32_t rf = (q.flags & 16u) ? PG_RENDER_GUIDE_ALMOST_DISCRETE : 0u;
                const bool gm = (q.flags & 4u) && guided_material(m, rf);
                const pg_vmm_theta *mix = (q.flags & 8u) ? &vmms[q.vmm] : nullptr;
                const double ua = q.u[4];
                const Continuation c = continue_path(m, wi * -1.0, n, front, x, gm, mix, par, q.c, q.u[0], q.u[1],
                                                     q.u[2], q.u[3], [&] { return ua; });
                put(0, c.wo);
                r[3] = c.pdf;
                put(4, c.tc);
                break;
            }
            case PG_PROBE_TO_WORLD:
                put(0, to_world(wo, n));
                break;
            case PG_PROBE_WEIGHT_WINDOW: {
                // applyWeightWindow (raytrace.rgen:830-869)
                const D3 r3 = d3(x.x / wo.x, x.y / wo.y, x.z / wo.z);
                const double center = sqrt(dot(r3, r3));
                const double s = q.a, lower = 2.0 * center / (1.0 + s), upper = s * lower;
                const double v = sqrt(dot(wi, wi));
                double qq = 1.0;
                int nn = 1;
                if (std::isnan(lower) || lower <= 0.0 || (lower <= v && v <= upper)) {
                    qq = 1.0;
                } else if (v <= lower) {
                    qq = std::max(v / lower, 0.1);
                } else {
                    qq = v / upper;
                    nn = (int)qq;
                    if (q.u[0] > (double)(nn + 1) - qq) ++nn;
                }
                r[0] = qq;
                r[1] = nn;
                break;
            }
            case PG_PROBE_APPROX_DIFFUSE: {
                // approxDiffuse (raytrace.rgen:815-828); GGX: its tint / pi
                const pg_material &m = mats[q.material];
                if (m.type == PG_MAT_BECKMANN) {
                    const double F = fresnel_conductor(dot(wi, n), m.eta, m.k) / PI;
                    put(0, d3(F, F, F));
                } else {
                    put(0, d3(m.albedo[0] / PI, m.albedo[1] / PI, m.albedo[2] / PI));
                }
                break;
            }
            default:
                break;
        }
    }
}

float pgo_rnd(uint32_t seed, uint32_t pixel, uint32_t sample, uint32_t dim) { return (float)rnd(seed, pixel, sample, dim); }

void pgo_trace_closest(const pgo_scene *s, const pg_ray *rays, uint32_t n, pg_hit *hits, int n_threads) {
    parallel_for(n, n_threads, [&](uint32_t i) { closest32(*s, rays[i], hits[i]); });
}

void pgo_trace_closest_counted(const pgo_scene *s, const pg_ray *rays, uint32_t n, pg_hit *hits, uint32_t *nodes,
                               uint32_t *tris, int n_threads) {
    parallel_for(n, n_threads, [&](uint32_t i) {
        uint32_t c[2];
        closest32(*s, rays[i], hits[i], c);
        nodes[i] = c[0];
        tris[i] = c[1];
    });
}

void pgo_trace_any(const pgo_scene *s, const pg_ray *rays, uint32_t n, uint32_t *occ, int n_threads) {
    parallel_for(n, n_threads, [&](uint32_t i) { occ[i] = any32(*s, rays[i]) ? 1u : 0u; });
}

void pgo_render_f64(const pgo_scene *s, const pg_render_params *rp, const pgo_guide *guide, double *image,
                    uint32_t row_begin, uint32_t row_end, int n_threads) {
    Scene64 sc;
    pgo_scene sa = *s;  // the frame's alpha-test salt, as the device renderer derives it
    sa.alpha_salt = fmix32(rp->seed ^ 0x5bd1e995u);
    sc.S = &sa;
    sc.tri_light.assign(s->n_tris, -1);
    // lights: one per emissive material over triangles (area-weighted), one per emissive sphere
    for (uint32_t m = 0; m < s->n_mats; ++m) {
        if (s->mats[m].type != PG_MAT_LIGHT) continue;
        Light L;
        L.type = 0;
        double acc = 0.0;
        for (uint32_t t = 0; t < s->n_tris; ++t) {
            if (s->tri_mat[t] != m) continue;
            const D3 a = fv(s->pos + 3 * (size_t)s->idx[3 * t]), b = fv(s->pos + 3 * (size_t)s->idx[3 * t + 1]),
                     c = fv(s->pos + 3 * (size_t)s->idx[3 * t + 2]);
            acc += 0.5 * sqrt(dot(cross(b - a, c - a), cross(b - a, c - a)));
            L.tris.push_back(t);
            L.cdf.push_back(acc);
            sc.tri_light[t] = (int)sc.lights.size();
        }
        if (L.tris.empty()) continue;
        for (double &c : L.cdf) c /= acc;
        L.cdf.back() = 1.0;
        L.area = acc;
        L.emission = fv(s->mats[m].emission);
        sc.lights.push_back(L);
    }
    for (uint32_t i = 0; i < s->n_spheres; ++i) {
        const pg_material &m = s->mats[s->spheres[i].material];
        if (m.type != PG_MAT_LIGHT) continue;
        Light L;
        L.type = 1;
        L.sphere = i;
        L.area = 4.0 * PI * (double)s->spheres[i].radius * s->spheres[i].radius;
        L.emission = fv(m.emission);
        sc.lights.push_back(L);
    }
    if (s->env && s->env_w && s->env_h) {  // the environment is the last light
        Light L;
        L.type = 2;
        L.sphere = 0;
        L.area = 0.0;
        L.emission = d3(0, 0, 0);
        sc.lights.push_back(L);
    }
    const uint32_t W = s->camera.width;
    row_end = std::min(row_end, s->camera.height);
    if (row_begin >= row_end) return;
    const uint32_t n = (row_end - row_begin) * W;
    parallel_for(n, n_threads, [&](uint32_t i) {
        const uint32_t pix = row_begin * W + i;
        D3 acc = d3(0, 0, 0);
        for (uint32_t smp = 0; smp < rp->spp; ++smp) acc = acc + render_pixel(sc, *rp, guide, pix, smp);
        image[3 * (size_t)pix] = acc.x;
        image[3 * (size_t)pix + 1] = acc.y;
        image[3 * (size_t)pix + 2] = acc.z;
    });
}

}  // extern "C"
