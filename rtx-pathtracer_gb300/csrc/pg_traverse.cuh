// pg_traverse.cuh - BVH traversal and ray-primitive tests on the device.
//
// Closest hit and any hit over the four-wide BVH of host/pg_scene.cpp.  The
// triangle test is the watertight algorithm of Woop, Benthin and Wald (JCGT
// 2013).  Every operation of the triangle and box tests is an explicit
// round-to-nearest one (__fmul_rn, __fadd_rn, __fmaf_rn, __fdiv_rn, ...), so the
// compiler contracts nothing and a CPU restatement with the same operations in
// the same order (fmaf where these use __fmaf_rn) reproduces the hit (triangle
// id and t) bit for bit.  The per-vertex shear and the numerator of t are fused
// multiply-adds; the edge functions are not, so an edge shared by two triangles
// gives exactly negated values in both (watertightness), nor is the slab test,
// whose widening bounds the error of a subtraction and a product.  Ties in t go
// to the lower triangle id.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pathguide.h"

namespace pg {

// Four-wide node (the host BvhNode): child boxes slot-major per coordinate.
struct DevBvhNode {
    float4 lox, loy, loz;
    float4 hix, hiy, hiz;
    int4 child;
    int4 count;
};
static_assert(sizeof(DevBvhNode) == 128, "node layout");

struct DevScene {
    const DevBvhNode *nodes;
    const float4 *tris;           // 3 float4 per triangle in BVH order; tris[3i].w = original id (bits),
                                  // tris[3i+1].w = the material's texture (bits; 0 none)
    const pg_sphere *spheres;
    uint32_t n_spheres;
    uint32_t n_triangles;
    const float *tri_uv;          // 6 per original triangle
    const uint4 *tex_info;        // per texture: first texel, width, height
    const uchar4 *tex_data;       // RGBA8 texels, rows from the top
    uint32_t alpha_salt;          // per-frame salt of the alpha test's hash
};

// ---- alpha-tested hits (raytrace.rahit:21-46) --------------------------------
// A hit on a textured triangle is ignored when a hash of (texture u, origin.x *
// t) and the frame's salt, as a number in [0, 1), exceeds the texture's alpha
// at the hit.  The arithmetic is spelled out with round-to-nearest operations
// so the CPU traversal twin reproduces every decision.
__host__ __device__ __forceinline__ uint32_t tea16(uint32_t v0, uint32_t v1) {
    uint32_t s0 = 0;
    for (int n = 0; n < 16; ++n) {
        s0 += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}

// Bilinear alpha (repeat addressing, texel centres at half-integers) of texture
// info {first, w, h} at (u, v).
__device__ __forceinline__ float tex_alpha(const DevScene &S, uint32_t tex, float u, float v) {
    const uint4 ti = __ldg(&S.tex_info[tex]);
    const int w = (int)ti.y, h = (int)ti.z;
    u = __fsub_rn(u, floorf(u));
    v = __fsub_rn(v, floorf(v));
    const float x = __fsub_rn(__fmul_rn(u, (float)w), 0.5f), y = __fsub_rn(__fmul_rn(v, (float)h), 0.5f);
    const float x0 = floorf(x), y0 = floorf(y);
    const float fx = __fsub_rn(x, x0), fy = __fsub_rn(y, y0);
    int ix0 = (int)x0, iy0 = (int)y0;
    int ix1 = ix0 + 1, iy1 = iy0 + 1;
    ix0 = ix0 < 0 ? ix0 + w : ix0;
    iy0 = iy0 < 0 ? iy0 + h : iy0;
    ix1 = ix1 >= w ? ix1 - w : ix1;
    iy1 = iy1 >= h ? iy1 - h : iy1;
    const uchar4 *d = S.tex_data + ti.x;
    const float k = 1.0f / 255.0f;
    const float a00 = __fmul_rn((float)__ldg(&d[iy0 * w + ix0]).w, k), a10 = __fmul_rn((float)__ldg(&d[iy0 * w + ix1]).w, k);
    const float a01 = __fmul_rn((float)__ldg(&d[iy1 * w + ix0]).w, k), a11 = __fmul_rn((float)__ldg(&d[iy1 * w + ix1]).w, k);
    const float gx = __fsub_rn(1.0f, fx), gy = __fsub_rn(1.0f, fy);
    const float top = __fadd_rn(__fmul_rn(a00, gx), __fmul_rn(a10, fx));
    const float bot = __fadd_rn(__fmul_rn(a01, gx), __fmul_rn(a11, fx));
    return __fadd_rn(__fmul_rn(top, gy), __fmul_rn(bot, fy));
}

// Whether the hit (barycentrics bu, bv of v1, v2; distance t) on original
// triangle `id` with texture `tex` (1-based) stands.
__device__ __noinline__ bool alpha_keep(const DevScene &S, const float org_x, uint32_t id, uint32_t tex, float bu,
                                           float bv, float t) {
    const float *uv = S.tri_uv + 6 * (size_t)id;
    const float w0 = __fsub_rn(__fsub_rn(1.0f, bu), bv);
    const float tu = __fadd_rn(__fadd_rn(__fmul_rn(__ldg(uv), w0), __fmul_rn(__ldg(uv + 2), bu)), __fmul_rn(__ldg(uv + 4), bv));
    const float tv = __fadd_rn(__fadd_rn(__fmul_rn(__ldg(uv + 1), w0), __fmul_rn(__ldg(uv + 3), bu)), __fmul_rn(__ldg(uv + 5), bv));
    const float a = tex_alpha(S, tex - 1u, tu, tv);
    // uint(textureUV * 1e8 + origin.x * t): the first component, converted through a
    // clamped 64-bit integer (the shader's conversion is undefined out of range)
    const float sx = fminf(fmaxf(__fadd_rn(__fmul_rn(tu, 100000000.0f), __fmul_rn(org_x, t)), -4.0e18f), 4.0e18f);
    uint32_t seed = tea16((uint32_t)(long long)sx, S.alpha_salt);
    seed = 1664525u * seed + 1013904223u;  // lcg, then rnd in [0, 1)
    const float r = (float)(seed & 0x00FFFFFFu) * (1.0f / 16777216.0f);
    return !(r > a);
}

struct RayPre {
    float org[3], dir[3], inv[3];
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

__device__ __forceinline__ RayPre ray_setup(const float o[3], const float d[3]) {
    RayPre r;
    for (int i = 0; i < 3; ++i) {
        r.org[i] = o[i];
        r.dir[i] = d[i];
        r.inv[i] = __fdiv_rn(1.0f, d[i]);
    }
    const float ax = fabsf(d[0]), ay = fabsf(d[1]), az = fabsf(d[2]);
    int kz = 0;
    if (ay > ax) kz = 1;
    if (az > fmaxf(ax, ay)) kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (d[kz] < 0.0f) {
        const int t = kx;
        kx = ky;
        ky = t;
    }
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.Sx = __fdiv_rn(d[kx], d[kz]);
    r.Sy = __fdiv_rn(d[ky], d[kz]);
    r.Sz = __fdiv_rn(1.0f, d[kz]);
    return r;
}

__device__ __forceinline__ float comp(const float4 &v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

// Watertight ray-triangle test; on a hit in (tmin, tmax) returns t and the
// barycentrics of v1 (u) and v2 (v).
__device__ __forceinline__ bool tri_intersect(const RayPre &r, const float4 &v0, const float4 &v1, const float4 &v2,
                                              float tmin, float tmax, float &t_out, float &u_out, float &v_out) {
    const float A[3] = {__fsub_rn(v0.x, r.org[0]), __fsub_rn(v0.y, r.org[1]), __fsub_rn(v0.z, r.org[2])};
    const float B[3] = {__fsub_rn(v1.x, r.org[0]), __fsub_rn(v1.y, r.org[1]), __fsub_rn(v1.z, r.org[2])};
    const float C[3] = {__fsub_rn(v2.x, r.org[0]), __fsub_rn(v2.y, r.org[1]), __fsub_rn(v2.z, r.org[2])};
    const float Akz = A[r.kz], Bkz = B[r.kz], Ckz = C[r.kz];
    const float Ax = __fmaf_rn(-r.Sx, Akz, A[r.kx]);
    const float Ay = __fmaf_rn(-r.Sy, Akz, A[r.ky]);
    const float Bx = __fmaf_rn(-r.Sx, Bkz, B[r.kx]);
    const float By = __fmaf_rn(-r.Sy, Bkz, B[r.ky]);
    const float Cx = __fmaf_rn(-r.Sx, Ckz, C[r.kx]);
    const float Cy = __fmaf_rn(-r.Sy, Ckz, C[r.ky]);
    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        // edge functions exactly zero: redo them in double (exact products)
        U = (float)__dsub_rn(__dmul_rn((double)Cx, (double)By), __dmul_rn((double)Cy, (double)Bx));
        V = (float)__dsub_rn(__dmul_rn((double)Ax, (double)Cy), __dmul_rn((double)Ay, (double)Cx));
        W = (float)__dsub_rn(__dmul_rn((double)Bx, (double)Ay), __dmul_rn((double)By, (double)Ax));
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.0f) return false;
    const float Az = __fmul_rn(r.Sz, Akz);
    const float Bz = __fmul_rn(r.Sz, Bkz);
    const float Cz = __fmul_rn(r.Sz, Ckz);
    const float T = __fmaf_rn(W, Cz, __fmaf_rn(V, Bz, __fmul_rn(U, Az)));
    const float t = __fdiv_rn(T, det);
    if (!(t > tmin && t < tmax)) return false;
    t_out = t;
    u_out = __fdiv_rn(V, det);
    v_out = __fdiv_rn(W, det);
    return true;
}

// Slab test with the exit distance widened by 4e-7 > 2 gamma_3 (Ize 2013) so the
// box test never rejects a triangle the triangle test would accept.
__device__ __forceinline__ float box_enter(const RayPre &r, float lx, float ly, float lz, float hx, float hy, float hz,
                                           float tmin, float tmax) {
    const float tx0 = __fmul_rn(__fsub_rn(lx, r.org[0]), r.inv[0]);
    const float tx1 = __fmul_rn(__fsub_rn(hx, r.org[0]), r.inv[0]);
    const float ty0 = __fmul_rn(__fsub_rn(ly, r.org[1]), r.inv[1]);
    const float ty1 = __fmul_rn(__fsub_rn(hy, r.org[1]), r.inv[1]);
    const float tz0 = __fmul_rn(__fsub_rn(lz, r.org[2]), r.inv[2]);
    const float tz1 = __fmul_rn(__fsub_rn(hz, r.org[2]), r.inv[2]);
    const float te = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), tmin));
    float tx = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tmax));
    tx = __fmul_rn(tx, 1.0000004f);
    return te <= tx ? te : INFINITY;
}

// Analytic sphere (raytrace.sphere.rint:11-29 solves the same quadratic).
__device__ __forceinline__ bool sphere_intersect(const RayPre &r, const pg_sphere &s, float tmin, float tmax,
                                                 float &t_out) {
    const float oc[3] = {__fsub_rn(r.org[0], s.center[0]), __fsub_rn(r.org[1], s.center[1]),
                         __fsub_rn(r.org[2], s.center[2])};
    const float a = __fadd_rn(__fadd_rn(__fmul_rn(r.dir[0], r.dir[0]), __fmul_rn(r.dir[1], r.dir[1])),
                              __fmul_rn(r.dir[2], r.dir[2]));
    const float b = __fadd_rn(__fadd_rn(__fmul_rn(r.dir[0], oc[0]), __fmul_rn(r.dir[1], oc[1])),
                              __fmul_rn(r.dir[2], oc[2]));
    const float c = __fsub_rn(__fadd_rn(__fadd_rn(__fmul_rn(oc[0], oc[0]), __fmul_rn(oc[1], oc[1])),
                                        __fmul_rn(oc[2], oc[2])),
                              __fmul_rn(s.radius, s.radius));
    const float disc = __fsub_rn(__fmul_rn(b, b), __fmul_rn(a, c));
    if (disc < 0.0f) return false;
    const float sq = __fsqrt_rn(disc);
    const float t1 = __fdiv_rn(__fsub_rn(-b, sq), a);
    if (t1 > tmin && t1 < tmax) {
        t_out = t1;
        return true;
    }
    const float t2 = __fdiv_rn(__fadd_rn(-b, sq), a);
    if (t2 > tmin && t2 < tmax) {
        t_out = t2;
        return true;
    }
    return false;
}

// Deep enough for any tree the builder makes (depth <= 60 binary levels, at
// most three pushes per four-wide level); a full stack drops the push, which
// the CPU twin does identically.
constexpr int kStackSize = 128;
// The short stack: the top kRegStack entries live in registers as a shift
// register (a push shifts them down, a pop up); only deeper entries go to the
// local-memory part of kStackSize - kRegStack.  The logical stack - order of
// entries and the dropped push when full - is that of one array of
// kStackSize, so the traversal order, and the CPU twin, do not change.
constexpr int kRegStack = 4;
constexpr int kDeepStack = kStackSize - kRegStack;

// Work counters of one traversal: NoCount compiles to nothing; WorkCount
// tallies the BVH nodes fetched and the triangles tested.
struct NoCount {
    __device__ __forceinline__ void node() {}
    __device__ __forceinline__ void tri() {}
};
struct WorkCount {
    uint32_t nodes = 0, tris = 0;
    __device__ __forceinline__ void node() { ++nodes; }
    __device__ __forceinline__ void tri() { ++tris; }
};

// Traversal state of one ray, advanced one BVH node per step, so a warp
// whose lanes finish at different times can hand finished lanes new rays
// (the persistent extension and shadow kernels).  The order of visits per
// ray does not depend on how the steps are scheduled.
struct TravState {
    RayPre r;
    float tmin, tmax;  // tmax: best t so far for closest-hit queries
    float best_u, best_v;
    uint32_t best_id;
    int node, sp;          // sp: entries on the stack
    int top[kRegStack];    // the stack's top entries, top[0] uppermost
};

// Push onto the short stack (deep: the local-memory part, kDeepStack entries).
__device__ __forceinline__ void stack_push(TravState &st, int *deep, int x) {
    if (st.sp >= kStackSize) return;
    if (st.sp >= kRegStack) deep[st.sp - kRegStack] = st.top[kRegStack - 1];
#pragma unroll
    for (int i = kRegStack - 1; i > 0; --i) st.top[i] = st.top[i - 1];
    st.top[0] = x;
    ++st.sp;
}
// Pop (the stack is not empty).
__device__ __forceinline__ int stack_pop(TravState &st, const int *deep) {
    const int x = st.top[0];
#pragma unroll
    for (int i = 0; i < kRegStack - 1; ++i) st.top[i] = st.top[i + 1];
    if (st.sp > kRegStack) st.top[kRegStack - 1] = deep[st.sp - 1 - kRegStack];
    --st.sp;
    return x;
}

// Spheres first (closest: they set the initial best; any: a hit ends the
// query), then the BVH from the root.  Returns true when the query is
// already decided (any-hit occluded by a sphere).
template <bool kAny>
__device__ __forceinline__ bool trav_begin(const DevScene &S, TravState &st, const float o[3], const float d[3],
                                           float tmin, float tmax) {
    st.r = ray_setup(o, d);
    st.tmin = tmin;
    st.tmax = tmax;
    st.best_u = st.best_v = 0.0f;
    st.best_id = PG_NO_HIT;
    st.node = 0;
    st.sp = 0;
    for (uint32_t i = 0; i < S.n_spheres; ++i) {
        float t;
        if (sphere_intersect(st.r, S.spheres[i], tmin, st.tmax, t)) {
            if (kAny) {
                st.best_id = PG_SPHERE_BIT | i;
                return true;
            }
            st.tmax = t;
            st.best_id = PG_SPHERE_BIT | i;
        }
    }
    return false;
}

__device__ __forceinline__ float f4(const float4 &v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w)); }
__device__ __forceinline__ int i4(const int4 &v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w)); }

// One node of a closest-hit (kAny false) or any-hit (kAny true) traversal:
// the four child boxes against the best t at the start of the step, leaf
// children tested in slot order, inner children visited nearest first
// (closest: entry distance, ties by slot; any: slot order), the others pushed
// so the next nearest is on top.  Returns true when the traversal is over; for
// any-hit, st.best_id != PG_NO_HIT then means occluded.
template <bool kAny, class Ctr>
__device__ __forceinline__ bool trav_step(const DevScene &S, TravState &st, int *deep, Ctr &ctr) {
    // read-only path: the scene never changes during a launch
    const DevBvhNode *np = S.nodes + st.node;
    const float4 lox = __ldg(&np->lox), loy = __ldg(&np->loy), loz = __ldg(&np->loz);
    const float4 hix = __ldg(&np->hix), hiy = __ldg(&np->hiy), hiz = __ldg(&np->hiz);
    const int4 child = __ldg(&np->child), count = __ldg(&np->count);
    ctr.node();
    float e[4];
#pragma unroll
    for (int j = 0; j < 4; ++j)
        e[j] = box_enter(st.r, f4(lox, j), f4(loy, j), f4(loz, j), f4(hix, j), f4(hiy, j), f4(hiz, j), st.tmin,
                         st.tmax);
    for (int j = 0; j < 4; ++j) {
        const int cnt = i4(count, j);
        if (e[j] == INFINITY || cnt <= 0) continue;
        const int first = i4(child, j);
        for (int k = 0; k < cnt; ++k) {
            const uint32_t ti = (uint32_t)(first + k);
            const float4 v0 = __ldg(&S.tris[3 * ti]), v1 = __ldg(&S.tris[3 * ti + 1]), v2 = __ldg(&S.tris[3 * ti + 2]);
            ctr.tri();
            float t, u, v;
            const uint32_t tex = __float_as_uint(v1.w);
            if (kAny) {
                if (tri_intersect(st.r, v0, v1, v2, st.tmin, st.tmax, t, u, v) &&
                    (tex == 0u || alpha_keep(S, st.r.org[0], __float_as_uint(v0.w), tex, u, v, t))) {
                    st.best_id = __float_as_uint(v0.w);
                    return true;
                }
            } else {
                const uint32_t id = __float_as_uint(v0.w);
                // one ulp above the best t, so an equal t is seen and the lower id wins
                const float lim = st.best_id == PG_NO_HIT ? st.tmax : __uint_as_float(__float_as_uint(st.tmax) + 1u);
                if (tri_intersect(st.r, v0, v1, v2, st.tmin, lim, t, u, v) &&
                    (t < st.tmax || (t == st.tmax && id < st.best_id)) &&
                    (tex == 0u || alpha_keep(S, st.r.org[0], id, tex, u, v, t))) {
                    st.tmax = t;
                    st.best_id = id;
                    st.best_u = u;
                    st.best_v = v;
                }
            }
        }
    }
    // inner children, sorted (insertion, stable) by entry distance for closest hits
    int cand[4];
    float ce[4];
    int nn = 0;
    for (int j = 0; j < 4; ++j) {
        if (e[j] == INFINITY || i4(count, j) > 0 || i4(child, j) < 0) continue;
        int pos = nn;
        if (!kAny)
            while (pos > 0 && ce[pos - 1] > e[j]) {
                ce[pos] = ce[pos - 1];
                cand[pos] = cand[pos - 1];
                --pos;
            }
        ce[pos] = e[j];
        cand[pos] = i4(child, j);
        ++nn;
    }
    if (nn > 0) {
        for (int q = nn - 1; q >= 1; --q) stack_push(st, deep, cand[q]);
        st.node = cand[0];
        return false;
    }
    if (st.sp == 0) return true;
    st.node = stack_pop(st, deep);
    return false;
}

// Closest hit.  Returns false if nothing is hit in (tmin, tmax).
template <class Ctr = NoCount>
__device__ __forceinline__ bool trace_closest(const DevScene &S, const float o[3], const float d[3], float tmin,
                                              float tmax, pg_hit &hit, Ctr &&ctr = Ctr()) {
    TravState st;
    int deep[kDeepStack];
    trav_begin<false>(S, st, o, d, tmin, tmax);
    while (!trav_step<false>(S, st, deep, ctr)) {
    }
    hit.t = st.tmax;
    hit.u = st.best_u;
    hit.v = st.best_v;
    hit.prim = st.best_id;
    return st.best_id != PG_NO_HIT;
}

// Any hit in (tmin, tmax).
template <class Ctr = NoCount>
__device__ __forceinline__ bool trace_any(const DevScene &S, const float o[3], const float d[3], float tmin,
                                          float tmax, Ctr &&ctr = Ctr()) {
    TravState st;
    int deep[kDeepStack];
    if (trav_begin<true>(S, st, o, d, tmin, tmax)) return true;
    while (!trav_step<true>(S, st, deep, ctr)) {
    }
    return st.best_id != PG_NO_HIT;
}

}  // namespace pg
