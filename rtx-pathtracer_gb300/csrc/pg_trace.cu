// pg_trace.cu - scenes on the device, ray queries, and the wavefront path
// tracer with NEE, MIS, vMF-mixture guiding and guiding-sample recording.
//
// The reference traces one megakernel per pixel on RT cores (shaders/
// raytrace.rgen:1623-1827, raytrace :992-1226).  Here each bounce of all pixels'
// paths runs as separate stages over compacted queues:
//   extend  - closest hit of every active path (BVH traversal, pg_traverse.cuh)
//   shade   - emission with MIS, next-event estimation (a shadow-ray entry in
//             a queue), BSDF or guided sampling of the continuation, guiding
//             record bookkeeping; survivors are appended to the next queue
//   shadow  - any hit of every shadow ray; unoccluded NEE is added to the
//             image and to the path's guiding records
//   commit  - after the last bounce, record weights |L| / pdf
//             (raytrace.rgen:980-990)
// Path state is structure-of-arrays indexed by pixel (one path per pixel per
// sample), so every stage reads coalesced rows.
//
// Estimator (ours, restated in FP64 by oracle/pg_oracle_trace.cpp):
//   lights are picked uniformly (getLightSamplingVector gives every light power
//   1, src/SceneLoader.cpp:923-944), mesh lights sample a triangle by area and
//   a uniform point on it (raytrace.rgen:436-472), sphere lights a uniform
//   point on the sphere (random.glsl:108-115); NEE and BSDF-sampled emission
//   are combined with the power heuristic (raytrace.rgen:488-493); BSDFs:
//   Lambert (cosine sampling), GGX conductor (Smith G, Schlick F, NDF
//   sampling), smooth dielectric (exact Fresnel, raytrace.rgen:145-160,
//   reflect/refract choice by Fresnel, raytrace.rgen:526-541), mirror.
//   Guided vertices draw from the region's vMF mixture with probability
//   guiding_prob and use the one-sample mixture pdf (raytrace.rgen:923-960).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "../host/pg_exr.h"
#include "../host/pg_png.h"
#include "../host/pg_scene.h"
#include "pg_internal.cuh"
#include "pg_traverse.cuh"

namespace pg {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kTMin = 0.001f;    // tMin of raytrace.rgen:51
constexpr float kTMax = 1.0e6f;    // tMax of raytrace.rgen:52
constexpr int kMaxRecords = 16;    // MAX_DIRECTIONAL_DATA_PER_PIXEL (shaders/limits.glsl:7)
constexpr int kNumStats = 8;       // device render statistics (see DevRender::stats)

struct DevLight {
    int32_t type;      // 0: triangle mesh, 1: sphere, 2: environment map
    uint32_t first;    // into light_tris / light_cdf
    uint32_t count;
    uint32_t sphere;
    float area;
    float emission[3];
};

// ---------------------------------------------------------------------------
// Random numbers: stateless hash of (seed, pixel, sample, dimension), so the
// FP64 oracle draws the same numbers.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint32_t fmix32(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}
__host__ __device__ __forceinline__ float rnd(uint32_t seed, uint32_t pixel, uint32_t sample, uint32_t dim) {
    const uint32_t h = fmix32(seed + fmix32(pixel + fmix32(sample * 1024u + dim)));
    return (float)(h >> 8) * (1.0f / 16777216.0f);
}
// dimension of the d-th number at bounce b
__host__ __device__ __forceinline__ uint32_t dimb(int b, int d) { return 2u + 16u * (uint32_t)b + (uint32_t)d; }

struct V {
    float x, y, z;
};
__device__ __forceinline__ V mk(float x, float y, float z) { return V{x, y, z}; }
__device__ __forceinline__ V add(V a, V b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V sub(V a, V b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V mul(V a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V hmul(V a, V b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float dot3(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V cross3(V a, V b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
__device__ __forceinline__ V nrm(V a) { return mul(a, rsqrtf(dot3(a, a))); }
__device__ __forceinline__ float maxc(V a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }

// Orthonormal frame around n (transform.glsl:7-16, coordinateAxis).
__device__ __forceinline__ void frame(V n, V &x, V &y) {
    if (fabsf(n.x) > fabsf(n.y)) {
        const float inv = rsqrtf(n.x * n.x + n.z * n.z);
        y = mk(n.z * inv, 0.0f, -n.x * inv);
    } else {
        const float inv = rsqrtf(n.y * n.y + n.z * n.z);
        y = mk(0.0f, n.z * inv, -n.y * inv);
    }
    x = cross3(y, n);
}
__device__ __forceinline__ V to_world(V l, V n) {
    V x, y;
    frame(n, x, y);
    return add(add(mul(x, l.x), mul(y, l.y)), mul(n, l.z));
}
__device__ __forceinline__ V reflect3(V i, V n) { return sub(i, mul(n, 2.0f * dot3(n, i))); }

// Fresnel of a dielectric (raytrace.rgen:145-160); eta = n_i / n_t.
__device__ __forceinline__ float fresnel_dielectric(float eta, float cos_i) {
    const float s2 = eta * eta * (1.0f - cos_i * cos_i);
    if (s2 > 1.0f) return 1.0f;
    const float cos_t = sqrtf(1.0f - s2);
    const float rs = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
    const float rp = (cos_i - eta * cos_t) / (cos_i + eta * cos_t);
    return 0.5f * (rs * rs + rp * rp);
}

// GGX microfacet conductor.
__device__ __forceinline__ float ggx_D(float a2, float cos_m) {
    const float c2 = cos_m * cos_m;
    const float d = c2 * (a2 - 1.0f) + 1.0f;
    return a2 / (kPi * d * d);
}
__device__ __forceinline__ float ggx_G1(float a2, float cos_v) {
    const float c = fabsf(cos_v);
    return 2.0f * c / (c + sqrtf(a2 + (1.0f - a2) * c * c));
}

// Fresnel of a conductor (raytrace.rgen:163-176), one spectrum value of eta and k.
__device__ __forceinline__ float fresnel_conductor(float ci, float eta, float k) {
    ci = fabsf(ci);
    const float ek = eta * eta + k * k, c2 = ci * ci;
    const float rs2 = (ek * c2 - 2.0f * eta * ci + 1.0f) / (ek * c2 + 2.0f * eta * ci + 1.0f);
    const float rp2 = (ek - 2.0f * eta * ci + c2) / (ek + 2.0f * eta * ci + c2);
    return 0.5f * (rs2 + rp2);
}

// The reference's Beckmann rough conductor (raytrace.rgen:178-231, 269-297):
// D with tan^2 = (1 - cos^2) / cos^2, and its G1 approximation as written
// there (the tangent taken of the cosine dot(v, n), and 2.577 a where the
// published rational fit has 2.577 a^2).
__device__ __forceinline__ float beckmann_D(float alpha, float c) {
    if (c <= 0.0f) return 0.0f;
    const float c2 = c * c, t2 = fmaxf(1.0f - c2, 0.0f) / c2, a2 = alpha * alpha;
    return expf(-t2 / a2) / (kPi * a2 * c2 * c2);
}
__device__ __forceinline__ float beckmann_G1(float alpha, V n, V m, V v) {
    const float tv = dot3(v, n);
    const float c = dot3(v, m) / tv;
    if (c <= 0.0f) return 0.0f;
    const float a = 1.0f / (alpha * tanf(tv));
    if (a >= 1.6f) return 1.0f;
    return (3.535f * a + 2.181f * a * a) / (1.0f + 2.276f * a + 2.577f * a);
}

struct MatEval {
    V f;        // BSDF * cos(theta_o)
    float pdf;  // solid-angle pdf of sampling wo
};

// BSDF value times cosine and sampling pdf for a non-delta material.
__device__ __forceinline__ MatEval bsdf_eval(const pg_material &m, V n, V wi, V wo) {
    MatEval r{mk(0, 0, 0), 0.0f};
    const float co = dot3(n, wo), ci = dot3(n, wi);
    if (co <= 0.0f || ci <= 0.0f) return r;
    if (m.type == PG_MAT_DIFFUSE) {
        r.f = mul(mk(m.albedo[0], m.albedo[1], m.albedo[2]), co / kPi);
        r.pdf = co / kPi;
    } else if (m.type == PG_MAT_GGX) {
        const V h = nrm(add(wi, wo));
        const float a2 = fmaxf(m.roughness * m.roughness, 1e-12f);
        const float ch = dot3(n, h), hi = dot3(wi, h);
        const float D = ggx_D(a2, ch);
        const float G = ggx_G1(a2, ci) * ggx_G1(a2, co);
        const float w = powf(1.0f - fmaxf(hi, 0.0f), 5.0f);
        const V F = mk(m.albedo[0] + (1.0f - m.albedo[0]) * w, m.albedo[1] + (1.0f - m.albedo[1]) * w,
                       m.albedo[2] + (1.0f - m.albedo[2]) * w);
        r.f = mul(F, D * G / (4.0f * ci));
        r.pdf = D * ch / (4.0f * fabsf(hi));
    } else if (m.type == PG_MAT_BECKMANN) {
        // roughConductor and pdfBSDF (raytrace.rgen:269-297)
        const V h = nrm(add(wi, wo));
        const float D = beckmann_D(m.roughness, dot3(n, h));
        float G = beckmann_G1(m.roughness, n, h, wi) * beckmann_G1(m.roughness, n, h, wo);
        G = G < 0.0f ? 0.0f : G;
        const float v = fresnel_conductor(dot3(wi, h), m.eta, m.k) * G * D / (4.0f * ci);
        r.f = isnan(v) ? mk(0, 0, 0) : mk(v, v, v);
        const float pm = D * fabsf(dot3(h, n)), oh = dot3(wo, h);
        r.pdf = (pm <= 0.0f || oh <= 0.0f) ? 0.0f : pm / (4.0f * fabsf(oh));
    } else if (m.type == PG_MAT_PHONG) {
        // phong and pdfBSDF (raytrace.rgen:242-267, 306-333)
        const V kd = mk(m.albedo[0], m.albedo[1], m.albedo[2]), ks = mk(m.specular[0], m.specular[1], m.specular[2]);
        V res = mul(kd, 1.0f / kPi);
        const float rw = dot3(reflect3(mul(wo, -1.0f), n), wi);
        if (rw > 0.0f) res = add(res, mul(ks, (m.exponent + 2.0f) / (2.0f * kPi) * powf(rw, m.exponent)));
        r.f = mul(res, co);
        const float ld = sqrtf(dot3(kd, kd)), ls = sqrtf(dot3(ks, ks)), sum = ld + ls;
        if (sum > 0.0f) {
            const float rr = dot3(reflect3(mul(wi, -1.0f), n), wo);
            const float pdf = rr > 0.0f ? (m.exponent + 1.0f) * powf(rr, m.exponent) / (2.0f * kPi) * (ls / sum) : 0.0f;
            r.pdf = pdf + co / kPi * (ld / sum);
        }
    }
    return r;
}

__device__ __forceinline__ bool is_delta(const pg_material &m) {  // hasDiscreteDirection (raytrace.rgen:733-741)
    return m.type == PG_MAT_DIELECTRIC || m.type == PG_MAT_SPECULAR || m.type == PG_MAT_CONDUCTOR;
}
// isMatAlmostDiscrete (raytrace.rgen:962-964): glossy lobes that are not recorded
__device__ __forceinline__ bool almost_delta(const pg_material &m) {
    return ((m.type == PG_MAT_GGX || m.type == PG_MAT_BECKMANN) && m.roughness <= 0.3f) ||
           (m.type == PG_MAT_PHONG && m.exponent >= 250.0f);
}
// Vertices whose continuation mixes in the guide.  The reference guides every
// non-discrete material (raytrace.rgen:926) but records only the ones that
// are not almost discrete; by default guiding here follows the recording
// rule, so a near-specular lobe is never sampled from a mixture learned at
// other surfaces of its region.  PG_RENDER_GUIDE_ALMOST_DISCRETE restores the
// reference's rule.
__device__ __forceinline__ bool guided_material(const pg_material &m, uint32_t render_flags) {
    return !is_delta(m) && ((render_flags & PG_RENDER_GUIDE_ALMOST_DISCRETE) || !almost_delta(m));
}

// Lambert (cosine), Phong (a lobe chosen by ul, sampleBSDF raytrace.rgen:
// 491-517), Beckmann (randomBeckmannNormal, random.glsl:127-136) or GGX
// (normal distribution, then reflection) sample.
__device__ __forceinline__ V sample_bsdf(const pg_material &m, V d, V n, float ul, float u1, float u2) {
    if (m.type == PG_MAT_PHONG) {
        const V kd = mk(m.albedo[0], m.albedo[1], m.albedo[2]), ks = mk(m.specular[0], m.specular[1], m.specular[2]);
        const float ld = sqrtf(dot3(kd, kd)), ls = sqrtf(dot3(ks, ks));
        if (ul * (ld + ls) > ld) {  // cosine power around the mirror direction
            const float ct = powf(u1, 1.0f / (m.exponent + 1.0f)), st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
            const float ph = 2.0f * kPi * u2;
            return to_world(mk(st * cosf(ph), st * sinf(ph), ct), reflect3(d, n));
        }
    }
    if (m.type == PG_MAT_DIFFUSE || m.type == PG_MAT_PHONG) {
        const float sr = sqrtf(u1), ph = 2.0f * kPi * u2;
        return to_world(mk(sr * cosf(ph), sr * sinf(ph), sqrtf(fmaxf(0.0f, 1.0f - u1))), n);
    }
    if (m.type == PG_MAT_BECKMANN) {
        const float th = atanf(sqrtf(-m.roughness * m.roughness * logf(1.0f - u1))), ph = 2.0f * kPi * u2;
        const V mh = to_world(mk(sinf(th) * cosf(ph), sinf(th) * sinf(ph), cosf(th)), n);
        return reflect3(d, mh);
    }
    const float a2 = fmaxf(m.roughness * m.roughness, 1e-12f);
    const float t2 = a2 * u1 / fmaxf(1.0f - u1, 1e-12f);
    const float cm = rsqrtf(1.0f + t2), sm = sqrtf(fmaxf(0.0f, 1.0f - cm * cm));
    const float ph = 2.0f * kPi * u2;
    const V mh = to_world(mk(sm * cosf(ph), sm * sinf(ph), cm), n);
    return reflect3(d, mh);
}

// ---------------------------------------------------------------------------
// Guiding: region lookup and the vMF mixture (shaders/guiding.glsl:32-96)
// ---------------------------------------------------------------------------
struct DevGuide {
    float root[6];
    uint32_t split_count;
    const int32_t *nodes;  // the region tree after region splits (null: the complete tree)
    const pg_vmm_theta *vmm;
    int use_parallax;
};

// Point -> region by descending the midpoint split tree with the same float
// arithmetic that built it; points outside the root box (or in a rounding gap)
// have no region (getGuidingRegion returns -1, raytrace.rgen:904-921).  The
// levels of pg_set_regions' complete tree are descended by arithmetic alone;
// once regions were split, the descent continues from that level's leaf
// through the node array (inner node v: children v, v + 1), so a region that
// was never split costs one load.
__device__ __forceinline__ bool descend_level(float lo[3], float hi[3], const float pp[3], int &side) {
    float size[3];
    for (int i = 0; i < 3; ++i) size[i] = __fsub_rn(hi[i], lo[i]);
    const int ax = size[0] > size[1] ? (size[0] > size[2] ? 0 : 2) : (size[1] > size[2] ? 1 : 2);
    const float lhi = __fsub_rn(hi[ax], __fmul_rn(0.5f, size[ax]));
    const float rlo = __fadd_rn(lo[ax], __fmul_rn(0.5f, size[ax]));
    if (pp[ax] <= lhi) {
        hi[ax] = lhi;
        side = 0;
    } else if (pp[ax] >= rlo) {
        lo[ax] = rlo;
        side = 1;
    } else {
        return false;
    }
    return true;
}

__device__ __forceinline__ uint32_t region_of(const DevGuide &g, V p) {
    float lo[3] = {g.root[0], g.root[1], g.root[2]}, hi[3] = {g.root[3], g.root[4], g.root[5]};
    const float pp[3] = {p.x, p.y, p.z};
    for (int i = 0; i < 3; ++i)
        if (!(pp[i] >= lo[i] && pp[i] <= hi[i])) return PG_INVALID_REGION;
    uint32_t id = 0;
    for (uint32_t l = 0; l < g.split_count; ++l) {
        int side;
        if (!descend_level(lo, hi, pp, side)) return PG_INVALID_REGION;
        id = 2u * id + (uint32_t)side;
    }
    if (!g.nodes) return id;
    int32_t node = (int32_t)((1u << g.split_count) - 1u + id);
    for (int depth = 0; depth < 64; ++depth) {
        const int32_t v = __ldg(g.nodes + node);
        if (v < 0) return (uint32_t)(-(v + 1));
        int side;
        if (!descend_level(lo, hi, pp, side)) return PG_INVALID_REGION;
        node = v + side;
    }
    return PG_INVALID_REGION;
}

__device__ __forceinline__ V lobe_mu(const pg_vmf_theta &t, V x, int par) {
    V mu = mk(t.mu[0], t.mu[1], t.mu[2]);
    if (par && t.distance > 0.0f) mu = nrm(sub(mk(t.target[0], t.target[1], t.target[2]), x));
    return mu;
}

// VMM pdf (guiding.glsl:32-60)
__device__ float vmm_pdf(const pg_vmm_theta &v, V wo, V x, int par) {
    float res = 0.0f;
    const int K = min(v.used_distributions, 16);
    for (int i = 0; i < K; ++i) {
        const pg_vmf_theta &t = v.thetas[i];
        float f;
        if (t.k == 0.0f) {
            f = 1.0f / (4.0f * kPi);
        } else {
            const V mu = lobe_mu(t, x, par);
            f = t.norm * expf(t.k * (dot3(mu, wo) - 1.0f));
        }
        res += v.pi[i] * f;
    }
    return res;
}

// sampleVMM (guiding.glsl:62-96): pick a lobe by walking the weights, then
// invert the vMF cosine CDF.
__device__ V vmm_sample(const pg_vmm_theta &v, V x, int par, float u_lobe, float u1, float u2) {
    const int K = min(v.used_distributions, 16);
    int i = 0;
    float acc = v.pi[0];
    while (acc < u_lobe && i < K - 1) {
        ++i;
        acc += v.pi[i];
    }
    const pg_vmf_theta &t = v.thetas[i];
    if (t.k > 0.0f) {
        const float ct = 1.0f + logf(1.0f + t.e_min2k * u1 - u1) / t.k;
        const float st = 1.0f - ct * ct <= 0.0f ? 0.0f : sqrtf(1.0f - ct * ct);
        const float ph = 2.0f * kPi * u2;
        return to_world(mk(st * cosf(ph), st * sinf(ph), ct), lobe_mu(t, x, par));
    }
    const float z = 1.0f - 2.0f * u1;  // uniform sphere
    const float r = sqrtf(fmaxf(0.0f, 1.0f - z * z));
    const float ph = 2.0f * kPi * u2;
    return mk(r * cosf(ph), r * sinf(ph), z);
}

// The continuation of a path at a vertex (getNewDirection, raytrace.rgen:
// 923-960, and the throughput change evalBsdf / pdf of :1176): delta
// materials reflect or refract (a dielectric picks by Fresnel with ul);
// others sample the BSDF or, with probability guiding_prob at a guided
// vertex (gm), the region's mixture `mix`, and weight by the one-sample
// mixture pdf.  A guided vertex without a region (mix null) ends the path
// (pdf 0).  draw_ua() supplies the lobe-choice number, drawn only when the
// guide is sampled.
struct Continuation {
    V wo;
    float pdf;
    V tc;        // throughput change f cos / pdf
    bool delta;  // discrete direction
};
template <typename DrawUa>
__device__ __forceinline__ Continuation continue_path(const pg_material &m, V d, V n, bool front, V x, bool gm,
                                                      const pg_vmm_theta *mix, int par, float guiding_prob,
                                                      float uch, float ul, float u1, float u2, DrawUa draw_ua) {
    Continuation c{mk(0, 0, 1), 0.0f, mk(0, 0, 0), false};
    const V wi = mul(d, -1.0f);
    if (m.type == PG_MAT_DIELECTRIC) {
        const float eta = front ? 1.0f / m.ior : m.ior;  // refractionIndexInv in front
        const float ci = dot3(wi, n);
        const float F = fresnel_dielectric(eta, ci);
        if (ul > F) {
            // refract(-wi, n, eta)
            const float k = 1.0f - eta * eta * (1.0f - ci * ci);
            c.wo = k < 0.0f ? reflect3(d, n) : sub(mul(d, eta), mul(n, eta * (-ci) + sqrtf(fmaxf(k, 0.0f))));
            c.wo = nrm(c.wo);
        } else {
            c.wo = reflect3(d, n);
        }
        c.pdf = 1.0f;
        c.tc = mk(m.albedo[0], m.albedo[1], m.albedo[2]);
        c.delta = true;
    } else if (m.type == PG_MAT_SPECULAR) {
        c.wo = reflect3(d, n);
        c.pdf = 1.0f;
        c.tc = mk(m.albedo[0], m.albedo[1], m.albedo[2]);
        c.delta = true;
    } else if (m.type == PG_MAT_CONDUCTOR) {
        // evalBsdf MAT_CONDUCTOR (raytrace.rgen:588-592)
        c.wo = reflect3(d, n);
        c.pdf = 1.0f;
        const float F = fresnel_conductor(dot3(wi, n), m.eta, m.k);
        c.tc = mk(F, F, F);
        c.delta = true;
    } else {
        if (gm && !mix) return c;  // no region: the path ends
        const bool use_guide = gm && uch < guiding_prob;
        V wo = use_guide ? vmm_sample(*mix, x, par, draw_ua(), u1, u2) : sample_bsdf(m, d, n, ul, u1, u2);
        MatEval me = bsdf_eval(m, n, wi, wo);
        float pdf = me.pdf;
        if (gm) {
            if (dot3(wo, n) < 0.0f || me.pdf <= 0.0f) {
                pdf = 0.0f;
            } else {
                const float pg = vmm_pdf(*mix, wo, x, par);
                if (isnan(pg)) {
                    // unusable mixture: a plain BSDF sample (raytrace.rgen:951-953)
                    if (use_guide) {
                        wo = sample_bsdf(m, d, n, ul, u1, u2);
                        me = bsdf_eval(m, n, wi, wo);
                    }
                    pdf = me.pdf;
                } else {
                    pdf = (1.0f - guiding_prob) * me.pdf + guiding_prob * pg;
                }
            }
        }
        c.wo = wo;
        if (dot3(wo, n) > 0.0f && pdf > 0.0f && me.pdf > 0.0f) {
            c.tc = mul(me.f, 1.0f / pdf);
            c.pdf = pdf;
        }
    }
    return c;
}

// ---------------------------------------------------------------------------
// Device scene and render state
// ---------------------------------------------------------------------------
// Per-frame salt of the alpha test (the reference's push-constant random number).
__host__ __device__ inline uint32_t alpha_salt(uint32_t seed) { return fmix32(seed ^ 0x5bd1e995u); }

// sRGB-encoded byte to linear (the sRGB texture format's decode before filtering).
__device__ __forceinline__ float srgb_to_linear(uint8_t b) {
    const float c = (float)b * (1.0f / 255.0f);
    return c <= 0.04045f ? c * (1.0f / 12.92f) : powf((c + 0.055f) * (1.0f / 1.055f), 2.4f);
}

// Bilinear linear-RGB colour of texture `tex` at the texture coordinate of the
// hit (barycentrics bu, bv) on original triangle `prim` (repeat addressing).
__device__ __forceinline__ void tex_rgb(const DevScene &S, uint32_t prim, uint32_t tex, float bu, float bv,
                                        float out[3]) {
    const float *uv = S.tri_uv + 6 * (size_t)prim;
    const float w0 = 1.0f - bu - bv;
    float u = uv[0] * w0 + uv[2] * bu + uv[4] * bv, v = uv[1] * w0 + uv[3] * bu + uv[5] * bv;
    const uint4 ti = S.tex_info[tex];
    const int w = (int)ti.y, h = (int)ti.z;
    u -= floorf(u);
    v -= floorf(v);
    const float x = u * (float)w - 0.5f, y = v * (float)h - 0.5f;
    const float x0 = floorf(x), y0 = floorf(y), fx = x - x0, fy = y - y0;
    int ix0 = (int)x0, iy0 = (int)y0, ix1 = ix0 + 1, iy1 = iy0 + 1;
    ix0 = ix0 < 0 ? ix0 + w : ix0;
    iy0 = iy0 < 0 ? iy0 + h : iy0;
    ix1 = ix1 >= w ? ix1 - w : ix1;
    iy1 = iy1 >= h ? iy1 - h : iy1;
    const uchar4 *d = S.tex_data + ti.x;
    const uchar4 t00 = d[iy0 * w + ix0], t10 = d[iy0 * w + ix1], t01 = d[iy1 * w + ix0], t11 = d[iy1 * w + ix1];
    const uint8_t c00[3] = {t00.x, t00.y, t00.z}, c10[3] = {t10.x, t10.y, t10.z}, c01[3] = {t01.x, t01.y, t01.z},
                  c11[3] = {t11.x, t11.y, t11.z};
    for (int c = 0; c < 3; ++c) {
        const float top = srgb_to_linear(c00[c]) * (1.0f - fx) + srgb_to_linear(c10[c]) * fx;
        const float bot = srgb_to_linear(c01[c]) * (1.0f - fx) + srgb_to_linear(c11[c]) * fx;
        out[c] = top * (1.0f - fy) + bot * fy;
    }
}

}  // namespace pg

#include "pg_icache.cuh"

namespace pg {

struct DevRender {
    DevScene S;
    const float *pos;            // 3 per vertex (original)
    const uint32_t *idx;         // 3 per triangle (original)
    const uint32_t *tri_mat;     // per original triangle
    const pg_material *mats;
    const DevLight *lights;
    uint32_t n_lights;
    const uint32_t *light_tris;  // original triangle ids of mesh lights
    const float *light_cdf;      // per light, cumulative area fraction
    const int32_t *tri_light;    // light index of each original triangle, -1 if none
    const float *env;            // environment map, RGB per texel (null: black)
    uint32_t env_w, env_h;
    unsigned long long *stats;   // [0] extension rays, [1] shadow rays, [2..5] traversal work (counting renders)
    pg_camera cam;
    float cam_fwd[3], cam_right[3], cam_up[3], tan_half;
    pg_render_params rp;
    uint32_t sample;             // sample index of this pass
    DevGuide guide;
    int guiding;
    int recording;
    // path state (indexed by pixel)
    float *ro, *rd, *thr;        // 3 per path
    float *prev_pdf;             // pdf of the sampled direction (0: camera or delta)
    uint8_t *alive;
    uint8_t *found;              // radiance reached the camera on this path
    pg_hit *hits;
    uint32_t *q_cur, *q_next;
    uint32_t *counters;          // [0] current queue, [1] next queue, [2] shadow queue, [4] records,
                                 // [6] / [7] extension / shadow fetch positions
    // shadow queue
    float *sh_o, *sh_d, *sh_tmax, *sh_c, *sh_l;  // origin, dir, tmax, contribution (thr * L), radiance L
    uint32_t *sh_pix, *sh_nrec;
    // guiding records
    pg_directional_data *rec;    // 16 per pixel
    float *rec_lsum, *rec_tc;    // 3 floats per slot: radiance sum, throughput change
    uint32_t *rec_count, *rec_start;
    int32_t *rec_pending;        // slot awaiting its distance, -1 if none
    float *rec_factor;           // apparent-distance factor through refraction
    float *image;
    DevIc ic;                    // irradiance cache (query / grow off: unused)
    // ADRRS and the split copies it makes: path ids below n_pix are camera
    // paths (their pixel); ids n_pix + k are split slot k
    const float *adrrs_est;      // pixels' mean radiance (null: ADRRS off)
    float adrrs_s;
    int adrrs_split;
    uint32_t n_pix, split_cap;
    uint32_t *split_pix, *split_stream;  // per split slot: pixel, random stream
    uint32_t *split_count;       // per pixel: copies made this pass
    uint32_t *q_copy;            // split copies made at this bounce (counters[9])
};

__device__ __forceinline__ V ld3(const float *a, uint32_t i) { return mk(a[3 * i], a[3 * i + 1], a[3 * i + 2]); }
__device__ __forceinline__ void st3(float *a, uint32_t i, V v) {
    a[3 * i] = v.x;
    a[3 * i + 1] = v.y;
    a[3 * i + 2] = v.z;
}

// A path's pixel and random stream: a camera path's are its id; a split
// copy's are recorded with its slot.
__device__ __forceinline__ uint32_t pixel_of(const DevRender &R, uint32_t p) {
    return p < R.n_pix ? p : R.split_pix[p - R.n_pix];
}
__device__ __forceinline__ uint32_t stream_of(const DevRender &R, uint32_t p) {
    return p < R.n_pix ? p : R.split_stream[p - R.n_pix];
}
__device__ __forceinline__ void add_image(const DevRender &R, uint32_t px, V c) {
    atomicAdd(&R.image[3 * px], c.x);
    atomicAdd(&R.image[3 * px + 1], c.y);
    atomicAdd(&R.image[3 * px + 2], c.z);
}

// applyWeightWindow (raytrace.rgen:830-869): the window around
// |estimate / adjoint| with upper = s * lower; returns q and the number of
// paths n (1: Russian roulette with survival probability q; more: an
// expected-value split into q paths, u deciding the rounding).
__device__ __forceinline__ float weight_window(V thr, V adjoint, V est, float s, float u, int &n) {
    const V r = mk(est.x / adjoint.x, est.y / adjoint.y, est.z / adjoint.z);
    const float center = sqrtf(dot3(r, r));
    const float lower = 2.0f * center / (1.0f + s);
    const float upper = s * lower;
    const float v = sqrtf(dot3(thr, thr));
    n = 1;
    if (isnan(lower) || lower <= 0.0f) return 1.0f;
    if (lower <= v && v <= upper) return 1.0f;
    if (v <= lower) return fmaxf(v / lower, 0.1f);
    const float q = v / upper;
    n = (int)q;
    if (u > (float)(n + 1) - q) ++n;
    return q;
}

__device__ __forceinline__ void warp_append(uint32_t *counter, uint32_t *queue, uint32_t value, bool pred) {
    const unsigned m = __ballot_sync(__activemask(), pred);
    if (!pred) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(m, base, leader);
    queue[base + __popc(m & ((1u << lane) - 1u))] = value;
}

// updateSamples (raytrace.rgen:973-978): radiance L arriving at the vertex
// after record slot n-1 flows back through the recorded throughput changes.
// Radiance L reaching a path: added to the light sums of its records
// [start, n), scaled back through each record's throughput change
// (updateSamples, raytrace.rgen:973-978).  lsum and tc are the path's
// record slots (3 floats each).
__device__ __forceinline__ void add_record_radiance(float *lsum, const float *tc, uint32_t start, uint32_t n, V L) {
    for (int i = (int)n - 1; i >= (int)start; --i) {
        lsum[3 * i] += L.x;
        lsum[3 * i + 1] += L.y;
        lsum[3 * i + 2] += L.z;
        L = hmul(L, ld3(tc, (uint32_t)i));
    }
}
__device__ __forceinline__ void update_records(const DevRender &R, uint32_t pix, uint32_t n, V L) {
    const uint32_t base = pix * kMaxRecords;
    add_record_radiance(R.rec_lsum + 3 * (size_t)base, R.rec_tc + 3 * (size_t)base, R.rec_start[pix], n, L);
}
// A record's weight |L| / pdf (commitSamples, raytrace.rgen:980-990); a
// weight that is not positive leaves the record invalid.
__device__ __forceinline__ float record_weight(V lsum, float pdf) { return sqrtf(dot3(lsum, lsum)) / pdf; }

// Environment radiance along a direction (raytrace.rmiss): the lat-long map
// at u = atan2(x, -z) / 2 pi, v = acos(y) / pi, bilinear with wrap-around in
// both axes as the reference's linear, repeating sampler.
__device__ __forceinline__ V env_radiance(const DevRender &R, V d) {
    const float kInv2Pi = 0.15915494309189535f;
    const float u = atan2f(d.x, -d.z) * kInv2Pi, v = acosf(fminf(fmaxf(d.y, -1.0f), 1.0f)) * (1.0f / kPi);
    const float sx = u * (float)R.env_w - 0.5f, sy = v * (float)R.env_h - 0.5f;
    const float fx0 = floorf(sx), fy0 = floorf(sy), fx = sx - fx0, fy = sy - fy0;
    const int W = (int)R.env_w, H = (int)R.env_h;
    int x0 = (int)fx0 % W, y0 = (int)fy0 % H;
    x0 += x0 < 0 ? W : 0;
    y0 += y0 < 0 ? H : 0;
    const int x1 = x0 + 1 == W ? 0 : x0 + 1, y1 = y0 + 1 == H ? 0 : y0 + 1;
    const V a = ld3(R.env, (uint32_t)(y0 * W + x0)), b = ld3(R.env, (uint32_t)(y0 * W + x1));
    const V c = ld3(R.env, (uint32_t)(y1 * W + x0)), e = ld3(R.env, (uint32_t)(y1 * W + x1));
    return add(mul(add(mul(a, 1.0f - fx), mul(b, fx)), 1.0f - fy), mul(add(mul(c, 1.0f - fx), mul(e, fx)), fy));
}

// Solid-angle pdf of NEE picking the emitter point hit at distance t with
// surface normal nl, seen along direction d.
__device__ __forceinline__ float light_pdf(const DevRender &R, uint32_t light, float t, float cos_l) {
    const DevLight &L = R.lights[light];
    return (t * t) / (fmaxf(cos_l, 1e-12f) * L.area) / (float)R.n_lights;
}

// One next-event sample from x (sampleLights, raytrace.rgen:358-473): a light
// picked uniformly by ul, then a point on it (u1, u2): the environment by a
// uniform direction in the hemisphere of n, a sphere uniformly over its
// surface, a mesh by area and uniformly within the triangle.  Returns false
// when the sample contributes nothing; else the direction, the shadow ray's
// extent, BSDF * cos * emitted radiance (fLe, to be divided by pl and weighted
// by the caller), the light pdf pl and the BSDF's pdf pb of the direction.
struct NeeSample {
    V wl;
    float tmax;
    V fLe;
    float pl, pb;
};
__device__ __forceinline__ bool nee_sample(const DevRender &R, const pg_material &m, V x, V n, V wi, float ul,
                                           float u1, float u2, NeeSample &ns) {
    const uint32_t l = min((uint32_t)(ul * (float)R.n_lights), R.n_lights - 1);
    const DevLight &L = R.lights[l];
    if (L.type == 2) {
        // environment: a uniform direction in the hemisphere (raytrace.rgen:406-421)
        const float ct = u1, st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct)), ph = 2.0f * kPi * u2;
        const V wl = to_world(mk(st * cosf(ph), st * sinf(ph), ct), n);
        const MatEval me = bsdf_eval(m, n, wi, wl);
        if (!(maxc(me.f) > 0.0f)) return false;
        ns.wl = wl;
        ns.tmax = 1e30f;
        ns.pl = 0.15915494309189535f / (float)R.n_lights;
        ns.pb = me.pdf;
        ns.fLe = hmul(me.f, env_radiance(R, wl));
        return true;
    }
    V lp, ln;
    if (L.type == 1) {
        const pg_sphere &sp = R.S.spheres[L.sphere];
        const float z = 1.0f - 2.0f * u1, rr = sqrtf(fmaxf(0.0f, 1.0f - z * z)), ph = 2.0f * kPi * u2;
        ln = mk(rr * cosf(ph), rr * sinf(ph), z);
        lp = add(mk(sp.center[0], sp.center[1], sp.center[2]), mul(ln, sp.radius));
    } else {
        // triangle by area, then a uniform point (raytrace.rgen:445-456)
        uint32_t lo = 0, hi = L.count - 1;
        const float uc = u1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) / 2;
            if (R.light_cdf[L.first + mid] < uc)
                lo = mid + 1;
            else
                hi = mid;
        }
        const float c0 = lo == 0 ? 0.0f : R.light_cdf[L.first + lo - 1];
        const float c1 = R.light_cdf[L.first + lo];
        const float ur = c1 > c0 ? fminf((uc - c0) / (c1 - c0), 0.99999994f) : 0.5f;
        const uint32_t t = R.light_tris[L.first + lo];
        const V a = ld3(R.pos, R.idx[3 * t]), bb = ld3(R.pos, R.idx[3 * t + 1]), c = ld3(R.pos, R.idx[3 * t + 2]);
        const float sx = sqrtf(ur);
        lp = add(add(mul(a, 1.0f - sx), mul(bb, sx * (1.0f - u2))), mul(c, u2 * sx));
        ln = nrm(cross3(sub(bb, a), sub(c, a)));
    }
    V tl = sub(lp, x);
    const float dist2 = dot3(tl, tl), dist = sqrtf(dist2);
    const V wl = mul(tl, 1.0f / dist);
    float cl = -dot3(wl, ln);
    if (L.type == 0) cl = fabsf(cl);  // two-sided mesh lights (raytrace.rgen:463-466)
    if (!(cl > 0.0f && dot3(n, wl) > 0.0f)) return false;
    const MatEval me = bsdf_eval(m, n, wi, wl);
    if (!(maxc(me.f) > 0.0f)) return false;
    ns.wl = wl;
    ns.tmax = dist * (1.0f - 0.0001f);
    ns.pl = dist2 / (cl * L.area) / (float)R.n_lights;
    ns.pb = me.pdf;
    ns.fLe = hmul(me.f, mk(L.emission[0], L.emission[1], L.emission[2]));
    return true;
}

}  // namespace pg

#include "pg_icache_paths.cuh"

namespace pg {

__global__ void k_camera(DevRender R) {
    const uint32_t W = R.cam.width, H = R.cam.height;
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= W * H) return;
    const uint32_t px = pix % W, py = pix / W;
    // getCameraRay (raytrace.rgen:1487-1494): jitter within the pixel
    const float jx = rnd(R.rp.seed, pix, R.sample, 0) - 0.5f, jy = rnd(R.rp.seed, pix, R.sample, 1) - 0.5f;
    const float aspect = (float)W / (float)H;
    const float sx = (2.0f * ((float)px + 0.5f + jx) / (float)W - 1.0f) * R.tan_half * aspect;
    const float sy = (1.0f - 2.0f * ((float)py + 0.5f + jy) / (float)H) * R.tan_half;
    const V f = mk(R.cam_fwd[0], R.cam_fwd[1], R.cam_fwd[2]);
    const V r = mk(R.cam_right[0], R.cam_right[1], R.cam_right[2]);
    const V u = mk(R.cam_up[0], R.cam_up[1], R.cam_up[2]);
    const V d = nrm(add(add(f, mul(r, sx)), mul(u, sy)));
    st3(R.ro, pix, mk(R.cam.origin[0], R.cam.origin[1], R.cam.origin[2]));
    st3(R.rd, pix, d);
    st3(R.thr, pix, mk(1, 1, 1));
    R.prev_pdf[pix] = 0.0f;
    R.alive[pix] = 1;
    R.found[pix] = 0;
    R.q_cur[pix] = pix;
    if (pix == 0) {
        R.counters[0] = W * H;
        R.counters[1] = 0;
        R.counters[2] = 0;
        R.counters[6] = 0;  // extension and shadow fetch positions
        R.counters[7] = 0;
    }
    if (R.recording) {
        R.rec_count[pix] = R.rec_start[pix];
        R.rec_pending[pix] = -1;
        R.rec_factor[pix] = 1.0f;
    }
    if (R.adrrs_split) R.split_count[pix] = 0;
    if (pix == 0) R.counters[8] = 0;  // split slots taken this pass
    if (R.ic.grow) {
        // main() of raytrace.rgen:1639-1641: an update of the next entry with probability update_prob
        R.ic.created[pix] = 0;
        if (rnd(R.rp.seed ^ kIcSalt, pix, R.sample, 1023u) < R.ic.update_prob)
            ic_push(R.ic, mk(0, 0, 0), mk(0, 0, 1), -1, pix, kIcUpdateBounce, R.sample);
    }
}

// Queue lengths live on the device (counters[0]: current queue, [1]: next
// queue being appended, [2]: shadow queue); kernels are launched over all
// pixels and threads past the length return, so a render needs no host sync.
// Persistent closest-hit stage: warps stay resident and every lane whose ray
// is finished takes the next queue entry (warp-aggregated fetch from
// counters[6]), so a warp's lanes stay busy instead of waiting for its
// slowest ray.  One BVH node per lane per loop trip (trav_step).
// kCount: also add the traversal work to stats[2] (nodes) and stats[3] (triangles).
template <bool kCount>
__global__ void __launch_bounds__(128, 8) k_extend(DevRender R) {
    const uint32_t n = R.counters[0];
    const int lane = threadIdx.x & 31;
    TravState st;
    int deep[kDeepStack];
    WorkCount wc;
    NoCount nc;
    uint32_t p = 0;
    bool have = false, exhausted = false;
    for (;;) {
        if (!exhausted) {
            const unsigned need = __ballot_sync(0xffffffffu, !have);
            if (need) {
                const int leader = __ffs(need) - 1;
                uint32_t base = 0;
                if (lane == leader) base = atomicAdd(&R.counters[6], (uint32_t)__popc(need));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (!have) {
                    const uint32_t idx = base + (uint32_t)__popc(need & ((1u << lane) - 1u));
                    if (idx < n) {
                        p = R.q_cur[idx];
                        const float o[3] = {R.ro[3 * p], R.ro[3 * p + 1], R.ro[3 * p + 2]};
                        const float d[3] = {R.rd[3 * p], R.rd[3 * p + 1], R.rd[3 * p + 2]};
                        trav_begin<false>(R.S, st, o, d, kTMin, kTMax);
                        have = true;
                    }
                }
                if (base + (uint32_t)__popc(need) >= n) exhausted = true;  // warp-uniform
            }
        }
        if (!__any_sync(0xffffffffu, have)) break;
        if (have) {
            const bool done = kCount ? trav_step<false>(R.S, st, deep, wc) : trav_step<false>(R.S, st, deep, nc);
            if (done) {
                pg_hit h;
                h.t = st.tmax;
                h.u = st.best_u;
                h.v = st.best_v;
                h.prim = st.best_id;
                R.hits[p] = h;
                have = false;
            }
        }
    }
    if (kCount) {
        atomicAdd(&R.stats[2], (unsigned long long)wc.nodes);
        atomicAdd(&R.stats[3], (unsigned long long)wc.tris);
    }
}

// Next-event estimation and the continuation at a non-emitting vertex x of
// path p (random stream `stream`, throughput thr before the vertex).  The
// shadow ray is queued with the radiance it would bring; the continuation
// (getNewDirection, raytrace.rgen:923-960) writes p's next ray and, with
// rec_on, the vertex's guiding record.  ic_end: the path ends at the
// irradiance cache here (next-event estimation always, unweighted: there is
// no continuation to pair it with).  Returns whether p continues.
__device__ bool shade_vertex(const DevRender &R, uint32_t p, uint32_t stream, int b, bool rec_on, bool ic_end,
                             const pg_material &m, V x, V n, V d, bool front, V thr) {
    const V wi = mul(d, -1.0f);
    // --- next-event estimation (raytrace.rgen:601-731), always at a cache end (:1122)
    if ((R.rp.use_nee || ic_end) && !is_delta(m) && R.n_lights > 0) {
        NeeSample ns;
        if (nee_sample(R, m, x, n, wi, rnd(R.rp.seed, stream, R.sample, dimb(b, 0)),
                       rnd(R.rp.seed, stream, R.sample, dimb(b, 1)), rnd(R.rp.seed, stream, R.sample, dimb(b, 2)),
                       ns)) {
            // pdf of the continuation sampler for this direction (MIS)
            float pb = ns.pb;
            if (R.guiding && guided_material(m, R.rp.flags)) {
                const uint32_t reg = region_of(R.guide, x);
                if (reg != PG_INVALID_REGION) {
                    const float pg = vmm_pdf(R.guide.vmm[reg], ns.wl, x, R.guide.use_parallax);
                    if (!isnan(pg)) pb = (1.0f - R.rp.guiding_prob) * pb + R.rp.guiding_prob * pg;
                }
            }
            const float pl = ns.pl;
            const float w = (R.rp.use_mis && !ic_end) ? pl * pl / (pl * pl + pb * pb) : 1.0f;
            const V Lnee = mul(ns.fLe, w / pl);
            const uint32_t s = atomicAdd(&R.counters[2], 1u);
            st3(R.sh_o, s, x);
            st3(R.sh_d, s, ns.wl);
            R.sh_tmax[s] = ns.tmax;
            st3(R.sh_c, s, hmul(thr, Lnee));
            st3(R.sh_l, s, Lnee);
            R.sh_pix[s] = p;
            R.sh_nrec[s] = (rec_on && !ic_end) ? R.rec_count[p] : 0u;
        }
    }
    if (ic_end) return false;
    // --- continuation (getNewDirection, raytrace.rgen:923-960)
    const float uch = rnd(R.rp.seed, stream, R.sample, dimb(b, 3));
    const float ul = rnd(R.rp.seed, stream, R.sample, dimb(b, 4));
    const float u1 = rnd(R.rp.seed, stream, R.sample, dimb(b, 5)), u2 = rnd(R.rp.seed, stream, R.sample, dimb(b, 6));
    const bool gm = R.guiding && guided_material(m, R.rp.flags);
    const pg_vmm_theta *mix = nullptr;
    if (gm) {
        const uint32_t reg = region_of(R.guide, x);
        if (reg != PG_INVALID_REGION) mix = &R.guide.vmm[reg];
    }
    const Continuation cn = continue_path(m, d, n, front, x, gm, mix, R.guide.use_parallax, R.rp.guiding_prob, uch,
                                          ul, u1, u2, [&] { return rnd(R.rp.seed, stream, R.sample, dimb(b, 7)); });
    const V wo = cn.wo, tc = cn.tc;
    const float pdf = cn.pdf;
    const bool delta = cn.delta;
    if (!(pdf > 0.0f && maxc(tc) > 0.0f)) return false;
    thr = hmul(thr, tc);
    // guiding record of this vertex (raytrace.rgen:1179-1200)
    if (rec_on) {
        const uint32_t cnt = R.rec_count[p];
        if (cnt < (uint32_t)kMaxRecords) {
            const uint32_t s = p * kMaxRecords + cnt;
            pg_directional_data rd;
            rd.position[0] = x.x;
            rd.position[1] = x.y;
            rd.position[2] = x.z;
            rd.direction[0] = wo.x;
            rd.direction[1] = wo.y;
            rd.direction[2] = wo.z;
            rd.weight = 0.0f;
            rd.pdf = pdf;
            rd.distance = 0.0f;
            if (delta || almost_delta(m)) {
                rd.flags = PG_INVALID_REGION;
            } else {
                rd.flags = region_of(R.guide, x);
                R.rec_pending[p] = (int32_t)cnt;
                R.rec_factor[p] = 1.0f;
            }
            R.rec[s] = rd;
            st3(R.rec_lsum, s, mk(0, 0, 0));
            st3(R.rec_tc, s, tc);
            R.rec_count[p] = cnt + 1;
        } else if (R.rec_pending[p] >= 0 && m.type == PG_MAT_DIELECTRIC && dot3(wo, n) < 0.0f) {
            const float eta = front ? m.ior : 1.0f / m.ior;
            R.rec_factor[p] = fabsf(dot3(n, d) / dot3(n, wo)) * eta;
        }
    }
    st3(R.ro, p, x);
    st3(R.rd, p, wo);
    st3(R.thr, p, thr);
    R.prev_pdf[p] = delta ? 0.0f : pdf;
    return true;
}

constexpr uint32_t kMaxSplits = 10;  // MAX_SPLITS (raytrace.rgen:82): copies per pixel and pass

// ADRRS at a vertex where the cache gives irradiance E (raytrace.rgen:
// 1086-1117): the weight window of the path's throughput thr against the
// pixel's estimate; Russian roulette (returns true when the path ends,
// otherwise divides thr by the survival probability) or splitting into
// `copies` paths (thr divided by their expected number; copies - 1 split
// slots from split_base, fewer within the pixel's budget and the slots, the
// throughput then shared by their number, raytrace.rgen:1103-1109).  Out of
// line: the shading kernel's registers stay with its common path.
__device__ __noinline__ bool adrrs_vertex(const DevRender &R, uint32_t px, uint32_t stream, int b, V E, V &thr,
                                          int &copies, uint32_t &split_base) {
    int nn;
    float q = weight_window(thr, E, ld3(R.adrrs_est, px), R.adrrs_s, rnd(R.rp.seed, stream, R.sample, dimb(b, 10)),
                            nn);
    if (nn == 1) {
        if (rnd(R.rp.seed, stream, R.sample, dimb(b, 9)) > q) return true;
        thr = mul(thr, 1.0f / q);
    } else if (R.adrrs_split) {
        const uint32_t want = (uint32_t)nn - 1u;
        const uint32_t used = atomicAdd(&R.split_count[px], want);
        uint32_t k = used < kMaxSplits ? min(want, kMaxSplits - used) : 0u;
        if (k) {
            split_base = atomicAdd(&R.counters[8], k);
            k = split_base < R.split_cap ? min(k, R.split_cap - split_base) : 0u;
        }
        if (k < want) {
            nn = (int)k + 1;
            q = (float)nn;
        }
        thr = mul(thr, 1.0f / q);
        copies = nn;
    }
    return false;
}

// One bounce of the paths in the current queue (copies 0), or of the split
// copies made at this bounce (copies 1: counters[9] of them in q_copy, each
// at its parent's vertex with the parent's ray and shared throughput; they
// take no roulette or split decision there again).  kCache: the irradiance
// cache or ADRRS is on (a render without them runs the leaner instance).
template <bool kCache>
__global__ void k_shade(DevRender R, int bounce, int last, int copies_pass) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= R.counters[copies_pass ? 9 : 0]) return;
    const uint32_t p = copies_pass ? R.q_copy[i] : R.q_cur[i];
    const uint32_t px = kCache ? pixel_of(R, p) : p, stream = kCache ? stream_of(R, p) : p;
    const pg_hit h = R.hits[p];
    const V d = ld3(R.rd, p);
    V thr = ld3(R.thr, p);
    bool cont = false;
    const bool rec_on = R.recording != 0;  // camera paths only: no split copies while recording
    if (h.prim == PG_NO_HIT) {
        // miss: a pending record saw infinity (distance 0)
        if (rec_on && R.rec_pending[p] >= 0) {
            R.rec[p * kMaxRecords + (uint32_t)R.rec_pending[p]].distance = 0.0f;
            R.rec_pending[p] = -1;
        }
        if (R.env) {
            // the environment (raytrace.rgen:1025-1037), MIS-weighted against its NEE:
            // a uniform direction in the hemisphere of the previous vertex
            float w = 1.0f;
            const float pp = R.prev_pdf[p];
            if (R.rp.use_nee && pp > 0.0f) {
                const float pl = 0.15915494309189535f / (float)R.n_lights;
                w = R.rp.use_mis ? pp * pp / (pp * pp + pl * pl) : 0.0f;
            }
            const V Le = mul(env_radiance(R, d), w);
            if (maxc(Le) > 0.0f) {
                add_image(R, px, hmul(thr, Le));
                R.found[p] = 1;
                if (rec_on) update_records(R, p, R.rec_count[p], Le);
            }
        }
    } else {
        const V o = ld3(R.ro, p);
        const V x = add(o, mul(d, h.t));
        V ng;
        uint32_t mat_id;
        uint32_t light_id = 0xFFFFFFFFu;
        if (h.prim & PG_SPHERE_BIT) {
            const pg_sphere &sp = R.S.spheres[h.prim & ~PG_SPHERE_BIT];
            ng = mul(sub(x, mk(sp.center[0], sp.center[1], sp.center[2])), 1.0f / sp.radius);
            mat_id = sp.material;
        } else {
            const uint32_t t = h.prim;
            const V v0 = ld3(R.pos, R.idx[3 * t]), v1 = ld3(R.pos, R.idx[3 * t + 1]), v2 = ld3(R.pos, R.idx[3 * t + 2]);
            ng = nrm(cross3(sub(v1, v0), sub(v2, v0)));
            mat_id = R.tri_mat[t];
        }
        pg_material m = R.mats[mat_id];
        if (m.texture > 0 && !(h.prim & PG_SPHERE_BIT) && (m.type == PG_MAT_DIFFUSE || m.type == PG_MAT_PHONG)) {
            // diffuse reflectance times the texture (raytrace.rgen:233-249)
            float tc[3];
            tex_rgb(R.S, h.prim, (uint32_t)m.texture - 1u, h.u, h.v, tc);
            for (int c = 0; c < 3; ++c) m.albedo[c] *= tc[c];
        }
        const bool front = dot3(d, ng) < 0.0f;  // raytrace.rchit:42-48
        const V n = front ? ng : mul(ng, -1.0f);
        const V wi = mul(d, -1.0f);
        // irradiance cache and ADRRS (raytrace.rgen:1080-1139): a vertex inside
        // cached spheres either takes their irradiance, adds next-event
        // estimation and ends the path, or (ADRRS) compares the path's
        // throughput with the weight window the cached irradiance gives:
        // Russian roulette below it, splitting above; a vertex outside every
        // sphere may queue a new entry
        bool ic_end = false, rr_end = false;
        V ic_L = mk(0, 0, 0);
        int copies = 1;
        uint32_t split_base = 0;
        if (kCache && (R.ic.query || (R.adrrs_est && bounce >= 1)) && !copies_pass && !last &&
            m.type != PG_MAT_LIGHT && ic_capable(R.ic, m)) {
            V E;
            if (ic_query(R.ic, x, n, E)) {
                if (R.adrrs_est) {
                    rr_end = adrrs_vertex(R, px, stream, bounce, E, thr, copies, split_base);
                } else {
                    ic_end = true;
                    ic_L = hmul(approx_diffuse(m, n, wi), E);
                }
            } else if (R.ic.grow && rnd(R.rp.seed, stream, R.sample, dimb(bounce, 8)) < R.ic.create_prob &&
                       R.ic.state[2] < R.ic.capacity && atomicAdd(&R.ic.created[px], 1u) < kIcMaxNewPerPixel) {
                ic_push(R.ic, x, n, -1, stream, (uint32_t)bounce, R.sample);
            }
        }
        // distance of a pending record (raytrace.rgen:1149-1156, 1201-1212); a
        // path that ends at the cache or in the roulette leaves it as it is
        if (rec_on && R.rec_pending[p] >= 0 && !ic_end && !rr_end) {
            pg_directional_data &rd = R.rec[p * kMaxRecords + (uint32_t)R.rec_pending[p]];
            rd.distance += h.t * R.rec_factor[p];
            if (!is_delta(m) && !almost_delta(m)) R.rec_pending[p] = -1;
        }
        if (m.type == PG_MAT_LIGHT) {
            // emission, MIS-weighted against NEE unless seen from the camera or a delta bounce
            float w = 1.0f;
            const float pp = R.prev_pdf[p];
            if (R.rp.use_nee && pp > 0.0f) {
                if (!R.rp.use_mis) {
                    w = 0.0f;
                } else {
                    // the light of this emitter
                    if (h.prim & PG_SPHERE_BIT) {
                        for (uint32_t l = 0; l < R.n_lights; ++l)
                            if (R.lights[l].type == 1 && R.lights[l].sphere == (h.prim & ~PG_SPHERE_BIT)) light_id = l;
                    } else if (R.tri_light[h.prim] >= 0) {
                        light_id = (uint32_t)R.tri_light[h.prim];
                    }
                    if (light_id != 0xFFFFFFFFu) {
                        const float cl = fabsf(dot3(ng, d));
                        const float pl = light_pdf(R, light_id, h.t, cl);
                        w = pp * pp / (pp * pp + pl * pl);
                    }
                }
            }
            if (front || (h.prim & PG_SPHERE_BIT) == 0) {
                const V Le = mul(mk(m.emission[0], m.emission[1], m.emission[2]), w);
                if (maxc(Le) > 0.0f) {
                    add_image(R, px, hmul(thr, Le));
                    R.found[p] = 1;
                    if (rec_on) update_records(R, p, R.rec_count[p], Le);
                }
            }
        } else if (!last && !rr_end) {
            if (kCache && ic_end) {
                // the cached irradiance; it reaches no guiding record (raytrace.rgen:1119)
                const V c = hmul(thr, ic_L);
                if (maxc(c) > 0.0f) {
                    add_image(R, px, c);
                    R.found[p] = 1;
                }
            }
            // split copies (raytrace.rgen:883-902, 1684-1708): paths of their own at
            // this vertex, shaded by the copies pass of this bounce with their own
            // next-event sample and continuation
            for (int c = 1; kCache && c < copies; ++c) {
                const uint32_t slot = split_base + (uint32_t)c - 1u, q2 = R.n_pix + slot;
                R.split_pix[slot] = px;
                R.split_stream[slot] = fmix32(stream * 0x9e3779b1u + (uint32_t)(bounce * (int)kMaxSplits + c));
                st3(R.ro, q2, o);
                st3(R.rd, q2, d);
                st3(R.thr, q2, thr);
                R.hits[q2] = h;
                R.prev_pdf[q2] = R.prev_pdf[p];
                R.found[q2] = 0;
                R.q_copy[atomicAdd(&R.counters[9], 1u)] = q2;
            }
            cont = shade_vertex(R, p, stream, bounce, rec_on, ic_end, m, x, n, d, front, thr);
        }
    }
    warp_append(&R.counters[1], R.q_next, p, cont);
}

// Unoccluded shadow ray i: its NEE contribution into the image and the
// path's guiding records.
__device__ __forceinline__ void shadow_finish(const DevRender &R, uint32_t i) {
    const uint32_t p = R.sh_pix[i];
    add_image(R, pixel_of(R, p), ld3(R.sh_c, i));
    R.found[p] = 1;
    if (R.recording) update_records(R, p, R.sh_nrec[i], ld3(R.sh_l, i));
}

// Persistent any-hit stage over the shadow queue (fetch from counters[7]),
// scheduled like k_extend.
// kCount: also add the traversal work to stats[4] (nodes) and stats[5] (triangles).
template <bool kCount>
__global__ void __launch_bounds__(128, 8) k_shadow(DevRender R) {
    const uint32_t n = R.counters[2];
    const int lane = threadIdx.x & 31;
    TravState st;
    int deep[kDeepStack];
    WorkCount wc;
    NoCount nc;
    uint32_t i = 0;
    bool have = false, exhausted = false;
    for (;;) {
        if (!exhausted) {
            const unsigned need = __ballot_sync(0xffffffffu, !have);
            if (need) {
                const int leader = __ffs(need) - 1;
                uint32_t base = 0;
                if (lane == leader) base = atomicAdd(&R.counters[7], (uint32_t)__popc(need));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (!have) {
                    const uint32_t idx = base + (uint32_t)__popc(need & ((1u << lane) - 1u));
                    if (idx < n) {
                        i = idx;
                        const float o[3] = {R.sh_o[3 * i], R.sh_o[3 * i + 1], R.sh_o[3 * i + 2]};
                        const float d[3] = {R.sh_d[3 * i], R.sh_d[3 * i + 1], R.sh_d[3 * i + 2]};
                        // a sphere in the way decides the query at once
                        have = !trav_begin<true>(R.S, st, o, d, kTMin, R.sh_tmax[i]);
                    }
                }
                if (base + (uint32_t)__popc(need) >= n) exhausted = true;  // warp-uniform
            }
        }
        if (!__any_sync(0xffffffffu, have)) break;
        if (have) {
            const bool done = kCount ? trav_step<true>(R.S, st, deep, wc) : trav_step<true>(R.S, st, deep, nc);
            if (done) {
                if (st.best_id == PG_NO_HIT) shadow_finish(R, i);
                have = false;
            }
        }
    }
    if (kCount) {
        atomicAdd(&R.stats[4], (unsigned long long)wc.nodes);
        atomicAdd(&R.stats[5], (unsigned long long)wc.tris);
    }
}

// commitSamples (raytrace.rgen:980-990) and slot reuse when the path found no light
__global__ void k_commit(DevRender R, uint32_t n_pix) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_pix) return;
    const uint32_t start = R.rec_start[p], cnt = R.rec_count[p];
    uint32_t valid = 0;
    for (uint32_t k = start; k < cnt; ++k) {
        const uint32_t s = p * kMaxRecords + k;
        pg_directional_data &rd = R.rec[s];
        const float w = record_weight(ld3(R.rec_lsum, s), rd.pdf);
        if (!(w > 0.0f) || rd.flags == PG_INVALID_REGION) {
            rd.flags = PG_INVALID_REGION;
        } else {
            rd.weight = w;
            ++valid;
        }
    }
    if (R.found[p]) {
        R.rec_start[p] = cnt;
        if (valid) atomicAdd(&R.counters[4], valid);
    } else {
        for (uint32_t k = start; k < cnt; ++k) R.rec[p * kMaxRecords + k].flags = PG_INVALID_REGION;
        R.rec_count[p] = start;
    }
}

// After a bounce: count the rays, make the next queue current.
__global__ void k_advance(DevRender R) {
    R.stats[0] += R.counters[0];
    R.stats[1] += R.counters[2];
    R.counters[0] = R.counters[1];
    R.counters[1] = 0;
    R.counters[2] = 0;
    R.counters[6] = 0;
    R.counters[7] = 0;
    R.counters[9] = 0;
}

__global__ void k_reset_records(pg_directional_data *rec, uint32_t n_slots, uint32_t *rec_start, uint32_t n_pix) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_slots) rec[i].flags = PG_INVALID_REGION;
    if (i < n_pix) rec_start[i] = 0;
}

// One shading-function call per probe (pg_probe_shading).
__global__ void k_probe_shading(const pg_material *mats, uint32_t n_mats, const pg_vmm_theta *vmms,
                                uint32_t n_vmms, const pg_shading_probe *P, uint32_t count, pg_shading_result *out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const pg_shading_probe q = P[i];
    pg_shading_result r;
    const bool uses_mat = q.op == PG_PROBE_BSDF_EVAL || q.op == PG_PROBE_BSDF_SAMPLE || q.op == PG_PROBE_CONTINUE ||
                          q.op == PG_PROBE_APPROX_DIFFUSE;
    const bool uses_vmm = q.op == PG_PROBE_VMM_PDF || q.op == PG_PROBE_VMM_SAMPLE ||
                          (q.op == PG_PROBE_CONTINUE && (q.flags & 8u));
    const bool bad = (uses_mat && q.material >= n_mats) || (uses_vmm && q.vmm >= n_vmms);
    for (int k = 0; k < 8; ++k) r.v[k] = bad ? __int_as_float(0x7fc00000) : 0.0f;
    if (bad) {
        out[i] = r;
        return;
    }
    const V n = mk(q.n[0], q.n[1], q.n[2]), wi = mk(q.wi[0], q.wi[1], q.wi[2]);
    const V wo = mk(q.wo[0], q.wo[1], q.wo[2]), x = mk(q.x[0], q.x[1], q.x[2]);
    const bool front = (q.flags & 1u) != 0;
    const int par = (q.flags & 2u) ? 1 : 0;
    auto put = [&](int at, V v) {
        r.v[at] = v.x;
        r.v[at + 1] = v.y;
        r.v[at + 2] = v.z;
    };
    switch (q.op) {
        case PG_PROBE_FRESNEL:
            r.v[0] = fresnel_dielectric(q.a, q.b);
            break;
        case PG_PROBE_FRESNEL_CONDUCTOR:
            r.v[0] = fresnel_conductor(q.a, q.b, q.c);
            break;
        case PG_PROBE_BSDF_EVAL: {
            const MatEval e = bsdf_eval(mats[q.material], n, wi, wo);
            put(0, e.f);
            r.v[3] = e.pdf;
            break;
        }
        case PG_PROBE_BSDF_SAMPLE: {
            const pg_material &m = mats[q.material];
            const V w = sample_bsdf(m, mul(wi, -1.0f), n, q.u[1], q.u[2], q.u[3]);
            put(0, w);
            r.v[3] = bsdf_eval(m, n, wi, w).pdf;
            break;
        }
        case PG_PROBE_VMM_PDF:
            r.v[0] = vmm_pdf(vmms[q.vmm], wo, x, par);
            break;
        case PG_PROBE_VMM_SAMPLE:
            put(0, vmm_sample(vmms[q.vmm], x, par, q.u[4], q.u[2], q.u[3]));
            break;
        case PG_PROBE_CONTINUE: {
            const pg_material &m = mats[q.material];
            const uint32_t rf = (q.flags & 16u) ? PG_RENDER_GUIDE_ALMOST_DISCRETE : 0u;
            const bool gm = (q.flags & 4u) && guided_material(m, rf);
            const pg_vmm_theta *mix = (q.flags & 8u) ? &vmms[q.vmm] : nullptr;
            const Continuation c = continue_path(m, mul(wi, -1.0f), n, front, x, gm, mix, par, q.c, q.u[0], q.u[1],
                                                 q.u[2], q.u[3], [&] { return q.u[4]; });
            put(0, c.wo);
            r.v[3] = c.pdf;
            put(4, c.tc);
            break;
        }
        case PG_PROBE_TO_WORLD:
            put(0, to_world(wo, n));
            break;
        case PG_PROBE_WEIGHT_WINDOW: {
            int nn;
            r.v[0] = weight_window(wi, wo, x, q.a, q.u[0], nn);
            r.v[1] = (float)nn;
            break;
        }
        case PG_PROBE_APPROX_DIFFUSE:
            put(0, approx_diffuse(mats[q.material], n, wi));
            break;
        default:
            break;
    }
    out[i] = r;
}

// Sample recording of one path per thread (pg_probe_records): the events in
// order through the renderer's record functions, then the commit.
__global__ void k_probe_records(const pg_record_event *ev, const uint32_t *offsets, uint32_t n_paths, float *weights,
                                uint32_t *flags, uint32_t *counts) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_paths) return;
    float lsum[3 * kMaxRecords], tc[3 * kMaxRecords], pdf[kMaxRecords];
    uint32_t region[kMaxRecords];
    uint32_t cnt = 0;
    for (uint32_t e = offsets[p]; e < offsets[p + 1]; ++e) {
        const pg_record_event q = ev[e];
        if (q.kind == 0) {
            if (cnt >= (uint32_t)kMaxRecords) continue;
            for (int c = 0; c < 3; ++c) {
                lsum[3 * cnt + c] = 0.0f;
                tc[3 * cnt + c] = q.tc[c];
            }
            pdf[cnt] = q.pdf;
            region[cnt] = q.region;
            ++cnt;
        } else {
            add_record_radiance(lsum, tc, 0u, cnt, mk(q.light[0], q.light[1], q.light[2]));
        }
    }
    for (uint32_t k = 0; k < cnt; ++k) {
        const float w = record_weight(ld3(lsum, k), pdf[k]);
        const bool valid = w > 0.0f && region[k] != PG_INVALID_REGION;
        weights[p * kMaxRecords + k] = valid ? w : 0.0f;
        flags[p * kMaxRecords + k] = valid ? region[k] : PG_INVALID_REGION;
    }
    counts[p] = cnt;
}

__global__ void k_trace_closest(DevScene S, const pg_ray *rays, uint32_t n, pg_hit *hits) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const pg_ray r = rays[i];
    pg_hit h;
    trace_closest(S, r.org, r.dir, r.tmin, r.tmax, h);
    hits[i] = h;
}

__global__ void k_trace_closest_counted(DevScene S, const pg_ray *rays, uint32_t n, pg_hit *hits, uint32_t *nodes,
                                        uint32_t *tris) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const pg_ray r = rays[i];
    pg_hit h;
    WorkCount c;
    trace_closest(S, r.org, r.dir, r.tmin, r.tmax, h, c);
    hits[i] = h;
    nodes[i] = c.nodes;
    tris[i] = c.tris;
}

__global__ void k_trace_any(DevScene S, const pg_ray *rays, uint32_t n, uint32_t *occ) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const pg_ray r = rays[i];
    occ[i] = trace_any(S, r.org, r.dir, r.tmin, r.tmax) ? 1u : 0u;
}

}  // namespace pg

using namespace pg;

// ---------------------------------------------------------------------------
// Scene object
// ---------------------------------------------------------------------------
struct pg_scene {
    SceneData host;
    DevBvhNode *d_nodes = nullptr;
    float4 *d_tris = nullptr;
    pg_sphere *d_spheres = nullptr;
    float *d_pos = nullptr;
    uint32_t *d_idx = nullptr;
    uint32_t *d_tri_mat = nullptr;
    pg_material *d_mats = nullptr;
    DevLight *d_lights = nullptr;
    uint32_t *d_light_tris = nullptr;
    float *d_light_cdf = nullptr;
    int32_t *d_tri_light = nullptr;
    float *d_env = nullptr;
    float *d_tri_uv = nullptr;
    uint4 *d_tex_info = nullptr;
    uchar4 *d_tex_data = nullptr;
    unsigned long long *d_stats = nullptr;
    uint32_t n_lights = 0;
    bool uploaded = false;
    std::vector<DevLight> h_lights;
    std::vector<uint32_t> h_light_tris;
    std::vector<float> h_light_cdf;
    std::vector<int32_t> h_tri_light;
    float aabb[6] = {0, 0, 0, 0, 0, 0};
    // render scratch
    uint32_t cap_pix = 0;
    uint32_t cap_paths = 0;       // path slots: pixels plus split copies
    uint32_t persist_blocks = 0;  // resident CTAs of the persistent traversal stages (all SMs)
    std::vector<void *> bufs;
    DevRender R{};
    uint32_t *d_counters = nullptr;
    pg_adrrs_config adrrs{nullptr, 5.0f, 1, {0, 0, 0, 0}};
    // irradiance cache
    struct IcStore {
        bool on = false;
        pg_irradiance_cache_config cfg{};
        pg_ic_entry *entries = nullptr;   // capacity
        uint32_t *state = nullptr;        // 4 words (DevIc::state)
        uint32_t *cell_start = nullptr;   // kIcCells + 1
        uint32_t *cell_count = nullptr;   // kIcCells
        uint32_t *cell_fill = nullptr;    // kIcCells
        uint32_t *refs = nullptr;
        uint32_t cap_refs = 0;
        IcRequest *requests = nullptr;    // req_cap
        IcResult *results = nullptr;      // req_cap
        float4 *samples = nullptr;        // req_cap x 200
        uint32_t req_cap = 0;
        uint32_t *created = nullptr;      // per pixel
        uint32_t cap_created = 0;
        bool grid_stale = true;
    } ic;
};

namespace {

int scene_error(int st, const std::string &m) { return set_error(nullptr, st, m); }

template <typename T>
int upload(T **dst, const std::vector<T> &src) {
    if (src.empty()) {
        *dst = nullptr;
        return PG_OK;
    }
    if (cudaMalloc(dst, sizeof(T) * src.size()) != cudaSuccess) return PG_ERR_CUDA;
    if (cudaMemcpy(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice) != cudaSuccess) return PG_ERR_CUDA;
    return PG_OK;
}

// Host side of scene creation: BVH, scene box and light tables.
void build_host(pg_scene *sc) {
    SceneData &s = sc->host;
    build_bvh(s, 4);
    // scene box (SceneLoader::calculateSceneSize, src/SceneLoader.cpp:350-368)
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t v = 0; v < s.pos.size() / 3; ++v)
        for (int i = 0; i < 3; ++i) {
            lo[i] = std::min(lo[i], s.pos[3 * v + i]);
            hi[i] = std::max(hi[i], s.pos[3 * v + i]);
        }
    for (const auto &sp : s.spheres)
        for (int i = 0; i < 3; ++i) {
            lo[i] = std::min(lo[i], sp.center[i] - sp.radius);
            hi[i] = std::max(hi[i], sp.center[i] + sp.radius);
        }
    for (int i = 0; i < 3; ++i) {
        sc->aabb[i] = lo[i];
        sc->aabb[3 + i] = hi[i];
    }
    // lights: one per emissive material over triangles, one per emissive sphere
    auto &lights = sc->h_lights;
    auto &ltris = sc->h_light_tris;
    auto &lcdf = sc->h_light_cdf;
    auto &tri_light = sc->h_tri_light;
    lights.clear();
    ltris.clear();
    lcdf.clear();
    tri_light.assign(s.tri_mat.size(), -1);
    for (uint32_t m = 0; m < s.mats.size(); ++m) {
        if (s.mats[m].type != PG_MAT_LIGHT) continue;
        DevLight L{};
        L.type = 0;
        L.first = (uint32_t)ltris.size();
        double acc = 0.0;
        std::vector<double> areas;
        for (uint32_t t = 0; t < s.tri_mat.size(); ++t) {
            if (s.tri_mat[t] != m) continue;
            const float *a = &s.pos[3 * (size_t)s.idx[3 * t]], *b = &s.pos[3 * (size_t)s.idx[3 * t + 1]],
                        *c = &s.pos[3 * (size_t)s.idx[3 * t + 2]];
            const double e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
            const double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
                         cz = e1[0] * e2[1] - e1[1] * e2[0];
            const double ar = 0.5 * sqrt(cx * cx + cy * cy + cz * cz);
            ltris.push_back(t);
            tri_light[t] = (int32_t)lights.size();
            areas.push_back(ar);
            acc += ar;
        }
        L.count = (uint32_t)(ltris.size() - L.first);
        if (L.count == 0) continue;
        double run = 0.0;
        for (double ar : areas) {
            run += ar;
            lcdf.push_back((float)(run / acc));
        }
        lcdf.back() = 1.0f;
        L.area = (float)acc;
        for (int i = 0; i < 3; ++i) L.emission[i] = s.mats[m].emission[i];
        lights.push_back(L);
    }
    for (uint32_t i = 0; i < s.spheres.size(); ++i) {
        const pg_material &m = s.mats[s.spheres[i].material];
        if (m.type != PG_MAT_LIGHT) continue;
        DevLight L{};
        L.type = 1;
        L.sphere = i;
        L.area = 4.0f * 3.14159265f * s.spheres[i].radius * s.spheres[i].radius;
        for (int k = 0; k < 3; ++k) L.emission[k] = m.emission[k];
        lights.push_back(L);
    }
    if (!s.env.empty()) {  // the environment is the last light (SceneLoader::parseEnvMap)
        DevLight L{};
        L.type = 2;
        lights.push_back(L);
    }
    sc->n_lights = (uint32_t)lights.size();
}

// Device copy of the scene, made on first use (so scenes can be built and
// inspected on a machine without a GPU).
int ensure_uploaded(pg_scene *sc) {
    if (sc->uploaded) return PG_OK;
    const SceneData &s = sc->host;
    static_assert(sizeof(DevBvhNode) == sizeof(BvhNode), "host and device nodes share one layout");
    std::vector<DevBvhNode> dn(s.nodes.size());
    memcpy(dn.data(), s.nodes.data(), sizeof(BvhNode) * s.nodes.size());
    std::vector<float4> tv(s.tri_verts.size() / 4);
    memcpy(tv.data(), s.tri_verts.data(), sizeof(float) * s.tri_verts.size());
    int st = upload(&sc->d_nodes, dn);
    if (!st) st = upload(&sc->d_tris, tv);
    if (!st) st = upload(&sc->d_spheres, s.spheres);
    if (!st) st = upload(&sc->d_pos, s.pos);
    if (!st) st = upload(&sc->d_idx, s.idx);
    if (!st) st = upload(&sc->d_tri_mat, s.tri_mat);
    if (!st) st = upload(&sc->d_mats, s.mats);
    if (!st) st = upload(&sc->d_lights, sc->h_lights);
    if (!st) st = upload(&sc->d_light_tris, sc->h_light_tris);
    if (!st) st = upload(&sc->d_light_cdf, sc->h_light_cdf);
    if (!st) st = upload(&sc->d_tri_light, sc->h_tri_light);
    if (!st) st = upload(&sc->d_env, s.env);
    if (!st) st = upload(&sc->d_tri_uv, s.tri_uv);
    if (!st && !s.textures.empty()) {
        std::vector<uint4> info;
        std::vector<uchar4> texels;
        for (const auto &t : s.textures) {
            info.push_back(make_uint4((uint32_t)texels.size(), t.w, t.h, 0u));
            for (size_t i = 0; i < (size_t)t.w * t.h; ++i)
                texels.push_back(make_uchar4(t.rgba[4 * i], t.rgba[4 * i + 1], t.rgba[4 * i + 2], t.rgba[4 * i + 3]));
        }
        st = upload(&sc->d_tex_info, info);
        if (!st) st = upload(&sc->d_tex_data, texels);
    }
    if (!st && cudaMalloc(&sc->d_counters, sizeof(uint32_t) * 16) != cudaSuccess) st = PG_ERR_CUDA;
    if (!st && cudaMalloc(&sc->d_stats, sizeof(unsigned long long) * kNumStats) != cudaSuccess) st = PG_ERR_CUDA;
    if (st) return scene_error(st, "scene upload failed (CUDA)");
    sc->uploaded = true;
    return PG_OK;
}

// Per-stage CUDA-event timing of a render (PG_RENDER_TIME_STAGES): an event
// pair around every launch, read back whenever the pool fills.
struct StageTimer {
    static constexpr uint32_t kPairs = 256;
    bool on = false;
    cudaStream_t s = nullptr;
    std::vector<cudaEvent_t> ev;
    int stage[kPairs] = {};
    uint32_t used = 0;
    float ms[PG_STAGE_COUNT] = {};
    uint32_t launches[PG_STAGE_COUNT] = {};
    bool failed = false;

    bool init(bool enable, cudaStream_t st) {
        on = enable;
        s = st;
        if (!on) return true;
        ev.assign(2 * kPairs, nullptr);
        for (auto &e : ev)
            if (cudaEventCreate(&e) != cudaSuccess) return false;
        return true;
    }
    void begin(int stg) {
        if (!on) return;
        if (used == kPairs) flush();
        stage[used] = stg;
        if (cudaEventRecord(ev[2 * used], s) != cudaSuccess) failed = true;
    }
    void end() {
        if (!on) return;
        if (cudaEventRecord(ev[2 * used + 1], s) != cudaSuccess) failed = true;
        ++used;
    }
    void flush() {
        if (!on || used == 0) return;
        if (cudaEventSynchronize(ev[2 * used - 1]) != cudaSuccess) failed = true;
        for (uint32_t i = 0; i < used; ++i) {
            float t = 0.0f;
            if (cudaEventElapsedTime(&t, ev[2 * i], ev[2 * i + 1]) != cudaSuccess) failed = true;
            ms[stage[i]] += t;
            launches[stage[i]] += 1;
        }
        used = 0;
    }
    ~StageTimer() {
        for (auto e : ev)
            if (e) cudaEventDestroy(e);
    }
};

DevScene dev_scene(const pg_scene *sc) {
    DevScene S;
    S.nodes = sc->d_nodes;
    S.tris = sc->d_tris;
    S.spheres = sc->d_spheres;
    S.n_spheres = (uint32_t)sc->host.spheres.size();
    S.n_triangles = (uint32_t)sc->host.tri_mat.size();
    S.tri_uv = sc->d_tri_uv;
    S.tex_info = sc->d_tex_info;
    S.tex_data = sc->d_tex_data;
    S.alpha_salt = 0u;
    return S;
}

// The state a render call shares with the cache's paths: the scene, the
// camera basis, the settings and the guide.  Path buffers are left as they are.
int setup_render(pg_scene *sc, const pg_render_params *rp, pg_ctx *guide, cudaStream_t s, DevRender &R) {
    R.S = dev_scene(sc);
    R.pos = sc->d_pos;
    R.idx = sc->d_idx;
    R.tri_mat = sc->d_tri_mat;
    R.mats = sc->d_mats;
    R.lights = sc->d_lights;
    R.n_lights = sc->n_lights;
    R.light_tris = sc->d_light_tris;
    R.light_cdf = sc->d_light_cdf;
    R.tri_light = sc->d_tri_light;
    R.env = sc->d_env;
    R.env_w = sc->host.env_w;
    R.env_h = sc->host.env_h;
    const pg_camera cam = sc->host.camera;
    R.cam = cam;
    {
        float f[3] = {cam.target[0] - cam.origin[0], cam.target[1] - cam.origin[1], cam.target[2] - cam.origin[2]};
        float l = sqrtf(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
        for (int i = 0; i < 3; ++i) f[i] /= l;
        float r[3] = {f[1] * cam.up[2] - f[2] * cam.up[1], f[2] * cam.up[0] - f[0] * cam.up[2],
                      f[0] * cam.up[1] - f[1] * cam.up[0]};
        l = sqrtf(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        for (int i = 0; i < 3; ++i) r[i] /= l;
        const float u[3] = {r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]};
        for (int i = 0; i < 3; ++i) {
            R.cam_fwd[i] = f[i];
            R.cam_right[i] = r[i];
            R.cam_up[i] = u[i];
        }
        R.tan_half = tanf(cam.vfov_deg * 0.5f * 3.14159265f / 180.0f);
    }
    R.rp = *rp;
    R.S.alpha_salt = alpha_salt(rp->seed);
    R.guiding = rp->use_guiding ? 1 : 0;
    R.recording = rp->record_samples ? 1 : 0;
    memset(&R.guide, 0, sizeof R.guide);
    if (guide) {
        GuideView gv;
        const int st = guide_view(guide, &gv, s);
        if (st) return scene_error(st, pg_last_error(guide));
        for (int i = 0; i < 6; ++i) R.guide.root[i] = gv.root[i];
        R.guide.split_count = gv.split_count;
        R.guide.nodes = gv.nodes;
        R.guide.vmm = gv.vmm;
        R.guide.use_parallax = gv.use_parallax;
    }
    memset(&R.ic, 0, sizeof R.ic);
    return PG_OK;
}

// ---------------------------------------------------------------------------
// Irradiance cache (host side)
// ---------------------------------------------------------------------------
constexpr uint32_t kIcRequestCap = 16384;  // requests one pass can queue

void ic_free(pg_scene::IcStore &c) {
    cudaFree(c.entries);
    cudaFree(c.state);
    cudaFree(c.cell_start);
    cudaFree(c.cell_count);
    cudaFree(c.cell_fill);
    cudaFree(c.refs);
    cudaFree(c.requests);
    cudaFree(c.results);
    cudaFree(c.samples);
    cudaFree(c.created);
    c = pg_scene::IcStore{};
}

// The device view of the scene's cache; the grid spans the scene box.
void ic_view(const pg_scene *sc, DevIc &D) {
    const auto &c = sc->ic;
    memset(&D, 0, sizeof D);
    D.entries = c.entries;
    D.cell_start = c.cell_start;
    D.cell_refs = c.refs;
    D.cap_refs = c.cap_refs;
    for (int i = 0; i < 3; ++i) {
        const float lo = sc->aabb[i], hi = sc->aabb[3 + i];
        const float ext = hi - lo, margin = 1e-3f * std::max(ext, 1e-3f);
        D.lo[i] = lo - margin;
        D.inv_cell[i] = (float)kIcGrid / (ext + 2.0f * margin);
    }
    D.a = c.cfg.a;
    D.min_radius = c.cfg.min_radius;
    D.create_prob = c.cfg.create_prob;
    D.update_prob = c.cfg.update_prob;
    D.grad_max = c.cfg.gradients_max_length;
    D.use_gradients = c.cfg.use_gradients ? 1 : 0;
    D.visibility = c.cfg.visibility_check ? 1 : 0;
    D.on_glossy = c.cfg.use_on_glossy ? 1 : 0;
    D.num_nee = c.cfg.num_nee ? c.cfg.num_nee : 1u;
    D.requests = c.requests;
    D.req_cap = c.req_cap;
    D.capacity = c.cfg.capacity;
    D.created = c.created;
    D.state = c.state;
}

uint32_t sm_count() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return (uint32_t)std::max(1, sms);
}

// Rebuilds the cell lists over the current entries (all on the stream).
int ic_build_grid(pg_scene *sc, const DevIc &D, cudaStream_t s) {
    auto &c = sc->ic;
    if (cudaMemsetAsync(c.cell_count, 0, sizeof(uint32_t) * kIcCells, s) != cudaSuccess ||
        cudaMemsetAsync(c.cell_fill, 0, sizeof(uint32_t) * kIcCells, s) != cudaSuccess)
        return scene_error(PG_ERR_CUDA, "irradiance cache grid reset");
    // (entry, z) slabs, grid-stride over the entries the device holds
    const uint32_t G = 16u * sm_count();
    k_ic_grid_count<<<G, 128, 0, s>>>(D, c.cell_count);
    k_ic_grid_scan<<<1, 1024, 0, s>>>(c.cell_count, c.cell_start);
    k_ic_grid_fill<<<G, 128, 0, s>>>(D, c.cell_start, c.cell_fill, c.refs);
    k_ic_grid_sort<<<kIcCells / 128, 128, 0, s>>>(c.cell_start, c.refs, c.cap_refs);
    if (cudaGetLastError() != cudaSuccess) return scene_error(PG_ERR_CUDA, "irradiance cache grid launch failed");
    c.grid_stale = false;
    return PG_OK;
}

// After a sample pass: the queued requests' entries computed and written, the
// grid rebuilt.  No host synchronization.
int ic_process(pg_scene *sc, const DevRender &R, cudaStream_t s) {
    auto &c = sc->ic;
    const DevIc &D = R.ic;
    const uint32_t sms = sm_count();
    const uint32_t gq = (c.req_cap + 127) / 128;
    k_ic_assign<<<gq, 128, 0, s>>>(D);
    k_ic_paths<<<8 * sms, 128, 0, s>>>(R, c.samples);
    k_ic_reduce<<<std::min((c.req_cap + 3) / 4, 8 * sms), 128, 0, s>>>(R, c.samples, c.results);
    k_ic_slots<<<gq, 128, 0, s>>>(D, c.results);
    k_ic_commit<<<gq, 128, 0, s>>>(D, c.results);
    k_ic_finish<<<1, 1, 0, s>>>(D);
    if (cudaGetLastError() != cudaSuccess) return scene_error(PG_ERR_CUDA, "irradiance cache launch failed");
    return ic_build_grid(sc, D, s);
}

int create_common(pg_scene *sc, pg_scene **out) {
    build_host(sc);
    *out = sc;
    return PG_OK;
}

}  // namespace

extern "C" {

int pg_scene_create_cornell(const pg_cornell_params *p, pg_scene **out) {
    if (!p || !out) return PG_ERR_ARG;
    if (p->width == 0 || p->height == 0 || p->ico_level < 0 || p->ico_level > 8)
        return scene_error(PG_ERR_ARG, "bad Cornell box parameters");
    pg_scene *sc = new pg_scene();
    make_cornell(sc->host, *p);
    return create_common(sc, out);
}

int pg_scene_create_plates(const pg_plates_params *p, pg_scene **out) {
    if (!p || !out) return PG_ERR_ARG;
    if (p->width == 0 || p->height == 0 || p->occluder_grid > 4096)
        return scene_error(PG_ERR_ARG, "bad plates-scene parameters");
    pg_scene *sc = new pg_scene();
    make_glossy_plates(sc->host, *p);
    return create_common(sc, out);
}

int pg_scene_load(const char *path, uint32_t width, uint32_t height, pg_scene **out) {
    if (!path || !out || width == 0 || height == 0) return PG_ERR_ARG;
    pg_scene *sc = new pg_scene();
    if (!load_mitsuba(sc->host, path, width, height)) {
        const std::string msg = sc->host.error;
        delete sc;
        const bool io = msg.rfind("cannot open", 0) == 0;
        return scene_error(io ? PG_ERR_IO : PG_ERR_PARSE, msg);
    }
    return create_common(sc, out);
}

int pg_scene_set_envmap(pg_scene *sc, const float *rgb, uint32_t width, uint32_t height) {
    if (!sc || (!rgb && (width || height)) || (width == 0) != (height == 0)) return PG_ERR_ARG;
    SceneData &s = sc->host;
    s.env.assign(rgb, rgb + 3 * (size_t)width * height);
    s.env_w = width;
    s.env_h = height;
    // the light table gains (or loses) the environment; device copies follow
    auto &L = sc->h_lights;
    if (!L.empty() && L.back().type == 2) L.pop_back();
    if (width) {
        DevLight e{};
        e.type = 2;
        L.push_back(e);
    }
    sc->n_lights = (uint32_t)L.size();
    if (sc->uploaded) {
        cudaFree(sc->d_env);
        cudaFree(sc->d_lights);
        sc->d_env = nullptr;
        sc->d_lights = nullptr;
        int st = upload(&sc->d_env, s.env);
        if (!st) st = upload(&sc->d_lights, L);
        if (st) return scene_error(st, "environment upload failed (CUDA)");
    }
    return PG_OK;
}

int pg_scene_get_envmap(const pg_scene *sc, float *rgb_out, uint32_t *width, uint32_t *height) {
    if (!sc) return PG_ERR_ARG;
    if (width) *width = sc->host.env_w;
    if (height) *height = sc->host.env_h;
    if (rgb_out && !sc->host.env.empty()) memcpy(rgb_out, sc->host.env.data(), sizeof(float) * sc->host.env.size());
    return PG_OK;
}

int pg_exr_read(const char *path, float *rgb_out, uint64_t capacity, uint32_t *width, uint32_t *height) {
    if (!path || !width || !height) return PG_ERR_ARG;
    ExrImage img;
    std::string err;
    if (!read_exr(path, img, err)) return scene_error(err.rfind("cannot open", 0) == 0 ? PG_ERR_IO : PG_ERR_PARSE, err);
    *width = img.width;
    *height = img.height;
    if (!rgb_out) return PG_OK;
    if (capacity < img.rgb.size()) return scene_error(PG_ERR_ARG, "EXR image larger than the buffer");
    memcpy(rgb_out, img.rgb.data(), sizeof(float) * img.rgb.size());
    return PG_OK;
}

int pg_exr_write(const char *path, const float *rgb, uint32_t width, uint32_t height) {
    if (!path || !rgb || !width || !height) return PG_ERR_ARG;
    std::string err;
    if (!write_exr(path, rgb, width, height, err)) return scene_error(PG_ERR_IO, err);
    return PG_OK;
}

int pg_scene_destroy(pg_scene *sc) {
    if (!sc) return PG_OK;
    cudaFree(sc->d_nodes);
    cudaFree(sc->d_tris);
    cudaFree(sc->d_spheres);
    cudaFree(sc->d_pos);
    cudaFree(sc->d_idx);
    cudaFree(sc->d_tri_mat);
    cudaFree(sc->d_mats);
    cudaFree(sc->d_lights);
    cudaFree(sc->d_light_tris);
    cudaFree(sc->d_light_cdf);
    cudaFree(sc->d_tri_light);
    cudaFree(sc->d_env);
    cudaFree(sc->d_tri_uv);
    cudaFree(sc->d_tex_info);
    cudaFree(sc->d_tex_data);
    cudaFree(sc->d_stats);
    cudaFree(sc->d_counters);
    for (void *b : sc->bufs) cudaFree(b);
    ic_free(sc->ic);
    delete sc;
    return PG_OK;
}

void pg_default_irradiance_cache_config(pg_irradiance_cache_config *out) {
    if (!out) return;
    memset(out, 0, sizeof *out);
    out->capacity = 100000;
    out->a = 0.2f;
    out->min_radius = 0.1f;
    out->create_prob = 0.0005f;
    out->update_prob = 0.00001f;
    out->use_gradients = 0;
    out->gradients_max_length = 5.0f;
    out->visibility_check = 0;
    out->use_on_glossy = 0;
    out->num_nee = 1;
}

int pg_scene_set_irradiance_cache(pg_scene *sc, const pg_irradiance_cache_config *cfg) {
    if (!sc || !cfg) return PG_ERR_ARG;
    if (cfg->capacity > (1u << 24)) return scene_error(PG_ERR_ARG, "irradiance cache capacity above 2^24 entries");
    if (cfg->num_nee > 64) return scene_error(PG_ERR_ARG, "irradiance cache: num_nee above 64");
    if (cfg->capacity && (!(cfg->a > 0.0f) || !std::isfinite(cfg->a) || !(cfg->min_radius >= 0.0f) ||
                          !(cfg->create_prob >= 0.0f && cfg->create_prob <= 1.0f) ||
                          !(cfg->update_prob >= 0.0f && cfg->update_prob <= 1.0f) ||
                          !(cfg->gradients_max_length >= 0.0f)))
        return scene_error(PG_ERR_ARG, "irradiance cache: a > 0, min_radius >= 0, probabilities in [0, 1], "
                                       "gradients_max_length >= 0");
    if (sc->ic.on) cudaDeviceSynchronize();  // a render may still read the old cache
    ic_free(sc->ic);
    if (cfg->capacity == 0) return PG_OK;
    auto &c = sc->ic;
    c.req_cap = kIcRequestCap;
    c.cap_refs = std::max(1u << 20, 8u * cfg->capacity);
    bool ok = cudaMalloc(&c.entries, sizeof(pg_ic_entry) * cfg->capacity) == cudaSuccess &&
              cudaMalloc(&c.state, 4 * sizeof(uint32_t)) == cudaSuccess &&
              cudaMalloc(&c.cell_start, sizeof(uint32_t) * (kIcCells + 1)) == cudaSuccess &&
              cudaMalloc(&c.cell_count, sizeof(uint32_t) * kIcCells) == cudaSuccess &&
              cudaMalloc(&c.cell_fill, sizeof(uint32_t) * kIcCells) == cudaSuccess &&
              cudaMalloc(&c.refs, sizeof(uint32_t) * c.cap_refs) == cudaSuccess &&
              cudaMalloc(&c.requests, sizeof(IcRequest) * c.req_cap) == cudaSuccess &&
              cudaMalloc(&c.results, sizeof(IcResult) * c.req_cap) == cudaSuccess &&
              cudaMalloc(&c.samples, sizeof(float4) * kIcSamples * (size_t)c.req_cap) == cudaSuccess;
    ok = ok && cudaMemset(c.state, 0, 4 * sizeof(uint32_t)) == cudaSuccess &&
         cudaMemset(c.cell_start, 0, sizeof(uint32_t) * (kIcCells + 1)) == cudaSuccess &&
         cudaDeviceSynchronize() == cudaSuccess;
    if (!ok) {
        ic_free(c);
        return scene_error(PG_ERR_NOMEM, "irradiance cache: out of device memory");
    }
    c.cfg = *cfg;
    c.on = true;
    c.grid_stale = false;  // empty lists
    return PG_OK;
}

int pg_scene_get_irradiance_cache(pg_scene *sc, pg_ic_entry *out, uint32_t capacity, uint32_t *n_entries) {
    if (!sc || !n_entries) return PG_ERR_ARG;
    *n_entries = 0;
    if (!sc->ic.on) return PG_OK;
    uint32_t st[4];
    if (cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(st, sc->ic.state, sizeof st, cudaMemcpyDeviceToHost) != cudaSuccess)
        return scene_error(PG_ERR_CUDA, "irradiance cache read");
    *n_entries = st[2];
    if (out && st[2]) {
        if (capacity < st[2]) return scene_error(PG_ERR_ARG, "irradiance cache: output holds fewer entries than the cache");
        if (cudaMemcpy(out, sc->ic.entries, sizeof(pg_ic_entry) * st[2], cudaMemcpyDeviceToHost) != cudaSuccess)
            return scene_error(PG_ERR_CUDA, "irradiance cache read");
    }
    return PG_OK;
}

int pg_scene_set_irradiance_cache_entries(pg_scene *sc, const pg_ic_entry *entries, uint32_t n) {
    if (!sc || (n && !entries)) return PG_ERR_ARG;
    if (!sc->ic.on) return scene_error(PG_ERR_ARG, "no irradiance cache on the scene (pg_scene_set_irradiance_cache)");
    if (n > sc->ic.cfg.capacity) return scene_error(PG_ERR_ARG, "more entries than the cache's capacity");
    const uint32_t st[4] = {0, 0, n, 0};
    if (cudaDeviceSynchronize() != cudaSuccess ||
        (n && cudaMemcpy(sc->ic.entries, entries, sizeof(pg_ic_entry) * n, cudaMemcpyHostToDevice) != cudaSuccess) ||
        cudaMemcpy(sc->ic.state, st, sizeof st, cudaMemcpyHostToDevice) != cudaSuccess)
        return scene_error(PG_ERR_CUDA, "irradiance cache write");
    sc->ic.grid_stale = true;
    // grow the reference list to what the grid will need
    DevIc D;
    ic_view(sc, D);
    if (int st2 = ic_build_grid(sc, D, nullptr)) return st2;
    uint32_t total = 0;
    if (cudaMemcpy(&total, sc->ic.cell_start + kIcCells, sizeof total, cudaMemcpyDeviceToHost) != cudaSuccess)
        return scene_error(PG_ERR_CUDA, "irradiance cache grid size");
    if (total > sc->ic.cap_refs) {
        cudaFree(sc->ic.refs);
        sc->ic.refs = nullptr;
        const uint64_t want = std::min<uint64_t>(2ull * total, 0xFFFFFFF0ull);
        if (cudaMalloc(&sc->ic.refs, sizeof(uint32_t) * want) != cudaSuccess) {
            sc->ic.cap_refs = 0;
            sc->ic.grid_stale = true;
            return scene_error(PG_ERR_NOMEM, "irradiance cache grid: out of device memory");
        }
        sc->ic.cap_refs = (uint32_t)want;
        ic_view(sc, D);
        if (int st2 = ic_build_grid(sc, D, nullptr)) return st2;
    }
    return cudaDeviceSynchronize() == cudaSuccess ? PG_OK : scene_error(PG_ERR_CUDA, "irradiance cache grid build");
}

int pg_scene_set_adrrs(pg_scene *sc, const pg_adrrs_config *cfg) {
    if (!sc || !cfg) return PG_ERR_ARG;
    if (!(cfg->s > 1.0f) || !std::isfinite(cfg->s)) return scene_error(PG_ERR_ARG, "ADRRS: s must be above 1");
    sc->adrrs = *cfg;
    return PG_OK;
}

int pg_ic_query(pg_scene *sc, const float *positions, const float *normals, uint32_t n, float *rgb, uint32_t *found,
                void *stream) {
    if (!sc || (n && (!positions || !normals || !rgb || !found))) return PG_ERR_ARG;
    if (!sc->ic.on) return scene_error(PG_ERR_ARG, "no irradiance cache on the scene (pg_scene_set_irradiance_cache)");
    if (n == 0) return PG_OK;
    cudaStream_t s = (cudaStream_t)stream;
    DevIc D;
    ic_view(sc, D);
    if (sc->ic.grid_stale)
        if (int st = ic_build_grid(sc, D, s)) return st;
    k_ic_query_probe<<<(n + 127) / 128, 128, 0, s>>>(D, positions, normals, n, rgb, found);
    return cudaGetLastError() == cudaSuccess ? PG_OK : scene_error(PG_ERR_CUDA, "irradiance cache query launch");
}

int pg_ic_compute(pg_scene *sc, const pg_render_params *rp, pg_ctx *guide, const pg_ic_request *requests, uint32_t n,
                  pg_ic_entry *out, void *stream) {
    if (!sc || !rp || (n && (!requests || !out))) return PG_ERR_ARG;
    if (!sc->ic.on) return scene_error(PG_ERR_ARG, "no irradiance cache on the scene (pg_scene_set_irradiance_cache)");
    if (rp->use_guiding && !guide) return scene_error(PG_ERR_ARG, "guiding needs a guiding context");
    if (n > 65536u) return scene_error(PG_ERR_ARG, "at most 65536 requests per call");
    if (n == 0) return PG_OK;
    if (int st = ensure_uploaded(sc)) return st;
    cudaStream_t s = (cudaStream_t)stream;
    DevRender R{};
    if (int st = setup_render(sc, rp, guide, s, R)) return st;
    ic_view(sc, R.ic);
    R.ic.query = 1;
    if (sc->ic.grid_stale)
        if (int st = ic_build_grid(sc, R.ic, s)) return st;
    IcRequest *req = nullptr;
    float4 *smp = nullptr;
    uint32_t *state = nullptr;
    const uint32_t st_host[4] = {n, 0, 0, 0};
    bool ok = cudaMalloc(&req, sizeof(IcRequest) * n) == cudaSuccess &&
              cudaMalloc(&smp, sizeof(float4) * kIcSamples * (size_t)n) == cudaSuccess &&
              cudaMalloc(&state, sizeof st_host) == cudaSuccess &&
              cudaMemcpyAsync(state, st_host, sizeof st_host, cudaMemcpyHostToDevice, s) == cudaSuccess;
    if (ok) {
        R.ic.requests = req;
        R.ic.req_cap = n;
        R.ic.state = state;
        R.ic.grow = 0;
        const uint32_t sms = sm_count();
        k_ic_load_requests<<<(n + 127) / 128, 128, 0, s>>>(requests, n, req);
        k_ic_paths<<<8 * sms, 128, 0, s>>>(R, smp);
        k_ic_compute_probe_reduce<<<std::min((n + 3) / 4, 8 * sms), 128, 0, s>>>(R, smp, n, out);
        ok = cudaGetLastError() == cudaSuccess && cudaStreamSynchronize(s) == cudaSuccess;
    }
    cudaFree(req);
    cudaFree(smp);
    cudaFree(state);
    return ok ? PG_OK : scene_error(PG_ERR_CUDA, "irradiance cache compute");
}

int pg_scene_texture_sizes(const pg_scene *sc, uint32_t *n_textures, uint64_t *n_texels) {
    if (!sc) return PG_ERR_ARG;
    uint64_t n = 0;
    for (const auto &t : sc->host.textures) n += (uint64_t)t.w * t.h;
    if (n_textures) *n_textures = (uint32_t)sc->host.textures.size();
    if (n_texels) *n_texels = n;
    return PG_OK;
}

int pg_scene_export_textures(const pg_scene *sc, float *tri_uv, uint32_t *tex_info, uint8_t *texels) {
    if (!sc) return PG_ERR_ARG;
    const SceneData &s = sc->host;
    if (tri_uv) memcpy(tri_uv, s.tri_uv.data(), sizeof(float) * s.tri_uv.size());
    uint64_t first = 0;
    for (size_t i = 0; i < s.textures.size(); ++i) {
        const auto &t = s.textures[i];
        if (tex_info) {
            tex_info[4 * i] = (uint32_t)first;
            tex_info[4 * i + 1] = t.w;
            tex_info[4 * i + 2] = t.h;
            tex_info[4 * i + 3] = 0;
        }
        if (texels) memcpy(texels + 4 * first, t.rgba.data(), t.rgba.size());
        first += (uint64_t)t.w * t.h;
    }
    return PG_OK;
}

int pg_png_read(const char *path, uint8_t *rgba_out, uint64_t capacity, uint32_t *width, uint32_t *height) {
    if (!path || !width || !height) return PG_ERR_ARG;
    uint32_t w = 0, h = 0;
    std::vector<uint8_t> rgba;
    std::string err;
    if (!pg::read_png(path, w, h, rgba, err))
        return set_error(nullptr, err.rfind("cannot open", 0) == 0 ? PG_ERR_IO : PG_ERR_PARSE, err);
    *width = w;
    *height = h;
    if (!rgba_out) return PG_OK;  // size query
    if (capacity < rgba.size()) return set_error(nullptr, PG_ERR_ARG, "PNG output buffer too small");
    memcpy(rgba_out, rgba.data(), rgba.size());
    return PG_OK;
}

int pg_scene_get_info(const pg_scene *sc, pg_scene_info *out) {
    if (!sc || !out) return PG_ERR_ARG;
    out->n_triangles = (uint32_t)sc->host.tri_mat.size();
    out->n_spheres = (uint32_t)sc->host.spheres.size();
    out->n_materials = (uint32_t)sc->host.mats.size();
    out->n_nodes = (uint32_t)sc->host.nodes.size();
    out->n_lights = sc->n_lights;
    for (int i = 0; i < 6; ++i) out->aabb[i] = sc->aabb[i];
    out->camera = sc->host.camera;
    return PG_OK;
}

int pg_scene_export(const pg_scene *sc, void *nodes, float *tri_verts, uint32_t *tri_order, uint32_t *tri_material,
                    pg_material *materials, pg_sphere *spheres) {
    if (!sc) return PG_ERR_ARG;
    const SceneData &s = sc->host;
    if (nodes) memcpy(nodes, s.nodes.data(), sizeof(BvhNode) * s.nodes.size());
    if (tri_verts) memcpy(tri_verts, s.tri_verts.data(), sizeof(float) * s.tri_verts.size());
    if (tri_order) memcpy(tri_order, s.tri_order.data(), sizeof(uint32_t) * s.tri_order.size());
    if (tri_material) memcpy(tri_material, s.tri_mat.data(), sizeof(uint32_t) * s.tri_mat.size());
    if (materials) memcpy(materials, s.mats.data(), sizeof(pg_material) * s.mats.size());
    if (spheres) memcpy(spheres, s.spheres.data(), sizeof(pg_sphere) * s.spheres.size());
    return PG_OK;
}

int pg_scene_set_camera(pg_scene *sc, const pg_camera *cam) {
    if (!sc || !cam || cam->width == 0 || cam->height == 0) return PG_ERR_ARG;
    sc->host.camera = *cam;
    return PG_OK;
}

int pg_scene_export_mesh(const pg_scene *sc, float *positions, uint32_t *indices, uint32_t *n_vertices) {
    if (!sc) return PG_ERR_ARG;
    const SceneData &s = sc->host;
    if (n_vertices) *n_vertices = (uint32_t)(s.pos.size() / 3);
    if (positions) memcpy(positions, s.pos.data(), sizeof(float) * s.pos.size());
    if (indices) memcpy(indices, s.idx.data(), sizeof(uint32_t) * s.idx.size());
    return PG_OK;
}

int pg_probe_shading(const pg_material *mats, uint32_t n_mats, const pg_vmm_theta *vmms, uint32_t n_vmms,
                     const pg_shading_probe *probes, uint32_t n, pg_shading_result *out, void *stream) {
    if (n == 0) return PG_OK;
    if (!probes || !out || (n_mats && !mats) || (n_vmms && !vmms)) return PG_ERR_ARG;
    k_probe_shading<<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(mats, n_mats, vmms, n_vmms, probes, n, out);
    return cudaGetLastError() == cudaSuccess ? PG_OK : scene_error(PG_ERR_CUDA, "probe launch");
}

int pg_probe_records(const pg_record_event *events, const uint32_t *path_offsets, uint32_t n_paths, float *weights,
                     uint32_t *flags, uint32_t *counts, void *stream) {
    if (n_paths == 0) return PG_OK;
    if (!events || !path_offsets || !weights || !flags || !counts) return PG_ERR_ARG;
    k_probe_records<<<(n_paths + 127) / 128, 128, 0, (cudaStream_t)stream>>>(events, path_offsets, n_paths, weights,
                                                                           flags, counts);
    return cudaGetLastError() == cudaSuccess ? PG_OK : scene_error(PG_ERR_CUDA, "probe launch");
}

int pg_trace_closest(pg_scene *sc, const pg_ray *rays, uint32_t n, pg_hit *hits, void *stream) {
    if (!sc || (!rays && n) || (!hits && n)) return PG_ERR_ARG;
    if (n == 0) return PG_OK;
    if (int st = ensure_uploaded(sc)) return st;
    k_trace_closest<<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(dev_scene(sc), rays, n, hits);
    return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ERR_CUDA;
}

int pg_trace_closest_counted(pg_scene *sc, const pg_ray *rays, uint32_t n, pg_hit *hits, uint32_t *node_visits,
                             uint32_t *triangle_tests, void *stream) {
    if (!sc || (n && (!rays || !hits || !node_visits || !triangle_tests))) return PG_ERR_ARG;
    if (n == 0) return PG_OK;
    if (int st = ensure_uploaded(sc)) return st;
    k_trace_closest_counted<<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(dev_scene(sc), rays, n, hits,
                                                                               node_visits, triangle_tests);
    return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ERR_CUDA;
}

int pg_trace_any(pg_scene *sc, const pg_ray *rays, uint32_t n, uint32_t *occluded, void *stream) {
    if (!sc || (!rays && n) || (!occluded && n)) return PG_ERR_ARG;
    if (n == 0) return PG_OK;
    if (int st = ensure_uploaded(sc)) return st;
    k_trace_any<<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(dev_scene(sc), rays, n, occluded);
    return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ERR_CUDA;
}

int pg_render(pg_scene *sc, const pg_render_params *rp, pg_ctx *guide, float *image, pg_directional_data *records,
              pg_render_stats *stats, void *stream) {
    if (!sc || !rp || !image) return PG_ERR_ARG;
    if (rp->max_depth == 0 || rp->max_depth > 64) return scene_error(PG_ERR_ARG, "max_depth must be in [1, 64]");
    if (rp->record_samples && !records) return scene_error(PG_ERR_ARG, "record_samples needs a records buffer");
    if ((rp->use_guiding || rp->record_samples) && !guide)
        return scene_error(PG_ERR_ARG, "guiding and sample recording need a guiding context (pg_set_regions)");
    if (int st = ensure_uploaded(sc)) return st;
    cudaStream_t s = (cudaStream_t)stream;
    const pg_camera cam = sc->host.camera;
    const uint32_t P = cam.width * cam.height;
    const bool adrrs = (rp->flags & PG_RENDER_ADRRS) != 0;
    if (adrrs && !sc->adrrs.estimate)
        return scene_error(PG_ERR_ARG, "PG_RENDER_ADRRS needs an estimate (pg_scene_set_adrrs)");
    if (adrrs && !sc->ic.on) return scene_error(PG_ERR_ARG, "PG_RENDER_ADRRS needs an irradiance cache");
    const bool splitting = adrrs && sc->adrrs.split;
    if (splitting && rp->record_samples)
        return scene_error(PG_ERR_ARG, "ADRRS splitting and record_samples exclude each other");
    // paths: one per pixel, plus up to two split copies per pixel and pass
    const uint32_t split_cap = splitting ? 2u * P : 0u;
    const uint32_t NP = P + split_cap;
    // grow the path and queue buffers
    if (P > sc->cap_pix || NP > sc->cap_paths) {
        for (void *b : sc->bufs) cudaFree(b);
        sc->bufs.clear();
        sc->cap_pix = 0;
        sc->cap_paths = 0;
        size_t want = 0;
        auto alloc = [&](size_t bytes) -> void * {
            ++want;
            void *p = nullptr;
            if (cudaMalloc(&p, std::max<size_t>(bytes, 4)) != cudaSuccess) return nullptr;
            sc->bufs.push_back(p);
            return p;
        };
        DevRender &R = sc->R;
        // per path
        R.ro = (float *)alloc(12ull * NP);
        R.rd = (float *)alloc(12ull * NP);
        R.thr = (float *)alloc(12ull * NP);
        R.prev_pdf = (float *)alloc(4ull * NP);
        R.alive = (uint8_t *)alloc(NP);
        R.found = (uint8_t *)alloc(NP);
        R.hits = (pg_hit *)alloc(sizeof(pg_hit) * (size_t)NP);
        R.q_cur = (uint32_t *)alloc(4ull * NP);
        R.q_next = (uint32_t *)alloc(4ull * NP);
        R.sh_o = (float *)alloc(12ull * NP);
        R.sh_d = (float *)alloc(12ull * NP);
        R.sh_tmax = (float *)alloc(4ull * NP);
        R.sh_c = (float *)alloc(12ull * NP);
        R.sh_l = (float *)alloc(12ull * NP);
        R.sh_pix = (uint32_t *)alloc(4ull * NP);
        R.sh_nrec = (uint32_t *)alloc(4ull * NP);
        // per pixel
        R.rec_lsum = (float *)alloc(12ull * P * kMaxRecords);
        R.rec_tc = (float *)alloc(12ull * P * kMaxRecords);
        R.rec_count = (uint32_t *)alloc(4ull * P);
        R.rec_start = (uint32_t *)alloc(4ull * P);
        R.rec_pending = (int32_t *)alloc(4ull * P);
        R.rec_factor = (float *)alloc(4ull * P);
        R.split_count = (uint32_t *)alloc(4ull * P);
        // per split slot
        R.split_pix = (uint32_t *)alloc(4ull * (NP - P));
        R.split_stream = (uint32_t *)alloc(4ull * (NP - P));
        R.q_copy = (uint32_t *)alloc(4ull * (NP - P));
        if (sc->bufs.size() != want) return scene_error(PG_ERR_NOMEM, "render buffers: out of device memory");
        sc->cap_pix = P;
        sc->cap_paths = NP;
    }
    DevRender R = sc->R;
    if (int st = setup_render(sc, rp, guide, s, R)) return st;
    R.image = image;
    R.counters = sc->d_counters;
    R.rec = records;
    R.n_pix = P;
    R.split_cap = split_cap;
    R.adrrs_est = adrrs ? sc->adrrs.estimate : nullptr;
    R.adrrs_s = sc->adrrs.s;
    R.adrrs_split = splitting ? 1 : 0;
    const bool ic_on = (rp->flags & PG_RENDER_IRRADIANCE_CACHE) != 0;
    if (ic_on || adrrs) {
        auto &c = sc->ic;
        if (!c.on) return scene_error(PG_ERR_ARG, "PG_RENDER_IRRADIANCE_CACHE needs a cache (pg_scene_set_irradiance_cache)");
        if (P > c.cap_created) {
            cudaFree(c.created);
            c.created = nullptr;
            c.cap_created = 0;
            if (cudaMalloc(&c.created, sizeof(uint32_t) * P) != cudaSuccess)
                return scene_error(PG_ERR_NOMEM, "irradiance cache pixel counters");
            c.cap_created = P;
        }
        ic_view(sc, R.ic);
        R.ic.query = ic_on ? 1 : 0;
        R.ic.grow = ic_on && !(rp->flags & PG_RENDER_IC_FROZEN) && (c.cfg.create_prob > 0.0f || c.cfg.update_prob > 0.0f);
        if (c.grid_stale)
            if (int st = ic_build_grid(sc, R.ic, s)) return st;
    }
    if (cudaMemsetAsync(sc->d_counters, 0, sizeof(uint32_t) * 16, s) != cudaSuccess)
        return scene_error(PG_ERR_CUDA, "counter reset");
    if (R.recording) {
        const uint32_t slots = P * kMaxRecords;
        k_reset_records<<<(slots + 255) / 256, 256, 0, s>>>(records, slots, R.rec_start, P);
    }
    R.stats = sc->d_stats;
    if (cudaMemsetAsync(sc->d_stats, 0, sizeof(unsigned long long) * kNumStats, s) != cudaSuccess)
        return scene_error(PG_ERR_CUDA, "stats reset");
    const bool count = (rp->flags & PG_RENDER_COUNT_WORK) != 0;
    StageTimer tm;
    if (!tm.init((rp->flags & PG_RENDER_TIME_STAGES) != 0, s)) return scene_error(PG_ERR_CUDA, "stage timer events");
    const uint32_t T = 128;
    const uint32_t G = (P + T - 1) / T;
    const uint32_t GS = (NP + T - 1) / T;                        // shading: camera paths and split copies
    const bool cache_paths = ic_on || adrrs;
    const uint32_t GC = std::max(1u, (split_cap + T - 1) / T);  // the copies made at a bounce
    if (sc->persist_blocks == 0) {
        int dev = 0, sms = 0, b_ext = 0, b_sh = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b_ext, k_extend<false>, (int)T, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b_sh, k_shadow<false>, (int)T, 0);
        sc->persist_blocks = (uint32_t)std::max(1, sms) * (uint32_t)std::max(1, std::min(b_ext, b_sh));
    }
    // persistent traversal grid: every SM full, never more CTAs than the full queue needs
    const uint32_t GP = std::min(G, sc->persist_blocks);
    for (uint32_t smp = 0; smp < rp->spp; ++smp) {
        R.sample = smp;
        DevRender Rb = R;
        tm.begin(PG_STAGE_CAMERA);
        k_camera<<<G, T, 0, s>>>(Rb);
        tm.end();
        for (uint32_t b = 0; b < rp->max_depth; ++b) {
            tm.begin(PG_STAGE_EXTEND);
            if (count)
                k_extend<true><<<GP, T, 0, s>>>(Rb);
            else
                k_extend<false><<<GP, T, 0, s>>>(Rb);
            tm.end();
            const int last = (b + 1 == rp->max_depth) ? 1 : 0;
            tm.begin(PG_STAGE_SHADE);
            if (cache_paths) {
                k_shade<true><<<GS, T, 0, s>>>(Rb, (int)b, last, 0);
                if (splitting) k_shade<true><<<GC, T, 0, s>>>(Rb, (int)b, last, 1);
            } else {
                k_shade<false><<<GS, T, 0, s>>>(Rb, (int)b, last, 0);
            }
            tm.end();
            tm.begin(PG_STAGE_SHADOW);
            if (count)
                k_shadow<true><<<GP, T, 0, s>>>(Rb);
            else
                k_shadow<false><<<GP, T, 0, s>>>(Rb);
            tm.end();
            tm.begin(PG_STAGE_ADVANCE);
            k_advance<<<1, 1, 0, s>>>(Rb);
            tm.end();
            std::swap(Rb.q_cur, Rb.q_next);
        }
        if (R.recording) {
            tm.begin(PG_STAGE_COMMIT);
            k_commit<<<G, T, 0, s>>>(R, P);
            tm.end();
        }
        if (R.ic.grow)
            if (int st = ic_process(sc, Rb, s)) return st;
    }
    if (R.ic.grow) {
        // grow the grid's reference list if the last build did not fit in it
        auto &c = sc->ic;
        uint32_t total = 0;
        if (cudaMemcpyAsync(&total, c.cell_start + kIcCells, sizeof total, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return scene_error(PG_ERR_CUDA, "irradiance cache grid size");
        if (total > c.cap_refs) {
            cudaFree(c.refs);
            c.refs = nullptr;
            const uint64_t want = std::min<uint64_t>(2ull * total, 0xFFFFFFF0ull);
            if (cudaMalloc(&c.refs, sizeof(uint32_t) * want) != cudaSuccess) {
                c.cap_refs = 0;
                c.grid_stale = true;
                return scene_error(PG_ERR_NOMEM, "irradiance cache grid: out of device memory");
            }
            c.cap_refs = (uint32_t)want;
            ic_view(sc, R.ic);
            if (int st = ic_build_grid(sc, R.ic, s)) return st;
        }
    }
    if (cudaGetLastError() != cudaSuccess) return scene_error(PG_ERR_CUDA, "render launch failed");
    tm.flush();
    if (tm.failed) return scene_error(PG_ERR_CUDA, "stage timing failed");
    if (stats) {
        uint32_t c[16];
        unsigned long long st2[kNumStats];
        if (cudaMemcpyAsync(c, sc->d_counters, sizeof c, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaMemcpyAsync(st2, sc->d_stats, sizeof st2, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return scene_error(PG_ERR_CUDA, "render stats");
        memset(stats, 0, sizeof *stats);
        stats->extension_rays = st2[0];
        stats->shadow_rays = st2[1];
        stats->samples_recorded = c[4];
        stats->paths = (uint64_t)P * rp->spp;
        stats->extension_node_visits = st2[2];
        stats->extension_triangle_tests = st2[3];
        stats->shadow_node_visits = st2[4];
        stats->shadow_triangle_tests = st2[5];
        for (int i = 0; i < PG_STAGE_COUNT; ++i) {
            stats->stage_ms[i] = tm.ms[i];
            stats->stage_launches[i] = tm.launches[i];
        }
    }
    return PG_OK;
}

}  // extern "C"
