// pg_splitmerge.cu - split and merge of mixture components after a region's
// fit (PathGuiding::postFit with splitAndMerge, src/PathGuiding.cpp:413-451).
//
// One CTA per region with samples in the pass.  Thread 0 runs the control
// logic of the reference - the Pearson chi-square merge metric of every pair
// (:709-760), greedy disjoint merges (:635-707, 762-781), split candidates by
// weighted divergence (:563-633), PCA splits along the principal axis of the
// component's 2-D covariance (:494-561) - on the mixture held in shared
// memory; all threads run the passes over the region's samples: the
// divergence statistic (incrementalpearsonchisquared.h:54-94), the
// covariance statistic (incrementalcovariance2d.h:54-106) and the masked EM
// refit of split components (VMMFactory.h:226-297, 458-485), with per-thread
// sums reduced in a fixed order.
//
// The statistics, the VMF products and divisions (VMFKernel.h:315-400), the
// component merge (:478-530) and the weight priors (ParametricMixtureModel.h:
// 339-370) follow the reference's formulas in FP32.  Its sorts are restated
// exactly: candidates are separated with the two-ended partition of
// libstdc++'s std::partition (whose order decides which components are split
// or merged first), then sorted by value.  The one substitution: the
// reference takes the PCA axis from an Eigen solver; here the principal
// eigenvector of the symmetric 2x2 covariance is computed in closed form.
#include <math.h>
#include <string.h>

#include <algorithm>

#include <cooperative_groups.h>

#include "pg_internal.cuh"

namespace cg = cooperative_groups;

namespace pg {
namespace sm {

// The control logic runs on thread 0 and is also host-callable.
#define SM_HD __host__ __device__

constexpr int NT = 128, NW = NT / 32, KM = 16;
constexpr float kPiF = 3.14159265358979323846f;

struct Mix {
    float w[KM], mx[KM], my[KM], mz[KM], k[KM], r[KM], nrm[KM], em2k[KM];
    uint32_t K;
    float sample_weight, num_samples;
    unsigned long long total;
};

struct Stats {
    float div[KM], dn[KM];   // chi-square: divergencePlusOneTimesIntegralSqr, numSamples
    float cov[KM][3], cw[KM];
    float dist[KM], dw[KM];  // IncrementalDistance
    float since;
};

// Pair candidates of one merge round (in shared memory on the device).
struct MergeScratch {
    float key[KM * (KM - 1) / 2];
    int ca[KM * (KM - 1) / 2], cb[KM * (KM - 1) / 2];
};

// The mixture as the sample passes read it (float4 / float2 broadcasts):
// log2 of weight x pdf of component c at direction d is
// min(e.xyz . d + e.w, l.x) with e = {kappa log2(e) mu, l.x - kappa log2(e)}
// and l.x = log2(weight norm) - the vMF pdf with the cosine clamped at 1.
struct PassMix {
    float4 e[KM];
    float2 l[KM];           // log2(weight norm), weight
    float4 sf[KM], tf[KM];  // covariance frames
};

struct Shared {
    Mix m;
    Stats s;
    PassMix pm;
    MergeScratch ms;
    float red[NW][4 * KM + 2];
    float part[2][4 * KM + 2];  // this CTA's sums of a pass, double-buffered (read by the cluster)
    float acc[4 * KM + 2];   // the region's sums of a pass
    uint32_t mask;           // components refitted by the masked EM
    int fit_iters;
    int stop;
    float old_active;        // masked EM: prior-free weight of the refitted components
    int merge, n_merged;     // mergeAll runs / merges of the last round
    uint32_t stat_passes, em_iters;  // work done, reported in the region's statistics
    float ll_last, ll_abs_inv;
    float sum_w;             // weight of the valid samples (masked EM, first iteration)
};

struct Args {
    pg_region_state *states;
    pg_region_extra *extras;
    const float4 *dirw;
    const float *pdf;
    const uint32_t *offsets;
    const uint32_t *order;   // region ids, largest first (the biggest regions start first)
    const uint32_t *n_large; // leading regions of `order` split by clusters
    uint32_t n_regions;
    pg_fit_config cfg;
    pg_split_merge_config sm;
};

SM_HD __forceinline__ uint32_t active_lanes(uint32_t K) { return (K + 3u) & ~3u; }

// kappaToMeanCosine / meanCosineToKappa (VMFKernel.h:46-66), one component
SM_HD __forceinline__ float k2r(float k) {
    if (k > 5.0f) return 1.0f - 1.0f / k;
    return k > 0.0f ? 1.0f / tanhf(k) - 1.0f / k : 0.0f;
}
SM_HD __forceinline__ float r2k(float r) { return (r * 3.0f - r * r * r) / (1.0f - r * r); }

// calNormalization (VMFKernel.h:620-628)
SM_HD __forceinline__ void normalise(Mix &m, int c) {
    m.em2k[c] = expf(-2.0f * m.k[c]);
    m.nrm[c] = m.k[c] > 0.0f ? m.k[c] / (2.0f * kPiF * (1.0f - m.em2k[c])) : 1.0f / (4.0f * kPiF);
}
SM_HD __forceinline__ void reset_comp(Mix &m, int c) {
    m.w[c] = 0.0f;
    m.k[c] = 0.0f;
    m.r[c] = 0.0f;
    m.mx[c] = m.my[c] = 0.0f;
    m.mz[c] = 1.0f;
    m.nrm[c] = 1.0f / (4.0f * kPiF);
    m.em2k[c] = 1.0f;
}
// setK / cutoff: components from K on are reset
SM_HD __forceinline__ void set_k(Mix &m, uint32_t K) {
    m.K = K;
    for (int c = (int)K; c < KM; ++c) reset_comp(m, c);
}
// setKappaAndR (VMFKernel.h:212-227)
SM_HD __forceinline__ void set_kappa_r(Mix &m, int c, float k, float r) {
    const bool small = k < 1e-3f;
    m.k[c] = small ? 0.0f : k;
    m.r[c] = small ? 0.0f : r;
    normalise(m, c);
}

// ParametricMixtureModel::removeWeightPrior / applyWeightPrior
SM_HD void remove_prior(Mix &m, float v) {
    const float inv = v * (float)m.K + 1.0f, wpn = 1.0f / inv, wptn = v * wpn;
    for (uint32_t c = 0; c < active_lanes(m.K); ++c) m.w[c] = (m.w[c] - wptn) * inv;
    for (uint32_t c = m.K; c < active_lanes(m.K); ++c) m.w[c] = 0.0f;
}
SM_HD void apply_prior(Mix &m, float v) {
    const float inv = v * (float)m.K + 1.0f, wpn = 1.0f / inv, wptn = v * wpn;
    for (uint32_t c = 0; c < active_lanes(m.K); ++c) m.w[c] = m.w[c] * wpn + wptn;
    for (uint32_t c = m.K; c < active_lanes(m.K); ++c) m.w[c] = 0.0f;
}

// lightpmm's exp of its 4-wide arithmetic (pmm-vcl.h:158-184): Mineiro's
// fastpow2 (fastapprox) of x log2(e), clipped at -126, with SSE2 truncation
// and round-to-nearest conversion.  Within 2e-5 of exp for x <= 0, but the
// offset of the fractional part is +1 for either sign, so for x > 0 it is off
// by up to 90%.  The vMF divisions of the merge metric take it at positive
// arguments, which moves the metric by more than its threshold: the
// reference's merges follow this function, so it is restated exactly (this
// file is compiled without FMA contraction, as the SSE2 build rounds every
// product and sum).
SM_HD __forceinline__ float lpmm_fastexp(float x) {
    const float p = 1.442695040f * x;
    const float clipp = (-126.0f > p) ? -126.0f : p;
    const float w = (clipp >= -2147483648.0f && clipp < 2147483648.0f) ? truncf(clipp) : clipp;
    const float z = (clipp - w) + 1.0f;
    const float t = ((clipp + 121.2740575f) + (27.7280233f / (4.84252568f - z))) - (1.49012907f * z);
    const float v = 8388608.0f * t;
    int32_t bits = INT32_MIN;  // cvtps2dq's answer out of range and for NaN
#ifdef __CUDA_ARCH__
    if (v >= -2147483648.0f && v < 2147483648.0f) bits = __float2int_rn(v);
    return __int_as_float(bits);
#else
    if (v >= -2147483648.0f && v < 2147483648.0f) bits = (int32_t)nearbyintf(v);
    float out;
    memcpy(&out, &bits, sizeof out);
    return out;
#endif
}

// A single vMF lobe as the merge metric manipulates it.
struct Lobe {
    float w, mx, my, mz, k, r, nrm, em2k;
};
SM_HD __forceinline__ Lobe lobe(const Mix &m, int c) {
    return Lobe{m.w[c], m.mx[c], m.my[c], m.mz[c], m.k[c], m.r[c], m.nrm[c], m.em2k[c]};
}

// VMFKernel::product (VMFKernel.h:315-355): a becomes a*b, returns its integral
SM_HD float product(Lobe &a, const Lobe &b) {
    float nx = a.mx * a.k + b.mx * b.k, ny = a.my * a.k + b.my * b.k, nz = a.mz * a.k + b.mz * b.k;
    float nk = sqrtf(nx * nx + ny * ny + nz * nz);
    const bool small = nk < 1e-3f;
    nk = small ? 0.0f : nk;
    if (small) {
        nx = a.mx, ny = a.my, nz = a.mz;
    } else {
        nx /= nk, ny /= nk, nz /= nk;
    }
    const float ci = a.nrm, cj = b.nrm;
    const float e2 = lpmm_fastexp(-2.0f * nk);
    const float cij = small ? 1.0f / (4.0f * kPiF) : (1.0f / (2.0f * kPiF)) * nk / (1.0f - e2);
    const float ti = nx * a.mx + ny * a.my + nz * a.mz, tj = nx * b.mx + ny * b.my + nz * b.mz;
    const float t = a.k * (ti - 1.0f) + b.k * (tj - 1.0f);
    const float s = lpmm_fastexp(t) * a.w * b.w * (ci * cj) / cij;
    a = Lobe{s, nx, ny, nz, nk, k2r(nk), cij, e2};
    return s;
}

// VMFKernel::division (VMFKernel.h:362-400): a becomes a/b, returns its integral
SM_HD float division(Lobe &a, const Lobe &b) {
    float nx = a.mx * a.k - b.mx * b.k, ny = a.my * a.k - b.my * b.k, nz = a.mz * a.k - b.mz * b.k;
    float nk = sqrtf(nx * nx + ny * ny + nz * nz);
    const bool small = nk < 1e-3f;
    nk = small ? 0.0f : nk;
    if (small) {
        nx = a.mx, ny = a.my, nz = a.mz;
    } else {
        nx /= nk, ny /= nk, nz /= nk;
    }
    const float ci = a.nrm, cj = b.nrm;
    const float e2 = lpmm_fastexp(-2.0f * nk);
    const float cij = small ? 1.0f / (4.0f * kPiF) : (1.0f / (2.0f * kPiF)) * nk / (1.0f - e2);
    const float mi = nx * a.mx + ny * a.my + nz * a.mz, mj = nx * b.mx + ny * b.my + nz * b.mz;
    const float t = a.k * (mi - 1.0f) - b.k * (mj - 1.0f);
    const float s = lpmm_fastexp(t) * a.w * ci / (b.w * cj * cij);
    a = Lobe{s, nx, ny, nz, nk, k2r(nk), cij, e2};
    return s;
}

// VMFKernel::mergeComponent (VMFKernel.h:478-530), the merged lobe of a and b
SM_HD Lobe merge_lobes(const Lobe &a, const Lobe &b) {
    const float w = a.w + b.w;
    float mx = (a.w * a.r * a.mx + b.w * b.r * b.mx) / w;
    float my = (a.w * a.r * a.my + b.w * b.r * b.my) / w;
    float mz = (a.w * a.r * a.mz + b.w * b.r * b.mz) / w;
    float r = mx * mx + my * my + mz * mz;
    float k = 0.0f, nrm = 1.0f / (4.0f * kPiF), em2k = 1.0f;
    if (r > 0.0f) {
        r = sqrtf(r);
        k = r2k(r);
        k = k < 1e-3f ? 0.0f : k;
        em2k = expf(-2.0f * k);
        nrm = k / (2.0f * kPiF * (1.0f - em2k));  // 0/0 when the merged lobe is flat, as in the reference
        mx /= r, my /= r, mz /= r;
    } else {
        mx = a.mx, my = a.my, mz = a.mz;
    }
    return Lobe{w, mx, my, mz, k, r, nrm, em2k};
}

// computePearsonChiSquaredMergeMetric for one pair (src/PathGuiding.cpp:709-760)
SM_HD float merge_metric(const Mix &m, int i, int j) {
    const Lobe ci = lobe(m, i), cj = lobe(m, j);
    Lobe si = ci, sj = cj, pij = ci;
    product(si, ci);
    product(sj, cj);
    product(pij, cj);
    const Lobe merged = merge_lobes(ci, cj);
    const float q1 = division(si, merged), q2 = division(pij, merged), q3 = division(sj, merged);
    return q1 + 2.0f * q2 + q3 - merged.w;
}

// lightpmm::coordinateAxis / Frame (pmm-glm.h:107-133).  Its unqualified
// sqrt resolves to the double one, so 1/length is taken in double and rounded.
SM_HD void coordinate_axis(const float z[3], float x[3], float y[3]) {
    if (fabsf(z[0]) > fabsf(z[1])) {
        const float inv = (float)(1.0 / sqrt((double)(z[0] * z[0] + z[2] * z[2])));
        y[0] = z[2] * inv, y[1] = 0.0f, y[2] = -z[0] * inv;
    } else {
        const float inv = (float)(1.0 / sqrt((double)(z[1] * z[1] + z[2] * z[2])));
        y[0] = 0.0f, y[1] = z[2] * inv, y[2] = -z[1] * inv;
    }
    x[0] = y[1] * z[2] - y[2] * z[1];
    x[1] = y[2] * z[0] - y[0] * z[2];
    x[2] = y[0] * z[1] - y[1] * z[0];
}

// Statistic merges (incrementaldistance.h:165-204, incrementalpearsonchisquared.h:176-204,
// incrementalcovariance2d.h:200-247) for components a < b with `last` the last component.
SM_HD void merge_stats(const Mix &m, Stats &s, int a, int b, int last) {
    const float wa = m.w[a], wb = m.w[b], mw = wa + wb;
    // parallax distance: harmonic means
    {
        const float msw = mw / (wa / s.dw[a] + wb / s.dw[b]);
        const float md = mw / (wa / s.dist[a] + wb / s.dist[b]);
        s.dist[a] = md;
        s.dw[a] = msw;
    }
    const float inv = 1.0f / mw;
    // chi-square
    if (!isinf(inv)) {
        const float sa = wa * inv, sb = wb * inv;
        const float d = sa * s.div[a] + sb * s.div[b];
        const float n = sa * s.dn[a] + sb * s.dn[b];
        s.div[a] = d;
        s.dn[a] = n;
    } else {
        s.div[a] = 0.0f;
        s.dn[a] = 0.0f;
    }
    // covariance; the merged mean is scaled by 1/3, what GLM's vec3::length() returns
    if (!isinf(inv)) {
        float mu[3] = {wa * m.mx[a] + wb * m.mx[b], wa * m.my[a] + wb * m.my[b], wa * m.mz[a] + wb * m.mz[b]};
        const float sc = 1.0f / 3.0f;
        for (int i = 0; i < 3; ++i) mu[i] *= sc;
        float fx[3], fy[3];
        coordinate_axis(mu, fx, fy);
        const float ax = m.mx[a] * fx[0] + m.my[a] * fx[1] + m.mz[a] * fx[2];
        const float ay = m.mx[a] * fy[0] + m.my[a] * fy[1] + m.mz[a] * fy[2];
        const float bx = m.mx[b] * fx[0] + m.my[b] * fx[1] + m.mz[b] * fx[2];
        const float by = m.mx[b] * fy[0] + m.my[b] * fy[1] + m.mz[b] * fy[2];
        const float msw = s.cw[a] + s.cw[b];
        const float f = wa * wb / mw;
        const float dx = ax - bx, dy = ay - by;
        const float dv[3] = {dx * dx, dy * dy, dx * dy};
        for (int i = 0; i < 3; ++i) s.cov[a][i] = (wa * s.cov[a][i] + wb * s.cov[b][i] + f * dv[i]) * inv;
        s.cw[a] = msw;
    } else {
        s.cov[a][0] = s.cov[a][1] = s.cov[a][2] = 0.0f;
        s.cw[a] = 0.0f;
    }
    if (b != last) {
        s.dist[b] = s.dist[last];
        s.dw[b] = s.dw[last];
        s.div[b] = s.div[last];
        s.dn[b] = s.dn[last];
        for (int i = 0; i < 3; ++i) s.cov[b][i] = s.cov[last][i];
        s.cw[b] = s.cw[last];
    }
}

// ParametricMixtureModel::mergeComponents: a takes the merge, b is reset and
// swapped with the last component, K decreases.
SM_HD void merge_components(Mix &m, Stats &s, int a, int b) {
    const int last = (int)m.K - 1;
    merge_stats(m, s, a, b, last);
    const Lobe mg = merge_lobes(lobe(m, a), lobe(m, b));
    m.w[a] = mg.w, m.k[a] = mg.k, m.r[a] = mg.r;
    m.mx[a] = mg.mx, m.my[a] = mg.my, m.mz[a] = mg.mz;
    m.nrm[a] = mg.nrm, m.em2k[a] = mg.em2k;
    reset_comp(m, b);
    m.K -= 1;
    if (b != (int)m.K) {  // swapComponents(b, K)
        const Lobe t = lobe(m, b);
        m.w[b] = m.w[m.K], m.k[b] = m.k[m.K], m.r[b] = m.r[m.K];
        m.mx[b] = m.mx[m.K], m.my[b] = m.my[m.K], m.mz[b] = m.mz[m.K];
        m.nrm[b] = m.nrm[m.K], m.em2k[b] = m.em2k[m.K];
        m.w[m.K] = t.w, m.k[m.K] = t.k, m.r[m.K] = t.r;
        m.mx[m.K] = t.mx, m.my[m.K] = t.my, m.mz[m.K] = t.mz;
        m.nrm[m.K] = t.nrm, m.em2k[m.K] = t.em2k;
    }
}

// libstdc++ std::partition (two-ended), over keys with their payload
template <class Pred>
SM_HD int hoare_partition(float *key, int *pa, int *pb, int n, Pred pred) {
    int first = 0, last = n;
    while (true) {
        while (true) {
            if (first == last) return first;
            if (pred(key[first])) ++first;
            else break;
        }
        --last;
        while (true) {
            if (first == last) return first;
            if (!pred(key[last])) --last;
            else break;
        }
        float tk = key[first];
        key[first] = key[last];
        key[last] = tk;
        int t = pa[first];
        pa[first] = pa[last];
        pa[last] = t;
        if (pb) {
            t = pb[first];
            pb[first] = pb[last];
            pb[last] = t;
        }
        ++first;
    }
}

// mergeAll (src/PathGuiding.cpp:635-707), thread 0
// Merge metric of the pairs [first, n (n - 1) / 2) with stride `step`, in the
// row-major order of (a, b), a < b.
SM_HD void merge_candidates(const Mix &m, MergeScratch &ms, int first, int step) {
    const int n = (int)m.K;
    const int np = n * (n - 1) / 2;
    for (int idx = first; idx < np; idx += step) {
        int a = 0, rem = idx;
        while (rem >= n - 1 - a) {
            rem -= n - 1 - a;
            ++a;
        }
        const int b = a + 1 + rem;
        ms.key[idx] = merge_metric(m, a, b);
        ms.ca[idx] = a;
        ms.cb[idx] = b;
    }
}

// One round of mergeAll (src/PathGuiding.cpp:635-707) on the candidates:
// pairs below the threshold, cheapest first, disjoint, merged from the highest
// second index down.  Returns the number of merges.
SM_HD int merge_round(Mix &m, Stats &s, const pg_split_merge_config &cfg, MergeScratch &ms) {
    float *key = ms.key;
    int *ca = ms.ca, *cb = ms.cb;
    const int n = (int)m.K;
    const int np = n * (n - 1) / 2;
    const float thr = cfg.merge_max_divergence;
    const int end = hoare_partition(key, ca, cb, np, [thr](float v) { return v <= thr; });
    // sort by metric ascending (insertion; the reference's std::sort on distinct values)
    for (int i = 1; i < end; ++i) {
        const float k = key[i];
        const int a = ca[i], b = cb[i];
        int j = i - 1;
        while (j >= 0 && key[j] > k) {
            key[j + 1] = key[j], ca[j + 1] = ca[j], cb[j + 1] = cb[j];
            --j;
        }
        key[j + 1] = k, ca[j + 1] = a, cb[j + 1] = b;
    }
    uint32_t used = 0;
    int ma[KM], mb[KM], nm = 0;
    for (int i = 0; i < end; ++i) {
        const int a = min(ca[i], cb[i]), b = max(ca[i], cb[i]);
        if ((used >> a) & 1u || (used >> b) & 1u) continue;
        ma[nm] = a, mb[nm] = b, ++nm;
        used |= (1u << a) | (1u << b);
    }
    // by second index, descending, so later merges keep their indices
    for (int i = 1; i < nm; ++i) {
        const int a = ma[i], b = mb[i];
        int j = i - 1;
        while (j >= 0 && mb[j] < b) {
            ma[j + 1] = ma[j], mb[j + 1] = mb[j];
            --j;
        }
        ma[j + 1] = a, mb[j + 1] = b;
    }
    for (int i = 0; i < nm; ++i) merge_components(m, s, ma[i], mb[i]);
    return nm;
}

// mergeAll on one thread (host checks)
SM_HD void merge_all(Mix &m, Stats &s, const pg_split_merge_config &cfg, MergeScratch &ms) {
    for (int round = 0; round < KM; ++round) {
        if (m.K <= 1) return;
        merge_candidates(m, ms, 0, 1);
        if (!merge_round(m, s, cfg, ms)) return;
    }
}

// Principal axis of the symmetric 2x2 covariance [[a, b], [b, c]]
SM_HD void principal_axis(float a, float b, float c, float &lambda, float &vx, float &vy) {
    const float h = 0.5f * (a - c);
    const float d = sqrtf(h * h + b * b);
    lambda = 0.5f * (a + c) + d;
    if (b == 0.0f) {
        vx = a >= c ? 1.0f : 0.0f;
        vy = a >= c ? 0.0f : 1.0f;
        return;
    }
    if (a >= c) {
        vx = lambda - c;
        vy = b;
    } else {
        vx = b;
        vy = lambda - a;
    }
    const float inv = 1.0f / sqrtf(vx * vx + vy * vy);
    vx *= inv;
    vy *= inv;
}

// splitComponentUsingPCA (src/PathGuiding.cpp:494-561), thread 0
SM_HD void split_component(Mix &m, Stats &s, int c, float max_kappa) {
    if (m.K == KM) return;
    const int dst = (int)m.K;
    const float z3[3] = {m.mx[c], m.my[c], m.mz[c]};
    float fx[3], fy[3];
    coordinate_axis(z3, fx, fy);
    const bool has = s.cw[c] > 0.0f;
    const float va = has ? s.cov[c][0] : 0.0f, vb = has ? s.cov[c][2] : 0.0f, vc = has ? s.cov[c][1] : 0.0f;
    float lambda, px, py;
    principal_axis(va, vb, vc, lambda, px, py);
    const float off = fminf(1.0f, 0.5f * sqrtf(lambda));
    px *= off;
    py *= off;
    const float z = sqrtf(1.0f - off * off);
    float a[3], b[3];
    for (int i = 0; i < 3; ++i) {
        a[i] = px * fx[i] + py * fy[i] + z * z3[i];
        b[i] = -px * fx[i] + -py * fy[i] + z * z3[i];
    }
    set_k(m, m.K + 1);
    const float src_r = m.r[c], src_w = m.w[c];
    const float split_w = src_w * 0.5f;
    const float max_r = k2r(max_kappa);
    const float split_r = z > 0.0f ? fminf(max_r, src_r / z) : max_r;
    const float split_k = r2k(split_r);
    set_kappa_r(m, c, split_k, split_r);
    m.mx[c] = a[0], m.my[c] = a[1], m.mz[c] = a[2];
    m.w[c] = split_w;
    set_kappa_r(m, dst, split_k, split_r);
    m.mx[dst] = b[0], m.my[dst] = b[1], m.mz[dst] = b[2];
    m.w[dst] = split_w;
    // statistics (incrementaldistance.h:206-216, chi-square and covariance reset)
    s.dist[dst] = s.dist[c];
    const float hw = 0.5f * s.dw[c];
    s.dw[c] = hw;
    s.dw[dst] = hw;
    s.div[c] = s.div[dst] = 0.0f;
    s.dn[c] = s.dn[dst] = 0.0f;
    for (int i = 0; i < 3; ++i) s.cov[c][i] = s.cov[dst][i] = 0.0f;
    s.cw[c] = s.cw[dst] = 0.0f;
}

__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float lg2_approx(float x) {
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// weight x vMF pdf (VMFKernel::pdf, cosine clamped at 1) of a component
__device__ __forceinline__ float weighted_pdf(float4 e, float lw, float4 d) {
    const float t = __fmaf_rn(e.x, d.x, __fmaf_rn(e.y, d.y, __fmaf_rn(e.z, d.z, e.w)));
    return ex2_approx(fminf(t, lw));
}
__device__ __forceinline__ float dot3(float4 a, float4 d) {
    return __fmaf_rn(a.z, d.z, __fmaf_rn(a.y, d.y, __fmul_rn(a.x, d.x)));
}

// incrementalcovariance2d.h:67-77: the tangent frame {s, t} of a component's mean
__device__ void cov_frame(float nx, float ny, float nz, float4 &sf, float4 &tf) {
    const bool xg = nx * nx > ny * ny;
    const float inv = 1.0f / sqrtf((xg ? nx * nx : ny * ny) + nz * nz);
    float t[3];
    if (xg) {
        t[0] = nz * inv, t[1] = 0.0f, t[2] = -nx * inv;
    } else {
        t[0] = 0.0f, t[1] = nz * inv, t[2] = -ny * inv;
    }
    tf = make_float4(t[0], t[1], t[2], 0.0f);
    sf = make_float4(t[1] * nz - t[2] * ny, t[2] * nx - t[0] * nz, t[0] * ny - t[1] * nx, 0.0f);
}

// Copies the mixture into the pass layout (and the covariance frames when
// asked); every thread calls it after the mixture's last change.
__device__ void load_pass_mix(Shared &S, bool frames) {
    __syncthreads();
    const int c = threadIdx.x;
    if (c < KM) {
        const Mix &m = S.m;
        const float kl = m.k[c] * 1.4426950408889634f;
        const float lw = log2f(m.w[c] * m.nrm[c]);  // -inf for an empty lane: its pdf term is 0
        S.pm.e[c] = make_float4(kl * m.mx[c], kl * m.my[c], kl * m.mz[c], lw - kl);
        S.pm.l[c] = make_float2(lw, m.w[c]);
        if (frames) cov_frame(m.mx[c], m.my[c], m.mz[c], S.pm.sf[c], S.pm.tf[c]);
    }
    __syncthreads();
}

// The CTAs that share a region: a thread-block cluster (size > 1) or one CTA.
// Every CTA of a cluster holds the same mixture and statistics and runs the
// same control code on the same sums, so all reach the same decisions; only
// rank 0 writes the region back.
struct Team {
    uint32_t rank, size;
    uint32_t phase;  // passes reduced so far: selects the partial-sum buffer
};

// Reduction of per-thread values v[0..N) in a fixed order (lanes, warps, then
// cluster ranks 0..size-1): value i goes to S.acc[i] below `tail`, to
// S.acc[4 KM + i - tail] from it on, in every CTA of the team.
template <int N, bool kCluster>
__device__ void block_sum(Shared &S, Team &T, const float (&v)[N], int tail) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        float x = v[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) S.red[warp][i] = x;
    }
    __syncthreads();
    const int i = threadIdx.x;
    if (!kCluster) {
        if (i < N) {
            float x = 0.0f;
            for (int w = 0; w < NW; ++w) x += S.red[w][i];
            S.acc[i < tail ? i : 4 * KM + i - tail] = x;
        }
        __syncthreads();
        return;
    }
    // Partials of consecutive passes alternate between two buffers: a rank
    // writes a buffer again two passes later, after the next cluster barrier,
    // which every rank reaches only once it has read this pass's partials.
    float *part = S.part[T.phase & 1u];
    ++T.phase;
    if (i < N) {
        float x = 0.0f;
        for (int w = 0; w < NW; ++w) x += S.red[w][i];
        part[i] = x;
    }
    cg::cluster_group cl = cg::this_cluster();
    cl.sync();  // every rank's partial sums are visible
    if (i < N) {
        const uint32_t nr = cl.num_blocks();
        float x = 0.0f;
        for (uint32_t r = 0; r < nr; ++r) x += cl.map_shared_rank(part, r)[i];
        S.acc[i < tail ? i : 4 * KM + i - tail] = x;
    }
    __syncthreads();
}

// Pass kinds over the region's samples
enum { PASS_CHI2 = 0, PASS_COV = 1, PASS_EM = 2 };

// One pass over the region's samples with L active component lanes (a
// compile-time count, so the per-thread sums stay in registers).  Sums land
// in S.acc: chi-square [c] = sum weight_c pdf_c w^2 pdf / mix^2 (divided by
// weight_c afterwards); covariance [4c..4c+3] = sum of gamma_c w, and its xx,
// yy, xy moments in the component's frame; EM [4c..4c+3] = sum of gamma_c w
// d.xyz and gamma_c w, [4 KM] = sum w, [4 KM + 1] = sum w log2(mix).
template <int KIND, int L, bool kCluster>
__device__ void sample_pass_l(Shared &S, const Args &A, Team &T, uint32_t b, uint32_t e) {
    constexpr int NV = KIND == PASS_CHI2 ? L : 4 * L + (KIND == PASS_EM ? 2 : 0);
    float v[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = 0.0f;
    for (uint32_t i = b + T.rank * NT + threadIdx.x; i < e; i += T.size * NT) {
        const float4 d = __ldg(A.dirw + i);
        float p[L];  // weight_c pdf_c
        float mix = 0.0f;
#pragma unroll
        for (int c = 0; c < L; ++c) {
            p[c] = weighted_pdf(S.pm.e[c], S.pm.l[c].x, d);
            mix += p[c];
        }
        if (!(mix > kPmmEps)) continue;
        if (KIND == PASS_CHI2) {
            const float f = d.w * d.w * __ldg(A.pdf + i) / (mix * mix);
#pragma unroll
            for (int c = 0; c < L; ++c) v[c] = __fmaf_rn(p[c], f, v[c]);
        } else if (KIND == PASS_COV) {
            const float inv = d.w / mix;
#pragma unroll
            for (int c = 0; c < L; ++c) {
                const float wt = p[c] * inv;
                const float lx = dot3(S.pm.sf[c], d), ly = dot3(S.pm.tf[c], d);
                v[4 * c] += wt;
                v[4 * c + 1] = __fmaf_rn(lx * lx, wt, v[4 * c + 1]);
                v[4 * c + 2] = __fmaf_rn(ly * ly, wt, v[4 * c + 2]);
                v[4 * c + 3] = __fmaf_rn(lx * ly, wt, v[4 * c + 3]);
            }
        } else {
            const float inv = d.w / mix;
#pragma unroll
            for (int c = 0; c < L; ++c) {
                const float g = p[c] * inv;
                v[4 * c] = __fmaf_rn(g, d.x, v[4 * c]);
                v[4 * c + 1] = __fmaf_rn(g, d.y, v[4 * c + 1]);
                v[4 * c + 2] = __fmaf_rn(g, d.z, v[4 * c + 2]);
                v[4 * c + 3] += g;
            }
            if (KIND == PASS_EM) {
                v[NV - 2] += d.w;
                v[NV - 1] = __fmaf_rn(d.w, lg2_approx(mix), v[NV - 1]);
            }
        }
    }
    block_sum<NV, kCluster>(S, T, v, KIND == PASS_CHI2 ? NV : 4 * L);
}

template <int KIND, bool kCluster>
__device__ void sample_pass(Shared &S, const Args &A, Team &T, uint32_t b, uint32_t e) {
    switch (active_lanes(S.m.K)) {
        case 4: sample_pass_l<KIND, 4, kCluster>(S, A, T, b, e); break;
        case 8: sample_pass_l<KIND, 8, kCluster>(S, A, T, b, e); break;
        case 12: sample_pass_l<KIND, 12, kCluster>(S, A, T, b, e); break;
        default: sample_pass_l<KIND, 16, kCluster>(S, A, T, b, e); break;
    }
}

// updateDivergence(Masked) and updateStatistics(Masked) over the region's samples
template <bool kCluster>
__device__ void update_stats(Shared &S, const Args &A, Team &T, uint32_t b, uint32_t e, uint32_t mask) {
    const int L = (int)active_lanes(S.m.K);
    const float n = (float)(e - b);
    if (threadIdx.x == 0) ++S.stat_passes;
    load_pass_mix(S, true);
    sample_pass<PASS_CHI2, kCluster>(S, A, T, b, e);
    const int c = threadIdx.x;  // one thread per component
    if (c < L && ((mask >> c) & 1u)) {
        const float w = S.pm.l[c].y;
        const float sum = w > 0.0f ? S.acc[c] / w : 0.0f;
        const float nn = S.s.dn[c] + n;
        S.s.div[c] = (S.s.div[c] * S.s.dn[c] + sum) / nn;
        S.s.dn[c] = nn;
    }
    __syncthreads();
    sample_pass<PASS_COV, kCluster>(S, A, T, b, e);
    if (c < L && ((mask >> c) & 1u)) {
        const float nw = S.s.cw[c] + S.acc[4 * c];
        for (int i = 0; i < 3; ++i)
            S.s.cov[c][i] = nw > 0.0f ? (S.s.cov[c][i] * S.s.cw[c] + S.acc[4 * c + 1 + i]) / nw : 0.0f;
        S.s.cw[c] = nw;
    }
    __syncthreads();
}

// VMMFactory::maskedFit with maskedParameterUpdate (VMMFactory.h:226-297, 458-485)
template <bool kCluster>
__device__ void masked_fit(Shared &S, const Args &A, Team &T, uint32_t b, uint32_t e) {
    const pg_fit_config &cfg = A.cfg;
    Mix &m = S.m;
    const uint32_t K = m.K;
    const float inv_wpn = cfg.v_prior * (float)K + 1.0f, wpn = 1.0f / inv_wpn, wptn = cfg.v_prior * wpn;
    const int L = (int)active_lanes(K);
    if (threadIdx.x == 0) {
        set_k(m, K);  // resetInactiveComponents
        float old_active = 0.0f;
        for (int c = 0; c < L; ++c)
            if ((S.mask >> c) & 1u) old_active += m.w[c] > wptn ? (m.w[c] - wptn) * inv_wpn : 0.0f;
        S.old_active = old_active;
        S.fit_iters = (e - b) > 2u * K ? (int)cfg.max_itr : 0;
        S.ll_last = 0.0f;
        S.ll_abs_inv = 0.0f;
    }
    __syncthreads();
    const int iters = S.fit_iters;
    const float max_r = k2r(cfg.max_kappa);
    for (int it = 0; it < iters; ++it) {
        load_pass_mix(S, false);
        sample_pass<PASS_EM, kCluster>(S, A, T, b, e);
        // M-step: one thread per refitted component
        const float sum_w = it == 0 ? S.acc[4 * KM] : S.sum_w;
        const int c = threadIdx.x;
        if (c < L && ((S.mask >> c) & 1u)) {
            float active = 0.0f;
            for (int j = 0; j < L; ++j)
                if ((S.mask >> j) & 1u) active += S.acc[4 * j + 3];
            const float norm = S.old_active * (sum_w / active);
            const float sx = S.acc[4 * c] * norm, sy = S.acc[4 * c + 1] * norm, sz = S.acc[4 * c + 2] * norm;
            const float sw = S.acc[4 * c + 3] * norm;
            const float mw = (sw / sum_w) * wpn + wptn;
            const float rl = sqrtf(sx * sx + sy * sy + sz * sz);
            if (rl > 0.0f) {
                m.mx[c] = sx / rl;
                m.my[c] = sy / rl;
                m.mz[c] = sz / rl;
            }
            const float avg = rl / sw;
            const float nsc = (float)m.total * mw;
            float ap = (avg * nsc + cfg.r_prior * cfg.r_prior_weight) / (nsc + cfg.r_prior_weight);
            ap = fminf(ap, max_r);
            m.w[c] = mw;
            set_kappa_r(m, c, r2k(ap), ap);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            ++S.em_iters;
            if (it == 0) S.sum_w = sum_w;
            set_k(m, K);
            // relative log-likelihood stop (VMMFactory.h:284-295), natural log
            int stop = 0;
            const float ll = S.acc[4 * KM + 1] * 0.6931471805599453f;
            if ((uint32_t)it >= cfg.min_itr) {
                if ((uint32_t)it > cfg.min_itr) {
                    const float rel = (ll - S.ll_last) * S.ll_abs_inv;
                    if (rel < cfg.rel_ll_threshold) stop = 1;
                }
                if (!stop) {
                    S.ll_last = ll;
                    S.ll_abs_inv = 1.0f / fabsf(ll);
                }
            }
            S.stop = stop;
        }
        __syncthreads();
        if (S.stop) break;
    }
}

// PathGuiding::postFit with splitAndMerge of region r by a team of CTAs.
template <bool kCluster>
__device__ void split_merge_region(Shared &S, const Args &A, Team &T, uint32_t r) {
    const uint32_t b = A.offsets[r], e = A.offsets[r + 1];
    if (e == b) return;  // PathGuiding::update skips empty regions
    pg_region_state *st = A.states + r;
    pg_region_extra *ex = A.extras + r;
    if (threadIdx.x == 0) {
        Mix &m = S.m;
        m.K = min(st->k, (uint32_t)KM);
        for (int c = 0; c < KM; ++c) {
            m.w[c] = st->weight[c];
            m.mx[c] = st->mu_x[c];
            m.my[c] = st->mu_y[c];
            m.mz[c] = st->mu_z[c];
            m.k[c] = st->kappa[c];
            m.r[c] = st->r[c];
            m.nrm[c] = st->norm[c];
            m.em2k[c] = st->e_min2k[c];
            S.s.div[c] = ex->chi2_div[c];
            S.s.dn[c] = ex->chi2_n[c];
            for (int i = 0; i < 3; ++i) S.s.cov[c][i] = ex->cov[c][i];
            S.s.cw[c] = ex->cov_w[c];
            S.s.dist[c] = st->distance[c];
            S.s.dw[c] = st->dist_sum_w[c];
        }
        m.sample_weight = st->sample_weight;
        m.num_samples = st->num_samples;
        m.total = st->total_num_samples;
        S.stat_passes = 0;
        S.em_iters = 0;
        S.s.since = ex->samples_since_merge + (float)(e - b);
        S.merge = S.s.since > (float)A.sm.min_samples_for_merging;
        if (S.merge) {
            remove_prior(m, A.cfg.v_prior);
            S.s.since = 0.0f;
        }
    }
    __syncthreads();
    if (S.merge) {
        // mergeAll: the pair metrics by all threads, each round's merges by thread 0
        for (int round = 0; round < KM && S.m.K > 1; ++round) {
            merge_candidates(S.m, S.ms, threadIdx.x, NT);
            __syncthreads();
            if (threadIdx.x == 0) S.n_merged = merge_round(S.m, S.s, A.sm, S.ms);
            __syncthreads();
            if (!S.n_merged) break;
        }
        if (threadIdx.x == 0) apply_prior(S.m, A.cfg.v_prior);
        __syncthreads();
    }
    update_stats<kCluster>(S, A, T, b, e, 0xFFFFu);
    const bool first = (unsigned long long)(e - b) == S.m.total;
    const bool fit = first || (e - b) > A.sm.min_samples_for_post_split_fitting;
    if (threadIdx.x == 0) remove_prior(S.m, A.cfg.v_prior);
    __syncthreads();
    if (S.m.K < (uint32_t)KM) {
        for (int round = 0; round < KM; ++round) {
            __shared__ int n_split;
            if (threadIdx.x == 0) {
                Mix &m = S.m;
                // split candidates by weighted divergence (computeDivergence,
                // incrementalpearsonchisquared.h:141-153)
                const float ia = (m.num_samples * m.num_samples) / (m.sample_weight * m.sample_weight);
                float key[KM];
                int cand[KM];
                for (int c = 0; c < (int)m.K; ++c) {
                    const float div = S.s.div[c] * ia - 1.0f;
                    const bool enough = S.s.dn[c] > (float)A.sm.min_samples_for_splitting;
                    key[c] = fabsf((first || enough) ? div * m.w[c] : 0.0f);
                    cand[c] = c;
                }
                const float thr = A.sm.split_min_divergence;
                const int nc = hoare_partition(key, cand, (int *)nullptr, (int)m.K,
                                               [thr](float v) { return v >= thr; });
                const int ns = min(nc, KM - (int)m.K);
                if (ns > 0 && nc > ns) {  // std::partial_sort: the ns largest, descending
                    for (int i = 1; i < nc; ++i) {
                        const float k = key[i];
                        const int c = cand[i];
                        int j = i - 1;
                        while (j >= 0 && key[j] < k) {
                            key[j + 1] = key[j], cand[j + 1] = cand[j];
                            --j;
                        }
                        key[j + 1] = k, cand[j + 1] = c;
                    }
                }
                uint32_t mask = 0;
                for (int i = 0; i < ns; ++i) {
                    mask |= 1u << cand[i];
                    mask |= 1u << m.K;
                    split_component(m, S.s, cand[i], A.cfg.max_kappa);
                }
                S.mask = mask;
                n_split = ns;
                if (ns > 0 && fit) apply_prior(m, A.cfg.v_prior);
            }
            __syncthreads();
            if (n_split == 0) break;
            if (fit) {
                masked_fit<kCluster>(S, A, T, b, e);
                update_stats<kCluster>(S, A, T, b, e, S.mask);
                if (threadIdx.x == 0) remove_prior(S.m, A.cfg.v_prior);
                __syncthreads();
            }
        }
    }
    if (threadIdx.x == 0 && T.rank == 0) {
        Mix &m = S.m;
        apply_prior(m, A.cfg.v_prior);
        st->k = m.K;
        for (int c = 0; c < KM; ++c) {
            st->weight[c] = m.w[c];
            st->mu_x[c] = m.mx[c];
            st->mu_y[c] = m.my[c];
            st->mu_z[c] = m.mz[c];
            st->kappa[c] = m.k[c];
            st->r[c] = m.r[c];
            st->norm[c] = m.nrm[c];
            st->e_min2k[c] = m.em2k[c];
            st->distance[c] = S.s.dist[c];
            st->dist_sum_w[c] = S.s.dw[c];
            ex->chi2_div[c] = S.s.div[c];
            ex->chi2_n[c] = S.s.dn[c];
            for (int i = 0; i < 3; ++i) ex->cov[c][i] = S.s.cov[c][i];
            ex->cov_w[c] = S.s.cw[c];
        }
        ex->samples_since_merge = S.s.since;
        ex->stat_passes = S.stat_passes;
        ex->em_iterations = S.em_iters;
    }
    // no rank leaves (or starts the next region) while another may still read
    // its last partial sums
    if (kCluster) cg::this_cluster().sync();
    else __syncthreads();
}

// Regions up to the cluster threshold: one CTA each, in the order after the
// large ones (A.order[n_large..]).
__global__ void __launch_bounds__(NT, 4) k_split_merge(Args A) {
    __shared__ Shared S;
    const uint32_t j = *A.n_large + blockIdx.x;
    if (j >= A.n_regions) return;
    Team T{0, 1, 0};
    split_merge_region<false>(S, A, T, A.order[j]);
}

// Regions above the cluster threshold (A.order[0..n_large), largest first):
// one cluster of CTAs per region, clusters striding over the regions.
__global__ void __launch_bounds__(NT, 4) k_split_merge_cluster(Args A) {
    __shared__ Shared S;
    cg::cluster_group cl = cg::this_cluster();
    const uint32_t size = cl.num_blocks(), n_clusters = gridDim.x / size;
    const uint32_t n_large = *A.n_large;
    Team T{cl.block_rank(), size, 0};
    for (uint32_t j = blockIdx.x / size; j < n_large; j += n_clusters) split_merge_region<true>(S, A, T, A.order[j]);
}

}  // namespace sm
}  // namespace pg

namespace pg {

int extras_ensure(pg_ctx *ctx, cudaStream_t s) {
    if (ctx->d_extras) return PG_OK;
    int st = check_cuda(ctx, cudaMalloc(&ctx->d_extras, sizeof(pg_region_extra) * (size_t)ctx->max_regions),
                        "split/merge statistics");
    if (!st) st = check_cuda(ctx, cudaStreamCreateWithFlags(&ctx->sm_aux, cudaStreamNonBlocking), "split/merge stream");
    if (!st) st = check_cuda(ctx, cudaEventCreateWithFlags(&ctx->sm_fork, cudaEventDisableTiming), "split/merge event");
    if (!st) st = check_cuda(ctx, cudaEventCreateWithFlags(&ctx->sm_join, cudaEventDisableTiming), "split/merge event");
    if (!st) st = extras_reset(ctx, 0, ctx->max_regions, s);
    return st;
}

void extras_release(pg_ctx *ctx) {
    if (!ctx) return;
    if (ctx->d_extras) cudaFree(ctx->d_extras);
    if (ctx->sm_aux) cudaStreamDestroy(ctx->sm_aux);
    if (ctx->sm_fork) cudaEventDestroy(ctx->sm_fork);
    if (ctx->sm_join) cudaEventDestroy(ctx->sm_join);
    ctx->d_extras = nullptr;
    ctx->sm_aux = nullptr;
    ctx->sm_fork = ctx->sm_join = nullptr;
}

int extras_reset(pg_ctx *ctx, uint32_t first, uint32_t n, cudaStream_t s) {
    if (!ctx->d_extras || n == 0) return PG_OK;
    return check_cuda(ctx, cudaMemsetAsync(ctx->d_extras + first, 0, sizeof(pg_region_extra) * (size_t)n, s),
                      "split/merge statistics reset");
}

}  // namespace pg

using namespace pg;

extern "C" {

void pg_default_split_merge_config(pg_split_merge_config *out) {
    if (!out) return;
    out->enabled = 1;
    out->min_samples_for_merging = 8192;
    out->min_samples_for_splitting = 4096;
    out->min_samples_for_post_split_fitting = 4096;
    out->split_min_divergence = 0.5f;
    out->merge_max_divergence = 0.025f;
    out->cluster_threshold = 0;
    out->cluster_size = 0;
}

int pg_set_split_merge(pg_ctx *ctx, const pg_split_merge_config *cfg) {
    if (!ctx || !cfg) return PG_ERR_ARG;
    if (cfg->enabled) {
        if (int st = extras_ensure(ctx, nullptr)) return st;
        if (cudaDeviceSynchronize() != cudaSuccess) return set_error(ctx, PG_ERR_CUDA, "split/merge setup");
    }
    ctx->sm = *cfg;
    return PG_OK;
}

int pg_split_merge(pg_ctx *ctx, const float *dirw, const float *pdf, const uint32_t *offsets, uint32_t n_regions,
                   void *stream) {
    if (!ctx || !dirw || !pdf || !offsets) return PG_ERR_ARG;
    if (n_regions > ctx->max_regions) return set_error(ctx, PG_ERR_ARG, "n_regions exceeds context capacity");
    if (n_regions == 0) return PG_OK;
    cudaStream_t s = (cudaStream_t)stream;
    guide_mark_stale(ctx);
    if (int st = extras_ensure(ctx, s)) return st;
    sm::Args A;
    A.states = ctx->d_states;
    A.extras = ctx->d_extras;
    A.dirw = reinterpret_cast<const float4 *>(dirw);
    A.pdf = pdf;
    A.offsets = offsets;
    A.order = ctx->d_order;
    A.n_large = ctx->d_counters + 8;
    A.n_regions = n_regions;
    A.cfg = ctx->cfg;
    A.sm = ctx->sm;
    if (!A.sm.min_samples_for_merging && !A.sm.split_min_divergence) pg_default_split_merge_config(&A.sm);
    A.sm.enabled = 1;
    const uint32_t threshold = A.sm.cluster_threshold ? A.sm.cluster_threshold : 8192u;
    const uint32_t csize = A.sm.cluster_size ? A.sm.cluster_size : 8u;
    if (csize > 16) return set_error(ctx, PG_ERR_ARG, "split/merge cluster size above 16");
    const bool clusters = threshold != 0xFFFFFFFFu && csize > 1;
    if (int st = order_regions(ctx, offsets, n_regions, clusters ? threshold : 0xFFFFFFFFu,
                               ctx->d_counters + 8, s))
        return st;
    if (clusters) {
        auto kern = sm::k_split_merge_cluster;
        if (csize > 8) {
            if (int st = check_cuda(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1),
                                    "split/merge cluster attribute"))
                return st;
        }
        cudaLaunchConfig_t lc = {};
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = csize;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        lc.blockDim = dim3(sm::NT, 1, 1);
        lc.stream = ctx->sm_aux;
        lc.attrs = attr;
        lc.numAttrs = 1;
        lc.gridDim = dim3(csize * (uint32_t)ctx->sm_count, 1, 1);
        int resident = 0;
        if (int st = check_cuda(ctx, cudaOccupancyMaxActiveClusters(&resident, kern, &lc), "split/merge occupancy"))
            return st;
        if (resident < 1) return set_error(ctx, PG_ERR_CUDA, "split/merge cluster does not fit on the device");
        lc.gridDim = dim3(csize * std::min<uint32_t>((uint32_t)resident, n_regions), 1, 1);
        // the large regions' clusters run on a side stream beside the per-CTA regions
        int st = check_cuda(ctx, cudaEventRecord(ctx->sm_fork, s), "split/merge fork");
        if (!st) st = check_cuda(ctx, cudaStreamWaitEvent(ctx->sm_aux, ctx->sm_fork, 0), "split/merge fork");
        if (!st) st = check_cuda(ctx, cudaLaunchKernelEx(&lc, kern, A), "split/merge cluster launch");
        if (!st) st = check_cuda(ctx, cudaEventRecord(ctx->sm_join, ctx->sm_aux), "split/merge join");
        if (st) return st;
    }
    sm::k_split_merge<<<n_regions, sm::NT, 0, s>>>(A);
    int st = check_cuda(ctx, cudaGetLastError(), "split/merge launch");
    if (!st && clusters) st = check_cuda(ctx, cudaStreamWaitEvent(s, ctx->sm_join, 0), "split/merge join");
    return st;
}

int pg_get_region_extra(pg_ctx *ctx, pg_region_extra *host_out, uint32_t count) {
    if (!ctx || (!host_out && count)) return PG_ERR_ARG;
    if (count > ctx->max_regions) return set_error(ctx, PG_ERR_ARG, "count exceeds context capacity");
    if (int st = extras_ensure(ctx, nullptr)) return st;
    return check_cuda(ctx, cudaMemcpy(host_out, ctx->d_extras, sizeof(pg_region_extra) * count, cudaMemcpyDeviceToHost),
                      "split/merge statistics download");
}

int pg_set_region_extra(pg_ctx *ctx, const pg_region_extra *host_in, uint32_t count) {
    if (!ctx || (!host_in && count)) return PG_ERR_ARG;
    if (count > ctx->max_regions) return set_error(ctx, PG_ERR_ARG, "count exceeds context capacity");
    if (int st = extras_ensure(ctx, nullptr)) return st;
    return check_cuda(ctx, cudaMemcpy(ctx->d_extras, host_in, sizeof(pg_region_extra) * count, cudaMemcpyHostToDevice),
                      "split/merge statistics upload");
}

}  // extern "C"
