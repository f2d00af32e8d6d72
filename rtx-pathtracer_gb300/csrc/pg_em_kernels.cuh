// pg_em_kernels.cuh - batched weighted EM fit of the per-region vMF mixtures
// (device code; instantiated per component count in pg_em_k8.cu / pg_em_k16.cu).
//
// One persistent launch fits every region.  CTAs pull regions from a device
// work queue ordered largest-first (LPT), so regions with uneven sample counts
// and uneven iteration counts (per-region relative log-likelihood test) share
// the GPU without a host round trip.  Per region, a CTA:
//   1. stages the region's float4 {direction.xyz, weight} samples into shared
//      memory with 1-D TMA bulk copies (cp.async.bulk, mbarrier completion) and
//      keeps them resident across all EM iterations; a slice larger than the
//      staging capacity streams from L2 every iteration through a ring of
//      TMA-filled stages, whose copies run ahead across iteration boundaries
//      (the next iteration's first chunks load during the M-step);
//   2. E-step: every thread evaluates all K components for its samples with
//      packed FP32x2 FMAs - the exponent of pi_k * vMF_k(d) is folded into one
//      affine form kappa_k log2(e) mu_k.d + log2(pi_k norm_k) - kappa_k log2(e),
//      clamped as the reference clamps cos(theta) <= 1, and fed to ex2 - then
//      accumulates the sufficient statistics sum gamma w d and sum gamma w in
//      FP32 registers;
//   3. reduces them with a warp reduce-scatter (shuffles) and merges the warps'
//      partial sums with Neumaier compensation;
//   4. M-step in one warp (lane = component): priors, mean direction, and the
//      kappa-from-mean-cosine inversion, whose 1 - r^2 cancellation is taken in
//      FP64; the log-likelihood convergence test runs in FP64.
//
// Reference: VMMFactory::fit / updateFit (external/lightpmm/include/pmm/
// VMMFactory.h:157-216, 305-362), computeSufficentStatsFromSamples (:497-536),
// parameterUpdate (:436-455), priors (:385-420), computeSufficentStatsFromMixture
// (:543-555); SoftAssignmentWeights (ParametricMixtureModel.h:501-522);
// VMFKernel::pdf / calNormalization / meanCosineToKappa (VMFKernel.h:57-66,
// 103-112, 620-628); the serial region loop of PathGuiding::update
// (src/PathGuiding.cpp:281-288).
#pragma once

#include <math.h>
#include <stdio.h>

#include <cooperative_groups.h>

#include <algorithm>

#include "pg_internal.cuh"

namespace cg = cooperative_groups;

namespace pg {

struct EmArgs {
    pg_region_state *states;
    const float4 *dirw;
    const uint32_t *offsets;
    const uint32_t *order;
    uint32_t n_regions;
    uint32_t *work_counter;
    uint32_t *error_word;
    const float *init_table;
    pg_fit_config cfg;
    int mode;
    uint32_t smem_cap;  // samples staged in shared memory
    double *ll_out;     // eval mode only
    uint32_t *large_counter;     // cluster work queue (largest regions)
    const uint32_t *n_large;     // number of regions fitted by a whole cluster
    uint32_t stages;             // ring stages for streamed slices (>= 1)
    uint32_t stage_n;            // samples per ring stage: a multiple of the E-step trip width
    HostSamples host;            // all null: every sample is in place in dirw
};

// Waits (one thread, bounded: about 2 s) until the chunk of samples holding
// offset b has arrived from the host; a wait that runs out reports
// PG_DEV_ERR_TIMEOUT.  The flags are written by host-to-device copies behind
// each chunk's copy on the copy stream, so the chunk's samples are in device
// memory once its flag reads non-zero.
__device__ __forceinline__ void wait_samples(const EmArgs &a, uint32_t b) {
    const HostSamples &ar = a.host;
    uint32_t c = 0;
    while (c + 1 < ar.n_chunks && ar.start[c + 1] <= b) ++c;
    const long long t0 = clock64();
    for (;;) {
        uint32_t v;
        asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(ar.ready + c) : "memory");
        if (v != 0u) break;
        if (clock64() - t0 > 4000000000LL) {
            atomicOr(a.error_word, PG_DEV_ERR_TIMEOUT);
            break;
        }
        __nanosleep(200);
    }
    __threadfence();
}

// At most kPullers CTAs read their slices from host memory at once, in the
// order they ask (about the fit's largest-first order): the host link then
// serves the first regions' samples first instead of sharing its bandwidth
// among every CTA of the first wave.  Thread 0; a wait that runs out (about
// 2 s) reports PG_DEV_ERR_TIMEOUT and reads anyway.
constexpr uint32_t kPullers = 32;
__device__ __forceinline__ void pull_gate_enter(const EmArgs &a) {
    const uint32_t t = atomicAdd(a.host.pulls, 1u);
    const long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(done) : "l"(a.host.pulls + 1) : "memory");
        if (done + kPullers > t) break;
        if (clock64() - t0 > 4000000000LL) {
            atomicOr(a.error_word, PG_DEV_ERR_TIMEOUT);
            break;
        }
        __nanosleep(256);
    }
}

// The CTA's threads copy samples [0, n) from src (page-locked host memory the
// device addresses) to dst (shared or device memory), eight 16-byte loads in
// flight per thread.
__device__ __forceinline__ void pull_samples(const float4 *__restrict__ src, float4 *__restrict__ dst, uint32_t n,
                                             uint32_t tid, uint32_t nt) {
    constexpr uint32_t D = 8;
    uint32_t i = tid;
    for (; i + (D - 1) * nt < n; i += D * nt) {
        float4 v[D];
#pragma unroll
        for (uint32_t k = 0; k < D; ++k) v[k] = __ldcs(src + i + k * nt);
#pragma unroll
        for (uint32_t k = 0; k < D; ++k) dst[i + k * nt] = v[k];
    }
    for (; i < n; i += nt) dst[i] = __ldcs(src + i);
}

constexpr uint32_t kMaxStages = 8;

// E-step constants of components 2j and 2j+1, laid out for two 128-bit and one
// 64-bit broadcast load: {ax, ay}, {az, c0}, {cm}.
struct __align__(16) ConstPair {
    float ax[2], ay[2], az[2], c0[2], cm[2], pad[2];
};

template <int KMAX, int NW>
struct EmShared {
    ConstPair cp[KMAX / 2];  // E-step constants
    float w[16], mx[16], my[16], mz[16], kap[16], rr[16], nrm[16], em2k[16];
    float osx[16], osy[16], osz[16], ow[16];  // statistics recovered from the prior mixture (updateFit)
    float red[NW][4 * KMAX];
    float red_ll[NW], red_sw[NW];
    float part[8][KMAX];  // this CTA's compensated statistics (cluster mode)
    float ptot[4];        // this CTA's log-likelihood and weight (hi, lo pairs)
    double last_ll, abs_inv_last, ll;
    float sample_weight, num_samples;
    unsigned long long total;
    uint32_t K, max_itr, item, stop, nonfinite;
    unsigned long long bar;
    unsigned long long ring_bar[kMaxStages];  // one per ring stage of a streamed slice
};

// E-step constants of component c from the model held in shared memory.
template <int KMAX, int NW>
__device__ __forceinline__ void make_consts(EmShared<KMAX, NW> &S, int c, uint32_t K) {
    if (c >= KMAX) return;
    const float kl = S.kap[c] * kLog2e;
    const float pn = S.w[c] * S.nrm[c];
    const float lw = (c < (int)K && pn > 0.0f) ? lg2_approx(pn) : -INFINITY;
    ConstPair &q = S.cp[c >> 1];
    const int i = c & 1;
    q.ax[i] = kl * S.mx[c];
    q.ay[i] = kl * S.my[c];
    q.az[i] = kl * S.mz[c];
    q.c0[i] = lw - kl;
    q.cm[i] = lw;
}

__device__ __forceinline__ void reset_component(float &w, float &mx, float &my, float &mz, float &k, float &r,
                                                float &n, float &e) {
    w = 0.0f;
    mx = 0.0f;
    my = 0.0f;
    mz = 1.0f;
    k = 0.0f;
    r = 0.0f;
    n = kInv4Pi;
    e = 1.0f;
}

__device__ __forceinline__ void normalization(float kappa, float &norm, float &em2k) {
    // VMFKernel::calNormalization (VMFKernel.h:620-628), with 1 - e^{-2k} as -expm1(-2k);
    // for kappa >= 10, e^{-2k} < 2.1e-9 and 1 - e^{-2k} rounds to 1 in FP32.
    if (kappa >= 10.0f) {
        em2k = ex2_approx(-2.0f * kLog2e * kappa);
        norm = kappa * (1.0f / kTwoPi);
    } else {
        em2k = expf(-2.0f * kappa);
        norm = kappa > 0.0f ? kappa / (kTwoPi * (-expm1f(-2.0f * kappa))) : kInv4Pi;
    }
}

// Warp 0: load (or initialise) the region's mixture into shared memory.
template <int KMAX, int NW>
__device__ void load_model(const EmArgs &a, EmShared<KMAX, NW> &S, pg_region_state *st, int lane, uint32_t N) {
    const pg_fit_config &cfg = a.cfg;
    float w, mx, my, mz, k, r, n, e;
    uint32_t K;
    if (a.mode == PG_FIT_INIT) {
        // VMMFactory::initialize (VMMFactory.h:132-148)
        K = cfg.num_initial_components;
        if (lane < (int)K) {
            w = 1.0f / (float)K;
            mx = a.init_table[lane];
            my = a.init_table[16 + lane];
            mz = a.init_table[32 + lane];
            k = cfg.init_kappa < kVmfMinKappa ? 0.0f : cfg.init_kappa;
            r = a.init_table[48 + lane];
            normalization(k, n, e);
        } else if (lane < 16) {
            reset_component(w, mx, my, mz, k, r, n, e);
        }
        if (lane == 0) {
            S.sample_weight = 0.0f;
            S.num_samples = 0.0f;
            S.total = 0ull;
        }
    } else {
        K = st->k;
        if (K > 16) K = 16;
        if (lane < 16) {
            w = st->weight[lane];
            mx = st->mu_x[lane];
            my = st->mu_y[lane];
            mz = st->mu_z[lane];
            k = st->kappa[lane];
            r = st->r[lane];
            n = st->norm[lane];
            e = st->e_min2k[lane];
            if (lane >= (int)K) reset_component(w, mx, my, mz, k, r, n, e);  // resetInactiveComponents
        }
        if (lane == 0) {
            S.sample_weight = st->sample_weight;
            S.num_samples = st->num_samples;
            S.total = st->total_num_samples;
        }
    }
    if (lane < 16) {
        S.w[lane] = w;
        S.mx[lane] = mx;
        S.my[lane] = my;
        S.mz[lane] = mz;
        S.kap[lane] = k;
        S.rr[lane] = r;
        S.nrm[lane] = n;
        S.em2k[lane] = e;
        // computeSufficentStatsFromMixture (VMMFactory.h:543-555) for updateFit.
        // A region without prior samples starts from its current mixture alone:
        // removeAvgCosinePrior divides by the prior sample count
        // (VMMFactory.h:428-433), which would make its statistics NaN for good.
        float ow = 0.0f, osx = 0.0f, osy = 0.0f, osz = 0.0f;
        if (a.mode == PG_FIT_UPDATE && lane < (int)K && st->total_num_samples > 0) {
            const float inv_wpn = cfg.v_prior * (float)K + 1.0f;
            const float wpn = 1.0f / inv_wpn;
            const float wptn = cfg.v_prior * wpn;
            const float rptw = cfg.r_prior * cfg.r_prior_weight;
            const float wnp = (w > wptn) ? (w - wptn) * inv_wpn : 0.0f;
            ow = wnp * st->sample_weight;
            const float nn = (float)st->total_num_samples * w;
            const float rr = (r * (nn + cfg.r_prior_weight) - rptw) / nn;
            const float f = rr * ow;
            osx = mx * f;
            osy = my * f;
            osz = mz * f;
        }
        S.ow[lane] = ow;
        S.osx[lane] = osx;
        S.osy[lane] = osy;
        S.osz[lane] = osz;
    }
    __syncwarp();
    make_consts(S, lane, K);
    if (lane == 0) {
        S.K = K;
        // maxItr = 0 unless N > 2K (VMMFactory.h:175-177)
        S.max_itr = (N > 2u * K) ? cfg.max_itr : 0u;
        S.stop = 0;
        S.nonfinite = 0;
        S.last_ll = 0.0;
        S.abs_inv_last = 0.0;
        S.ll = 0.0;
    }
}

// Warp reduce-scatter of M floats over the lanes that share lane bits below
// 5-STEPS (STEPS = 5: the whole warp; STEPS = 4: lanes of equal parity).
// Afterwards lane L holds the sums of elements [(L >> (5-STEPS)) * Q, ... + Q)
// in v[0 .. Q), Q = M >> STEPS.
template <int M, int STEPS>
__device__ __forceinline__ void reduce_scatter(float (&v)[M], int lane) {
#pragma unroll
    for (int s = 0; s < STEPS; ++s) {
        const int o = 16 >> s;
        const int half = M >> (s + 1);
        const bool upper = (lane & o) != 0;
#pragma unroll
        for (int j = 0; j < half; ++j) {
            const float send = upper ? v[j] : v[j + half];
            const float keep = upper ? v[j + half] : v[j];
            v[j] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
}

__device__ __forceinline__ float warp_sum(float x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

// E-step contribution of one sample to this thread's CPT components
// (components [h*CPT, (h+1)*CPT) when TPS = KMAX/CPT threads share a sample).
// Accumulates sum v_k s d and sum v_k s with s = w / p (p = mixture pdf, summed
// over the TPS threads of the sample), and - in the thread with h == 0 -
// sum w log2 p and sum w over valid samples.
template <int CPT, int TPS>
__device__ __forceinline__ void estep_sample(float4 s, bool count_totals, const float2 (&AX)[CPT / 2],
                                             const float2 (&AY)[CPT / 2], const float2 (&AZ)[CPT / 2],
                                             const float2 (&C0)[CPT / 2], const float (&CM)[CPT],
                                             float2 (&SX)[CPT / 2], float2 (&SY)[CPT / 2], float2 (&SZ)[CPT / 2],
                                             float2 (&SW)[CPT / 2], float &ll, float &sw) {
    const float2 dx2 = make_float2(s.x, s.x);
    const float2 dy2 = make_float2(s.y, s.y);
    const float2 dz2 = make_float2(s.z, s.z);
    float v[CPT];
    float2 p2 = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int j = 0; j < CPT / 2; ++j) {
        float2 t = __ffma2_rn(AZ[j], dz2, C0[j]);
        t = __ffma2_rn(AY[j], dy2, t);
        t = __ffma2_rn(AX[j], dx2, t);
        v[2 * j] = ex2_approx(fminf(t.x, CM[2 * j]));
        v[2 * j + 1] = ex2_approx(fminf(t.y, CM[2 * j + 1]));
        p2 = __fadd2_rn(p2, make_float2(v[2 * j], v[2 * j + 1]));
    }
    float p = p2.x + p2.y;
    if (TPS == 2) p += __shfl_xor_sync(0xffffffffu, p, 1);
    const bool valid = p > kPmmEps;
    const float wt = s.w;
    const float sc = valid ? wt * rcp_approx(p) : 0.0f;
    if (count_totals) {
        ll = valid ? fmaf(wt, lg2_approx(p), ll) : ll;
        sw = valid ? sw + wt : sw;
    }
    const float2 sx = make_float2(sc * s.x, sc * s.x);
    const float2 sy = make_float2(sc * s.y, sc * s.y);
    const float2 sz = make_float2(sc * s.z, sc * s.z);
    const float2 s2 = make_float2(sc, sc);
#pragma unroll
    for (int j = 0; j < CPT / 2; ++j) {
        const float2 vv = make_float2(v[2 * j], v[2 * j + 1]);
        SX[j] = __ffma2_rn(vv, sx, SX[j]);
        SY[j] = __ffma2_rn(vv, sy, SY[j]);
        SZ[j] = __ffma2_rn(vv, sz, SZ[j]);
        SW[j] = __ffma2_rn(vv, s2, SW[j]);
    }
}

// E-step over n samples of src (shared memory): thread pairs (TPS = 2) or single
// threads share a sample; U samples per loop trip for instruction-level
// parallelism.  The trip
// count is the same for every thread of the CTA, so the pair shuffle is always
// executed by full warps; samples past n enter with zero weight.
template <int CPT, int TPS, int U>
__device__ __forceinline__ void estep(const float4 *__restrict__ src, uint32_t n, int tid, int nt,
                                      const float2 (&AX)[CPT / 2], const float2 (&AY)[CPT / 2],
                                      const float2 (&AZ)[CPT / 2], const float2 (&C0)[CPT / 2],
                                      const float (&CM)[CPT], float2 (&SX)[CPT / 2], float2 (&SY)[CPT / 2],
                                      float2 (&SZ)[CPT / 2], float2 (&SW)[CPT / 2], float &ll, float &sw) {
    const uint32_t g = (uint32_t)tid / TPS;
    const uint32_t stride = (uint32_t)nt / TPS;
    const bool lead = (tid % TPS) == 0;
    for (uint32_t i0 = 0; i0 < n; i0 += stride * U) {
        float4 sm[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t idx = i0 + g + (uint32_t)u * stride;
            if (idx < n)
                sm[u] = src[idx];
            else
                sm[u] = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            estep_sample<CPT, TPS>(sm[u], lead, AX, AY, AZ, C0, CM, SX, SY, SZ, SW, ll, sw);
    }
}

// Shared-memory loads kept in place: the loop-invariant constants are re-read
// every trip instead of being hoisted into registers.
__device__ __forceinline__ float4 lds_f4(const float *p) {
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"(smem_u32(p)));
    return v;
}
__device__ __forceinline__ float2 lds_f2(const float *p) {
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(smem_u32(p)));
    return v;
}

// The E-step with the constants read from shared memory (broadcast loads, once
// per pair of components per loop trip of U samples) instead of held in
// registers: the same arithmetic in the same order, about 80 fewer registers
// per thread, so more CTAs fit on an SM.
template <int CPT, int TPS, int U>
__device__ __forceinline__ void estep_sc(const float4 *__restrict__ src, uint32_t n, int tid, int nt,
                                         const ConstPair *__restrict__ cpb, float2 (&SX)[CPT / 2],
                                         float2 (&SY)[CPT / 2], float2 (&SZ)[CPT / 2], float2 (&SW)[CPT / 2],
                                         float &ll, float &sw) {
    const uint32_t g = (uint32_t)tid / TPS;
    const uint32_t stride = (uint32_t)nt / TPS;
    const bool lead = (tid % TPS) == 0;
    for (uint32_t i0 = 0; i0 < n; i0 += stride * U) {
        float4 sm[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t idx = i0 + g + (uint32_t)u * stride;
            sm[u] = idx < n ? src[idx] : make_float4(0.0f, 0.0f, 1.0f, 0.0f);
        }
        float v[U][CPT];
        float2 p2[U];
#pragma unroll
        for (int u = 0; u < U; ++u) p2[u] = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int j = 0; j < CPT / 2; ++j) {
            const float4 qa = lds_f4(cpb[j].ax);  // ax0 ax1 ay0 ay1
            const float4 qb = lds_f4(cpb[j].az);  // az0 az1 c00 c01
            const float2 qm = lds_f2(cpb[j].cm);
#pragma unroll
            for (int u = 0; u < U; ++u) {
                float2 t = __ffma2_rn(make_float2(qb.x, qb.y), make_float2(sm[u].z, sm[u].z),
                                      make_float2(qb.z, qb.w));
                t = __ffma2_rn(make_float2(qa.z, qa.w), make_float2(sm[u].y, sm[u].y), t);
                t = __ffma2_rn(make_float2(qa.x, qa.y), make_float2(sm[u].x, sm[u].x), t);
                v[u][2 * j] = ex2_approx(fminf(t.x, qm.x));
                v[u][2 * j + 1] = ex2_approx(fminf(t.y, qm.y));
                p2[u] = __fadd2_rn(p2[u], make_float2(v[u][2 * j], v[u][2 * j + 1]));
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const float4 s = sm[u];
            float p = p2[u].x + p2[u].y;
            if (TPS == 2) p += __shfl_xor_sync(0xffffffffu, p, 1);
            const bool valid = p > kPmmEps;
            const float wt = s.w;
            const float sc = valid ? wt * rcp_approx(p) : 0.0f;
            if (lead) {
                ll = valid ? fmaf(wt, lg2_approx(p), ll) : ll;
                sw = valid ? sw + wt : sw;
            }
            const float2 sx = make_float2(sc * s.x, sc * s.x);
            const float2 sy = make_float2(sc * s.y, sc * s.y);
            const float2 sz = make_float2(sc * s.z, sc * s.z);
            const float2 s2 = make_float2(sc, sc);
#pragma unroll
            for (int j = 0; j < CPT / 2; ++j) {
                const float2 vv = make_float2(v[u][2 * j], v[u][2 * j + 1]);
                SX[j] = __ffma2_rn(vv, sx, SX[j]);
                SY[j] = __ffma2_rn(vv, sy, SY[j]);
                SZ[j] = __ffma2_rn(vv, sz, SZ[j]);
                SW[j] = __ffma2_rn(vv, s2, SW[j]);
            }
        }
    }
}

// Compensated statistics of one component: (hi, lo) pairs of sum gamma w d.xyz, sum gamma w.
struct Stats4 {
    float sxh, sxc, syh, syc, szh, szc, wh, wc;
};

__device__ __forceinline__ Stats4 stats_zero() { return Stats4{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f}; }

// Adds a compensated pair (h, l) into (s, c).
__device__ __forceinline__ void neumaier_add2(float &s, float &c, float h, float l) {
    neumaier_add(s, c, h);
    c += l;
}

// Warp 0, lane c < KMAX: the CTA's statistics of component c, merged over warps.
template <int KMAX, int NW>
__device__ __forceinline__ Stats4 merge_warps(const EmShared<KMAX, NW> &S, int c) {
    Stats4 m = stats_zero();
#pragma unroll
    for (int w = 0; w < NW; ++w) {
        neumaier_add(m.sxh, m.sxc, S.red[w][c]);
        neumaier_add(m.syh, m.syc, S.red[w][KMAX + c]);
        neumaier_add(m.szh, m.szc, S.red[w][2 * KMAX + c]);
        neumaier_add(m.wh, m.wc, S.red[w][3 * KMAX + c]);
    }
    return m;
}

// Lane 0: the CTA's log-likelihood (log2 units) and valid weight, merged over warps.
template <int KMAX, int NW>
__device__ __forceinline__ void merge_totals(const EmShared<KMAX, NW> &S, float &llh, float &llc, float &swh,
                                             float &swc) {
    llh = llc = swh = swc = 0.0f;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
        neumaier_add(llh, llc, S.red_ll[w]);
        neumaier_add(swh, swc, S.red_sw[w]);
    }
}

// The log-likelihood of iteration `it` (FP64) and the relative log-likelihood
// test (VMMFactory.h:201-212): one thread of a warp other than the M-step's, so
// this FP64 chain runs beside the component updates.
template <int KMAX, int NW>
__device__ void mstep_loglik(const EmArgs &a, EmShared<KMAX, NW> &S, uint32_t it, float llh, float llc) {
    const pg_fit_config &cfg = a.cfg;
    S.ll = ((double)llh + (double)llc) * 0.6931471805599453;
    uint32_t stop = 0;
    if (it >= cfg.min_itr) {
        if (it > cfg.min_itr) {
            // (LL - last) * (1/|last|) < thr, evaluated without the division:
            // (LL - last) < thr * |last| gives the same decision for every
            // finite or infinite operand (|last| = 0 included).
            if ((S.ll - S.last_ll) < (double)cfg.rel_ll_threshold * fabs(S.last_ll)) stop = 1;
        }
        if (!stop) S.last_ll = S.ll;
    }
    S.stop = stop;
}

// Warp 0 of the CTA that owns the region: the component updates of iteration
// `it` from merged statistics m (lane c < KMAX) and the region's valid weight
// (lane 0); the log-likelihood and the stopping test are mstep_loglik's.
template <int KMAX, int NW>
__device__ void mstep_apply(const EmArgs &a, EmShared<KMAX, NW> &S, int lane, uint32_t it, uint32_t N, Stats4 m,
                            float swh, float swc) {
    const pg_fit_config &cfg = a.cfg;
    const uint32_t K = S.K;
    if (lane == 0) {
        if (it == 0) {
            const float sum_w = swh + swc;
            if (a.mode == PG_FIT_UPDATE) {
                S.sample_weight += sum_w;
                S.num_samples += (float)N;
                S.total += N;
            } else {
                S.sample_weight = sum_w;
                S.num_samples = (float)N;
                S.total = N;
            }
        }
    }
    __syncwarp();
    if (lane < KMAX) {
        const int c = lane;
        if (a.mode == PG_FIT_UPDATE) {
            neumaier_add(m.sxh, m.sxc, S.osx[c]);
            neumaier_add(m.syh, m.syc, S.osy[c]);
            neumaier_add(m.szh, m.szc, S.osz[c]);
            neumaier_add(m.wh, m.wc, S.ow[c]);
        }
        const float Sx = m.sxh + m.sxc, Sy = m.syh + m.syc, Sz = m.szh + m.szc, W = m.wh + m.wc;
        // Non-finite statistics (corrupt samples) keep the reference's arithmetic
        // but are reported: the region is flagged and pg_sync_status fails.
        if (!(isfinite(Sx) && isfinite(Sy) && isfinite(Sz) && isfinite(W))) S.nonfinite = 1;
        // parameterUpdate (VMMFactory.h:436-455)
        const float inv_wpn = cfg.v_prior * (float)K + 1.0f;
        const float wpn = 1.0f / inv_wpn;
        const float wptn = cfg.v_prior * wpn;
        // Quotients use the fast reciprocal (within 2 ulp): the M-step is on the
        // critical path of every iteration.
        const float mw = __fdividef(W, S.sample_weight) * wpn + wptn;
        const float rl2 = fmaf(Sx, Sx, fmaf(Sy, Sy, Sz * Sz));
        const float irl = rsqrtf(rl2);
        const float rl = rl2 > 0.0f ? rl2 * irl : 0.0f;
        float mx = S.mx[c], my = S.my[c], mz = S.mz[c];
        if (rl2 > 0.0f) {
            mx = Sx * irl;
            my = Sy * irl;
            mz = Sz * irl;
        }
        const float avg = __fdividef(rl, W);
        const float ns = (float)S.total * mw;
        const float a_p = cfg.r_prior * cfg.r_prior_weight;
        const float b_p = cfg.r_prior_weight;
        const float inv_nb = __fdividef(1.0f, ns + b_p);
        float rp = (avg * ns + a_p) * inv_nb;
        // 1 - r_p without cancellation: 1 - avg = (W^2 - |S|^2) / (W (W + |S|)),
        // with W^2 - |S|^2 evaluated in FP64 from the compensated sums.
        const double Wd = (double)m.wh + (double)m.wc;
        const double Xd = (double)m.sxh + (double)m.sxc, Yd = (double)m.syh + (double)m.syc,
                     Zd = (double)m.szh + (double)m.szc;
        const double gap = fma(Wd, Wd, -fma(Xd, Xd, fma(Yd, Yd, Zd * Zd)));
        const float one_m_avg = __fdividef((float)gap, W * (W + rl));
        float one_m_rp = (ns * one_m_avg + (b_p - a_p)) * inv_nb;
        // kappaToMeanCosine(maxKappa) (VMFKernel.h:47-55)
        const float maxk = cfg.max_kappa;
        float maxr, one_m_maxr;
        if (maxk > 5.0f) {
            one_m_maxr = 1.0f / maxk;
            maxr = 1.0f - one_m_maxr;
        } else {
            maxr = 1.0f / tanhf(maxk) - 1.0f / maxk;
            one_m_maxr = 1.0f - maxr;
        }
        if (!(rp < maxr) || !(one_m_rp > one_m_maxr)) {  // min(r, maxr); NaN takes the bound
            rp = maxr;
            one_m_rp = one_m_maxr;
        }
        // meanCosineToKappa (VMFKernel.h:57-66): (3r - r^3) / (1 - r^2)
        float kap = __fdividef(rp * (3.0f - rp * rp), one_m_rp * (1.0f + rp));
        const bool small = kap < kVmfMinKappa;
        kap = small ? 0.0f : kap;
        rp = small ? 0.0f : rp;
        float nrm, em2k;
        normalization(kap, nrm, em2k);
        const bool active = c < (int)K;
        float w_ = mw, r_ = rp;
        if (!active) reset_component(w_, mx, my, mz, kap, r_, nrm, em2k);
        if (!(isfinite(kap) && isfinite(mx) && isfinite(my) && isfinite(mz) && isfinite(w_))) S.nonfinite = 1;
        S.w[c] = w_;
        S.mx[c] = mx;
        S.my[c] = my;
        S.mz[c] = mz;
        S.kap[c] = kap;
        S.rr[c] = r_;
        S.nrm[c] = nrm;
        S.em2k[c] = em2k;
        make_consts(S, c, K);
    }
}

template <int KMAX, int NW>
__device__ void store_model(const EmArgs &a, EmShared<KMAX, NW> &S, pg_region_state *st, int lane, uint32_t iters) {
    if (lane < 16) {
        float w, mx, my, mz, k, r, n, e;
        if (lane < KMAX) {
            w = S.w[lane];
            mx = S.mx[lane];
            my = S.my[lane];
            mz = S.mz[lane];
            k = S.kap[lane];
            r = S.rr[lane];
            n = S.nrm[lane];
            e = S.em2k[lane];
        } else {
            reset_component(w, mx, my, mz, k, r, n, e);
        }
        st->weight[lane] = w;
        st->mu_x[lane] = mx;
        st->mu_y[lane] = my;
        st->mu_z[lane] = mz;
        st->kappa[lane] = k;
        st->r[lane] = r;
        st->norm[lane] = n;
        st->e_min2k[lane] = e;
        if (a.mode == PG_FIT_INIT) {
            st->distance[lane] = INFINITY;
            st->dist_sum_w[lane] = 0.0f;
        }
    }
    if (lane == 0) {
        const uint32_t prev_iters = (a.mode == PG_FIT_INIT) ? 0u : st->num_em_iterations;
        st->k = S.K;
        st->sample_weight = S.sample_weight;
        st->num_samples = S.num_samples;
        st->total_num_samples = S.total;
        st->num_em_iterations = prev_iters + iters;
        st->iters_last = iters;
        st->ll_last = (float)S.ll;
        uint32_t flags = (a.mode == PG_FIT_INIT) ? 0u : st->flags;
        flags &= ~PG_STATE_NONFINITE;
        if (iters > 0) flags |= PG_STATE_FITTED;
        if (S.nonfinite) flags |= PG_STATE_NONFINITE;
        st->flags = flags;
        if (a.mode == PG_FIT_INIT) {
            for (int i = 0; i < 3; ++i) {
                st->parallax_mean[i] = 0.0f;
                st->last_parallax_mean[i] = 0.0f;
            }
        }
        if (S.nonfinite) atomicOr(a.error_word, PG_DEV_ERR_NUMERIC);
    }
}

// Copies the E-step constants, K, the iteration bound and the stop flag from
// the shared memory of cluster rank 0 (warp 0 of a non-zero rank).
template <int KMAX, int NW>
__device__ __forceinline__ void pull_consts(cg::cluster_group &cluster, EmShared<KMAX, NW> &S, int lane) {
    EmShared<KMAX, NW> *R0 = cluster.map_shared_rank(&S, 0);
    constexpr int kWords = (int)sizeof(S.cp) / 4;
    const float *src = reinterpret_cast<const float *>(R0->cp);
    float *dst = reinterpret_cast<float *>(S.cp);
    for (int i = lane; i < kWords; i += 32) dst[i] = src[i];
    if (lane == 0) {
        S.K = R0->K;
        S.max_itr = R0->max_itr;
        S.stop = R0->stop;
    }
}

// One region (or, in a cluster, this CTA's slice of one region): stage the
// samples, iterate E-step / reduction / M-step, store the mixture.
// Issues ring use q of a streamed slice [sb, sb + n_local): chunk q mod nch of
// stage_n samples into stage (g0 + q) mod stages, completing on that stage's
// mbarrier.  One thread; the stage's previous readers have passed a CTA barrier.
template <int KMAX, int NW>
__device__ __forceinline__ void ring_issue(const EmArgs &a, EmShared<KMAX, NW> &S, float4 *s_samp, uint32_t sb,
                                           uint32_t n_local, uint32_t nch, uint32_t g0, uint32_t q) {
    const uint32_t stage_n = a.stage_n;
    const uint32_t c = q % nch;
    const uint32_t stg = (g0 + q) % a.stages;
    const uint32_t n0 = c * stage_n;
    const uint32_t bytes = min(stage_n, n_local - n0) * 16u;
    uint64_t *rb = reinterpret_cast<uint64_t *>(&S.ring_bar[stg]);
    mbar_arrive_expect_tx(rb, bytes);
    const char *src = reinterpret_cast<const char *>(a.dirw + sb + n0);
    char *dst = reinterpret_cast<char *>(s_samp + (size_t)stg * stage_n);
    for (uint32_t off = 0; off < bytes; off += 32768u) tma_bulk_g2s(dst + off, src + off, min(32768u, bytes - off), rb);
}

template <int KMAX, int NT, bool kCluster, int CPT, int U, bool SC>
__device__ void process_region(const EmArgs &a, EmShared<KMAX, NT / 32> &S, float4 *s_samp, uint64_t *bar,
                               uint32_t &phase, uint32_t &ring_pos, uint32_t item, cg::cluster_group &cluster) {
    constexpr int NW = NT / 32;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t crank = kCluster ? cluster.block_rank() : 0u;
    const uint32_t csize = kCluster ? cluster.num_blocks() : 1u;
    const uint32_t r = a.order[item];
    const uint32_t b = a.offsets[r], e = a.offsets[r + 1];
    const uint32_t N = e > b ? e - b : 0u;
    pg_region_state *st = a.states + r;
    if (a.host.ready) {
        // samples copied from the host while the fit runs: wait for this region's chunk
        if (tid == 0) wait_samples(a, b);
        __syncthreads();
    }
    // this CTA's slice [sb, se)
    const uint32_t chunk = (N + csize - 1) / csize;
    const uint32_t sb = min(e, b + crank * chunk);
    const uint32_t se = min(e, sb + chunk);
    const uint32_t n_local = se - sb;
    const bool owner = crank == 0;
    if (owner && warp == 0) load_model(a, S, st, lane, N);
    if (kCluster) {
        cluster.sync();
        if (!owner && warp == 0) pull_consts(cluster, S, lane);
    }
    __syncthreads();
    const uint32_t max_itr = S.max_itr;
    const bool resident = n_local <= a.smem_cap;
    bool ok = true;
    if (resident && max_itr > 0 && n_local > 0 && a.host.mapped) {
        // samples in page-locked host memory: the CTA reads its slice itself
        if (tid == 0) pull_gate_enter(a);
        __syncthreads();
        pull_samples(a.host.mapped + sb, s_samp, n_local, tid, NT);
        fence_proxy_async_smem();  // later TMA writes to this shared memory come after these stores
        __syncthreads();
        if (tid == 0) atomicAdd(a.host.pulls + 1, 1u);
    } else if (resident && max_itr > 0 && n_local > 0) {
        if (tid == 0) {
            fence_proxy_async_smem();
            const uint32_t bytes = n_local * 16u;
            mbar_arrive_expect_tx(bar, bytes);
            const char *src = reinterpret_cast<const char *>(a.dirw + sb);
            char *dst = reinterpret_cast<char *>(s_samp);
            for (uint32_t off = 0; off < bytes; off += 32768u) {
                const uint32_t ch = min(32768u, bytes - off);
                tma_bulk_g2s(dst + off, src + off, ch, bar);
            }
        }
        ok = mbar_wait_bounded(bar, phase, a.error_word);
        phase ^= 1u;
    }
    // A timed-out copy leaves the slice's statistics at zero; the error word reports it.
    uint32_t it = 0;
    constexpr int TPS = KMAX / CPT;  // threads per sample
    const int h = tid % TPS;         // this thread's component block
    // A slice larger than the staging capacity streams through a ring of
    // a.stages stages of stage_n samples.  stage_n is a multiple of the E-step's
    // trip width (NT / TPS threads x U samples), so every thread meets the same
    // samples in the same order as in one pass over the slice.  Ring use q
    // (chunk q mod nch of iteration q / nch) lives in stage (ring_pos + q) mod
    // stages and completes phase ((ring_pos + q) / stages) & 1 of that stage's
    // mbarrier; ring_pos carries over from region to region so the phases stay
    // in step.  A resident slice is one "chunk" that stays in place.
    const uint32_t stages = a.stages, stage_n = a.stage_n;
    const bool ring = !resident && max_itr > 0;  // then n_local > smem_cap >= stage_n > 0
    const uint32_t nch = ring ? (n_local + stage_n - 1) / stage_n : 1u;
    const unsigned long long uses = ring ? (unsigned long long)nch * max_itr : 0ull;
    uint32_t consumed = 0;  // ring uses completed
    if (ring && a.host.mapped) {
        // streamed slice from host memory: copy it once to its place in the
        // device sample buffer, which the ring's TMA copies then read
        if (tid == 0) pull_gate_enter(a);
        __syncthreads();
        pull_samples(a.host.mapped + sb, const_cast<float4 *>(a.dirw) + sb, n_local, tid, NT);
        fence_proxy_async_global();
        __syncthreads();
        if (tid == 0) atomicAdd(a.host.pulls + 1, 1u);
    }
    if (ring && tid == 0) {
        fence_proxy_async_smem();
        const uint32_t first = (uint32_t)min(uses, (unsigned long long)stages);
        for (uint32_t q = 0; q < first; ++q) ring_issue(a, S, s_samp, sb, n_local, nch, ring_pos, q);
    }
    for (; it < max_itr; ++it) {
        float2 AX[CPT / 2], AY[CPT / 2], AZ[CPT / 2], C0[CPT / 2];
        float CM[CPT];
        const ConstPair *cpb = S.cp + h * (CPT / 2);  // this thread's component block
        if constexpr (!SC) {
#pragma unroll
            for (int j = 0; j < CPT / 2; ++j) {
                const ConstPair &q = cpb[j];
                AX[j] = make_float2(q.ax[0], q.ax[1]);
                AY[j] = make_float2(q.ay[0], q.ay[1]);
                AZ[j] = make_float2(q.az[0], q.az[1]);
                C0[j] = make_float2(q.c0[0], q.c0[1]);
                CM[2 * j] = q.cm[0];
                CM[2 * j + 1] = q.cm[1];
            }
        }
        float2 SX[CPT / 2], SY[CPT / 2], SZ[CPT / 2], SW[CPT / 2];
#pragma unroll
        for (int j = 0; j < CPT / 2; ++j) SX[j] = SY[j] = SZ[j] = SW[j] = make_float2(0.0f, 0.0f);
        float ll = 0.0f, sw = 0.0f;
        for (uint32_t c = 0; c < nch && ok; ++c) {
            const float4 *src = s_samp;
            uint32_t n = n_local;
            bool got = true;
            if (ring) {
                const uint32_t g = ring_pos + consumed;
                const uint32_t stg = g % stages;
                got = mbar_wait_bounded(reinterpret_cast<uint64_t *>(&S.ring_bar[stg]), (g / stages) & 1u,
                                        a.error_word);
                src = s_samp + (size_t)stg * stage_n;
                n = min(stage_n, n_local - c * stage_n);
            }
            if (got) {
                if constexpr (SC)
                    estep_sc<CPT, TPS, U>(src, n, tid, NT, cpb, SX, SY, SZ, SW, ll, sw);
                else
                    estep<CPT, TPS, U>(src, n, tid, NT, AX, AY, AZ, C0, CM, SX, SY, SZ, SW, ll, sw);
            }
            if (ring) {
                // Every thread is done with the stage: refill it with use consumed + stages.
                if (__syncthreads_or(!got)) {  // a copy timed out: stop streaming (reported)
                    ok = false;
                    break;
                }
                if ((unsigned long long)consumed + stages < uses && tid == 0) {
                    fence_proxy_async_smem();
                    ring_issue(a, S, s_samp, sb, n_local, nch, ring_pos, consumed + stages);
                }
                ++consumed;
            }
        }
        float f[4 * CPT];
#pragma unroll
        for (int j = 0; j < CPT / 2; ++j) {
            f[2 * j] = SX[j].x;
            f[2 * j + 1] = SX[j].y;
            f[CPT + 2 * j] = SY[j].x;
            f[CPT + 2 * j + 1] = SY[j].y;
            f[2 * CPT + 2 * j] = SZ[j].x;
            f[2 * CPT + 2 * j + 1] = SZ[j].y;
            f[3 * CPT + 2 * j] = SW[j].x;
            f[3 * CPT + 2 * j + 1] = SW[j].y;
        }
        // Lanes of equal component block reduce together (TPS = 2: 4 shuffle steps).
        constexpr int STEPS = (TPS == 2) ? 4 : 5;
        reduce_scatter<4 * CPT, STEPS>(f, lane);
        constexpr int Q = (4 * CPT) >> STEPS;
        const int base = (lane / TPS) * Q;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const int idx = base + q;  // stat * CPT + component-in-block
            S.red[warp][(idx / CPT) * KMAX + h * CPT + (idx % CPT)] = f[q];
        }
        ll = warp_sum(ll);
        sw = warp_sum(sw);
        if (lane == 0) {
            S.red_ll[warp] = ll;
            S.red_sw[warp] = sw;
        }
        __syncthreads();
        if (!kCluster) {
            if (warp == 0) {
                Stats4 m = stats_zero();
                if (lane < KMAX) m = merge_warps(S, lane);
                float llh = 0.f, llc = 0.f, swh = 0.f, swc = 0.f;
                if (lane == 0 && it == 0) merge_totals(S, llh, llc, swh, swc);
                mstep_apply(a, S, lane, it, N, m, swh, swc);
            } else if (warp == 1 && lane == 0) {
                float llh, llc, swh, swc;
                merge_totals(S, llh, llc, swh, swc);
                mstep_loglik(a, S, it, llh, llc);
            }
            __syncthreads();
        } else {
            // CTA partial -> own shared memory; rank 0 merges the cluster's partials.
            if (warp == 0) {
                if (lane < KMAX) {
                    const Stats4 m = merge_warps(S, lane);
                    S.part[0][lane] = m.sxh;
                    S.part[1][lane] = m.sxc;
                    S.part[2][lane] = m.syh;
                    S.part[3][lane] = m.syc;
                    S.part[4][lane] = m.szh;
                    S.part[5][lane] = m.szc;
                    S.part[6][lane] = m.wh;
                    S.part[7][lane] = m.wc;
                }
                if (lane == 0) merge_totals(S, S.ptot[0], S.ptot[1], S.ptot[2], S.ptot[3]);
            }
            cluster.sync();
            if (owner && warp == 0) {
                Stats4 m = stats_zero();
                float swh = 0.f, swc = 0.f;
                for (uint32_t q = 0; q < csize; ++q) {
                    const EmShared<KMAX, NW> *P = cluster.map_shared_rank(&S, q);
                    if (lane < KMAX) {
                        neumaier_add2(m.sxh, m.sxc, P->part[0][lane], P->part[1][lane]);
                        neumaier_add2(m.syh, m.syc, P->part[2][lane], P->part[3][lane]);
                        neumaier_add2(m.szh, m.szc, P->part[4][lane], P->part[5][lane]);
                        neumaier_add2(m.wh, m.wc, P->part[6][lane], P->part[7][lane]);
                    }
                    if (lane == 0 && it == 0) neumaier_add2(swh, swc, P->ptot[2], P->ptot[3]);
                }
                mstep_apply(a, S, lane, it, N, m, swh, swc);
            } else if (owner && warp == 1 && lane == 0) {
                float llh = 0.f, llc = 0.f;
                for (uint32_t q = 0; q < csize; ++q) {
                    const EmShared<KMAX, NW> *P = cluster.map_shared_rank(&S, q);
                    neumaier_add2(llh, llc, P->ptot[0], P->ptot[1]);
                }
                mstep_loglik(a, S, it, llh, llc);
            }
            cluster.sync();
            if (!owner && warp == 0) pull_consts(cluster, S, lane);
            __syncthreads();
        }
        if (S.stop) break;
    }
    if (ring) {
        // An early stop leaves copies in flight: let them land before the
        // shared memory is reused, so every issued use completes its phase.
        const uint32_t issued = (uint32_t)min(uses, (unsigned long long)consumed + stages);
        if (tid == 0)
            for (uint32_t q = consumed; q < issued; ++q) {
                const uint32_t g = ring_pos + q;
                mbar_wait_bounded(reinterpret_cast<uint64_t *>(&S.ring_bar[g % stages]), (g / stages) & 1u,
                                  a.error_word);
            }
        ring_pos += issued;
    }
    if (owner && warp == 0) store_model(a, S, st, lane, it);
    __syncthreads();
}

// MINB: CTAs per SM the register allocation is sized for (0: no limit); SC:
// E-step constants read from shared memory rather than held in registers.
template <int KMAX, int NT, bool kCluster, int CPT, int U, int MINB = 0, bool SC = false>
__global__ void __launch_bounds__(NT, MINB) em_fit_kernel(EmArgs a) {
    constexpr int NW = NT / 32;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float4 *s_samp = reinterpret_cast<float4 *>(smem_raw);
    EmShared<KMAX, NW> &S = *reinterpret_cast<EmShared<KMAX, NW> *>(smem_raw + (size_t)a.smem_cap * 16);
    const int tid = threadIdx.x;
    uint64_t *bar = reinterpret_cast<uint64_t *>(&S.bar);
    cg::cluster_group cluster = cg::this_cluster();
    if (tid == 0) {
        mbar_init(bar, 1);
        for (uint32_t i = 0; i < kMaxStages; ++i) mbar_init(reinterpret_cast<uint64_t *>(&S.ring_bar[i]), 1);
        fence_mbar_init();
    }
    __syncthreads();
    uint32_t phase = 0, ring_pos = 0;
    const uint32_t n_large = kCluster ? *a.n_large : 0u;
    if constexpr (kCluster) {
        // Phase 1: the largest regions, each shared by all CTAs of a cluster.
        for (;;) {
            if (cluster.block_rank() == 0 && tid == 0) S.item = atomicAdd(a.large_counter, 1u);
            cluster.sync();
            const uint32_t item = *cluster.map_shared_rank(&S.item, 0);
            cluster.sync();
            if (item >= n_large) break;
            process_region<KMAX, NT, true, CPT, U, SC>(a, S, s_samp, bar, phase, ring_pos, item, cluster);
        }
    }
    // Phase 2: the remaining regions, one CTA each, largest first.
    for (;;) {
        if (tid == 0) S.item = n_large + atomicAdd(a.work_counter, 1u);
        __syncthreads();
        const uint32_t item = S.item;
        __syncthreads();
        if (item >= a.n_regions) break;
        process_region<KMAX, NT, false, CPT, U, SC>(a, S, s_samp, bar, phase, ring_pos, item, cluster);
    }
}


template <int KMAX, int NT>
inline size_t fit_smem_bytes(uint32_t cap) {
    return (size_t)cap * 16 + sizeof(EmShared<KMAX, NT / 32>);
}

// Ring shape for a launch whose E-step trip covers `grain` samples: at least
// one trip per stage (the staging capacity grows to one trip if smaller, and
// the stage count shrinks until a stage holds a trip), stages a whole number
// of trips.
inline void ring_shape(EmArgs &a, uint32_t grain) {
    a.smem_cap = std::max(a.smem_cap, grain);
    a.stages = std::min(std::max(a.stages, 1u), kMaxStages);
    while (a.stages > 1 && a.smem_cap / a.stages < grain) --a.stages;
    a.stage_n = (a.smem_cap / a.stages) / grain * grain;
}

template <int KMAX, int NT, int CPT, int U, int MINB = 0, bool SC = false>
static int launch_fit(pg_ctx *ctx, const EmArgs &args_in, cudaStream_t s, uint32_t ctas_per_sm, uint32_t cluster) {
    EmArgs args = args_in;
    ring_shape(args, (uint32_t)(NT / (KMAX / CPT)) * U);
    const size_t smem = fit_smem_bytes<KMAX, NT>(args.smem_cap);
    cudaLaunchConfig_t lc = {};
    cudaLaunchAttribute attr[1];
    lc.blockDim = dim3(NT, 1, 1);
    lc.dynamicSmemBytes = smem;
    lc.stream = s;
    int st;
    if (cluster > 1) {
        auto kern = em_fit_kernel<KMAX, NT, true, CPT, U, MINB, SC>;
        st = check_cuda(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                        "em_fit smem attribute");
        if (st) return st;
        if (cluster > 8) {
            st = check_cuda(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1),
                            "em_fit cluster attribute");
            if (st) return st;
        }
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = cluster;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        lc.attrs = attr;
        lc.numAttrs = 1;
        lc.gridDim = dim3(cluster * (uint32_t)ctx->sm_count, 1, 1);
        int nclusters = 0;
        st = check_cuda(ctx, cudaOccupancyMaxActiveClusters(&nclusters, kern, &lc), "em_fit cluster occupancy");
        if (st) return st;
        if (nclusters < 1) return set_error(ctx, PG_ERR_ARG, "em_fit: cluster configuration does not fit");
        uint32_t grid = (uint32_t)nclusters * cluster;
        if (ctas_per_sm) grid = std::min<uint32_t>(grid, ctas_per_sm * (uint32_t)ctx->sm_count / cluster * cluster);
        if (grid < cluster) grid = cluster;
        lc.gridDim = dim3(grid, 1, 1);
        st = check_cuda(ctx, cudaLaunchKernelEx(&lc, kern, args), "em_fit launch");
    } else {
        auto kern = em_fit_kernel<KMAX, NT, false, CPT, U, MINB, SC>;
        st = check_cuda(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                        "em_fit smem attribute");
        if (st) return st;
        int occ = 0;
        st = check_cuda(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, NT, smem), "em_fit occupancy");
        if (st) return st;
        if (occ < 1) return set_error(ctx, PG_ERR_ARG, "em_fit: launch configuration does not fit on an SM");
        const uint32_t per_sm = ctas_per_sm ? std::min<uint32_t>(ctas_per_sm, (uint32_t)occ) : (uint32_t)occ;
        uint32_t grid = per_sm * (uint32_t)ctx->sm_count;
        if (grid > args.n_regions) grid = args.n_regions;
        if (grid == 0) grid = 1;
        lc.gridDim = dim3(grid, 1, 1);
        lc.numAttrs = 0;
        st = check_cuda(ctx, cudaLaunchKernelEx(&lc, kern, args), "em_fit launch");
    }
    return st;
}


// Orders region ids by expected work, largest first (LPT), with a stable
// counting sort over 128 logarithmic buckets (4 per octave).  The work of a
// region is its sample count times its iteration count over 20: a fitted
// region's last fit's count (states, may be null) predicts this fit's, others
// count 20 - so with forced iterations (always 20) the order is by sample
// count, and with the convergence test a region that iterated long last time
// starts early and, above the threshold, gets a cluster (the tail of a
// 100-iteration region on one CTA otherwise outlasts the rest of the fit).
// One CTA of 1024 threads; n_regions of any size.  NB = 128 buckets.
template <int NB>
__global__ void __launch_bounds__(1024) order_regions_kernel(const uint32_t *offsets, uint32_t n_regions,
                                                             uint32_t *order, uint32_t large_threshold,
                                                             uint32_t *n_large_out,
                                                             const pg_region_state *states = nullptr) {
    __shared__ uint32_t hist[NB];
    __shared__ uint32_t base[NB];
    __shared__ uint32_t warp_cnt[32][NB];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    auto bucket_of = [&](uint32_t r) -> int {
        float n = (float)(offsets[r + 1] - offsets[r]);
        if (states) {
            const pg_region_state &st = states[r];
            const uint32_t it = (st.flags & PG_STATE_FITTED) ? st.iters_last : 0u;
            if (it > 0) n = n * (float)it * (1.0f / 20.0f);
        }
        // descending: bucket 0 = largest
        const float l = log2f(n + 1.0f) * 4.0f;
        int k = (int)l;
        k = k < 0 ? 0 : (k > NB - 1 ? NB - 1 : k);
        return NB - 1 - k;
    };
    for (int i = tid; i < NB; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    for (uint32_t r = tid; r < n_regions; r += blockDim.x) atomicAdd(&hist[bucket_of(r)], 1u);
    __syncthreads();
    if (tid == 0) {
        uint32_t acc = 0;
        for (int i = 0; i < NB; ++i) {
            base[i] = acc;
            acc += hist[i];
        }
        // regions whose size bucket is at or above the threshold's bucket come
        // first in the order and are fitted by a whole cluster
        uint32_t nl = 0;
        if (large_threshold != 0xFFFFFFFFu) {
            const float l = log2f((float)large_threshold + 1.0f) * 4.0f;
            int k = (int)l;
            k = k < 0 ? 0 : (k > NB - 1 ? NB - 1 : k);
            const int bt = NB - 1 - k;
            for (int i = 0; i <= bt; ++i) nl += hist[i];
        }
        *n_large_out = nl;
    }
    __syncthreads();
    for (uint32_t chunk = 0; chunk < n_regions; chunk += blockDim.x) {
        const uint32_t r = chunk + tid;
        const bool valid = r < n_regions;
        const int bk = valid ? bucket_of(r) : -1;
        for (int i = lane; i < NB; i += 32) warp_cnt[warp][i] = 0;
        __syncwarp();
        const unsigned mask = __match_any_sync(0xffffffffu, bk);
        const unsigned lt = mask & ((1u << lane) - 1u);
        const uint32_t rank_in_warp = __popc(lt);
        if (valid && lt == 0) warp_cnt[warp][bk] = __popc(mask);
        __syncthreads();
        if (valid) {
            uint32_t before = 0;
            for (int w = 0; w < warp; ++w) before += warp_cnt[w][bk];
            order[base[bk] + before + rank_in_warp] = r;
        }
        __syncthreads();
        // advance bucket bases by this chunk's counts
        for (int i = tid; i < NB; i += blockDim.x) {
            uint32_t add = 0;
            for (int w = 0; w < 32; ++w) add += warp_cnt[w][i];
            base[i] += add;
        }
        __syncthreads();
    }
}


// Launchers of one component bound (pg_em_k8.cu / pg_em_k16.cu): pick the
// instantiation for the tuning's threads per CTA, components per thread and
// unroll, and launch it (clustered when cluster > 1).
int launch_fit_k8(pg_ctx *ctx, const EmArgs &args, cudaStream_t s, const pg_fit_tuning &t, uint32_t cluster);
int launch_fit_k16(pg_ctx *ctx, const EmArgs &args, cudaStream_t s, const pg_fit_tuning &t, uint32_t cluster);

}  // namespace pg
