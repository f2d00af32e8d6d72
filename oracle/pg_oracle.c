/*
 * pg_oracle.c - TEST INFRASTRUCTURE (see pg_oracle.h).  Plain-C restatement of
 * the reference's guiding-fit arithmetic.  Compiled with -ffp-contract=off so
 * that every product and sum rounds the way the reference's SSE2 build does.
 *
 * Citations are to the rtx-pathtracer tree: lightpmm is vendored under
 * external/lightpmm/include/pmm, the guiding statistics under external/guiding.
 */
#include "pg_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define INV_4PI_F ((float)(1.0 / (4.0 * 3.14159265358979323846)))
#define TWO_PI_F ((float)(2.0 * 3.14159265358979323846))
#define PMM_EPS 1.0e-8f       /* PMM_EPSILON, pmm.h:40 */
#define VMF_MIN_KAPPA 1e-3f   /* VMF_MinKappa, VMFKernel.h:42 */

static float bits_to_float(int32_t i) {
    float f;
    memcpy(&f, &i, sizeof f);
    return f;
}

/* SSE2 cvtps2dq: round to nearest even, out of range or NaN -> INT32_MIN. */
static int32_t cvt_rne(float v) {
    if (!(v >= -2147483648.0f && v < 2147483648.0f)) return INT32_MIN;
    return (int32_t)nearbyintf(v);
}

/* fastpow2 (pmm-vcl.h:161-176): Mineiro's rational approximation of 2^p,
 * with the clip at -126 and truncation of the SSE2 build (INSTRSET 2). */
static float fastpow2_f(float p) {
    const float clipp = (-126.0f > p) ? -126.0f : p; /* _mm_max_ps(-126, p) */
    float w;
    {
        /* vcl::truncate, SSE2 path: cvttps2dq, back to float, keep input on overflow */
        if (clipp >= -2147483648.0f && clipp < 2147483648.0f)
            w = (float)(int32_t)clipp;
        else
            w = clipp;
    }
    const float z = (clipp - w) + 1.0f;
    const float t = ((clipp + 121.2740575f) + (27.7280233f / (4.84252568f - z))) - (1.49012907f * z);
    return bits_to_float(cvt_rne(8388608.0f * t));
}

float pgo_fastexp(float x) { return fastpow2_f(1.442695040f * x); }

/* fasttanh (pmm-vcl.h:187-222) for one lane. */
static float fasttanh_f(float x0) {
    const float r0 = -3.33332819422E-1f, r1 = 1.33314422036E-1f, r2 = -5.37397155531E-2f,
                r3 = 2.06390887954E-2f, r4 = -5.70498872745E-3f;
    const float x = fabsf(x0);
    float y;
    if (x <= 0.625f) {
        const float x2 = x * x;
        /* polynomial_4(x2, r0..r4) (vectormath_common.h:136-143), mul_add = a*b+c */
        const float X2 = x2 * x2;
        const float X4 = X2 * X2;
        const float p = (r3 * x2 + r2) * X2 + ((r1 * x2 + r0) + r4 * X4);
        y = p * (x2 * x) + x;
    } else {
        float e = pgo_fastexp(x + x);
        y = 1.0f - 2.0f / (e + 1.0f);
    }
    if (x > 44.4f) y = 1.0f;
    return copysignf(y, x0);
}

/* kappaToMeanCosine (VMFKernel.h:47-55) on one 4-lane group: the cheap
 * 1 - 1/kappa form only when all four lanes exceed 5. */
static void kappa_to_mean_cosine4(const float *kappa, float *r) {
    int all = 1;
    for (int i = 0; i < 4; ++i) all &= (kappa[i] > 5.0f);
    for (int i = 0; i < 4; ++i) {
        if (all) {
            r[i] = 1.0f - 1.0f / kappa[i];
        } else {
            const float v = 1.0f / fasttanh_f(kappa[i]) - 1.0f / kappa[i];
            r[i] = (kappa[i] > 0.0f) ? v : 0.0f;
        }
    }
}

void pgo_initial_mus(uint32_t num_components, float *out) {
    /* computeUniformMus (VMMFactory.h:594-632) for l = K-1, in the reference's
     * float arithmetic: phi is formed in double (2.0f*M_PI is a double) and
     * stored as float; acos/sin/cos are the float functions. */
    const float gr = 1.618033988749895f;
    for (uint32_t n = 0; n < 16; ++n) {
        float x = 0.0f, y = 0.0f, z = 1.0f;
        if (n < num_components) {
            const float phi = (float)(2.0f * M_PI * (double)((float)n / gr));
            const float zz = 1.0f - ((2.0f * (float)n + 1.0f) / (float)num_components);
            const float theta = acosf(zz);
            const float st = sinf(theta);
            x = st * cosf(phi);
            y = st * sinf(phi);
            z = cosf(theta);
        }
        out[n] = x;
        out[16 + n] = y;
        out[32 + n] = z;
    }
}

/* reset of an inactive lane (VMFKernel.h:554-568) */
static void reset_lane(pg_region_state *s, int c) {
    s->weight[c] = 0.0f;
    s->kappa[c] = 0.0f;
    s->r[c] = 0.0f;
    s->mu_x[c] = 0.0f;
    s->mu_y[c] = 0.0f;
    s->mu_z[c] = 1.0f;
    s->norm[c] = INV_4PI_F;
    s->e_min2k[c] = 1.0f;
}

static void cal_normalization_f32(pg_region_state *s, int c) {
    /* VMFKernel::calNormalization (VMFKernel.h:620-628) */
    const float k = s->kappa[c];
    const float e = pgo_fastexp(-2.0f * k);
    s->e_min2k[c] = e;
    const float norm = k / (TWO_PI_F * (1.0f - e));
    s->norm[c] = (k > 0.0f) ? norm : INV_4PI_F;
}

static void cal_normalization_f64(double k, double *norm, double *em2k) {
    *em2k = exp(-2.0 * k);
    *norm = (k > 0.0) ? k / (2.0 * M_PI * (-expm1(-2.0 * k))) : 1.0 / (4.0 * M_PI);
}

void pgo_init_states(const pg_fit_config *cfg, uint32_t n, pg_region_state *states, int exact) {
    const uint32_t K = cfg->num_initial_components;
    float mus[48];
    pgo_initial_mus(K, mus);
    for (uint32_t rg = 0; rg < n; ++rg) {
        pg_region_state *s = &states[rg];
        memset(s, 0, sizeof *s);
        s->k = K;
        const float w0 = 1.0f / (float)K;
        float kap = cfg->init_kappa;
        if (kap < VMF_MIN_KAPPA) kap = 0.0f;
        for (int c = 0; c < 16; ++c) {
            s->distance[c] = INFINITY;
            s->dist_sum_w[c] = 0.0f;
            if ((uint32_t)c >= K) {
                reset_lane(s, c);
                continue;
            }
            s->weight[c] = w0;
            s->mu_x[c] = mus[c];
            s->mu_y[c] = mus[16 + c];
            s->mu_z[c] = mus[32 + c];
            s->kappa[c] = kap;
        }
        for (int g = 0; g < 4; ++g) {
            if ((uint32_t)(4 * g) >= K) break;
            float kk[4] = {kap, kap, kap, kap};
            float rr[4];
            if (exact) {
                for (int i = 0; i < 4; ++i) {
                    const double kd = kap;
                    rr[i] = kd > 0.0 ? (float)(1.0 / tanh(kd) - 1.0 / kd) : 0.0f;
                }
            } else {
                kappa_to_mean_cosine4(kk, rr);
            }
            for (int i = 0; i < 4; ++i) {
                const int c = 4 * g + i;
                if ((uint32_t)c >= K) continue;
                s->r[c] = rr[i];
                if (exact) {
                    double nm, em;
                    cal_normalization_f64(kap, &nm, &em);
                    s->norm[c] = (float)nm;
                    s->e_min2k[c] = (float)em;
                } else {
                    cal_normalization_f32(s, c);
                }
            }
        }
    }
}

/* ------------------------------------------------------------------ */
/* lightpmm-faithful FP32 fit                                          */
/* ------------------------------------------------------------------ */

typedef struct {
    float sx[16], sy[16], sz[16], w[16];
} stats32;

/* computeSufficentStatsFromSamples (VMMFactory.h:497-536) with
 * SoftAssignmentWeights (ParametricMixtureModel.h:501-522). */
static void estep32(const pg_region_state *s, const float *dirw, uint32_t b, uint32_t e,
                    stats32 *st, float *sum_w, float *ll) {
    const uint32_t K = s->k;
    const uint32_t nk = (K + 3) / 4;
    memset(st, 0, sizeof *st);
    if (sum_w) *sum_w = 0.0f;
    if (ll) *ll = 0.0f;
    for (uint32_t n = b; n < e; ++n) {
        const float dx = dirw[4 * (size_t)n], dy = dirw[4 * (size_t)n + 1],
                    dz = dirw[4 * (size_t)n + 2], wt = dirw[4 * (size_t)n + 3];
        float sa[16];
        float part[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (uint32_t k = 0; k < nk; ++k) {
            for (int i = 0; i < 4; ++i) {
                const int c = 4 * k + i;
                const float cs = (s->mu_x[c] * dx + s->mu_y[c] * dy) + s->mu_z[c] * dz;
                const float tm = cs - 1.0f;
                const float t = (tm < 0.0f) ? tm : 0.0f; /* _mm_min_ps(cos-1, 0) */
                const float ex = pgo_fastexp(s->kappa[c] * t);
                const float pdf = s->norm[c] * ex;
                sa[c] = s->weight[c] * pdf;
                part[i] = part[i] + sa[c];
            }
        }
        const float mix = (part[0] + part[2]) + (part[1] + part[3]);
        const float inv = 1.0f / mix;
        if (!(mix > PMM_EPS)) continue;
        for (uint32_t k = 0; k < nk; ++k)
            for (int i = 0; i < 4; ++i) {
                const int c = 4 * k + i;
                const float a = sa[c] * inv;
                const float sw = a * wt;
                st->sx[c] = st->sx[c] + dx * sw;
                st->sy[c] = st->sy[c] + dy * sw;
                st->sz[c] = st->sz[c] + dz * sw;
                st->w[c] = st->w[c] + sw;
            }
        if (sum_w) *sum_w = *sum_w + wt;
        if (ll) *ll = *ll + wt * logf(mix);
    }
}

/* parameterUpdate (VMMFactory.h:436-455) with the priors of :385-420. */
static void mstep32(const pg_fit_config *cfg, pg_region_state *s, const stats32 *st) {
    const uint32_t K = s->k;
    const uint32_t nk = (K + 3) / 4;
    float mk[4] = {cfg->max_kappa, cfg->max_kappa, cfg->max_kappa, cfg->max_kappa};
    float maxr[4];
    kappa_to_mean_cosine4(mk, maxr);
    const float inv_wpn = cfg->v_prior * (float)K + 1.0f;
    const float wpn = 1.0f / inv_wpn;
    const float wptn = cfg->v_prior * wpn;
    const float rptw = cfg->r_prior * cfg->r_prior_weight;
    for (uint32_t c = 0; c < 4 * nk; ++c) {
        const float mw = (st->w[c] / s->sample_weight) * wpn + wptn;
        const float rl = sqrtf((st->sx[c] * st->sx[c] + st->sy[c] * st->sy[c]) + st->sz[c] * st->sz[c]);
        float mx = s->mu_x[c], my = s->mu_y[c], mz = s->mu_z[c];
        if (rl > 0.0f) {
            mx = st->sx[c] / rl;
            my = st->sy[c] / rl;
            mz = st->sz[c] / rl;
        }
        const float avg = rl / st->w[c];
        const float ns = (float)s->total_num_samples * mw;
        float rp = (avg * ns + rptw) / (ns + cfg->r_prior_weight);
        rp = (rp < maxr[c & 3]) ? rp : maxr[c & 3]; /* _mm_min_ps: NaN -> second operand */
        float kap = (rp * 3.0f - ((rp * rp) * rp)) / (1.0f - rp * rp);
        const int small = kap < VMF_MIN_KAPPA;
        s->weight[c] = mw;
        s->mu_x[c] = mx;
        s->mu_y[c] = my;
        s->mu_z[c] = mz;
        s->kappa[c] = small ? 0.0f : kap;
        s->r[c] = small ? 0.0f : rp;
        cal_normalization_f32(s, (int)c);
    }
    /* resetInactiveComponents (VMMFactory.h:110-118) */
    for (uint32_t c = K; c < 4 * nk; ++c) reset_lane(s, (int)c);
}

/* computeSufficentStatsFromMixture (VMMFactory.h:543-555) */
static void stats_from_mixture32(const pg_fit_config *cfg, const pg_region_state *s, stats32 *st) {
    const uint32_t K = s->k;
    const uint32_t nk = (K + 3) / 4;
    const float inv_wpn = cfg->v_prior * (float)K + 1.0f;
    const float wpn = 1.0f / inv_wpn;
    const float wptn = cfg->v_prior * wpn;
    const float rptw = cfg->r_prior * cfg->r_prior_weight;
    memset(st, 0, sizeof *st);
    for (uint32_t c = 0; c < 4 * nk; ++c) {
        const float w = s->weight[c];
        const float wnp = (w > wptn) ? (w - wptn) * inv_wpn : 0.0f;
        const float sw = wnp * s->sample_weight;
        const float n = (float)s->total_num_samples * w;
        const float rr = (s->r[c] * (n + cfg->r_prior_weight) - rptw) / n;
        const float f = rr * sw;
        st->w[c] = sw;
        st->sx[c] = s->mu_x[c] * f;
        st->sy[c] = s->mu_y[c] * f;
        st->sz[c] = s->mu_z[c] * f;
    }
}

static void fit_region32(const pg_fit_config *cfg, int mode, const float *dirw, uint32_t b,
                         uint32_t e, pg_region_state *s, float *ll_final) {
    if (mode == PG_FIT_INIT) pgo_init_states(cfg, 1, s, 0);
    const uint32_t K = s->k;
    const uint32_t nk = (K + 3) / 4;
    for (uint32_t c = K; c < 4 * nk; ++c) reset_lane(s, (int)c);
    stats32 old;
    memset(&old, 0, sizeof old);
    const int update = (mode == PG_FIT_UPDATE);
    /* A region without prior samples starts from its current mixture alone:
     * lightpmm's removeAvgCosinePrior divides by the prior sample count
     * (VMMFactory.h:428-433), which would make its statistics NaN for good. */
    if (update && s->total_num_samples > 0) stats_from_mixture32(cfg, s, &old);
    const uint32_t N = e - b;
    const uint32_t max_itr = (N > 2 * K) ? cfg->max_itr : 0;
    float sum_w = 0.0f, ll = 0.0f, last_ll = 0.0f, abs_inv_last = 0.0f;
    uint32_t i = 0;
    for (; i < max_itr; ++i) {
        stats32 st;
        estep32(s, dirw, b, e, &st, i == 0 ? &sum_w : NULL, i >= cfg->min_itr ? &ll : NULL);
        if (i == 0) {
            if (update) {
                s->sample_weight += sum_w;
                s->num_samples += (float)N;
                s->total_num_samples += N;
            } else {
                s->sample_weight = sum_w;
                s->num_samples = (float)N;
                s->total_num_samples = N;
            }
        }
        if (update)
            for (int c = 0; c < 16; ++c) {
                st.sx[c] = old.sx[c] + st.sx[c];
                st.sy[c] = old.sy[c] + st.sy[c];
                st.sz[c] = old.sz[c] + st.sz[c];
                st.w[c] = old.w[c] + st.w[c];
            }
        mstep32(cfg, s, &st);
        if (i >= cfg->min_itr) {
            if (i > cfg->min_itr) {
                const float rel = (ll - last_ll) * abs_inv_last;
                if (rel < cfg->rel_ll_threshold) break;
            }
            last_ll = ll;
            abs_inv_last = 1.0f / fabsf(ll);
        }
    }
    s->num_em_iterations += i;
    s->iters_last = i;
    s->ll_last = ll;
    s->flags |= PG_STATE_FITTED;
    if (ll_final) {
        stats32 st;
        float l = 0.0f;
        if (e > b) estep32(s, dirw, b, e, &st, NULL, &l);
        *ll_final = l;
    }
}

/* ------------------------------------------------------------------ */
/* FP64 fit                                                            */
/* ------------------------------------------------------------------ */

typedef struct {
    double sx[16], sy[16], sz[16], w[16];
} stats64;

typedef struct {
    double w[16], mx[16], my[16], mz[16], kappa[16], r[16], norm[16];
    double sample_weight;
} mix64;

static void load64(const pg_region_state *s, mix64 *m) {
    for (int c = 0; c < 16; ++c) {
        m->w[c] = s->weight[c];
        m->mx[c] = s->mu_x[c];
        m->my[c] = s->mu_y[c];
        m->mz[c] = s->mu_z[c];
        m->kappa[c] = s->kappa[c];
        m->r[c] = s->r[c];
        m->norm[c] = s->norm[c];
    }
    m->sample_weight = s->sample_weight;
}

static void estep64(const mix64 *m, uint32_t K, const float *dirw, uint32_t b, uint32_t e,
                    stats64 *st, double *sum_w, double *ll) {
    memset(st, 0, sizeof *st);
    if (sum_w) *sum_w = 0.0;
    if (ll) *ll = 0.0;
    for (uint32_t n = b; n < e; ++n) {
        const double dx = dirw[4 * (size_t)n], dy = dirw[4 * (size_t)n + 1],
                     dz = dirw[4 * (size_t)n + 2], wt = dirw[4 * (size_t)n + 3];
        double v[16];
        double p = 0.0;
        for (uint32_t c = 0; c < K; ++c) {
            double cs = m->mx[c] * dx + m->my[c] * dy + m->mz[c] * dz;
            double t = cs - 1.0;
            if (t > 0.0) t = 0.0;
            v[c] = m->w[c] * m->norm[c] * exp(m->kappa[c] * t);
            p += v[c];
        }
        if (!(p > (double)PMM_EPS)) continue;
        const double sc = wt / p;
        for (uint32_t c = 0; c < K; ++c) {
            const double g = v[c] * sc;
            st->sx[c] += g * dx;
            st->sy[c] += g * dy;
            st->sz[c] += g * dz;
            st->w[c] += g;
        }
        if (sum_w) *sum_w += wt;
        if (ll) *ll += wt * log(p);
    }
}

static void mstep64(const pg_fit_config *cfg, mix64 *m, uint32_t K, double total, const stats64 *st) {
    const double maxk = cfg->max_kappa;
    const double maxr = maxk > 0.0 ? 1.0 / tanh(maxk) - 1.0 / maxk : 0.0;
    const double inv_wpn = (double)cfg->v_prior * K + 1.0;
    const double wpn = 1.0 / inv_wpn;
    const double wptn = cfg->v_prior * wpn;
    const double rptw = (double)cfg->r_prior * cfg->r_prior_weight;
    for (uint32_t c = 0; c < K; ++c) {
        const double mw = (st->w[c] / m->sample_weight) * wpn + wptn;
        const double rl = sqrt(st->sx[c] * st->sx[c] + st->sy[c] * st->sy[c] + st->sz[c] * st->sz[c]);
        if (rl > 0.0) {
            m->mx[c] = st->sx[c] / rl;
            m->my[c] = st->sy[c] / rl;
            m->mz[c] = st->sz[c] / rl;
        }
        const double avg = rl / st->w[c];
        const double ns = total * mw;
        double rp = (avg * ns + rptw) / (ns + cfg->r_prior_weight);
        if (!(rp < maxr)) rp = maxr; /* min with NaN taking the bound */
        const double kap = (3.0 * rp - rp * rp * rp) / (1.0 - rp * rp);
        const int small = kap < (double)VMF_MIN_KAPPA;
        m->w[c] = mw;
        m->kappa[c] = small ? 0.0 : kap;
        m->r[c] = small ? 0.0 : rp;
        double em;
        cal_normalization_f64(m->kappa[c], &m->norm[c], &em);
    }
}

static void fit_region64(const pg_fit_config *cfg, int mode, const float *dirw, uint32_t b,
                         uint32_t e, pg_region_state *s, double *ll_final) {
    if (mode == PG_FIT_INIT) pgo_init_states(cfg, 1, s, 1);
    const uint32_t K = s->k;
    for (uint32_t c = K; c < 16; ++c) reset_lane(s, (int)c);
    mix64 m;
    load64(s, &m);
    const int update = (mode == PG_FIT_UPDATE);
    stats64 old;
    memset(&old, 0, sizeof old);
    double total = (double)s->total_num_samples;
    if (update && s->total_num_samples > 0) {  /* no prior samples: no prior statistics */
        const double inv_wpn = (double)cfg->v_prior * K + 1.0;
        const double wptn = cfg->v_prior / inv_wpn;
        const double rptw = (double)cfg->r_prior * cfg->r_prior_weight;
        for (uint32_t c = 0; c < K; ++c) {
            const double w = m.w[c];
            const double sw = (w > wptn ? (w - wptn) * inv_wpn : 0.0) * m.sample_weight;
            const double n = total * w;
            const double rr = (m.r[c] * (n + cfg->r_prior_weight) - rptw) / n;
            old.w[c] = sw;
            old.sx[c] = m.mx[c] * rr * sw;
            old.sy[c] = m.my[c] * rr * sw;
            old.sz[c] = m.mz[c] * rr * sw;
        }
    }
    const uint32_t N = e - b;
    const uint32_t max_itr = (N > 2 * K) ? cfg->max_itr : 0;
    double sum_w = 0.0, ll = 0.0, last_ll = 0.0, abs_inv_last = 0.0;
    double num_samples = s->num_samples;
    uint32_t i = 0;
    for (; i < max_itr; ++i) {
        stats64 st;
        estep64(&m, K, dirw, b, e, &st, i == 0 ? &sum_w : NULL, i >= cfg->min_itr ? &ll : NULL);
        if (i == 0) {
            if (update) {
                m.sample_weight += sum_w;
                num_samples += N;
                total += N;
            } else {
                m.sample_weight = sum_w;
                num_samples = N;
                total = N;
            }
        }
        if (update)
            for (uint32_t c = 0; c < K; ++c) {
                st.sx[c] += old.sx[c];
                st.sy[c] += old.sy[c];
                st.sz[c] += old.sz[c];
                st.w[c] += old.w[c];
            }
        mstep64(cfg, &m, K, total, &st);
        if (i >= cfg->min_itr) {
            if (i > cfg->min_itr) {
                const double rel = (ll - last_ll) * abs_inv_last;
                if (rel < (double)cfg->rel_ll_threshold) break;
            }
            last_ll = ll;
            abs_inv_last = 1.0 / fabs(ll);
        }
    }
    for (uint32_t c = 0; c < K; ++c) {
        s->weight[c] = (float)m.w[c];
        s->mu_x[c] = (float)m.mx[c];
        s->mu_y[c] = (float)m.my[c];
        s->mu_z[c] = (float)m.mz[c];
        s->kappa[c] = (float)m.kappa[c];
        s->r[c] = (float)m.r[c];
        double nm, em;
        cal_normalization_f64(m.kappa[c], &nm, &em);
        s->norm[c] = (float)nm;
        s->e_min2k[c] = (float)em;
    }
    s->sample_weight = (float)m.sample_weight;
    s->num_samples = (float)num_samples;
    s->total_num_samples = (uint64_t)total;
    s->num_em_iterations += i;
    s->iters_last = i;
    s->ll_last = (float)ll;
    s->flags |= PG_STATE_FITTED;
    if (ll_final) {
        stats64 st;
        double l = 0.0;
        if (e > b) estep64(&m, K, dirw, b, e, &st, NULL, &l);
        *ll_final = l;
    }
}

void pgo_eval_ll_f64(uint32_t n_regions, const float *dirw, const uint32_t *offsets,
                     const pg_region_state *states, double *ll_out) {
    for (uint32_t r = 0; r < n_regions; ++r) {
        mix64 m;
        load64(&states[r], &m);
        stats64 st;
        double l = 0.0;
        estep64(&m, states[r].k, dirw, offsets[r], offsets[r + 1], &st, NULL, &l);
        ll_out[r] = l;
    }
}

/* ------------------------------------------------------------------ */
/* Region-parallel driver                                              */
/* ------------------------------------------------------------------ */

typedef struct {
    const pg_fit_config *cfg;
    int mode;
    uint32_t n_regions;
    const float *dirw;
    const uint32_t *offsets;
    pg_region_state *states;
    float *ll32;
    double *ll64;
    int f64;
    uint32_t next; /* atomic */
} job_t;

static void *worker(void *arg) {
    job_t *j = (job_t *)arg;
    for (;;) {
        const uint32_t r = __atomic_fetch_add(&j->next, 1u, __ATOMIC_RELAXED);
        if (r >= j->n_regions) break;
        if (j->f64)
            fit_region64(j->cfg, j->mode, j->dirw, j->offsets[r], j->offsets[r + 1], &j->states[r],
                         j->ll64 ? &j->ll64[r] : NULL);
        else
            fit_region32(j->cfg, j->mode, j->dirw, j->offsets[r], j->offsets[r + 1], &j->states[r],
                         j->ll32 ? &j->ll32[r] : NULL);
    }
    return NULL;
}

static int run_job(job_t *j, int n_threads) {
    if (n_threads <= 1) {
        worker(j);
        return 0;
    }
    if (n_threads > 256) n_threads = 256;
    pthread_t th[256];
    int started = 0;
    for (int t = 0; t < n_threads; ++t)
        if (pthread_create(&th[t], NULL, worker, j) == 0) ++started;
    if (started == 0) worker(j);
    for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
    return 0;
}

int pgo_fit_lpmm32(const pg_fit_config *cfg, int mode, uint32_t n_regions, const float *dirw,
                   const uint32_t *offsets, pg_region_state *states, float *ll_final, int n_threads) {
    job_t j = {cfg, mode, n_regions, dirw, offsets, states, ll_final, NULL, 0, 0};
    return run_job(&j, n_threads);
}

int pgo_fit_f64(const pg_fit_config *cfg, int mode, uint32_t n_regions, const float *dirw,
                const uint32_t *offsets, pg_region_state *states, double *ll_final, int n_threads) {
    job_t j = {cfg, mode, n_regions, dirw, offsets, states, NULL, ll_final, 1, 0};
    return run_job(&j, n_threads);
}

/* ------------------------------------------------------------------ */
/* Parallax, distances, packing, regions, sort                         */
/* ------------------------------------------------------------------ */

void pgo_prefit_parallax(uint32_t n_regions, const pg_directional_data *sorted,
                         const uint32_t *offsets, const float *means, float *dirw_out,
                         float *dist_out) {
    for (uint32_t r = 0; r < n_regions; ++r) {
        const float *m = means + 3 * (size_t)r;
        for (uint32_t i = offsets[r]; i < offsets[r + 1]; ++i) {
            const pg_directional_data *d = &sorted[i];
            float dx = d->direction[0], dy = d->direction[1], dz = d->direction[2];
            float dist;
            if (d->distance > 0.0f) {
                /* pos + distance*direction - parallaxMean, then glm::normalize / length */
                const float nx = (d->position[0] + d->distance * dx) - m[0];
                const float ny = (d->position[1] + d->distance * dy) - m[1];
                const float nz = (d->position[2] + d->distance * dz) - m[2];
                const float l2 = (nx * nx + ny * ny) + nz * nz;
                const float inv = 1.0f / sqrtf(l2);
                dx = nx * inv;
                dy = ny * inv;
                dz = nz * inv;
                dist = sqrtf(l2);
            } else {
                dist = INFINITY;
            }
            dirw_out[4 * (size_t)i] = dx;
            dirw_out[4 * (size_t)i + 1] = dy;
            dirw_out[4 * (size_t)i + 2] = dz;
            dirw_out[4 * (size_t)i + 3] = d->weight;
            dist_out[i] = dist;
        }
    }
}

void pgo_update_distances(uint32_t n_regions, const float *dirw, const float *dist,
                          const uint32_t *offsets, pg_region_state *states) {
    for (uint32_t r = 0; r < n_regions; ++r) {
        /* postFit runs only for regions with samples (PathGuiding.cpp:281-288) */
        if (offsets[r + 1] == offsets[r]) continue;
        pg_region_state *s = &states[r];
        const uint32_t K = s->k;
        double bw[16] = {0}, bwd[16] = {0};
        for (uint32_t i = offsets[r]; i < offsets[r + 1]; ++i) {
            const double t_n = dist[i];
            if (!(t_n > 0.0)) continue;
            const double dx = dirw[4 * (size_t)i], dy = dirw[4 * (size_t)i + 1],
                         dz = dirw[4 * (size_t)i + 2], wt = dirw[4 * (size_t)i + 3];
            double pdf[16], v[16], p = 0.0;
            for (uint32_t c = 0; c < K; ++c) {
                double t = s->mu_x[c] * dx + s->mu_y[c] * dy + s->mu_z[c] * dz - 1.0;
                if (t > 0.0) t = 0.0;
                pdf[c] = s->norm[c] * exp((double)s->kappa[c] * t);
                v[c] = s->weight[c] * pdf[c];
                p += v[c];
            }
            if (!(p > (double)PMM_EPS)) continue;
            const double sc = wt / p;
            for (uint32_t c = 0; c < K; ++c) {
                const double a = v[c] * pdf[c] * sc;
                bw[c] += a;
                bwd[c] += a / t_n;
            }
        }
        for (uint32_t c = 0; c < K; ++c) {
            const float nw = (float)((double)s->dist_sum_w[c] + bw[c]);
            const float den = (float)((double)s->dist_sum_w[c] / (double)s->distance[c] + bwd[c]);
            s->distance[c] = nw / den;
            s->dist_sum_w[c] = nw;
        }
    }
}

void pgo_reposition(pg_region_state *s, const float d[3]) {
    for (uint32_t c = 0; c < s->k; ++c) {
        const int invalid = isinf(s->distance[c]) || s->dist_sum_w[c] <= 0.0f;
        if (invalid) continue;
        const float x = s->mu_x[c] * s->distance[c] + d[0];
        const float y = s->mu_y[c] * s->distance[c] + d[1];
        const float z = s->mu_z[c] * s->distance[c] + d[2];
        const float l = sqrtf((x * x + y * y) + z * z);
        s->distance[c] = l;
        s->mu_x[c] = x / l;
        s->mu_y[c] = y / l;
        s->mu_z[c] = z / l;
    }
}

void pgo_pack_vmm_theta(uint32_t n_regions, const pg_region_state *states, int use_parallax,
                        pg_vmm_theta *out) {
    for (uint32_t r = 0; r < n_regions; ++r) {
        const pg_region_state *s = &states[r];
        pg_vmm_theta *v = &out[r];
        memset(v, 0, sizeof *v);
        for (int c = 0; c < 16; ++c) v->thetas[c].distance = -1.0f;
        v->used_distributions = (int32_t)s->k;
        for (uint32_t c = 0; c < s->k; ++c) {
            v->pi[c] = s->weight[c];
            v->thetas[c].mu[0] = s->mu_x[c];
            v->thetas[c].mu[1] = s->mu_y[c];
            v->thetas[c].mu[2] = s->mu_z[c];
            /* VMF_Theta::setK (src/PathGuiding.h:44-50), evaluated in double */
            float k = s->kappa[c];
            k = k < VMF_MIN_KAPPA ? 0.0f : k;
            v->thetas[c].k = k;
            v->thetas[c].norm = (float)((double)k / (2.0 * M_PI * (1.0 - exp(-2.0 * (double)k))));
            v->thetas[c].e_min2k = (float)exp(-2.0 * (double)k);
        }
        if (use_parallax) {
            for (int i = 0; i < 3; ++i) v->mean_position[i] = s->parallax_mean[i];
            for (int c = 0; c < 16; ++c) {
                float dd = s->distance[c];
                dd = (dd == INFINITY) ? -1.0f : dd;
                v->thetas[c].distance = dd;
                for (int i = 0; i < 3; ++i) {
                    const float mu = v->thetas[c].mu[i];
                    v->thetas[c].target[i] = s->parallax_mean[i] + dd * mu;
                }
            }
        }
    }
}

void pgo_region_aabbs(uint32_t split_count, const float a[6], float *out) {
    /* Aabb::addEpsilon (src/Shapes.h:48-53) */
    float mn[3], mx[3];
    for (int i = 0; i < 3; ++i) {
        const float ext = a[3 + i] - a[i];
        const float cen = a[i] + 0.5f * ext;
        mn[i] = cen - 0.50001f * ext;
        mx[i] = cen + 0.50001f * ext;
    }
    const uint32_t n = 1u << split_count;
    float *cur = (float *)malloc(sizeof(float) * 6 * n);
    float *nxt = (float *)malloc(sizeof(float) * 6 * n);
    for (int i = 0; i < 3; ++i) {
        cur[i] = mn[i];
        cur[3 + i] = mx[i];
    }
    uint32_t count = 1;
    for (uint32_t s = 0; s < split_count; ++s) {
        for (uint32_t b = 0; b < count; ++b) {
            const float *bx = cur + 6 * b;
            float size[3];
            for (int i = 0; i < 3; ++i) size[i] = bx[3 + i] - bx[i];
            const int axis = size[0] > size[1] ? (size[0] > size[2] ? 0 : 2) : (size[1] > size[2] ? 1 : 2);
            float *L = nxt + 6 * (2 * b), *R = nxt + 6 * (2 * b + 1);
            memcpy(L, bx, sizeof(float) * 6);
            memcpy(R, bx, sizeof(float) * 6);
            L[3 + axis] -= 0.5f * size[axis];
            R[axis] += 0.5f * size[axis];
        }
        count *= 2;
        float *t = cur;
        cur = nxt;
        nxt = t;
    }
    memcpy(out, cur, sizeof(float) * 6 * n);
    free(cur);
    free(nxt);
}

uint64_t pgo_sort_samples(const pg_directional_data *rec, uint64_t n, uint32_t n_regions,
                          pg_directional_data *sorted, uint32_t *offsets) {
    memset(offsets, 0, sizeof(uint32_t) * (n_regions + 1));
    for (uint64_t i = 0; i < n; ++i)
        if (rec[i].flags < n_regions) offsets[rec[i].flags + 1]++;
    for (uint32_t r = 0; r < n_regions; ++r) offsets[r + 1] += offsets[r];
    uint32_t *cursor = (uint32_t *)malloc(sizeof(uint32_t) * (n_regions + 1));
    memcpy(cursor, offsets, sizeof(uint32_t) * (n_regions + 1));
    for (uint64_t i = 0; i < n; ++i)
        if (rec[i].flags < n_regions) sorted[cursor[rec[i].flags]++] = rec[i];
    free(cursor);
    return offsets[n_regions];
}

/* ------------------------------------------------------------------ */
/* Split and merge after the fit (PathGuiding::postFit)                */
/* ------------------------------------------------------------------ */
/*
 * PathGuiding::postFit with splitAndMerge (src/PathGuiding.cpp:413-451) on
 * lightpmm's FP32 4-lane arithmetic: component pdfs with fastexp, per-lane
 * partial sums folded as (l0 + l2) + (l1 + l3), a whole kernel's norms
 * recomputed whenever one lane's kappa is set.  The statistics follow
 * external/guiding/incrementalpearsonchisquared.h:53-204,
 * incrementalcovariance2d.h:53-263 and incrementaldistance.h:165-216; the
 * merge metric and merges src/PathGuiding.cpp:635-781 with
 * VMFKernel.h:315-400, 478-530; the splits :494-633 with VMMFactory.h:226-297,
 * 458-485.  The principal axis of the PCA split is the closed-form eigenvector
 * of the symmetric 2x2 covariance (the reference calls Eigen there).
 */

#define SM_KM 16

static float hsum4(const float p[4]) { return (p[0] + p[2]) + (p[1] + p[3]); }

static float lane_pdf(const pg_region_state *s, int c, float dx, float dy, float dz) {
    const float cs = (s->mu_x[c] * dx + s->mu_y[c] * dy) + s->mu_z[c] * dz;
    const float tm = cs - 1.0f;
    const float t = (tm < 0.0f) ? tm : 0.0f;
    return s->norm[c] * pgo_fastexp(s->kappa[c] * t);
}

/* kappaToMeanCosine for one scalar (the 4-lane rule with all lanes equal) */
static float k2r_scalar(float k) {
    float kk[4] = {k, k, k, k}, r[4];
    kappa_to_mean_cosine4(kk, r);
    return r[0];
}

static float r2k_f(float r) { return (r * 3.0f - ((r * r) * r)) / (1.0f - r * r); }

/* VMFKernel::setKappaAndR(idx, ...) then calNormalization of the whole kernel */
static void set_kappa_r_lane(pg_region_state *s, int c, float kappa, float r) {
    const int small = kappa < VMF_MIN_KAPPA;
    s->kappa[c] = small ? 0.0f : kappa;
    s->r[c] = small ? 0.0f : r;
    const int k0 = c & ~3;
    for (int i = 0; i < 4; ++i) cal_normalization_f32(s, k0 + i);
}

/* ParametricMixtureModel::removeWeightPrior / applyWeightPrior (:339-370) */
static void pmm_remove_prior(pg_region_state *s, float v) {
    const uint32_t K = s->k, nk = (K + 3) / 4;
    const float inv = v * (float)K + 1.0f, wpn = 1.0f / inv, wptn = v * wpn;
    for (uint32_t c = 0; c < 4 * nk; ++c) s->weight[c] = (s->weight[c] - wptn) * inv;
    for (uint32_t c = K; c < 4 * nk; ++c) s->weight[c] = 0.0f;
}
static void pmm_apply_prior(pg_region_state *s, float v) {
    const uint32_t K = s->k, nk = (K + 3) / 4;
    const float inv = v * (float)K + 1.0f, wpn = 1.0f / inv, wptn = v * wpn;
    for (uint32_t c = 0; c < 4 * nk; ++c) s->weight[c] = s->weight[c] * wpn + wptn;
    for (uint32_t c = K; c < 4 * nk; ++c) s->weight[c] = 0.0f;
}

/* VMFKernel::cutoff of the lanes from K in K's kernel (resetInactiveComponents) */
static void cutoff_last(pg_region_state *s) {
    const uint32_t K = s->k;
    if (K % 4 == 0) return;
    for (uint32_t c = K; c < (K + 3) / 4 * 4; ++c) reset_lane(s, (int)c);
}

/* ParametricMixtureModel::setK (:426-440): lanes beyond K in K's kernel are
 * cut off, the kernels after the next are reset */
static void set_k(pg_region_state *s, uint32_t K) {
    s->k = K;
    const uint32_t full = K / 4, rem = K % 4;
    if (rem) for (uint32_t c = K; c < 4 * full + 4; ++c) reset_lane(s, (int)c);
    for (uint32_t k = full + 1; k < 4; ++k)
        for (int i = 0; i < 4; ++i) reset_lane(s, (int)(4 * k + i));
}

/* Component pdfs and weight x pdf of one sample over the active kernels */
static float sample_pdfs(const pg_region_state *s, uint32_t nk, float dx, float dy, float dz, float *pdf,
                         float *wpdf) {
    float part[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (uint32_t k = 0; k < nk; ++k)
        for (int i = 0; i < 4; ++i) {
            const int c = 4 * (int)k + i;
            pdf[c] = lane_pdf(s, c, dx, dy, dz);
            wpdf[c] = s->weight[c] * pdf[c];
            part[i] = part[i] + wpdf[c];
        }
    return hsum4(part);
}

/* IncrementalPearsonChiSquared::updateDivergence(Masked) */
static void chi2_update(const pg_region_state *s, pg_region_extra *x, const float *dirw, const float *pdf_s,
                        uint32_t b, uint32_t e, uint32_t mask) {
    if (e == b) return;
    const uint32_t nk = (s->k + 3) / 4;
    float batch[SM_KM] = {0};
    for (uint32_t n = b; n < e; ++n) {
        const float *d = dirw + 4 * (size_t)n;
        float pdf[SM_KM], wpdf[SM_KM];
        const float mix = sample_pdfs(s, nk, d[0], d[1], d[2], pdf, wpdf);
        if (!(mix > PMM_EPS)) continue;
        const float f = ((d[3] * d[3]) * pdf_s[n]) / (mix * mix);
        for (uint32_t c = 0; c < 4 * nk; ++c)
            if ((mask >> c) & 1u) batch[c] = batch[c] + pdf[c] * f;
    }
    const float N = (float)(e - b);
    for (uint32_t c = 0; c < 4 * nk; ++c) {
        if (!((mask >> c) & 1u)) continue;
        const float nn = x->chi2_n[c] + N;
        x->chi2_div[c] = (x->chi2_div[c] * x->chi2_n[c] + batch[c]) / nn;
        x->chi2_n[c] = nn;
    }
}

/* IncrementalCovariance2D::updateStatistics(Masked) */
static void cov_update(const pg_region_state *s, pg_region_extra *x, const float *dirw, uint32_t b, uint32_t e,
                       uint32_t mask) {
    const uint32_t nk = (s->k + 3) / 4;
    float sv[SM_KM][3], tv[SM_KM][3];
    for (uint32_t c = 0; c < 4 * nk; ++c) {
        const float nx = s->mu_x[c], ny = s->mu_y[c], nz = s->mu_z[c];
        const float sx = nx * nx, sy = ny * ny, sz = nz * nz;
        const int xg = sx > sy;
        const float inv = 1.0f / sqrtf((xg ? sx : sy) + sz);
        const float t0 = xg ? nz * inv : 0.0f, t1 = xg ? 0.0f : nz * inv, t2 = xg ? -nx * inv : -ny * inv;
        tv[c][0] = t0, tv[c][1] = t1, tv[c][2] = t2;
        sv[c][0] = (t1 * nz) - (t2 * ny);
        sv[c][1] = (t2 * nx) - (t0 * nz);
        sv[c][2] = (t0 * ny) - (t1 * nx);
    }
    float bw[SM_KM] = {0}, bv[SM_KM][3] = {{0}};
    for (uint32_t n = b; n < e; ++n) {
        const float *d = dirw + 4 * (size_t)n;
        float pdf[SM_KM], wpdf[SM_KM];
        const float mix = sample_pdfs(s, nk, d[0], d[1], d[2], pdf, wpdf);
        const float inv = 1.0f / mix;
        if (!(mix > PMM_EPS)) continue;
        for (uint32_t c = 0; c < 4 * nk; ++c) {
            if (!((mask >> c) & 1u)) continue;
            const float wt = d[3] * (wpdf[c] * inv);
            bw[c] = bw[c] + wt;
            const float lx = (sv[c][0] * d[0] + sv[c][1] * d[1]) + sv[c][2] * d[2];
            const float ly = (tv[c][0] * d[0] + tv[c][1] * d[1]) + tv[c][2] * d[2];
            bv[c][0] = bv[c][0] + (lx * lx) * wt;
            bv[c][1] = bv[c][1] + (ly * ly) * wt;
            bv[c][2] = bv[c][2] + (lx * ly) * wt;
        }
    }
    for (uint32_t c = 0; c < 4 * nk; ++c) {
        if (!((mask >> c) & 1u)) continue;
        const float ns = x->cov_w[c] + bw[c];
        for (int i = 0; i < 3; ++i) x->cov[c][i] = ns > 0.0f ? (x->cov[c][i] * x->cov_w[c] + bv[c][i]) / ns : 0.0f;
        x->cov_w[c] = ns;
    }
}

/* VMMFactory::maskedFit with maskedParameterUpdate (prior applied on entry) */
static void masked_fit32(const pg_fit_config *cfg, pg_region_state *s, const float *dirw, uint32_t b, uint32_t e,
                         uint32_t mask, uint32_t *iters) {
    const uint32_t K = s->k, nk = (K + 3) / 4;
    cutoff_last(s);
    const float inv_wpn = cfg->v_prior * (float)K + 1.0f, wpn = 1.0f / inv_wpn, wptn = cfg->v_prior * wpn;
    const float rptw = cfg->r_prior * cfg->r_prior_weight;
    float part[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (uint32_t c = 0; c < 4 * nk; ++c) {
        const float w = s->weight[c];
        const float wnp = (w > wptn) ? (w - wptn) * inv_wpn : 0.0f;
        part[c & 3] = part[c & 3] + (((mask >> c) & 1u) ? wnp : 0.0f);
    }
    const float old_active = hsum4(part);
    float mk[4] = {cfg->max_kappa, cfg->max_kappa, cfg->max_kappa, cfg->max_kappa}, maxr[4];
    kappa_to_mean_cosine4(mk, maxr);
    const uint32_t max_itr = (e - b) > 2u * K ? cfg->max_itr : 0;
    float sum_w = 0.0f, ll = 0.0f, last_ll = 0.0f, abs_inv_last = 0.0f;
    uint32_t i = 0;
    for (; i < max_itr; ++i) {
        stats32 st;
        estep32(s, dirw, b, e, &st, i == 0 ? &sum_w : NULL, i >= cfg->min_itr ? &ll : NULL);
        float ap[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (uint32_t k = 0; k < nk; ++k) {
            if (!((mask >> (4 * k)) & 0xFu)) continue;
            for (int l = 0; l < 4; ++l)
                ap[l] = ap[l] + (((mask >> (4 * k + l)) & 1u) ? st.w[4 * k + l] : 0.0f);
        }
        const float norm = old_active * (sum_w / hsum4(ap));
        for (uint32_t c = 0; c < 4 * nk; ++c)
            if ((mask >> c) & 1u) {
                st.sx[c] = st.sx[c] * norm;
                st.sy[c] = st.sy[c] * norm;
                st.sz[c] = st.sz[c] * norm;
                st.w[c] = st.w[c] * norm;
            }
        for (uint32_t k = 0; k < nk; ++k) {
            if (!((mask >> (4 * k)) & 0xFu)) continue;
            float kap[4], rr[4];
            for (int l = 0; l < 4; ++l) {
                const int c = 4 * (int)k + l;
                if (!((mask >> c) & 1u)) {
                    kap[l] = s->kappa[c];
                    rr[l] = s->r[c];
                    continue;
                }
                const float mw = (st.w[c] / sum_w) * wpn + wptn;
                const float rl = sqrtf((st.sx[c] * st.sx[c] + st.sy[c] * st.sy[c]) + st.sz[c] * st.sz[c]);
                if (rl > 0.0f) {
                    s->mu_x[c] = st.sx[c] / rl;
                    s->mu_y[c] = st.sy[c] / rl;
                    s->mu_z[c] = st.sz[c] / rl;
                }
                const float avg = rl / st.w[c];
                const float ns = (float)s->total_num_samples * mw;
                float rp = (avg * ns + rptw) / (ns + cfg->r_prior_weight);
                rp = (rp < maxr[l]) ? rp : maxr[l];
                s->weight[c] = mw;
                kap[l] = r2k_f(rp);
                rr[l] = rp;
            }
            for (int l = 0; l < 4; ++l) {
                const int c = 4 * (int)k + l;
                const int small = kap[l] < VMF_MIN_KAPPA;
                s->kappa[c] = small ? 0.0f : kap[l];
                s->r[c] = small ? 0.0f : rr[l];
            }
            for (int l = 0; l < 4; ++l) cal_normalization_f32(s, 4 * (int)k + l);
        }
        cutoff_last(s);
        if (i >= cfg->min_itr) {
            if (i > cfg->min_itr) {
                const float rel = (ll - last_ll) * abs_inv_last;
                if (rel < cfg->rel_ll_threshold) {
                    ++i;
                    break;
                }
            }
            last_ll = ll;
            abs_inv_last = 1.0f / fabsf(ll);
        }
    }
    *iters += i;
}

typedef struct {
    float w, mx, my, mz, k, nrm;
} lobe_t;

static lobe_t lobe_of(const pg_region_state *s, int c) {
    lobe_t l = {s->weight[c], s->mu_x[c], s->mu_y[c], s->mu_z[c], s->kappa[c], s->norm[c]};
    return l;
}

/* VMFKernel::product (sign +1) and division (sign -1): a becomes a*b or a/b,
 * the integral is returned */
static float vmf_combine(lobe_t *a, const lobe_t *b, int sign) {
    float nx, ny, nz;
    if (sign > 0) {
        nx = a->mx * a->k + b->mx * b->k, ny = a->my * a->k + b->my * b->k, nz = a->mz * a->k + b->mz * b->k;
    } else {
        nx = a->mx * a->k - b->mx * b->k, ny = a->my * a->k - b->my * b->k, nz = a->mz * a->k - b->mz * b->k;
    }
    float nk = sqrtf((nx * nx + ny * ny) + nz * nz);
    const int small = nk < VMF_MIN_KAPPA;
    if (small) {
        nk = 0.0f;
        nx = a->mx, ny = a->my, nz = a->mz;
    } else {
        nx = nx / nk, ny = ny / nk, nz = nz / nk;
    }
    const float ci = a->nrm, cj = b->nrm;
    const float e2 = pgo_fastexp(-2.0f * nk);
    const float cij = small ? INV_4PI_F : ((float)(1.0 / (2.0 * 3.14159265358979323846)) * nk) / (1.0f - e2);
    const float ti = (nx * a->mx + ny * a->my) + nz * a->mz, tj = (nx * b->mx + ny * b->my) + nz * b->mz;
    float s;
    if (sign > 0) {
        const float t = a->k * (ti - 1.0f) + b->k * (tj - 1.0f);
        s = (((pgo_fastexp(t) * a->w) * b->w) * (ci * cj)) / cij;
    } else {
        const float t = a->k * (ti - 1.0f) - b->k * (tj - 1.0f);
        s = ((pgo_fastexp(t) * a->w) * ci) / ((b->w * cj) * cij);
    }
    a->w = s, a->mx = nx, a->my = ny, a->mz = nz, a->k = nk, a->nrm = cij;
    return s;
}

/* VMFKernel::mergeComponent (:478-530): the merged lobe of two components,
 * with its r and exp(-2 kappa) */
static void merge_lobes(const pg_region_state *s, int a, int b, float out[8]) {
    const float w0 = s->weight[a], w1 = s->weight[b], r0 = s->r[a], r1 = s->r[b];
    float kappa = 0.0f, norm = INV_4PI_F, em2k = 1.0f;
    const float w = w0 + w1;
    float mx = w0 * r0 * s->mu_x[a] + w1 * r1 * s->mu_x[b];
    float my = w0 * r0 * s->mu_y[a] + w1 * r1 * s->mu_y[b];
    float mz = w0 * r0 * s->mu_z[a] + w1 * r1 * s->mu_z[b];
    mx /= w, my /= w, mz /= w;
    float r = mx * mx + my * my + mz * mz;
    if (r > 0.0f) {
        r = sqrtf(r);
        kappa = r2k_f(r);
        kappa = kappa < VMF_MIN_KAPPA ? 0.0f : kappa;
        em2k = expf(-2.0f * kappa);
        norm = (float)((double)kappa / (2.0 * 3.14159265358979323846 * (double)(1.0f - em2k)));
        mx /= r, my /= r, mz /= r;
    } else {
        mx = s->mu_x[a], my = s->mu_y[a], mz = s->mu_z[a];
    }
    out[0] = w, out[1] = mx, out[2] = my, out[3] = mz, out[4] = kappa, out[5] = r, out[6] = norm, out[7] = em2k;
}

/* computePearsonChiSquaredMergeMetric for the pair a < b */
static float merge_metric(const pg_region_state *s, int a, int b) {
    const lobe_t ci = lobe_of(s, a), cj = lobe_of(s, b);
    lobe_t si = ci, sj = cj, pij = ci;
    vmf_combine(&si, &ci, 1);
    vmf_combine(&sj, &cj, 1);
    vmf_combine(&pij, &cj, 1);
    float m[8];
    merge_lobes(s, a, b, m);
    const lobe_t mg = {m[0], m[1], m[2], m[3], m[4], m[6]};
    const float q1 = vmf_combine(&si, &mg, -1), q2 = vmf_combine(&pij, &mg, -1), q3 = vmf_combine(&sj, &mg, -1);
    return ((q1 + 2.0f * q2) + q3) - mg.w;
}

/* lightpmm::coordinateAxis (pmm-glm.h:107-117); its unqualified sqrt is the
 * double one: 1/length in double, rounded to float */
static void coordinate_axis(const float z[3], float x[3], float y[3]) {
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

/* VMFKernel::swapComponent across kernels */
static void swap_lanes(pg_region_state *s, int i, int j) {
    float *f[8] = {s->weight, s->mu_x, s->mu_y, s->mu_z, s->kappa, s->r, s->norm, s->e_min2k};
    for (int q = 0; q < 8; ++q) {
        const float t = f[q][i];
        f[q][i] = f[q][j];
        f[q][j] = t;
    }
}

/* PathGuiding::mergeComponents (:762-781): statistics first, then the
 * mixture (a takes the merge, b is reset and swapped with the last) */
static void merge_pair(pg_region_state *s, pg_region_extra *x, int a, int b) {
    const float wa = s->weight[a], wb = s->weight[b], mw = wa + wb;
    const int last = (int)s->k - 1;
    /* incrementaldistance.h:165-204 */
    {
        const float msw = mw / (wa / s->dist_sum_w[a] + wb / s->dist_sum_w[b]);
        const float md = mw / (wa / s->distance[a] + wb / s->distance[b]);
        s->distance[a] = md;
        s->dist_sum_w[a] = msw;
        if (b != last) {
            s->distance[b] = s->distance[last];
            s->dist_sum_w[b] = s->dist_sum_w[last];
        }
    }
    const float inv = 1.0f / mw;
    /* incrementalpearsonchisquared.h:176-204 */
    if (!isinf(inv)) {
        const float sa = wa * inv, sb = wb * inv;
        const float d = sa * x->chi2_div[a] + sb * x->chi2_div[b];
        const float n = sa * x->chi2_n[a] + sb * x->chi2_n[b];
        x->chi2_div[a] = d;
        x->chi2_n[a] = n;
    } else {
        x->chi2_div[a] = 0.0f;
        x->chi2_n[a] = 0.0f;
    }
    if (b != last) {
        x->chi2_div[b] = x->chi2_div[last];
        x->chi2_n[b] = x->chi2_n[last];
    }
    /* incrementalcovariance2d.h:200-247; the merged mean is scaled by 1/3,
     * what the reference's glm::vec3::length() (the component count) gives */
    if (!isinf(inv)) {
        float mu[3] = {wa * s->mu_x[a] + wb * s->mu_x[b], wa * s->mu_y[a] + wb * s->mu_y[b],
                       wa * s->mu_z[a] + wb * s->mu_z[b]};
        const float sc = 1.0f / 3.0f;
        for (int i = 0; i < 3; ++i) mu[i] *= sc;
        float fx[3], fy[3];
        coordinate_axis(mu, fx, fy);
        const float ax = (s->mu_x[a] * fx[0] + s->mu_y[a] * fx[1]) + s->mu_z[a] * fx[2];
        const float ay = (s->mu_x[a] * fy[0] + s->mu_y[a] * fy[1]) + s->mu_z[a] * fy[2];
        const float bx = (s->mu_x[b] * fx[0] + s->mu_y[b] * fx[1]) + s->mu_z[b] * fx[2];
        const float by = (s->mu_x[b] * fy[0] + s->mu_y[b] * fy[1]) + s->mu_z[b] * fy[2];
        const float msw = x->cov_w[a] + x->cov_w[b];
        const float f = wa * wb / mw;
        const float dx = ax - bx, dy = ay - by;
        const float dv[3] = {dx * dx, dy * dy, dx * dy};
        for (int i = 0; i < 3; ++i) x->cov[a][i] = ((wa * x->cov[a][i] + wb * x->cov[b][i]) + f * dv[i]) * inv;
        x->cov_w[a] = msw;
    } else {
        x->cov[a][0] = x->cov[a][1] = x->cov[a][2] = 0.0f;
        x->cov_w[a] = 0.0f;
    }
    if (b != last) {
        for (int i = 0; i < 3; ++i) x->cov[b][i] = x->cov[last][i];
        x->cov_w[b] = x->cov_w[last];
    }
    /* the mixture */
    float m[8];
    merge_lobes(s, a, b, m);
    s->weight[a] = m[0], s->mu_x[a] = m[1], s->mu_y[a] = m[2], s->mu_z[a] = m[3];
    s->kappa[a] = m[4], s->r[a] = m[5], s->norm[a] = m[6], s->e_min2k[a] = m[7];
    reset_lane(s, b);
    s->k -= 1;
    if (b != (int)s->k) swap_lanes(s, b, (int)s->k);
}

/* libstdc++'s two-ended std::partition over keys with one or two payloads */
static int partition_keys(float *key, int *pa, int *pb, int n, float thr, int keep_le) {
    int first = 0, last = n;
#define PRED(v) (keep_le ? ((v) <= thr) : ((v) >= thr))
    for (;;) {
        for (;;) {
            if (first == last) return first;
            if (PRED(key[first])) ++first;
            else break;
        }
        --last;
        for (;;) {
            if (first == last) return first;
            if (!PRED(key[last])) --last;
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
#undef PRED
}

/* PathGuiding::mergeAll (:635-707), prior removed */
static void merge_all(pg_region_state *s, pg_region_extra *x, const pg_split_merge_config *sm) {
    for (;;) {
        const int n = (int)s->k;
        if (n <= 1) return;
        float key[SM_KM * (SM_KM - 1) / 2];
        int ca[SM_KM * (SM_KM - 1) / 2], cb[SM_KM * (SM_KM - 1) / 2];
        int idx = 0;
        for (int a = 0; a < n; ++a)
            for (int b = a + 1; b < n; ++b, ++idx) {
                key[idx] = merge_metric(s, a, b);
                ca[idx] = a;
                cb[idx] = b;
            }
        const int end = partition_keys(key, ca, cb, idx, sm->merge_max_divergence, 1);
        for (int i = 1; i < end; ++i) { /* ascending by metric */
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
        int ma[SM_KM], mb[SM_KM], nm = 0;
        for (int i = 0; i < end; ++i) {
            const int a = ca[i] < cb[i] ? ca[i] : cb[i], b = ca[i] < cb[i] ? cb[i] : ca[i];
            if (((used >> a) & 1u) || ((used >> b) & 1u)) continue;
            ma[nm] = a, mb[nm] = b, ++nm;
            used |= (1u << a) | (1u << b);
        }
        if (nm == 0) return;
        for (int i = 1; i < nm; ++i) { /* by second index, descending */
            const int a = ma[i], b = mb[i];
            int j = i - 1;
            while (j >= 0 && mb[j] < b) {
                ma[j + 1] = ma[j], mb[j + 1] = mb[j];
                --j;
            }
            ma[j + 1] = a, mb[j + 1] = b;
        }
        for (int i = 0; i < nm; ++i) merge_pair(s, x, ma[i], mb[i]);
    }
}

/* The larger eigenvalue of the symmetric 2x2 [[a, b], [b, c]] and its unit
 * eigenvector, in closed form */
static void principal_axis(float a, float b, float c, float *lambda, float *vx, float *vy) {
    const float h = 0.5f * (a - c);
    const float d = sqrtf(h * h + b * b);
    *lambda = 0.5f * (a + c) + d;
    if (b == 0.0f) {
        *vx = a >= c ? 1.0f : 0.0f;
        *vy = a >= c ? 0.0f : 1.0f;
        return;
    }
    float x, y;
    if (a >= c) {
        x = *lambda - c;
        y = b;
    } else {
        x = b;
        y = *lambda - a;
    }
    const float inv = 1.0f / sqrtf(x * x + y * y);
    *vx = x * inv;
    *vy = y * inv;
}

/* splitComponentUsingPCA (:494-561) */
static void split_component(pg_region_state *s, pg_region_extra *x, int c, float max_kappa) {
    if (s->k == SM_KM) return;
    const int dst = (int)s->k;
    const float z3[3] = {s->mu_x[c], s->mu_y[c], s->mu_z[c]};
    float fx[3], fy[3];
    coordinate_axis(z3, fx, fy);
    const int has = x->cov_w[c] > 0.0f;
    const float va = has ? x->cov[c][0] : 0.0f, vb = has ? x->cov[c][2] : 0.0f, vc = has ? x->cov[c][1] : 0.0f;
    float lambda, px, py;
    principal_axis(va, vb, vc, &lambda, &px, &py);
    const float hv = 0.5f * sqrtf(lambda);
    const float off = (hv < 1.0f) ? hv : 1.0f;
    px *= off;
    py *= off;
    const float z = sqrtf(1.0f - off * off);
    float ma[3], mbv[3];
    for (int i = 0; i < 3; ++i) {
        ma[i] = (px * fx[i] + py * fy[i]) + z * z3[i];
        mbv[i] = (-px * fx[i] + -py * fy[i]) + z * z3[i];
    }
    set_k(s, (uint32_t)dst + 1);
    const float src_r = s->r[c], src_w = s->weight[c];
    const float split_w = src_w * 0.5f;
    const float max_r = k2r_scalar(max_kappa);
    float split_r = max_r;
    if (z > 0.0f) {
        const float q = src_r / z;
        split_r = (q < max_r) ? q : max_r;
    }
    const float split_k = r2k_f(split_r);
    set_kappa_r_lane(s, c, split_k, split_r);
    s->mu_x[c] = ma[0], s->mu_y[c] = ma[1], s->mu_z[c] = ma[2];
    s->weight[c] = split_w;
    set_kappa_r_lane(s, dst, split_k, split_r);
    s->mu_x[dst] = mbv[0], s->mu_y[dst] = mbv[1], s->mu_z[dst] = mbv[2];
    s->weight[dst] = split_w;
    s->distance[dst] = s->distance[c];
    const float hw = 0.5f * s->dist_sum_w[c];
    s->dist_sum_w[c] = hw;
    s->dist_sum_w[dst] = hw;
    x->chi2_div[c] = x->chi2_div[dst] = 0.0f;
    x->chi2_n[c] = x->chi2_n[dst] = 0.0f;
    for (int i = 0; i < 3; ++i) x->cov[c][i] = x->cov[dst][i] = 0.0f;
    x->cov_w[c] = x->cov_w[dst] = 0.0f;
}

/* splitAll (:563-633), iterative, prior removed on entry and exit */
static void split_all(const pg_fit_config *cfg, const pg_split_merge_config *sm, pg_region_state *s,
                      pg_region_extra *x, const float *dirw, const float *pdf, uint32_t b, uint32_t e, int fit) {
    if (s->k >= SM_KM) return;
    const int first = (uint64_t)(e - b) == s->total_num_samples;
    for (;;) {
        const int K = (int)s->k;
        const float ia = (s->num_samples * s->num_samples) / (s->sample_weight * s->sample_weight);
        float key[SM_KM];
        int cand[SM_KM];
        for (int c = 0; c < K; ++c) {
            const float div = x->chi2_div[c] * ia - 1.0f;
            const int enough = x->chi2_n[c] > (float)sm->min_samples_for_splitting;
            key[c] = fabsf((first || enough) ? div * s->weight[c] : 0.0f);
            cand[c] = c;
        }
        const int nc = partition_keys(key, cand, NULL, K, sm->split_min_divergence, 0);
        const int room = SM_KM - K;
        const int ns = nc < room ? nc : room;
        if (ns == 0) break;
        if (nc > ns)
            for (int i = 1; i < nc; ++i) { /* the ns largest first, descending */
                const float k = key[i];
                const int c = cand[i];
                int j = i - 1;
                while (j >= 0 && key[j] < k) {
                    key[j + 1] = key[j], cand[j + 1] = cand[j];
                    --j;
                }
                key[j + 1] = k, cand[j + 1] = c;
            }
        uint32_t mask = 0;
        for (int i = 0; i < ns; ++i) {
            mask |= 1u << cand[i];
            mask |= 1u << s->k;
            split_component(s, x, cand[i], cfg->max_kappa);
        }
        if (fit) {
            pmm_apply_prior(s, cfg->v_prior);
            masked_fit32(cfg, s, dirw, b, e, mask, &x->em_iterations);
            chi2_update(s, x, dirw, pdf, b, e, mask);
            cov_update(s, x, dirw, b, e, mask);
            x->stat_passes += 1;
            pmm_remove_prior(s, cfg->v_prior);
        }
    }
}

static void postfit_region32(const pg_fit_config *cfg, const pg_split_merge_config *sm, const float *dirw,
                             const float *pdf, uint32_t b, uint32_t e, pg_region_state *s, pg_region_extra *x) {
    if (e == b) return;
    x->stat_passes = 0;
    x->em_iterations = 0;
    x->samples_since_merge += (float)(e - b);
    if (x->samples_since_merge > (float)sm->min_samples_for_merging) {
        pmm_remove_prior(s, cfg->v_prior);
        merge_all(s, x, sm);
        pmm_apply_prior(s, cfg->v_prior);
        x->samples_since_merge = 0.0f;
    }
    chi2_update(s, x, dirw, pdf, b, e, 0xFFFFu);
    cov_update(s, x, dirw, b, e, 0xFFFFu);
    x->stat_passes += 1;
    const int first = (uint64_t)(e - b) == s->total_num_samples;
    const int fit = first || (e - b) > sm->min_samples_for_post_split_fitting;
    pmm_remove_prior(s, cfg->v_prior);
    split_all(cfg, sm, s, x, dirw, pdf, b, e, fit);
    pmm_apply_prior(s, cfg->v_prior);
}

typedef struct {
    const pg_fit_config *cfg;
    const pg_split_merge_config *sm;
    uint32_t n_regions;
    const float *dirw, *pdf;
    const uint32_t *offsets;
    pg_region_state *states;
    pg_region_extra *extras;
    uint32_t next; /* atomic */
} postfit_job_t;

static void *postfit_worker(void *arg) {
    postfit_job_t *j = (postfit_job_t *)arg;
    for (;;) {
        const uint32_t r = __atomic_fetch_add(&j->next, 1u, __ATOMIC_RELAXED);
        if (r >= j->n_regions) break;
        postfit_region32(j->cfg, j->sm, j->dirw, j->pdf, j->offsets[r], j->offsets[r + 1], &j->states[r],
                         &j->extras[r]);
    }
    return NULL;
}

int pgo_postfit_lpmm32(const pg_fit_config *cfg, const pg_split_merge_config *sm, uint32_t n_regions,
                       const float *dirw, const float *pdf, const uint32_t *offsets, pg_region_state *states,
                       pg_region_extra *extras, int n_threads) {
    postfit_job_t j = {cfg, sm, n_regions, dirw, pdf, offsets, states, extras, 0};
    if (n_threads <= 1) {
        postfit_worker(&j);
        return 0;
    }
    if (n_threads > 256) n_threads = 256;
    pthread_t th[256];
    int started = 0;
    for (int t = 0; t < n_threads; ++t)
        if (pthread_create(&th[t], NULL, postfit_worker, &j) == 0) ++started;
    if (started == 0) postfit_worker(&j);
    for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Region splitting (PathGuiding::update's split check, splitRegion)   */
/* ------------------------------------------------------------------ */

/* src/PathGuiding.cpp:290-348 with Aabb::splitAabb (src/Shapes.h:32-46):
 * regions [0, n) in order; one whose m_numSamples exceeds `thr` keeps the
 * lower half of its box, the upper half becomes the next new region, both
 * with the mixture (and statistics) whose sample count and weight were
 * multiplied by 0.25.  The tree: node v >= 0 has children v, v + 1; a node
 * < 0 is the leaf of region -v - 1; leaf_of maps regions to their leaves.
 * Stops creating regions at `cap`.  Returns the new region count. */
uint32_t pgo_split_regions(uint32_t n, uint32_t cap, float thr, pg_region_state *states, pg_region_extra *extras,
                           float *aabbs, int32_t *nodes, uint32_t *leaf_of, uint32_t *n_nodes) {
    uint32_t count = n;
    for (uint32_t r = 0; r < n; ++r) {
        if (!(states[r].num_samples > thr) || count >= cap) continue;
        const uint32_t nr = count++;
        pg_region_state *st = &states[r];
        st->num_samples = st->num_samples * 0.25f;
        st->sample_weight = st->sample_weight * 0.25f;
        states[nr] = *st;
        if (extras) extras[nr] = extras[r];
        float *b = aabbs + 6 * (size_t)r, *c = aabbs + 6 * (size_t)nr;
        float size[3];
        for (int i = 0; i < 3; ++i) size[i] = b[3 + i] - b[i];
        const int ax = size[0] > size[1] ? (size[0] > size[2] ? 0 : 2) : (size[1] > size[2] ? 1 : 2);
        for (int i = 0; i < 6; ++i) c[i] = b[i];
        b[3 + ax] -= 0.5f * size[ax];
        c[ax] += 0.5f * size[ax];
        const uint32_t a = *n_nodes;
        *n_nodes += 2;
        nodes[leaf_of[r]] = (int32_t)a;
        nodes[a] = -(int32_t)r - 1;
        nodes[a + 1] = -(int32_t)nr - 1;
        leaf_of[r] = a;
        leaf_of[nr] = a + 1;
    }
    return count;
}

/* Point -> region by descending the tree from the padded scene box (the
 * region boxes' midpoint rule); PG_INVALID_REGION outside it or in a rounding
 * gap between halves. */
uint32_t pgo_region_of(const float root[6], const int32_t *nodes, const float p[3]) {
    float lo[3] = {root[0], root[1], root[2]}, hi[3] = {root[3], root[4], root[5]};
    for (int i = 0; i < 3; ++i)
        if (!(p[i] >= lo[i] && p[i] <= hi[i])) return PG_INVALID_REGION;
    int32_t node = 0;
    for (int depth = 0; depth < 64; ++depth) {
        const int32_t v = nodes[node];
        if (v < 0) return (uint32_t)(-(v + 1));
        float size[3];
        for (int i = 0; i < 3; ++i) size[i] = hi[i] - lo[i];
        const int ax = size[0] > size[1] ? (size[0] > size[2] ? 0 : 2) : (size[1] > size[2] ? 1 : 2);
        const float lhi = hi[ax] - 0.5f * size[ax];
        const float rlo = lo[ax] + 0.5f * size[ax];
        if (p[ax] <= lhi) {
            hi[ax] = lhi;
            node = v;
        } else if (p[ax] >= rlo) {
            lo[ax] = rlo;
            node = v + 1;
        } else {
            return PG_INVALID_REGION;
        }
    }
    return PG_INVALID_REGION;
}
