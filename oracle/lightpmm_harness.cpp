// lightpmm_harness.cpp - TEST INFRASTRUCTURE (oracle), never shipped or measured
// as the product.
//
// Compiles the reference's own vendored lightpmm fit (external/lightpmm/include/pmm)
// and its parallax-distance statistics (external/guiding/incrementaldistance.h)
// where they lie in the reference tree, and exposes them through a C entry point
// that speaks the pg_region_state layout of include/pathguide.h.  The build
// recipe is oracle/build_oracle.py; the output goes to oracle/_ref/ only.
//
// The per-region flow restates PathGuiding::updateRegion
// (src/PathGuiding.cpp:350-368): optional parallax pre-pass (preFit, :370-411),
// VMMFactory::fit / updateFit (VMMFactory.h:157-216, 305-362), then the parallax
// distance update (postFit, :445-448).  lpmm_ref_postfit adds the split/merge
// part of postFit (:413-451) restated from src/PathGuiding.cpp:494-781 around
// the reference's own IncrementalPearsonChiSquared, IncrementalCovariance2D,
// IncrementalDistance and VMMFactory::maskedFit; the one substitution is the
// 2x2 eigen decomposition of the PCA split (the reference calls Eigen, which is
// not vendored): the principal eigenvector of the symmetric covariance in
// closed form.
#include <algorithm>
#include <atomic>
#include <thread>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <sstream>
#include <vector>

#include "pmm/DirectionalData.h"
#include "pmm/ParametricMixtureModel.h"
#include "pmm/VMFKernel.h"
#include "pmm/VMMFactory.h"
// incrementaldistance.h declares the Vector alias incrementalcovariance2d.h uses
#include "guiding/incrementaldistance.h"
#include "guiding/incrementalcovariance2d.h"
#include "guiding/incrementalpearsonchisquared.h"
#include "guiding/Range.h"

#include "pathguide.h"

namespace {

using Scalar = lightpmm::Scalar4;
using VMF = lightpmm::VMFKernel<Scalar>;
using PMM = lightpmm::ParametricMixtureModel<VMF, 4>;
using Factory = lightpmm::VMMFactory<PMM>;
using DData = lightpmm::DirectionalData;

lightpmm::VMMFactoryProperties props_from(const pg_fit_config *c) {
    lightpmm::VMMFactoryProperties p;
    p.minItr = c->min_itr;
    p.maxItr = c->max_itr;
    p.relLogLikelihoodThreshold = c->rel_ll_threshold;
    p.numInitialComponents = c->num_initial_components;
    p.initKappa = c->init_kappa;
    p.maxKappa = c->max_kappa;
    p.vPrior = c->v_prior;
    p.rPrior = c->r_prior;
    p.rPriorWeight = c->r_prior_weight;
    return p;
}

// VMFKernel keeps kappa/r/norm/eMin2Kappa private; its public binary
// serialize/deserialize (VMFKernel.h:590-600) is the documented way in and out.
struct KernelBytes {
    alignas(16) float w[4];
    alignas(16) float mx[4];
    alignas(16) float my[4];
    alignas(16) float mz[4];
    alignas(16) float kappa[4];
    alignas(16) float r[4];
    alignas(16) float norm[4];
    alignas(16) float em2k[4];
};
static_assert(sizeof(KernelBytes) == sizeof(VMF), "VMFKernel<Scalar4> layout");

void state_to_pmm(const pg_region_state &s, PMM &pmm) {
    pmm.m_K = s.k;
    pmm.m_sampleWeight = s.sample_weight;
    pmm.m_numSamples = s.num_samples;
    pmm.m_totalNumSamples = s.total_num_samples;
    pmm.m_numEMIterations = s.num_em_iterations;
    for (int k = 0; k < 4; ++k) {
        KernelBytes b;
        for (int i = 0; i < 4; ++i) {
            const int c = 4 * k + i;
            b.w[i] = s.weight[c];
            b.mx[i] = s.mu_x[c];
            b.my[i] = s.mu_y[c];
            b.mz[i] = s.mu_z[c];
            b.kappa[i] = s.kappa[c];
            b.r[i] = s.r[c];
            b.norm[i] = s.norm[c];
            b.em2k[i] = s.e_min2k[c];
        }
        std::string bytes(reinterpret_cast<const char *>(&b), sizeof(b));
        std::istringstream in(bytes);
        pmm.m_comps[k].deserialize(in);
    }
}

void pmm_to_state(const PMM &pmm, pg_region_state &s) {
    s.k = pmm.m_K;
    s.sample_weight = pmm.m_sampleWeight;
    s.num_samples = pmm.m_numSamples;
    s.total_num_samples = pmm.m_totalNumSamples;
    s.num_em_iterations = pmm.m_numEMIterations;
    for (int k = 0; k < 4; ++k) {
        std::ostringstream out;
        pmm.m_comps[k].serialize(out);
        const std::string bytes = out.str();
        KernelBytes b;
        std::memcpy(&b, bytes.data(), sizeof(b));
        for (int i = 0; i < 4; ++i) {
            const int c = 4 * k + i;
            s.weight[c] = b.w[i];
            s.mu_x[c] = b.mx[i];
            s.mu_y[c] = b.my[i];
            s.mu_z[c] = b.mz[i];
            s.kappa[c] = b.kappa[i];
            s.r[c] = b.r[i];
            s.norm[c] = b.norm[i];
            s.e_min2k[c] = b.em2k[i];
        }
    }
}

using IDist = guiding::IncrementalDistance<PMM>;

void state_to_dist(const pg_region_state &s, IDist &d) {
    for (int k = 0; k < 4; ++k)
        for (int i = 0; i < 4; ++i) {
            d.distances[k].insert(i, s.distance[4 * k + i]);
            d.sumWeights[k].insert(i, s.dist_sum_w[4 * k + i]);
        }
}

void dist_to_state(const IDist &d, pg_region_state &s) {
    for (int k = 0; k < 4; ++k)
        for (int i = 0; i < 4; ++i) {
            s.distance[4 * k + i] = d.distances[k][i];
            s.dist_sum_w[4 * k + i] = d.sumWeights[k][i];
        }
}

using IChi = guiding::IncrementalPearsonChiSquared<PMM>;
using ICov = guiding::IncrementalCovariance2D<PMM>;
using Samples = guiding::Range<std::vector<DData>>;

struct Extra {
    IDist dist;
    IChi chi;
    ICov cov;
    float since_merge = 0.0f;
};

void extra_in(const pg_region_state &s, const pg_region_extra &e, Extra &x) {
    state_to_dist(s, x.dist);
    for (int k = 0; k < 4; ++k)
        for (int i = 0; i < 4; ++i) {
            const int c = 4 * k + i;
            x.chi.divergencePlusOneTimesIntegralSqr[k].insert(i, e.chi2_div[c]);
            x.chi.numSamples[k].insert(i, e.chi2_n[c]);
            x.cov.varianceAndCovariance[k].x.insert(i, e.cov[c][0]);
            x.cov.varianceAndCovariance[k].y.insert(i, e.cov[c][1]);
            x.cov.varianceAndCovariance[k].z.insert(i, e.cov[c][2]);
            x.cov.sumWeights[k].insert(i, e.cov_w[c]);
        }
    x.since_merge = e.samples_since_merge;
}

void extra_out(const Extra &x, pg_region_state &s, pg_region_extra &e) {
    dist_to_state(x.dist, s);
    for (int k = 0; k < 4; ++k)
        for (int i = 0; i < 4; ++i) {
            const int c = 4 * k + i;
            e.chi2_div[c] = x.chi.divergencePlusOneTimesIntegralSqr[k][i];
            e.chi2_n[c] = x.chi.numSamples[k][i];
            e.cov[c][0] = x.cov.varianceAndCovariance[k].x[i];
            e.cov[c][1] = x.cov.varianceAndCovariance[k].y[i];
            e.cov[c][2] = x.cov.varianceAndCovariance[k].z[i];
            e.cov_w[c] = x.cov.sumWeights[k][i];
        }
    e.samples_since_merge = x.since_merge;
}

// std::partition as libstdc++ implements it for random-access ranges (the
// order of the kept elements decides the order of splits and merges).
template <typename It, typename P>
It hoare_partition(It first, It last, P pred) {
    while (true) {
        while (true) {
            if (first == last) return first;
            if (pred(*first)) ++first;
            else break;
        }
        --last;
        while (true) {
            if (first == last) return first;
            if (!pred(*last)) --last;
            else break;
        }
        std::iter_swap(first, last);
        ++first;
    }
}

// Principal axis of the symmetric 2x2 covariance [[a, b], [b, c]]: the
// larger eigenvalue and its unit eigenvector (closed form; stands in for the
// Eigen call of src/PathGuiding.cpp:454-484).
void principal_axis(float a, float b, float c, float &lambda, float &vx, float &vy) {
    const float h = 0.5f * (a - c);
    const float d = std::sqrt(h * h + b * b);
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
    const float inv = 1.0f / std::sqrt(vx * vx + vy * vy);
    vx *= inv;
    vy *= inv;
}

// splitComponentUsingPCA (src/PathGuiding.cpp:494-561)
void split_component(Extra &st, PMM &pmm, uint32_t component, float max_kappa) {
    if (pmm.getK() == PMM::MaxK::value) return;
    const uint32_t src = component, dst = pmm.getK();
    VMF &sc = pmm.getComponent(src / 4);
    VMF &tc = pmm.getComponent(dst / 4);
    const lightpmm::Frame frame{sc.getMu(src % 4)};
    const lightpmm::Matrix2x2 cov = st.cov.computeCovarianceMatrix(component);
    float lambda, px, py;
    principal_axis(cov[0][0], cov[0][1], cov[1][1], lambda, px, py);
    const float off = std::min(1.0f, 0.5f * std::sqrt(lambda));
    px *= off;
    py *= off;
    const float z = std::sqrt(1.0f - off * off);
    const lightpmm::Vector3 muA{frame.toWorld({px, py, z})};
    const lightpmm::Vector3 muB{frame.toWorld({-px, -py, z})};
    pmm.setK(dst + 1);
    const float src_r = sc.getR()[src % 4];
    const float src_w = sc.getWeight(src % 4);
    const float split_w = src_w * 0.5f;
    const float max_r = lightpmm::kappaToMeanCosine(max_kappa);
    const float split_r = (z > 0.0f) ? std::min(max_r, src_r / z) : max_r;
    const float split_k = lightpmm::meanCosineToKappa(split_r);
    sc.setKappaAndR(src % 4, split_k, split_r);
    sc.setMu(src % 4, muA);
    sc.setWeight(src % 4, split_w);
    tc.setKappaAndR(dst % 4, split_k, split_r);
    tc.setMu(dst % 4, muB);
    tc.setWeight(dst % 4, split_w);
    st.dist.split(pmm, component);
    st.chi.split(pmm, component);
    st.cov.split(pmm, component);
}

// splitAll (src/PathGuiding.cpp:563-633)
uint32_t split_all(Extra &st, PMM &pmm, const Samples &samples, bool iterative, bool fit, const Factory &factory,
                   const lightpmm::VMMFactoryProperties &props, const pg_split_merge_config &sm) {
    if (pmm.getK() >= PMM::MaxK::value) return 0;
    const bool first_fit = samples.size() == pmm.m_totalNumSamples;
    uint32_t total = 0, num = 0;
    do {
        const uint32_t nk = (pmm.getK() + 3) / 4;
        const std::array<Scalar, PMM::NumKernels::value> div = st.chi.computeDivergence(pmm);
        std::array<std::pair<float, uint32_t>, PMM::MaxK::value> cand;
        for (uint32_t k = 0; k < nk; ++k) {
            const auto enough = st.chi.numSamples[k] > (float)sm.min_samples_for_splitting;
            const Scalar wd = lightpmm::ifthen(first_fit || enough, div[k] * pmm.getComponent(k).m_weights, 0.0f);
            for (uint32_t i = 0; i < 4; ++i) cand[k * 4 + i] = std::make_pair(std::fabs(wd[i]), k * 4 + i);
        }
        const auto last = hoare_partition(cand.begin(), cand.begin() + pmm.getK(),
                                          [&](const std::pair<float, uint32_t> &x) {
                                              return x.first >= sm.split_min_divergence;
                                          });
        const uint32_t n_cand = (uint32_t)std::distance(cand.begin(), last);
        const uint32_t max_splits = PMM::MaxK::value - pmm.getK();
        num = std::min(n_cand, max_splits);
        if (num == 0) break;
        if (n_cand > num)
            std::partial_sort(cand.begin(), cand.begin() + num, last,
                              [](const std::pair<float, uint32_t> a, const std::pair<float, uint32_t> b) {
                                  return a.first > b.first;
                              });
        std::array<Scalar::BooleanType, PMM::NumKernels::value> mask;
        std::fill(mask.begin(), mask.end(), Scalar::BooleanType{false});
        for (uint32_t i = 0; i < num; ++i) {
            mask[cand[i].second / 4].insert(cand[i].second % 4, true);
            mask[pmm.getK() / 4].insert(pmm.getK() % 4, true);
            split_component(st, pmm, cand[i].second, props.maxKappa);
        }
        if (fit) {
            pmm.applyWeightPrior(props.vPrior);
            factory.maskedFit(samples.begin(), samples.end(), pmm, mask);
            st.chi.updateDivergenceMasked(pmm, samples, mask);
            st.cov.updateStatisticsMasked(pmm, samples, mask);
            pmm.removeWeightPrior(props.vPrior);
        }
        total += num;
    } while (iterative);
    return total;
}

// computePearsonChiSquaredMergeMetric (src/PathGuiding.cpp:709-760)
std::array<float, PMM::MaxK::value *(PMM::MaxK::value - 1) / 2> merge_metric(const PMM &d) {
    const uint32_t n = d.getK();
    const uint32_t nk = (n + 3) / 4;
    std::array<VMF, PMM::NumKernels::value> self;
    for (uint32_t k = 0; k < nk; ++k) {
        self[k] = d.getComponent(k);
        self[k].product(self[k]);
    }
    std::array<Scalar, PMM::NumKernels::value * PMM::MaxK::value> vals;
    for (uint32_t i = 0; i + 1 < n; ++i) {
        const VMF ci = d.getComponent(i / 4).extract(i % 4);
        const VMF ci2 = self[i / 4].extract(i % 4);
        for (uint32_t j = (i + 1) / 4; j < nk; ++j) {
            VMF pij{ci};
            pij.product(d.getComponent(j));
            const VMF kj{d.getComponent(j)};
            VMF merged{ci};
            {
                VMF kjm{kj};
                for (uint32_t l = 0; l < 4; ++l) merged.mergeComponent(l, l, kjm);
            }
            const Scalar q1 = VMF{ci2}.division(merged);
            const Scalar q2 = VMF{pij}.division(merged);
            const Scalar q3 = VMF{self[j]}.division(merged);
            vals[i * PMM::NumKernels::value + j] = q1 + 2.0f * q2 + q3 - merged.m_weights;
        }
    }
    std::array<float, PMM::MaxK::value *(PMM::MaxK::value - 1) / 2> out;
    uint32_t idx = 0;
    for (uint32_t i = 0; i + 1 < n; ++i)
        for (uint32_t j = i + 1; j < n; ++j, ++idx) out[idx] = vals[i * PMM::NumKernels::value + j / 4][j % 4];
    return out;
}

// mergeComponents (src/PathGuiding.cpp:762-781)
void merge_components(Extra &st, PMM &pmm, uint32_t a, uint32_t b) {
    st.dist.merge(pmm, a, b);
    st.chi.merge(pmm, a, b);
    st.cov.merge(pmm, a, b);
    pmm.mergeComponents(a, b);
}

// mergeAll (src/PathGuiding.cpp:635-707)
uint32_t merge_all(Extra &st, PMM &pmm, const pg_split_merge_config &sm) {
    uint32_t total = 0;
    while (true) {
        const uint32_t n = pmm.getK();
        uint32_t num = 0;
        if (n <= 1) return total;
        const uint32_t n_sim = n * (n - 1) / 2;
        const auto metric = merge_metric(pmm);
        std::array<std::pair<float, std::pair<uint32_t, uint32_t>>, PMM::MaxK::value *(PMM::MaxK::value - 1) / 2> cand;
        for (uint32_t a = 0, oa = 0; a < n; ++a, oa += n - a)
            for (uint32_t b = a + 1, ob = 0; b < n; ++b, ++ob) cand[oa + ob] = std::make_pair(metric[oa + ob], std::make_pair(a, b));
        const auto end = hoare_partition(cand.begin(), cand.begin() + n_sim, [&](const auto &c) {
            return c.first <= sm.merge_max_divergence;
        });
        std::sort(cand.begin(), end, [](const auto &x, const auto &y) { return x.first < y.first; });
        uint32_t used = 0;
        std::array<std::pair<uint32_t, uint32_t>, PMM::MaxK::value> merges;
        for (auto it = cand.begin(); it != end; ++it) {
            const uint32_t a = std::min(it->second.first, it->second.second);
            const uint32_t b = std::max(it->second.first, it->second.second);
            if ((used & (1u << a)) || (used & (1u << b))) continue;
            merges[num++] = std::make_pair(a, b);
            used |= (1u << a) | (1u << b);
        }
        if (num == 0) break;
        std::sort(merges.begin(), merges.begin() + num, [](const auto &x, const auto &y) { return x.second > y.second; });
        for (uint32_t i = 0; i < num; ++i) merge_components(st, pmm, merges[i].first, merges[i].second);
        total += num;
    }
    return total;
}

}  // namespace

extern "C" {

// PathGuiding::postFit (src/PathGuiding.cpp:413-451) of one region after its
// fit: merges (when enough samples were seen since the last merge), the
// divergence and covariance statistics, splits with masked refits, then the
// parallax distances.  dirw / pdf / dist: the region's samples after preFit.
int lpmm_ref_postfit(const pg_fit_config *cfg, const pg_split_merge_config *sm, uint32_t n, const float *dirw,
                     const float *pdf, const float *dist, pg_region_state *state, pg_region_extra *extra) {
    const lightpmm::VMMFactoryProperties props = props_from(cfg);
    Factory factory(props);
    std::vector<DData> data(n);
    for (uint32_t i = 0; i < n; ++i) {
        const float *p = dirw + 4 * size_t(i);
        data[i] = DData(lightpmm::Point3(0.f, 0.f, 0.f), lightpmm::Vector3(p[0], p[1], p[2]), p[3], pdf[i],
                        dist ? dist[i] : 0.0f, 0);
    }
    Samples range(data.begin(), data.end());
    PMM pmm{};
    state_to_pmm(*state, pmm);
    Extra st;
    extra_in(*state, *extra, st);
    if (sm->enabled) {
        st.since_merge += (float)n;
        if (st.since_merge > (float)sm->min_samples_for_merging) {
            pmm.removeWeightPrior(props.vPrior);
            merge_all(st, pmm, *sm);
            pmm.applyWeightPrior(props.vPrior);
            st.since_merge = 0.0f;
        }
        st.chi.updateDivergence(pmm, range);
        st.cov.updateStatistics(pmm, range);
        const bool first = n == pmm.m_totalNumSamples;
        const bool fit = first || n > sm->min_samples_for_post_split_fitting;
        pmm.removeWeightPrior(props.vPrior);
        split_all(st, pmm, range, true, fit, factory, props, *sm);
        pmm.applyWeightPrior(props.vPrior);
    }
    if (cfg->use_parallax && dist) st.dist.updateDistances(pmm, range);
    pmm_to_state(pmm, *state);
    extra_out(st, *state, *extra);
    return 0;
}

// Initialises `n` states as PathGuiding::createPMMs does (src/PathGuiding.cpp:42-51).
int lpmm_ref_init(const pg_fit_config *cfg, uint32_t n, pg_region_state *states) {
    Factory factory(props_from(cfg));
    for (uint32_t r = 0; r < n; ++r) {
        PMM pmm{};  // zeroed (the reference default-initialises it): components beyond K stay defined
        factory.initialize(pmm);
        pg_region_state &s = states[r];
        std::memset(&s, 0, sizeof(s));
        pmm_to_state(pmm, s);
        for (int c = 0; c < 16; ++c) {
            s.distance[c] = std::numeric_limits<float>::infinity();
            s.dist_sum_w[c] = 0.0f;
        }
    }
    return 0;
}

}  // extern "C"

namespace {
// One region of lpmm_ref_fit: the reference's VMMFactory::initialize / fit /
// updateFit on the region's samples.
void fit_region(Factory &factory, std::vector<DData> &data, const pg_fit_config *cfg, int mode, uint32_t r,
                const float *dirw, const uint32_t *offsets, pg_region_state *states, float *ll_final) {
    (void)cfg;
    const uint32_t b = offsets[r], e = offsets[r + 1];
    data.resize(e - b);
    for (uint32_t i = b; i < e; ++i) {
        const float *p = dirw + 4 * size_t(i);
        data[i - b] = DData(lightpmm::Point3(0.f, 0.f, 0.f), lightpmm::Vector3(p[0], p[1], p[2]), p[3], 1.0f, 1.0f,
                            r);
    }
    PMM pmm{};
    if (mode == PG_FIT_INIT) {
        factory.initialize(pmm);
    } else {
        state_to_pmm(states[r], pmm);
    }
    const uint32_t before = pmm.m_numEMIterations;
    if (e > b) {
        if (mode == PG_FIT_UPDATE)
            factory.updateFit(data.begin(), data.end(), pmm);
        else
            factory.fit(data.begin(), data.end(), pmm, false);
    }
    pg_region_state &s = states[r];
    if (mode == PG_FIT_INIT) {
        std::memset(&s, 0, sizeof(s));
        for (int c = 0; c < 16; ++c) s.distance[c] = std::numeric_limits<float>::infinity();
    }
    pmm_to_state(pmm, s);
    s.iters_last = pmm.m_numEMIterations - before;
    if (ll_final) {
        float ll = 0.0f;
        if (e > b) factory.computeSufficentStatsFromSamples(data.begin(), data.end(), pmm, nullptr, &ll);
        ll_final[r] = ll;
    }
}
}  // namespace

extern "C" {

// Fits each region with the reference's VMMFactory.  `dirw` holds float4
// {dir.xyz, weight} per sample grouped by region (offsets[n_regions+1]).
// mode: PG_FIT_INIT / PG_FIT_CONTINUE / PG_FIT_UPDATE.  ll_final[r] receives
// the weighted log-likelihood of the fitted mixture over the region's samples,
// computed by VMMFactory::computeSufficentStatsFromSamples (VMMFactory.h:497-536).
int lpmm_ref_fit(const pg_fit_config *cfg, int mode, uint32_t n_regions, const float *dirw,
                 const uint32_t *offsets, pg_region_state *states, float *ll_final) {
    Factory factory(props_from(cfg));
    std::vector<DData> data;
    for (uint32_t r = 0; r < n_regions; ++r) fit_region(factory, data, cfg, mode, r, dirw, offsets, states, ll_final);
    return 0;
}

// lpmm_ref_fit with the regions spread over n_threads host threads (each with
// its own factory), taking the next region from a shared counter - the
// reference's per-region fit run region-parallel, as a multi-core host would.
int lpmm_ref_fit_threads(const pg_fit_config *cfg, int mode, uint32_t n_regions, const float *dirw,
                         const uint32_t *offsets, pg_region_state *states, float *ll_final, int n_threads) {
    std::atomic<uint32_t> next{0};
    auto body = [&] {
        Factory factory(props_from(cfg));
        std::vector<DData> data;
        for (uint32_t r = next.fetch_add(1); r < n_regions; r = next.fetch_add(1))
            fit_region(factory, data, cfg, mode, r, dirw, offsets, states, ll_final);
    };
    const int T = std::max(1, n_threads);
    std::vector<std::thread> pool;
    for (int t = 1; t < T; ++t) pool.emplace_back(body);
    body();
    for (auto &th : pool) th.join();
    return 0;
}

// The reference's parallax distance update (IncrementalDistance::updateDistances,
// external/guiding/incrementaldistance.h:57-107) over one pass of samples; `dist`
// holds the per-sample (re-centred) distance.
int lpmm_ref_update_distances(uint32_t n_regions, const float *dirw, const float *dist,
                              const uint32_t *offsets, pg_region_state *states) {
    std::vector<DData> data;
    for (uint32_t r = 0; r < n_regions; ++r) {
        const uint32_t b = offsets[r], e = offsets[r + 1];
        data.resize(e - b);
        for (uint32_t i = b; i < e; ++i) {
            const float *p = dirw + 4 * size_t(i);
            data[i - b] = DData(lightpmm::Point3(0.f, 0.f, 0.f), lightpmm::Vector3(p[0], p[1], p[2]),
                                p[3], 1.0f, dist[i], r);
        }
        PMM pmm{};
        state_to_pmm(states[r], pmm);
        IDist d;
        state_to_dist(states[r], d);
        guiding::Range<std::vector<DData>> range(data.begin(), data.end());
        d.updateDistances(pmm, range);
        dist_to_state(d, states[r]);
    }
    return 0;
}

// IncrementalDistance::reposition (incrementaldistance.h:109-131) applied as
// PathGuiding::preFit does (src/PathGuiding.cpp:404-409).
int lpmm_ref_reposition(pg_region_state *s, const float new_to_old[3]) {
    PMM pmm{};
    state_to_pmm(*s, pmm);
    IDist d;
    state_to_dist(*s, d);
    d.reposition(pmm, lightpmm::Vector3(new_to_old[0], new_to_old[1], new_to_old[2]));
    pmm_to_state(pmm, *s);
    dist_to_state(d, *s);
    return 0;
}

// lightpmm's vectorised exp approximation (pmm-vcl.h:158-184), for measuring
// its error against exact exp when deriving tolerances.
void lpmm_ref_fastexp(const float *x, float *y, uint32_t n) {
    for (uint32_t i = 0; i < n; i += 4) {
        float in[4] = {0, 0, 0, 0};
        for (uint32_t j = 0; j < 4 && i + j < n; ++j) in[j] = x[i + j];
        lightpmm::float4 v;
        v.load(in);
        lightpmm::float4 o = lightpmm::exp(v);
        float out[4];
        o.store(out);
        for (uint32_t j = 0; j < 4 && i + j < n; ++j) y[i + j] = out[j];
    }
}

uint32_t lpmm_ref_state_size(void) { return sizeof(pg_region_state); }

}  // extern "C"
