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
// distance update (postFit, :445-448).  Split/merge is not part of this path.
#include <cstdint>
#include <cstring>
#include <limits>
#include <sstream>
#include <vector>

#include "pmm/DirectionalData.h"
#include "pmm/ParametricMixtureModel.h"
#include "pmm/VMFKernel.h"
#include "pmm/VMMFactory.h"
#include "guiding/incrementaldistance.h"
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

}  // namespace

extern "C" {

// Initialises `n` states as PathGuiding::createPMMs does (src/PathGuiding.cpp:42-51).
int lpmm_ref_init(const pg_fit_config *cfg, uint32_t n, pg_region_state *states) {
    Factory factory(props_from(cfg));
    for (uint32_t r = 0; r < n; ++r) {
        PMM pmm;
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

// Fits each region with the reference's VMMFactory.  `dirw` holds float4
// {dir.xyz, weight} per sample grouped by region (offsets[n_regions+1]).
// mode: PG_FIT_INIT / PG_FIT_CONTINUE / PG_FIT_UPDATE.  ll_final[r] receives
// the weighted log-likelihood of the fitted mixture over the region's samples,
// computed by VMMFactory::computeSufficentStatsFromSamples (VMMFactory.h:497-536).
int lpmm_ref_fit(const pg_fit_config *cfg, int mode, uint32_t n_regions, const float *dirw,
                 const uint32_t *offsets, pg_region_state *states, float *ll_final) {
    Factory factory(props_from(cfg));
    std::vector<DData> data;
    for (uint32_t r = 0; r < n_regions; ++r) {
        const uint32_t b = offsets[r], e = offsets[r + 1];
        data.resize(e - b);
        for (uint32_t i = b; i < e; ++i) {
            const float *p = dirw + 4 * size_t(i);
            data[i - b] = DData(lightpmm::Point3(0.f, 0.f, 0.f), lightpmm::Vector3(p[0], p[1], p[2]),
                                p[3], 1.0f, 1.0f, r);
        }
        PMM pmm;
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
        PMM pmm;
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
    PMM pmm;
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
