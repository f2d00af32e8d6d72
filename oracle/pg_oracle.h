/*
 * pg_oracle.h - TEST INFRASTRUCTURE.  CPU restatements of the reference's
 * path-guiding arithmetic, used only by tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py, as the checker.  Nothing in the
 * product links or calls this library.
 *
 * Two restatements of the lightpmm MAP-EM fit (external/lightpmm/include/pmm/
 * VMMFactory.h:157-216, 305-362, 385-455, 497-555; VMFKernel.h:46-66, 103-112,
 * 620-628, 674-681; ParametricMixtureModel.h:501-522):
 *   - pgo_fit_lpmm32: FP32, the reference's own operation order, its
 *     fastexp/fasttanh approximations (pmm-vcl.h:158-222) and its 4-lane
 *     grouping.  This is the "port" of the reference CPU fit.
 *   - pgo_fit_f64: the same equations in double with exact exp/tanh; the
 *     tight parity target for the GPU fit.
 * Both use the pg_region_state layout of include/pathguide.h.
 */
#ifndef PG_ORACLE_H
#define PG_ORACLE_H

#include <stdint.h>

#include "pathguide.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Spherical Fibonacci initial means (VMMFactory.h:594-632), computed in double
 * and rounded to float; out has 3*16 floats (x[16], y[16], z[16]). */
void pgo_initial_mus(uint32_t num_components, float *out_xyz);

/* VMMFactory::initialize (VMMFactory.h:132-148) for n regions.  The r of the
 * initial lobes follows kappaToMeanCosine (VMFKernel.h:47-55); `exact` selects
 * exact tanh/exp (1) or lightpmm's fast approximations (0). */
void pgo_init_states(const pg_fit_config *cfg, uint32_t n, pg_region_state *states, int exact);

/* lightpmm-faithful FP32 fit of n_regions regions over `n_threads` host threads
 * (regions are independent).  ll_final (may be NULL) gets the weighted
 * log-likelihood of the fitted mixture over the region's samples. */
int pgo_fit_lpmm32(const pg_fit_config *cfg, int mode, uint32_t n_regions, const float *dirw,
                   const uint32_t *offsets, pg_region_state *states, float *ll_final,
                   int n_threads);

/* FP64 fit of the same equations (exact exp, tanh, log). */
int pgo_fit_f64(const pg_fit_config *cfg, int mode, uint32_t n_regions, const float *dirw,
                const uint32_t *offsets, pg_region_state *states, double *ll_final,
                int n_threads);

/* Weighted log-likelihood of each region's samples under its mixture, FP64. */
void pgo_eval_ll_f64(uint32_t n_regions, const float *dirw, const uint32_t *offsets,
                     const pg_region_state *states, double *ll_out);

/* PathGuiding::postFit with splitAndMerge (src/PathGuiding.cpp:413-451):
 * merges, divergence and covariance statistics, PCA splits with masked refits,
 * on lightpmm's FP32 4-lane arithmetic, for regions [0, n_regions) over
 * `n_threads` host threads; regions without samples are untouched.  pdf = the
 * records' sampling pdf, grouped like dirw.  The parallax distances are not
 * updated here (pgo_update_distances). */
int pgo_postfit_lpmm32(const pg_fit_config *cfg, const pg_split_merge_config *sm, uint32_t n_regions,
                       const float *dirw, const float *pdf, const uint32_t *offsets, pg_region_state *states,
                       pg_region_extra *extras, int n_threads);

/* PathGuiding::update's region split check and splitRegion
 * (src/PathGuiding.cpp:290-348, Aabb::splitAabb src/Shapes.h:32-46) over
 * regions [0, n); returns the new region count (at most cap).  nodes /
 * leaf_of / n_nodes: the region tree (node v >= 0: children v, v + 1; v < 0:
 * leaf of region -v - 1). */
uint32_t pgo_split_regions(uint32_t n, uint32_t cap, float thr, pg_region_state *states, pg_region_extra *extras,
                           float *aabbs, int32_t *nodes, uint32_t *leaf_of, uint32_t *n_nodes);
/* Point -> region by descent of that tree from the padded scene box. */
uint32_t pgo_region_of(const float root[6], const int32_t *nodes, const float p[3]);

/* lightpmm fastexp (pmm-vcl.h:158-184), scalar restatement. */
float pgo_fastexp(float x);

/* Parallax pre-pass (PathGuiding::preFit, src/PathGuiding.cpp:370-402):
 * re-centres each sample of region r on `mean` (3 floats per region),
 * writing dirw (float4) and the new distance (+inf for misses). */
void pgo_prefit_parallax(uint32_t n_regions, const pg_directional_data *sorted,
                         const uint32_t *offsets, const float *means, float *dirw_out,
                         float *dist_out);

/* Harmonic-mean lobe distance update (the statistic of
 * external/guiding/incrementaldistance.h:57-107), FP64 accumulation. */
void pgo_update_distances(uint32_t n_regions, const float *dirw, const float *dist,
                          const uint32_t *offsets, pg_region_state *states);

/* Re-aims lobes with a finite distance at a moved parallax mean
 * (incrementaldistance.h:109-131). */
void pgo_reposition(pg_region_state *s, const float new_to_old[3]);

/* PathGuiding::pmmToVMM_Theta + syncPMMsToVMM_Thetas
 * (src/PathGuiding.cpp:53-69, 106-132). */
void pgo_pack_vmm_theta(uint32_t n_regions, const pg_region_state *states, int use_parallax,
                        pg_vmm_theta *out);

/* Region boxes of `split_count` midpoint splits along the largest axis of the
 * padded scene box (src/PathGuiding.cpp:81-104, src/Shapes.h:32-53); out has
 * 6 floats (min xyz, max xyz) per region, (1 << split_count) regions. */
void pgo_region_aabbs(uint32_t split_count, const float scene_aabb[6], float *out);

/* SampleCollector::getSortedData (src/SampleCollector.cpp:76-131): stable
 * bucket of records by region id (flags); INVALID records dropped.  Returns
 * the number of valid records; offsets has n_regions+1 entries. */
uint64_t pgo_sort_samples(const pg_directional_data *records, uint64_t n, uint32_t n_regions,
                          pg_directional_data *sorted_out, uint32_t *offsets_out);

#ifdef __cplusplus
}
#endif

#endif /* PG_ORACLE_H */
