/*
 * pathguide.h - C ABI of the GB300 path-guiding library (libpathguide.so).
 *
 * Plain C: pointers, sizes and integer status codes; no CUDA or torch types.
 * Streams are passed as `void*` holding a cudaStream_t (NULL = legacy default
 * stream).  Every entry point returns a pg_status; the text of the last error
 * of a context is available from pg_last_error().
 *
 * Each entry point names the reference interface it stands in for
 * (paths relative to the rtx-pathtracer source tree).
 */
#ifndef PATHGUIDE_H
#define PATHGUIDE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* MAX_DISTRIBUTIONS in shaders/limits.glsl:6; four 4-wide lightpmm kernels
 * (src/PathGuiding.h:28-30). */
#define PG_MAX_COMPONENTS 16u
/* INVALID region id of a sample slot (src/SampleCollector.h:13). */
#define PG_INVALID_REGION 0xFFFFFFFFu

typedef enum pg_status {
    PG_OK = 0,
    PG_ERR_ARG = 1,      /* bad argument (null pointer, size out of range)   */
    PG_ERR_CUDA = 2,     /* a CUDA runtime call failed                        */
    PG_ERR_TIMEOUT = 3,  /* a bounded device-side wait ran out               */
    PG_ERR_NUMERIC = 4,  /* non-finite result detected                        */
    PG_ERR_NOMEM = 5,    /* capacity of the context exceeded                  */
    PG_ERR_IO = 6,       /* file could not be read or written                 */
    PG_ERR_PARSE = 7,    /* scene file malformed                              */
    PG_ERR_STATE = 8     /* call made in the wrong order                      */
} pg_status;

/* Fit modes of pg_fit_regions. */
typedef enum pg_fit_mode {
    /* VMMFactory::initialize + VMMFactory::fit(..., initialize=false)
     * (external/lightpmm/include/pmm/VMMFactory.h:132-216), which is what
     * PathGuiding::createPMMs + the first updateRegion do
     * (src/PathGuiding.cpp:42-51, 357-359). */
    PG_FIT_INIT = 0,
    /* VMMFactory::fit(..., initialize=false) from the current state. */
    PG_FIT_CONTINUE = 1,
    /* VMMFactory::updateFit: stepwise EM that adds the statistics recovered
     * from the current parameters (VMMFactory.h:305-362, 543-555); used by
     * PathGuiding::updateRegion on every pass after the first
     * (src/PathGuiding.cpp:360-363). */
    PG_FIT_UPDATE = 2
} pg_fit_mode;

/* lightpmm::DirectionalData (external/lightpmm/include/pmm/DirectionalData.h:44-101)
 * and the GLSL record (shaders/guiding.glsl:99-111): 40 bytes, AoS.
 * `flags` holds the guiding region id or PG_INVALID_REGION. */
typedef struct pg_directional_data {
    float position[3];
    float direction[3];
    float weight;
    float pdf;
    float distance;
    uint32_t flags;
} pg_directional_data;

/* lightpmm::VMMFactoryProperties (VMMFactory.h:45-61) with the overrides of
 * PathGuiding::configureVMMFactory (src/PathGuiding.cpp:33-40), plus the
 * parallax switch of PathGuiding (src/PathGuiding.h:103). */
typedef struct pg_fit_config {
    uint32_t min_itr;
    uint32_t max_itr;
    float rel_ll_threshold;
    uint32_t num_initial_components; /* 1..16 */
    float init_kappa;
    float max_kappa;
    float v_prior;
    float r_prior;
    float r_prior_weight;
    uint32_t use_parallax;
} pg_fit_config;

/* Per-region mixture state held in device memory (one 704-byte record per
 * region).  It carries what lightpmm::ParametricMixtureModel
 * (ParametricMixtureModel.h:69-81), its VMFKernel lanes (VMFKernel.h:75-86)
 * and PMM_ExtraData's parallax fields (src/PathGuiding.h:77-84) hold, in
 * structure-of-arrays form over the 16 components. */
typedef struct pg_region_state {
    float weight[16];      /* mixture weights (weight prior applied)          */
    float mu_x[16];        /* mean directions                                 */
    float mu_y[16];
    float mu_z[16];
    float kappa[16];       /* concentrations                                  */
    float r[16];           /* mean cosines                                    */
    float norm[16];        /* kappa / (2 pi (1 - exp(-2 kappa)))              */
    float e_min2k[16];     /* exp(-2 kappa)                                   */
    float distance[16];    /* parallax distance per lobe (+inf: unknown)      */
    float dist_sum_w[16];  /* accumulated weight of the distance estimate     */
    float parallax_mean[3];
    float last_parallax_mean[3];
    uint32_t k;            /* active components                               */
    float sample_weight;   /* m_sampleWeight                                  */
    float num_samples;     /* m_numSamples                                    */
    uint32_t num_em_iterations;
    uint64_t total_num_samples;
    float ll_last;         /* weighted log-likelihood of the last E-step      */
    uint32_t iters_last;   /* EM iterations run by the last fit               */
    uint32_t flags;        /* PG_STATE_* bits                                 */
    uint32_t reserved;
} pg_region_state;

#define PG_STATE_FITTED 1u     /* region has been fitted at least once        */
#define PG_STATE_NONFINITE 2u  /* last fit produced a non-finite parameter    */
/* Set by pg_fit_regions_noalloc on every region of a call in which a bounded
 * device wait ran out or an index check failed (the fit of those regions is
 * incomplete); that entry point clears it on a clean call, the others leave it
 * as they find it.  Context-based fits report the same events through their
 * status codes instead. */
#define PG_STATE_FIT_FAILED 4u

/* VMF_Theta / VMM_Theta as uploaded to the tracer (src/PathGuiding.h:36-75,
 * shaders/guiding.glsl:14-51): 40 and 720 bytes, scalar layout. */
typedef struct pg_vmf_theta {
    float mu[3];
    float k;
    float norm;
    float e_min2k;
    float distance;
    float target[3];
} pg_vmf_theta;

typedef struct pg_vmm_theta {
    pg_vmf_theta thetas[16];
    float pi[16];
    float mean_position[3];
    int32_t used_distributions;
} pg_vmm_theta;

typedef struct pg_ctx pg_ctx;

/* ------------------------------------------------------------------ */
/* Context                                                             */
/* ------------------------------------------------------------------ */

/* Reference defaults: VMMFactoryProperties (VMMFactory.h:45-61) overridden by
 * PathGuiding::configureVMMFactory (src/PathGuiding.cpp:33-40): K=8,
 * maxItr=100, maxKappa=50000; parallax on (src/RayTracingApp.h:117). */
void pg_default_fit_config(pg_fit_config *out);

/* Creates a context on the current CUDA device.  The context owns the
 * per-region mixture states (max_regions records) and the scratch of the
 * fit (work queues, region order) and of the sample sort (max_samples
 * records).  Replaces the constructor PathGuiding::PathGuiding
 * (src/PathGuiding.cpp:11-24) minus its Vulkan objects. */
int pg_ctx_create(const pg_fit_config *cfg, uint32_t max_regions, uint64_t max_samples,
                  pg_ctx **out);
int pg_ctx_destroy(pg_ctx *ctx);
const char *pg_last_error(const pg_ctx *ctx);
const char *pg_status_string(int status);
int pg_get_fit_config(const pg_ctx *ctx, pg_fit_config *out);
int pg_set_fit_config(pg_ctx *ctx, const pg_fit_config *cfg);

/* ------------------------------------------------------------------ */
/* Mixture state                                                       */
/* ------------------------------------------------------------------ */

/* Initialises n_regions mixtures as VMMFactory::initialize does
 * (VMMFactory.h:132-148): K components, weights 1/K, kappa = init_kappa,
 * means on the spherical Fibonacci set (VMMFactory.h:594-632); distances
 * +inf (external/guiding/incrementaldistance.h:52-55).  Device-side. */
int pg_init_regions(pg_ctx *ctx, uint32_t n_regions, void *stream);

/* Host copies of the device states (ParametricMixtureModel::serialize /
 * deserialize, ParametricMixtureModel.h:373-397, in this layout). */
int pg_get_region_states(pg_ctx *ctx, pg_region_state *host_out, uint32_t first,
                         uint32_t count, void *stream);
int pg_set_region_states(pg_ctx *ctx, const pg_region_state *host_in, uint32_t first,
                         uint32_t count, void *stream);
/* Device pointer to the state array (valid until pg_ctx_destroy). */
int pg_region_states_device(pg_ctx *ctx, pg_region_state **dev_out);

/* ------------------------------------------------------------------ */
/* Batched weighted EM                                                 */
/* ------------------------------------------------------------------ */

/* Fits the mixtures of regions [0, n_regions) to their samples in one
 * launch.  `dirw` (device, 16-byte aligned) holds one float4
 * {direction.xyz, weight} per sample, grouped by region; `offsets` (device)
 * holds n_regions+1 sample offsets.  Regions run different iteration counts
 * (relative log-likelihood test per region).  The launch takes regions in
 * order of expected work - samples times the iteration count of the region's
 * last fit (20 where it has none) - and gives those above the tuning's
 * large_threshold (in samples at 20 iterations) a cluster of CTAs, so a
 * region's team, and with it the low bits of its statistics' sums, follows
 * its state's last iteration count.  Replaces the serial loop
 * PathGuiding::update -> updateRegion -> VMMFactory::fit / updateFit
 * (src/PathGuiding.cpp:281-288, 350-368; VMMFactory.h:157-216, 305-362). */
int pg_fit_regions(pg_ctx *ctx, const float *dirw, const uint32_t *offsets,
                   uint32_t n_regions, int mode, void *stream);

/* VMMFactory::fit / updateFit over regions whose samples are in HOST memory
 * (the reference fits the host copy of the records, src/PathGuiding.cpp:
 * 276-312): dirw_host holds float4 {direction, weight} per sample grouped by
 * region, offsets_host n_regions + 1 sample offsets.  Page-locked samples
 * (cudaHostAlloc, cudaHostRegister, a pinned torch tensor) at a 16-byte aligned
 * address are read by the fit itself: each region's samples are read from host
 * memory when the fit reaches the region (largest regions first), so the
 * transfer overlaps the fit; slices larger than the staging capacity are
 * copied once to a context-owned device buffer.  Other host memory goes to
 * that buffer on a copy stream that starts behind the work already queued on
 * `stream`, in up to 16 chunks cut at region boundaries, the chunks holding
 * the largest regions first, while the fit runs: each region waits for its
 * chunk, and a region whose chunk has not arrived after about two seconds
 * stops waiting and pg_sync_status then reports PG_ERR_TIMEOUT.  Same results
 * as pg_fit_regions on the same samples; the states stay on the device
 * (pg_get_region_states).  Both buffers must stay valid and unchanged until
 * the stream has completed the fit. */
int pg_fit_regions_host(pg_ctx *ctx, const float *dirw_host, const uint32_t *offsets_host, uint32_t n_regions,
                        int mode, void *stream);

/* Weighted log-likelihood sum_n w_n log p(d_n) of each region's samples under
 * the current mixtures (the quantity of VMMFactory.h:531-532), written as
 * double to ll_out (device, n_regions entries). */
int pg_eval_loglik(pg_ctx *ctx, const float *dirw, const uint32_t *offsets,
                   uint32_t n_regions, double *ll_out, void *stream);

/* Tuning of the fit launch (chosen by the autotuner; 0 = default). */
typedef struct pg_fit_tuning {
    uint32_t threads_per_cta;       /* 128 or 256                               */
    uint32_t smem_samples;          /* samples kept in shared memory per CTA    */
    uint32_t ctas_per_sm;           /* cap on resident CTAs per SM (0: maximum);
                                       with 128 threads, 3 (16 components per
                                       thread, unroll 2) and 4 (8 components per
                                       thread) also cap the registers per thread
                                       so that as many CTAs fit                 */
    uint32_t cluster_size;          /* CTAs sharing one large region: 1..16     */
    uint32_t components_per_thread; /* 8 or 16: K=16 mixtures use 2 or 1 threads per sample */
    uint32_t unroll;                /* samples per loop trip: 1, 2 or 4 (4: 128
                                       threads per CTA)                         */
    uint32_t large_threshold;       /* regions with more expected work (samples
                                       x last iterations / 20) are shared by a
                                       cluster (0: 24576)                       */
    uint32_t stream_stages;         /* slices larger than smem_samples stream
                                       from L2 through a ring of this many
                                       TMA-filled shared-memory stages (0: 2; at
                                       most 8; fewer when a stage would hold
                                       less than one E-step loop trip)          */
} pg_fit_tuning;
int pg_set_fit_tuning(pg_ctx *ctx, const pg_fit_tuning *t);
int pg_get_fit_tuning(const pg_ctx *ctx, pg_fit_tuning *t);

/* Synchronises `stream` and reports errors recorded by device code since the
 * last pg_fit_regions: PG_ERR_TIMEOUT (a bounded wait ran out),
 * PG_ERR_NUMERIC (a fit produced a non-finite parameter, e.g. from corrupt
 * samples; the region's state carries PG_STATE_NONFINITE). */
int pg_sync_status(pg_ctx *ctx, void *stream);

/* Device kernels launched by the last pg_fit_regions call (for counting
 * launches in benchmarks). */
int pg_last_launch_count(const pg_ctx *ctx, uint32_t *count);

/* ------------------------------------------------------------------ */
/* Split and merge of mixture components                               */
/* ------------------------------------------------------------------ */

/* PathGuiding::postFit with splitAndMerge (src/PathGuiding.cpp:413-451):
 * components whose Pearson chi-square divergence is large are split along
 * the principal axis of their 2-D covariance (PCA split, :494-561) and
 * refitted by a masked EM; pairs whose merged component would barely change
 * the mixture are merged (:635-781).  The statistics it keeps per region and
 * component (incrementalpearsonchisquared.h, incrementalcovariance2d.h): */
typedef struct pg_region_extra {
    float chi2_div[16];        /* divergencePlusOneTimesIntegralSqr */
    float chi2_n[16];          /* numSamples                        */
    float cov[16][3];          /* variance x, variance y, covariance (component frame) */
    float cov_w[16];           /* sumWeights                        */
    float samples_since_merge; /* samplesSinceLastMerge             */
    /* work of the last pg_split_merge on the region (not in the reference):
     * passes of the divergence + covariance statistics over its samples and
     * masked EM iterations */
    uint32_t stat_passes;
    uint32_t em_iterations;
    uint32_t reserved;
} pg_region_extra;

/* The reference's knobs (src/PathGuiding.h:124-129). */
typedef struct pg_split_merge_config {
    uint32_t enabled;                            /* splitAndMerge                 */
    uint32_t min_samples_for_merging;            /* 8192                          */
    uint32_t min_samples_for_splitting;          /* 4096                          */
    uint32_t min_samples_for_post_split_fitting; /* 4096                          */
    float split_min_divergence;                  /* 0.5                           */
    float merge_max_divergence;                  /* 0.025                         */
    /* GPU work split (not in the reference): regions above cluster_threshold
     * samples are processed by a cluster of cluster_size CTAs, the others by
     * one CTA each, both at once.  0 selects the defaults (8192 samples, 8 CTAs);
     * cluster_threshold 0xFFFFFFFF keeps every region on one CTA. */
    uint32_t cluster_threshold;
    uint32_t cluster_size;
} pg_split_merge_config;

/* The reference's defaults, enabled. */
void pg_default_split_merge_config(pg_split_merge_config *out);
/* Sets the context's split/merge configuration (contexts start with it
 * disabled); pg_update then runs it after each fit, before the distances. */
int pg_set_split_merge(pg_ctx *ctx, const pg_split_merge_config *cfg);
/* The post-fit split/merge of regions [0, n_regions) on one pass of samples:
 * dirw as for pg_fit_regions, pdf = the records' sampling pdf per sample
 * (device, grouped like dirw).  Regions without samples are untouched.
 * Mixture components may change in number (1..16). */
int pg_split_merge(pg_ctx *ctx, const float *dirw, const float *pdf, const uint32_t *offsets, uint32_t n_regions,
                   void *stream);
/* Host copies of the per-region split/merge statistics. */
int pg_get_region_extra(pg_ctx *ctx, pg_region_extra *host_out, uint32_t count);
int pg_set_region_extra(pg_ctx *ctx, const pg_region_extra *host_in, uint32_t count);

/* Autotuner (no counterpart in the reference, which fits on the host): times
 * the fit on the caller's own samples for each candidate tuning (the built-in
 * grid of CTA size, samples staged per CTA, components per thread, cluster
 * size and cluster threshold when candidates is NULL) with CUDA events on
 * `stream`, keeps the fastest in the context and returns it in best_out with
 * its time in best_ms_out (either may be NULL).  The mixture states are saved
 * before and restored after, so the call leaves them as it found them;
 * candidates the device cannot launch are skipped.  Synchronises the stream. */
int pg_autotune_fit(pg_ctx *ctx, const float *dirw, const uint32_t *offsets, uint32_t n_regions, int mode,
                    const pg_fit_tuning *candidates, uint32_t n_candidates, pg_fit_tuning *best_out,
                    float *best_ms_out, void *stream);

/* The fit as a CUDA graph: pg_fit_graph_create captures pg_fit_regions on
 * `stream` (a non-default stream) with the given buffers and the context's
 * current tuning; every pg_fit_graph_launch replays it - the caller refills
 * the same sample and offset buffers between launches.  The graph holds
 * pointers into the context: destroy it before the context. */
typedef struct pg_fit_graph pg_fit_graph;
int pg_fit_graph_create(pg_ctx *ctx, const float *dirw, const uint32_t *offsets, uint32_t n_regions, int mode,
                        void *stream, pg_fit_graph **out);
int pg_fit_graph_launch(pg_fit_graph *graph, void *stream);
int pg_fit_graph_destroy(pg_fit_graph *graph);

/* ------------------------------------------------------------------ */
/* Regions, sample bucketing, parallax, distances, VMM_Theta            */
/* ------------------------------------------------------------------ */

/* Builds 2^split_count regions by repeated midpoint splits of the padded scene
 * box along its largest axis (PathGuiding::createRegions,
 * src/PathGuiding.cpp:81-104; Aabb::splitAabb / addEpsilon, src/Shapes.h:32-53)
 * and initialises their mixtures (pg_init_regions).  scene_aabb = min xyz, max xyz. */
int pg_set_regions(pg_ctx *ctx, uint32_t split_count, const float scene_aabb[6], void *stream);
/* PathGuiding::getRegionCount (src/PathGuiding.h:136). */
int pg_region_count(const pg_ctx *ctx, uint32_t *out);
/* The region boxes, 6 floats each (host copy / device pointer). */
int pg_get_region_aabbs(pg_ctx *ctx, float *host_out, uint32_t count);
int pg_region_aabbs_device(pg_ctx *ctx, const float **dev_out);

/* Adaptive region splitting (PathGuiding::update's split check and
 * splitRegion, src/PathGuiding.cpp:290-348; the reference's knobs
 * splitRegions = false and samplesForRegionSplit = 10000, src/PathGuiding.h:121-122). */
typedef struct pg_region_split_config {
    uint32_t enabled;
    float samples_for_region_split; /* a region splits when its mixture's sample count exceeds this */
} pg_region_split_config;
/* The reference's threshold, enabled (the reference leaves it off by default). */
void pg_default_region_split_config(pg_region_split_config *out);
/* Sets the context's region splitting (off until set); pg_update then runs
 * pg_split_regions after each fit, before VMM_Theta packing. */
int pg_set_region_split(pg_ctx *ctx, const pg_region_split_config *cfg);
/* The split check over the current regions, in region order: a region whose
 * mixture has seen more than samples_for_region_split samples (m_numSamples)
 * is halved along the largest axis of its box (Aabb::splitAabb); it keeps the
 * lower half and the upper half becomes region n, n+1, ... in that order; both
 * start from its mixture and split/merge statistics with the sample count and
 * sample weight decayed by 0.25.  Regions that would exceed the context's
 * capacity are not created.  Synchronises the stream; *n_regions_out = the new
 * region count (a split happened if it grew). */
int pg_split_regions(pg_ctx *ctx, uint32_t *n_regions_out, void *stream);
/* The region tree the renderer descends: 2 n_regions - 1 nodes; a node >= 0
 * is an inner node whose children are nodes v and v + 1 (lower half first,
 * the midpoint split of the node's box along its largest axis), a node < 0 is
 * the leaf of region -v - 1.  Node 0 is the padded scene box. */
int pg_get_region_tree(pg_ctx *ctx, int32_t *host_nodes, uint32_t capacity, uint32_t *n_nodes_out);

/* SampleCollector::getSortedData (src/SampleCollector.cpp:76-131) on the
 * device: buckets n_records records by region id (flags), stably (equal ids
 * keep their order); INVALID or out-of-range ids are dropped.  offsets_out
 * (device, n_regions+1) receives the region offsets; sorted_out (device, may
 * be NULL) the bucketed records. */
int pg_sort_samples(pg_ctx *ctx, const pg_directional_data *records, uint64_t n_records, uint32_t n_regions,
                    pg_directional_data *sorted_out, uint32_t *offsets_out, void *stream);

/* PathGuiding::preFit (src/PathGuiding.cpp:370-411): sets each region's
 * parallax mean to its box centre, re-aims its lobes at the new mean after the
 * first fit (incrementaldistance.h:109-131) - both only for regions with
 * records in this pass, as PathGuiding::update skips empty ones - and writes for each bucketed
 * record the float4 {direction, weight} seen from the mean and the distance
 * (+inf for misses).  Without parallax the directions pass through. */
int pg_prefit_parallax(pg_ctx *ctx, const pg_directional_data *sorted, const uint32_t *offsets,
                       uint32_t n_regions, uint64_t n_valid, float *dirw_out, float *dist_out, void *stream);

/* Harmonic-mean lobe distances over one pass of samples (the statistic of
 * external/guiding/incrementaldistance.h:57-107, PathGuiding::postFit,
 * src/PathGuiding.cpp:445-448).  Regions without samples are left unchanged,
 * as PathGuiding::update runs postFit only for non-empty regions.  The pass
 * takes up to the context's max_samples, or as many samples as the largest
 * record set sorted by the context (pg_sort_samples, pg_update); more than
 * that leave every distance unchanged and report a bounds error through
 * pg_sync_status. */
int pg_update_distances(pg_ctx *ctx, const float *dirw, const float *dist, const uint32_t *offsets,
                        uint32_t n_regions, void *stream);

/* PathGuiding::pmmToVMM_Theta + syncPMMsToVMM_Thetas (src/PathGuiding.cpp:53-69,
 * 106-132): the tracer's per-region VMM_Theta (device, n_regions x 720 B). */
int pg_pack_vmm_theta(pg_ctx *ctx, uint32_t n_regions, pg_vmm_theta *out, void *stream);

/* PathGuiding::update (src/PathGuiding.cpp:276-312) as one device-resident
 * pass: bucket the tracer's records by region, parallax pre-pass, fit
 * (VMMFactory::fit on the first pass after pg_set_regions, updateFit after),
 * distance update, and - when vmm_out is not NULL - VMM_Theta packing. */
int pg_update(pg_ctx *ctx, const pg_directional_data *records, uint64_t n_records, pg_vmm_theta *vmm_out,
              void *stream);

/* ------------------------------------------------------------------ */
/* Scenes, traversal and the wavefront path tracer                       */
/* ------------------------------------------------------------------ */

/* Material types: the reference's EMatType (src/SceneLoader.h:31-39) - diffuse,
 * specular, dielectric, light, Phong, conductor - plus GGX (the project's
 * glossy lobe) and the reference's Beckmann rough conductor. */
enum {
    PG_MAT_DIFFUSE = 0,
    PG_MAT_SPECULAR = 1,
    PG_MAT_DIELECTRIC = 2,
    PG_MAT_LIGHT = 3,
    PG_MAT_PHONG = 4,
    PG_MAT_CONDUCTOR = 5,
    PG_MAT_GGX = 6,
    PG_MAT_BECKMANN = 7
};

typedef struct pg_material {
    int32_t type;
    float albedo[3];    /* diffuse reflectance (diffuse, Phong); specular / GGX tint (Fresnel F0) */
    float emission[3];  /* radiance of a light (lightColor) */
    float roughness;    /* GGX and Beckmann alpha */
    float ior;          /* dielectric index of refraction (intIOR / extIOR) */
    float specular[3];  /* Phong specular reflectance */
    float exponent;     /* Phong exponent (specularHighlight) */
    float eta, k;       /* conductor and Beckmann conductor: Fresnel eta and k (one spectrum value) */
    int32_t texture;    /* 0: none; t: scene texture t - 1, which scales a diffuse albedo
                           (textureIdDiffuse) and alpha-tests every hit (raytrace.rahit) */
} pg_material;

typedef struct pg_sphere {
    float center[3];
    float radius;
    uint32_t material;
    uint32_t reserved[3];
} pg_sphere;

typedef struct pg_camera {
    float origin[3];
    float target[3];
    float up[3];
    float vfov_deg;
    uint32_t width, height;
} pg_camera;

/* One ray: origin, t_min, direction, t_max (32 B). */
typedef struct pg_ray {
    float org[3];
    float tmin;
    float dir[3];
    float tmax;
} pg_ray;

#define PG_NO_HIT 0xFFFFFFFFu
#define PG_SPHERE_BIT 0x80000000u
/* Closest hit: t, barycentrics (u, v) and the original triangle id, or
 * PG_SPHERE_BIT | sphere index, or PG_NO_HIT. */
typedef struct pg_hit {
    float t;
    float u, v;
    uint32_t prim;
} pg_hit;

/* Procedural Cornell box: five walls (10 triangles, albedo 0.7 / red /
 * green), a 0.25 x 0.25 area light on the ceiling, and a dielectric icosphere
 * with 20 * 4^ico_level triangles. */
typedef struct pg_cornell_params {
    uint32_t width, height;
    int32_t ico_level;
    float light_radiance;
    float ior;
} pg_cornell_params;

/* Multi-light glossy scene: four GGX plates (roughness 0.005, 0.02, 0.07,
 * 0.2) facing four spherical lights (radii 0.03, 0.1, 0.3, 1.0, power
 * proportional to 1/r^2) over a diffuse floor, plus a seeded displaced plane of
 * 2 * grid^2 triangles between lights and plates. */
typedef struct pg_plates_params {
    uint32_t width, height;
    uint32_t occluder_grid;
    uint32_t seed;
} pg_plates_params;

typedef struct pg_scene_info {
    uint32_t n_triangles, n_spheres, n_materials, n_nodes, n_lights;
    float aabb[6];       /* SceneLoader::getSceneSize (src/SceneLoader.h:118) */
    pg_camera camera;
} pg_scene_info;

/* Render settings: the push constants of the reference's ray-generation
 * shader that this path uses (src/RayTracingApp.h:81-130). */
typedef struct pg_render_params {
    uint32_t spp;
    uint32_t max_depth;
    uint32_t seed;
    uint32_t use_nee;          /* next-event estimation */
    uint32_t use_mis;          /* power-heuristic MIS of NEE and BSDF samples */
    uint32_t use_guiding;      /* sample directions from the context's mixtures */
    float guiding_prob;        /* one-sample mixture weight of the guide (0.5) */
    uint32_t record_samples;   /* write DirectionalData records for the next fit */
    uint32_t flags;            /* PG_RENDER_* instrumentation bits (0 for plain rendering) */
    uint32_t reserved[3];
} pg_render_params;

/* Count BVH node visits and triangle tests of every ray into the stats (a
 * separately compiled traversal; the image is unchanged). */
#define PG_RENDER_COUNT_WORK 1u
/* Time each stage with CUDA events on the render stream (the call then
 * synchronises the stream before returning). */
#define PG_RENDER_TIME_STAGES 2u
/* Guide near-specular lobes too (Beckmann / GGX roughness <= 0.3, Phong
 * exponent >= 250), as the reference does: it mixes the guide into every
 * non-discrete material (raytrace.rgen:926) while recording only the others
 * (:962-964, 1180).  Off by default: guiding then follows the recording rule. */
#define PG_RENDER_GUIDE_ALMOST_DISCRETE 4u

/* Irradiance cache (raytrace.rgen:745-813, 1231-1421; raytrace.irradiance.rint,
 * raytrace.irradiance.rahit): with a cache set on the scene
 * (pg_scene_set_irradiance_cache), a path that reaches a diffuse vertex (or any
 * non-discrete one with use_on_glossy) inside cached spheres takes the cached
 * irradiance there times the surface's diffuse reflectance / pi, adds one
 * next-event sample and ends.  Elsewhere the vertex queues a new entry with
 * probability create_prob (at most 5 per pixel and pass), and every pixel
 * queues an update of the next entry (round robin) with probability
 * update_prob.  The queued entries are computed after each sample pass (20 x 10
 * stratified hemisphere paths each), written in pixel order, and used from the
 * next pass on: one pass here is one frame of the reference at one sample per
 * pixel.  A render call that grows the cache synchronizes its stream once at
 * the end.  Requires a cache on the scene. */
#define PG_RENDER_IRRADIANCE_CACHE 8u
/* With PG_RENDER_IRRADIANCE_CACHE: query the cache only (no creation, no
 * update, no synchronization). */
#define PG_RENDER_IC_FROZEN 16u
/* ADRRS, adjoint-driven Russian roulette and splitting (raytrace.rgen:830-869,
 * 883-902, 1080-1117, 1684-1708): at a cache-capable vertex after the first bounce
 * where the scene's irradiance cache applies, the path's throughput is
 * compared with a weight window centred on |estimate / cached irradiance|
 * (estimate: the pixel's value from pg_scene_set_adrrs).  Below the window
 * the path continues with probability max(v / lower, 0.1) and its
 * throughput is divided by it; above it, with split set, it is split into
 * about v / upper copies (at most 10 copies per pixel and pass) that share
 * the throughput and continue independently.  The cache is only read (a path
 * does not end at it).  Requires a cache and an estimate on the scene; not
 * with record_samples when splitting (the reference collects no samples
 * then either). */
#define PG_RENDER_ADRRS 32u

enum pg_render_stage {
    PG_STAGE_CAMERA = 0, PG_STAGE_EXTEND, PG_STAGE_SHADE, PG_STAGE_SHADOW, PG_STAGE_ADVANCE, PG_STAGE_COMMIT,
    PG_STAGE_COUNT
};

typedef struct pg_render_stats {
    uint64_t extension_rays;
    uint64_t shadow_rays;
    uint64_t samples_recorded;
    uint64_t paths;
    /* with PG_RENDER_COUNT_WORK: traversal work of extension and shadow rays */
    uint64_t extension_node_visits, extension_triangle_tests;
    uint64_t shadow_node_visits, shadow_triangle_tests;
    /* with PG_RENDER_TIME_STAGES: summed duration and launch count per stage */
    float stage_ms[PG_STAGE_COUNT];
    uint32_t stage_launches[PG_STAGE_COUNT];
} pg_render_stats;

typedef struct pg_scene pg_scene;

/* SceneLoader(filepath) (src/SceneLoader.cpp:29-65): Mitsuba-XML subset
 * (sensor lookAt/fov, bsdf diffuse/dielectric/conductor/roughconductor,
 * shape obj/sphere/rectangle/cube, area emitters).  Builds the BVH on the host;
 * the device copy is made on first use.  On failure the message is in
 * pg_last_error(NULL) (PG_ERR_IO: unreadable file, PG_ERR_PARSE: malformed). */
int pg_scene_load(const char *path, uint32_t width, uint32_t height, pg_scene **out);
int pg_scene_create_cornell(const pg_cornell_params *p, pg_scene **out);
int pg_scene_create_plates(const pg_plates_params *p, pg_scene **out);
int pg_scene_destroy(pg_scene *scene);
int pg_scene_get_info(const pg_scene *scene, pg_scene_info *out);
/* Host copies of the built scene: BVH nodes (128 B each, four-wide), triangles in BVH
 * order (12 floats each), their original ids, per-triangle materials, the
 * materials and the spheres.  Any pointer may be NULL. */
int pg_scene_export(const pg_scene *scene, void *nodes, float *tri_verts, uint32_t *tri_order,
                    uint32_t *tri_material, pg_material *materials, pg_sphere *spheres);
/* Host copies of the vertex positions (3 floats each, n_vertices of them) and
 * triangle indices (3 per triangle, original order). */
int pg_scene_export_mesh(const pg_scene *scene, float *positions, uint32_t *indices, uint32_t *n_vertices);
/* Material textures (Mitsuba bitmap textures, PNG; SceneLoader::addTexture,
 * src/SceneLoader.cpp:184-233): the count and total texel count, then host
 * copies of the texture coordinates (6 floats per triangle, original order),
 * per texture {first texel, width, height, 0} and the RGBA8 texels (rows from
 * the top).  Any output pointer may be NULL. */
int pg_scene_texture_sizes(const pg_scene *scene, uint32_t *n_textures, uint64_t *n_texels);
int pg_scene_export_textures(const pg_scene *scene, float *tri_uv, uint32_t *tex_info, uint8_t *texels);
/* Decodes a PNG file (8-bit grey, grey + alpha, RGB, RGBA or palette,
 * non-interlaced) to RGBA8: *width and *height are set; rgba_out (NULL: a size
 * query) receives width * height * 4 bytes, PG_ERR_ARG if capacity is smaller. */
int pg_png_read(const char *path, uint8_t *rgba_out, uint64_t capacity, uint32_t *width, uint32_t *height);
/* Replaces the camera (SceneLoader origin/target/upDir/vfov, src/SceneLoader.h:147-150)
 * and the image size. */
int pg_scene_set_camera(pg_scene *scene, const pg_camera *cam);
/* Environment map (SceneLoader::parseEnvMap, src/SceneLoader.cpp:370-401;
 * shaders/raytrace.rmiss): a lat-long RGB image, width x height texels, row 0
 * looking up (+y), column u = atan2(x, -z) / 2 pi; sampled bilinearly with
 * wrap-around.  It lights misses and is one more light for next-event
 * estimation (a uniform direction in the hemisphere, raytrace.rgen:406-421).
 * width = height = 0 removes it.  A Mitsuba file's envmap emitter sets it. */
int pg_scene_set_envmap(pg_scene *scene, const float *rgb, uint32_t width, uint32_t height);
/* Its size, and a copy when rgb_out is not NULL (3 * width * height floats). */
int pg_scene_get_envmap(const pg_scene *scene, float *rgb_out, uint32_t *width, uint32_t *height);

/* OpenEXR images (writeEXR / readEXR, src/CommonOps.cpp:12-65): scanline
 * files with HALF, FLOAT or UINT channels, uncompressed, ZIPS, ZIP or PIZ
 * compressed (the project decodes both itself); RGB floats row-major from the
 * top row (a Y-only image fills all three).  With rgb_out NULL only the size
 * is returned; capacity counts floats.  The writer stores FLOAT R, G, B
 * without compression. */
int pg_exr_read(const char *path, float *rgb_out, uint64_t capacity, uint32_t *width, uint32_t *height);
int pg_exr_write(const char *path, const float *rgb, uint32_t width, uint32_t height);

/* The irradiance cache of a scene: the reference's push constants
 * (src/RayTracingApp.h:97-113) and IC_SIZE.  Defaults: a 0.2, min_radius 0.1,
 * create_prob 0.0005, update_prob 0.00001, gradients off (max length 5),
 * visibility check off, one NEE sample, diffuse surfaces only. */
typedef struct pg_irradiance_cache_config {
    uint32_t capacity;            /* IC_SIZE: maximum entries (0 removes the cache) */
    float a;                      /* irradianceA: sphere radius = a * harmonic mean distance */
    float min_radius;             /* irradianceCacheMinRadius: lower bound of the harmonic distance */
    float create_prob;            /* irradianceCreateProb, per vertex without a cache hit */
    float update_prob;            /* irradianceUpdateProb, per pixel sample */
    uint32_t use_gradients;       /* useIrradianceGradients */
    float gradients_max_length;   /* irradianceGradientsMaxLength */
    uint32_t visibility_check;    /* irradianceCachePerformVisibilityCheck */
    uint32_t use_on_glossy;       /* useIrradianceCacheOnGlossy */
    uint32_t num_nee;             /* irradianceNumNEE: light samples averaged at each
                                     vertex of an entry's hemisphere paths (0: 1; at most 64) */
    uint32_t reserved[2];
} pg_irradiance_cache_config;

/* One cache entry (cacheSpheres[i] and cache[i] of raytrace.rgen:118-119): the
 * sphere (centre, radius = a * harmonic_r), the surface normal, the cached
 * irradiance and its rotation and translation gradients. */
typedef struct pg_ic_entry {
    float center[3];
    float radius;
    float normal[3];
    float harmonic_r;
    float color[3];
    uint32_t num_updates;
    float rot_grad[3];
    float trans_grad[3];
} pg_ic_entry;

void pg_default_irradiance_cache_config(pg_irradiance_cache_config *out);
/* Sets (and empties) the scene's irradiance cache; capacity 0 removes it. */
int pg_scene_set_irradiance_cache(pg_scene *scene, const pg_irradiance_cache_config *cfg);
/* The entries (host copy; NULL out: count only) and their count. */
int pg_scene_get_irradiance_cache(pg_scene *scene, pg_ic_entry *out, uint32_t capacity, uint32_t *n_entries);
/* Replaces the entries (host array, at most the capacity) - e.g. a cache
 * computed elsewhere, for rendering with PG_RENDER_IC_FROZEN - and restarts
 * the round-robin update position. */
int pg_scene_set_irradiance_cache_entries(pg_scene *scene, const pg_ic_entry *entries, uint32_t n);

/* ADRRS settings (src/RayTracingApp.h:111-113).  estimate: a device array
 * of width * height * 3 floats for the scene's camera, each pixel's mean
 * radiance (the reference renders it with its estimate settings,
 * src/RayTracingApp.cpp:1206-1217), owned by the caller and read by every
 * render with PG_RENDER_ADRRS until replaced.  s: the window's ratio
 * upper / lower (adrrsS, default 5).  split: split paths above the window
 * (adrrsSplit, default 1). */
typedef struct pg_adrrs_config {
    const float *estimate;
    float s;
    uint32_t split;
    uint32_t reserved[4];
} pg_adrrs_config;
int pg_scene_set_adrrs(pg_scene *scene, const pg_adrrs_config *cfg);

/* Cache queries at n points with their surface normals (device arrays, 3
 * floats each): rgb the weighted mean of the applicable entries
 * (queryIrradianceCache, raytrace.rgen:748-773), found 1 where one applied. */
int pg_ic_query(pg_scene *scene, const float *positions, const float *normals, uint32_t n, float *rgb,
                uint32_t *found, void *stream);

/* A request for a cache entry at a surface point.  pixel, bounce and pass
 * name the random numbers its paths use: a render queues the request of the
 * vertex at `bounce` of the path `pixel` (a camera path: its pixel) in sample
 * pass `pass` (bounce 255: the update request of that pixel). */
typedef struct pg_ic_request {
    float position[3];
    float normal[3];
    uint32_t pixel, bounce, pass, reserved;
} pg_ic_request;

/* The entries calculateCacheData (raytrace.rgen:1231-1316) and
 * createIrradianceCache (:1383-1421) make at n requests (device arrays), with
 * the render settings rp (seed, next-event estimation, guiding with `guide`)
 * and the scene's cache for the lookups of their paths; the cache is not
 * changed.  A request whose hemisphere saw nothing gets harmonic_r -1 and
 * num_updates 0 (no entry would be made). */
int pg_ic_compute(pg_scene *scene, const pg_render_params *rp, pg_ctx *guide, const pg_ic_request *requests,
                  uint32_t n, pg_ic_entry *out, void *stream);

/* Closest hit / any hit of n rays (device arrays).  Traversal: four-wide BVH,
 * near child first, watertight FP32 ray-triangle test (Woop, Benthin and
 * Wald 2013); ties in t go to the lower triangle id. */
int pg_trace_closest(pg_scene *scene, const pg_ray *rays, uint32_t n, pg_hit *hits, void *stream);
int pg_trace_any(pg_scene *scene, const pg_ray *rays, uint32_t n, uint32_t *occluded, void *stream);
/* pg_trace_closest that also writes, per ray, the BVH nodes visited and the
 * triangles tested (device arrays of n).  The traversal order is that of
 * pg_trace_closest, so the counts are the algorithm's work for those rays. */
int pg_trace_closest_counted(pg_scene *scene, const pg_ray *rays, uint32_t n, pg_hit *hits, uint32_t *node_visits,
                             uint32_t *triangle_tests, void *stream);

/* Renders params->spp samples per pixel with the wavefront integrator and
 * adds the radiance sums into image (device, width * height * 3 floats).
 * With `guide` (a context after pg_set_regions / pg_update) and
 * use_guiding, BSDF sampling is mixed with the regions' vMF mixtures
 * (shaders/guiding.glsl:32-96, raytrace.rgen:923-960).  With record_samples,
 * up to 16 guiding records per pixel (raytrace.rgen:966-990, 1179-1200) are
 * written to records (device, width * height * 16), INVALID where empty. */
int pg_render(pg_scene *scene, const pg_render_params *params, pg_ctx *guide, float *image,
              pg_directional_data *records, pg_render_stats *stats, void *stream);

/* Shading-function probes (diagnostics; no counterpart in the reference,
 * whose functions run inside its ray-generation shader).  Each probe runs one
 * of the renderer's own device functions on explicit inputs and random
 * numbers, so the functions can be compared with the reference's shader
 * functions (shaders/raytrace.rgen, guiding.glsl, random.glsl) one call at a
 * time:
 *   PG_PROBE_FRESNEL            fresnel(a = eta, b = cos_i)            raytrace.rgen:145-160
 *   PG_PROBE_FRESNEL_CONDUCTOR  fresnelConductor(a = cos_i, b = eta, c = k)  :163-175
 *   PG_PROBE_BSDF_EVAL          evalBsdf * and pdfBSDF at (n, wi, wo)   :284-332, 557-599
 *   PG_PROBE_BSDF_SAMPLE        sampleBSDF with u[1..3]; v[3] = its pdf :483-552
 *   PG_PROBE_VMM_PDF            VMM(wo) of mixture `vmm` seen from x     guiding.glsl:53-60
 *   PG_PROBE_VMM_SAMPLE         sampleVMM from x with u[4], u[2], u[3]  guiding.glsl:62-96
 *   PG_PROBE_CONTINUE           getNewDirection and evalBsdf / pdf      raytrace.rgen:923-960, 1176
 *                               (u = choice, lobe/ul, u1, u2, lobe choice; c = guiding prob;
 *                               result: direction, pdf, throughput change)
 *   PG_PROBE_TO_WORLD           toWorld(wo, n)                          transform.glsl:7-38
 *   PG_PROBE_WEIGHT_WINDOW      applyWeightWindow(throughput = wi, adjoint = wo, estimate = x,
 *                               s = a, rounding number u[0]): v[0] = q, v[1] = n   raytrace.rgen:830-869
 *   PG_PROBE_APPROX_DIFFUSE     approxDiffuse(material, n, wi)          raytrace.rgen:815-828
 * (* the library's BSDF value includes the cosine, as evalBsdf's does.)
 * flags: bit 0 front face, bit 1 parallax re-aiming, bit 2 the vertex is
 * guided, bit 3 its region exists (else the path ends), bit 4 the guide-all
 * rule (PG_RENDER_GUIDE_ALMOST_DISCRETE).  mats, vmms, probes and out are
 * device arrays; a probe whose material or mixture index is out of range
 * writes NaN results. */
enum {
    PG_PROBE_FRESNEL = 0, PG_PROBE_FRESNEL_CONDUCTOR = 1, PG_PROBE_BSDF_EVAL = 2, PG_PROBE_BSDF_SAMPLE = 3,
    PG_PROBE_VMM_PDF = 4, PG_PROBE_VMM_SAMPLE = 5, PG_PROBE_CONTINUE = 6, PG_PROBE_TO_WORLD = 7,
    PG_PROBE_WEIGHT_WINDOW = 8, PG_PROBE_APPROX_DIFFUSE = 9
};
typedef struct pg_shading_probe {
    int32_t op;
    uint32_t material;  /* index into mats */
    uint32_t vmm;       /* index into vmms */
    uint32_t flags;
    float n[3], wi[3], wo[3], x[3];
    float u[5];
    float a, b, c;
} pg_shading_probe;
typedef struct pg_shading_result {
    float v[8];  /* direction or value (3), pdf, throughput change (3), unused */
} pg_shading_result;
int pg_probe_shading(const pg_material *mats, uint32_t n_mats, const pg_vmm_theta *vmms, uint32_t n_vmms,
                     const pg_shading_probe *probes, uint32_t n, pg_shading_result *out, void *stream);

/* Sample-recording probe (diagnostics; no counterpart in the reference):
 * replays paths through the renderer's record functions - radiance reaching
 * a path is added to its earlier records through their throughput changes
 * (updateSamples, raytrace.rgen:973-978), then each record is committed with
 * weight |L| / pdf or marked invalid (commitSamples, :980-990).  Path p's
 * events are events[path_offsets[p] .. path_offsets[p + 1]); kind 0 records a
 * vertex (pdf, throughput change tc, region id; at most 16 per path, later
 * ones dropped), kind 1 is radiance `light` reaching the path.  Per path:
 * counts[p] records, weights / flags [p * 16 + k] (flags = region id or
 * PG_INVALID_REGION).  All arrays are device arrays. */
typedef struct pg_record_event {
    int32_t kind;
    float pdf;
    float tc[3];
    uint32_t region;
    float light[3];
} pg_record_event;
int pg_probe_records(const pg_record_event *events, const uint32_t *path_offsets, uint32_t n_paths, float *weights,
                     uint32_t *flags, uint32_t *counts, void *stream);

/* ------------------------------------------------------------------ */
/* Allocation-free fit                                                 */
/* ------------------------------------------------------------------ */

/* No counterpart in the reference: the reference fits on the host.
 *
 * pg_fit_regions_noalloc runs the same batched fit as pg_fit_regions for
 * callers that cannot allocate device memory: renderers that own all device
 * memory through their own arena (another allocator would fragment it and
 * defeat its accounting), and plugin hosts that hand the guiding step only its
 * own buffers and no right to allocate.  It needs no pg_ctx: the caller passes
 * the fit properties, the device array of n_regions mixture states (read and
 * written in place) and the samples and offsets as for pg_fit_regions.  The
 * fit's scratch lives in one static device array of the library, sized for
 * PG_NOALLOC_MAX_REGIONS regions (about 257 KB per GPU, held until the process
 * exits); nothing is allocated and nothing is read from host memory after the
 * call returns.  The first call on a device looks up that array's device
 * address (cudaGetSymbolAddress) and keeps it for the life of the process; a
 * device reset (cudaDeviceReset) invalidates the kept address, so do not call
 * this entry point after one.  All calls share the array: calls whose work may
 * overlap on the GPU race and must be ordered (same stream or events).
 * Returns PG_ERR_NOMEM when n_regions exceeds PG_NOALLOC_MAX_REGIONS,
 * PG_ERR_ARG for bad arguments, PG_ERR_CUDA when a CUDA call fails.  Errors
 * found on the device are reported in the states, stream-ordered: non-finite
 * results per region (PG_STATE_NONFINITE), and a bounded wait that ran out or
 * a failed index check on every region of the call (PG_STATE_FIT_FAILED). */
#define PG_NOALLOC_MAX_REGIONS 65536u
int pg_fit_regions_noalloc(const pg_fit_config *cfg, pg_region_state *states, const float *dirw,
                           const uint32_t *offsets, uint32_t n_regions, int mode, void *stream);

/* ------------------------------------------------------------------ */
/* Learned guiding surrogate                                           */
/* ------------------------------------------------------------------ */

/* No counterpart in the reference (it fits one mixture per region,
 * src/PathGuiding.cpp:350-368).  A small MLP maps a position to a
 * 16-component vMF mixture: Fourier features of the position in the scene box
 * (16 octaves per axis, 112 inputs), three hidden layers of 64 ReLU units,
 * 80 outputs (per component: weight logit, mean direction, log kappa).  BF16
 * weights and activations on the tensor cores, FP32 accumulation, FP32 master
 * weights and Adam.  Trained on the tracer's guiding records by maximising
 * their weighted log-likelihood; the per-region EM fit stays the fallback and
 * the judge of its KL error.  Parameters are one float vector of
 * PG_MLP_PARAMS values: W1 (64 x 112), b1, W2 (64 x 64), b2, W3 (64 x 64), b3,
 * W4 (80 x 64), b4, matrices row-major with one row per output unit. */
#define PG_MLP_PARAMS 20752u
#define PG_MLP_COMPONENTS 16u

typedef struct pg_mlp pg_mlp;

typedef struct pg_mlp_config {
    uint32_t batch;       /* samples per Adam step (e.g. 65536) */
    float lr;             /* 1e-3 */
    float beta1, beta2, eps;
    uint32_t seed;        /* initial weights */
    float scene_aabb[6];  /* positions are encoded relative to this box */
} pg_mlp_config;

void pg_mlp_default_config(pg_mlp_config *out);
int pg_mlp_create(const pg_mlp_config *cfg, pg_mlp **out);
int pg_mlp_destroy(pg_mlp *mlp);
/* Host copies of the FP32 master parameters (PG_MLP_PARAMS floats); setting
 * them also resets Adam's moments and step count. */
int pg_mlp_get_params(pg_mlp *mlp, float *host_out);
int pg_mlp_set_params(pg_mlp *mlp, const float *host_in);
/* Weighted NLL of n records (device) under the current network, and its
 * gradient (device, PG_MLP_PARAMS floats; may be NULL) - no update.  Records
 * flagged PG_INVALID_REGION carry no weight.  *loss_out is written after a
 * stream synchronisation. */
int pg_mlp_loss_grad(pg_mlp *mlp, const pg_directional_data *records, uint32_t n, float *grad_out, float *loss_out,
                     void *stream);
/* One training pass: the records in batches of cfg.batch, one Adam step per
 * batch.  loss_out (host, may be NULL) receives the mean batch loss, read
 * after a stream synchronisation. */
int pg_mlp_train(pg_mlp *mlp, const pg_directional_data *records, uint64_t n, float *loss_out, void *stream);
/* Implementation of the training step: PG_MLP_PATH_TCGEN05 (default) runs one
 * persistent kernel per batch on the tcgen05 tensor cores (forward, loss,
 * backward and weight gradients of 128-record tiles, gradient sums kept in
 * tensor memory); PG_MLP_PATH_WARP_MMA runs warp-level mma.sync kernels with
 * a DRAM scratch between the forward/backward and weight-gradient passes.
 * Both compute the same quantities in the same precision. */
#define PG_MLP_PATH_TCGEN05 0
#define PG_MLP_PATH_WARP_MMA 1
int pg_mlp_set_path(pg_mlp *mlp, int path);
/* Mixture parameters at n positions (device, 3 floats each): per position 16
 * components of {weight, mu x, mu y, mu z, kappa} (80 floats, device).
 * Stream-ordered and not synchronised: a bounded tensor-core wait that ran out
 * is reported (PG_ERR_TIMEOUT) by the next call of this surrogate that
 * synchronises - pg_mlp_loss_grad / pg_mlp_train with a loss, or
 * pg_mlp_write_guide / pg_mlp_judge_guide, which check right after their own
 * inference. */
int pg_mlp_infer(pg_mlp *mlp, const float *positions, uint32_t n, float *mixtures_out, void *stream);
/* Evaluates the network at the centres of the regions of a guiding context
 * (after pg_set_regions) and installs the mixtures as the context's packed
 * guide, so pg_render guides with the network (no parallax re-aiming). */
int pg_mlp_write_guide(pg_mlp *mlp, pg_ctx *guide, void *stream);
/* The network beside the per-region fit, the fit staying the fallback and
 * the judge: for each region of `guide`, the weighted NLL (the KL divergence
 * up to a constant) of the given records (device; flags = region id, as the
 * tracer writes them) under the context's own mixture and under the
 * network's mixture at the region centre are compared; regions with at least
 * min_records records where the network's is lower take the network's
 * mixture.  *switched_out (host, may be NULL) receives the number of regions
 * switched, after a stream synchronisation. */
int pg_mlp_judge_guide(pg_mlp *mlp, pg_ctx *guide, const pg_directional_data *records, uint64_t n,
                       uint32_t min_records, uint32_t *switched_out, void *stream);
/* Weighted NLL, sum w (-log q(d)) / sum w, of records (device; flags = region
 * id) under a context's current guide - the fitted mixtures or what
 * pg_mlp_write_guide / pg_mlp_judge_guide installed - with parallax re-aiming
 * when the context uses it.  *nll_out is written after a stream
 * synchronisation. */
int pg_guide_nll(pg_ctx *guide, const pg_directional_data *records, uint64_t n, double *nll_out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PATHGUIDE_H */
