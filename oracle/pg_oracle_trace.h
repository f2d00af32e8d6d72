/*
 * pg_oracle_trace.h - TEST INFRASTRUCTURE.  CPU twins of the tracer:
 *   - pgo_trace_closest / pgo_trace_any: the same BVH walk and watertight
 *     triangle test as the device traversal, in FP32 with the same operation
 *     order (compiled with -ffp-contract=off), for bit-exact hit comparison;
 *   - pgo_render_f64: the path-tracing estimator restated in double precision
 *     (per-pixel loop, double-precision Moller-Trumbore intersection), drawing
 *     the same hashed random numbers as the GPU renderer, for image parity and
 *     for converged reference images.
 * Used only by tests/ and bench.py's reference leg, as the checker.
 */
#ifndef PG_ORACLE_TRACE_H
#define PG_ORACLE_TRACE_H

#include <stdint.h>

#include "pathguide.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pgo_scene {
    const void *nodes;          /* 64-byte BVH nodes */
    uint32_t n_nodes;
    const float *tri_verts;     /* 12 floats per triangle, BVH order; [3] = original id bits */
    uint32_t n_tris;
    const float *pos;           /* original vertices */
    uint32_t n_vertices;
    const uint32_t *idx;        /* original triangles */
    const uint32_t *tri_mat;
    const pg_material *mats;
    uint32_t n_mats;
    const pg_sphere *spheres;
    uint32_t n_spheres;
    pg_camera camera;
    const float *env;           /* environment map, RGB per texel, or NULL */
    uint32_t env_w, env_h;
    const float *tri_uv;        /* 6 per original triangle, or NULL */
    const uint32_t *tex_info;   /* per texture: first texel, width, height, 0 */
    const uint8_t *tex_data;    /* RGBA8 texels */
    uint32_t n_tex;
    uint32_t alpha_salt;        /* the alpha test's per-frame salt (traversal queries) */
} pgo_scene;

typedef struct pgo_guide {
    float root[6];
    uint32_t split_count;
    const int32_t *nodes; /* the region tree after region splits, or NULL (complete tree) */
    const pg_vmm_theta *vmm;
    int32_t use_parallax;
} pgo_guide;

void pgo_trace_closest(const pgo_scene *s, const pg_ray *rays, uint32_t n, pg_hit *hits, int n_threads);
/* pgo_trace_closest that also reports, per ray, BVH nodes fetched and triangles tested. */
void pgo_trace_closest_counted(const pgo_scene *s, const pg_ray *rays, uint32_t n, pg_hit *hits, uint32_t *nodes,
                               uint32_t *tris, int n_threads);
void pgo_trace_any(const pgo_scene *s, const pg_ray *rays, uint32_t n, uint32_t *occluded, int n_threads);

/* Renders rows [row_begin, row_end) of the image with params->spp samples per
 * pixel; image receives width*height*3 radiance sums (rows outside the range
 * are left untouched).  guide may be NULL (unguided). */
void pgo_render_f64(const pgo_scene *s, const pg_render_params *params, const pgo_guide *guide, double *image,
                    uint32_t row_begin, uint32_t row_end, int n_threads);

/* The renderer's shading functions in double precision on the probes of
 * pg_probe_shading (same records and result layout: 8 values per probe). */
void pgo_probe_shading(const pg_material *mats, uint32_t n_mats, const pg_vmm_theta *vmms, uint32_t n_vmms,
                       const pg_shading_probe *probes, uint32_t n, double *out);

/* The renderer's random number (seed, pixel, sample, dimension). */
float pgo_rnd(uint32_t seed, uint32_t pixel, uint32_t sample, uint32_t dim);

#ifdef __cplusplus
}
#endif

#endif
