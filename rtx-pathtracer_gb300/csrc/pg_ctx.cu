// pg_ctx.cu - context lifetime, errors, mixture-state transfer and the
// initial-mixture table (the C-ABI entry points of include/pathguide.h that do
// not launch the fit).
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <string>

#include "pg_internal.cuh"

namespace {
thread_local std::string g_last_error;
}

namespace pg {

int set_error(pg_ctx *ctx, int status, const std::string &msg) {
    if (ctx)
        ctx->last_error = msg;
    else
        g_last_error = msg;
    return status;
}

int check_cuda(pg_ctx *ctx, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return PG_OK;
    return set_error(ctx, PG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// The initial means of VMMFactory::initialize (VMMFactory.h:594-632, l = K-1),
// evaluated with the reference's float arithmetic, and the initial mean cosine
// coth(kappa) - 1/kappa (VMFKernel.h:47-55) in double.
int upload_init_table(pg_ctx *ctx, cudaStream_t s) {
    const uint32_t K = ctx->cfg.num_initial_components;
    const float kap = ctx->cfg.init_kappa;
    if (ctx->init_k == K && ctx->init_kappa == kap) return PG_OK;
    float t[64];
    const float gr = 1.618033988749895f;
    for (uint32_t n = 0; n < 16; ++n) {
        float x = 0.0f, y = 0.0f, z = 1.0f;
        if (n < K) {
            const float phi = (float)(2.0f * M_PI * (double)((float)n / gr));
            const float zz = 1.0f - ((2.0f * (float)n + 1.0f) / (float)K);
            const float theta = acosf(zz);
            const float st = sinf(theta);
            x = st * cosf(phi);
            y = st * sinf(phi);
            z = cosf(theta);
        }
        t[n] = x;
        t[16 + n] = y;
        t[32 + n] = z;
        const double kd = kap < 1e-3f ? 0.0 : (double)kap;
        t[48 + n] = kd > 0.0 ? (float)(1.0 / tanh(kd) - 1.0 / kd) : 0.0f;
    }
    int st = check_cuda(ctx, cudaMemcpyAsync(ctx->d_init, t, sizeof(t), cudaMemcpyHostToDevice, s),
                        "init table upload");
    if (st) return st;
    st = check_cuda(ctx, cudaStreamSynchronize(s), "init table sync");
    if (st) return st;
    ctx->init_k = K;
    ctx->init_kappa = kap;
    return PG_OK;
}

}  // namespace pg

using namespace pg;

extern "C" {

void pg_default_fit_config(pg_fit_config *c) {
    if (!c) return;
    c->min_itr = 1;
    c->max_itr = 100;
    c->rel_ll_threshold = 0.005f;
    c->num_initial_components = 8;
    c->init_kappa = 5.0f;
    c->max_kappa = 50000.0f;
    c->v_prior = 0.01f;
    c->r_prior = 0.0f;
    c->r_prior_weight = 1.0f;
    c->use_parallax = 1;
}

static int validate_cfg(pg_ctx *ctx, const pg_fit_config *c) {
    if (!c) return set_error(ctx, PG_ERR_ARG, "null fit config");
    if (c->num_initial_components < 1 || c->num_initial_components > PG_MAX_COMPONENTS)
        return set_error(ctx, PG_ERR_ARG, "num_initial_components must be in [1, 16]");
    if (!(c->max_kappa > 0.0f)) return set_error(ctx, PG_ERR_ARG, "max_kappa must be > 0");
    if (!(c->r_prior_weight >= 0.0f) || !(c->v_prior >= 0.0f))
        return set_error(ctx, PG_ERR_ARG, "priors must be >= 0");
    return PG_OK;
}

int pg_ctx_create(const pg_fit_config *cfg, uint32_t max_regions, uint64_t max_samples, pg_ctx **out) {
    if (!out) return set_error(nullptr, PG_ERR_ARG, "null output pointer");
    *out = nullptr;
    int st = validate_cfg(nullptr, cfg);
    if (st) return st;
    if (max_regions == 0) return set_error(nullptr, PG_ERR_ARG, "max_regions must be > 0");
    pg_ctx *ctx = new pg_ctx();
    ctx->cfg = *cfg;
    ctx->max_regions = max_regions;
    ctx->max_samples = max_samples;
    cudaError_t e = cudaGetDevice(&ctx->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, ctx->device);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_states, sizeof(pg_region_state) * (size_t)max_regions);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_order, sizeof(uint32_t) * (size_t)max_regions);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_counters, sizeof(uint32_t) * 64);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_init, sizeof(float) * 64);
    if (e == cudaSuccess) e = cudaMemset(ctx->d_counters, 0, sizeof(uint32_t) * 64);
    if (e == cudaSuccess) e = cudaMemset(ctx->d_states, 0, sizeof(pg_region_state) * (size_t)max_regions);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_zero_offsets, sizeof(uint32_t) * ((size_t)max_regions + 1));
    if (e == cudaSuccess) e = cudaMemset(ctx->d_zero_offsets, 0, sizeof(uint32_t) * ((size_t)max_regions + 1));
    if (e != cudaSuccess) {
        set_error(nullptr, PG_ERR_CUDA, std::string("pg_ctx_create: ") + cudaGetErrorString(e));
        pg_ctx_destroy(ctx);
        return PG_ERR_CUDA;
    }
    *out = ctx;
    return PG_OK;
}

int pg_ctx_destroy(pg_ctx *ctx) {
    if (!ctx) return PG_OK;
    guide_release(ctx);
    extras_release(ctx);
    cudaFree(ctx->h2d_dirw);
    cudaFree(ctx->h2d_offsets);
    cudaFree(ctx->h2d_ready);
    if (ctx->h2d_ones) cudaFreeHost(ctx->h2d_ones);
    if (ctx->h2d_stream) cudaStreamDestroy(ctx->h2d_stream);
    for (cudaEvent_t e : ctx->h2d_events)
        if (e) cudaEventDestroy(e);
    cudaFree(ctx->d_states);
    cudaFree(ctx->d_order);
    cudaFree(ctx->d_counters);
    cudaFree(ctx->d_init);
    cudaFree(ctx->d_zero_offsets);
    delete ctx;
    return PG_OK;
}

const char *pg_last_error(const pg_ctx *ctx) {
    return ctx ? ctx->last_error.c_str() : g_last_error.c_str();
}

const char *pg_status_string(int status) {
    switch (status) {
        case PG_OK: return "PG_OK";
        case PG_ERR_ARG: return "PG_ERR_ARG";
        case PG_ERR_CUDA: return "PG_ERR_CUDA";
        case PG_ERR_TIMEOUT: return "PG_ERR_TIMEOUT";
        case PG_ERR_NUMERIC: return "PG_ERR_NUMERIC";
        case PG_ERR_NOMEM: return "PG_ERR_NOMEM";
        case PG_ERR_IO: return "PG_ERR_IO";
        case PG_ERR_PARSE: return "PG_ERR_PARSE";
        case PG_ERR_STATE: return "PG_ERR_STATE";
        default: return "PG_ERR_UNKNOWN";
    }
}

int pg_get_fit_config(const pg_ctx *ctx, pg_fit_config *out) {
    if (!ctx || !out) return PG_ERR_ARG;
    *out = ctx->cfg;
    return PG_OK;
}

int pg_set_fit_config(pg_ctx *ctx, const pg_fit_config *cfg) {
    if (!ctx) return PG_ERR_ARG;
    int st = validate_cfg(ctx, cfg);
    if (st) return st;
    ctx->cfg = *cfg;
    return PG_OK;
}

int pg_get_region_states(pg_ctx *ctx, pg_region_state *host_out, uint32_t first, uint32_t count,
                         void *stream) {
    if (!ctx || (!host_out && count)) return PG_ERR_ARG;
    if ((uint64_t)first + count > ctx->max_regions) return set_error(ctx, PG_ERR_ARG, "region range out of bounds");
    cudaStream_t s = (cudaStream_t)stream;
    int st = check_cuda(ctx,
                        cudaMemcpyAsync(host_out, ctx->d_states + first, sizeof(pg_region_state) * (size_t)count,
                                        cudaMemcpyDeviceToHost, s),
                        "state download");
    if (st) return st;
    return check_cuda(ctx, cudaStreamSynchronize(s), "state download sync");
}

int pg_set_region_states(pg_ctx *ctx, const pg_region_state *host_in, uint32_t first, uint32_t count,
                         void *stream) {
    if (!ctx || (!host_in && count)) return PG_ERR_ARG;
    if ((uint64_t)first + count > ctx->max_regions) return set_error(ctx, PG_ERR_ARG, "region range out of bounds");
    cudaStream_t s = (cudaStream_t)stream;
    guide_mark_stale(ctx);
    int st = check_cuda(ctx,
                        cudaMemcpyAsync(ctx->d_states + first, host_in, sizeof(pg_region_state) * (size_t)count,
                                        cudaMemcpyHostToDevice, s),
                        "state upload");
    if (st) return st;
    return check_cuda(ctx, cudaStreamSynchronize(s), "state upload sync");
}

int pg_region_states_device(pg_ctx *ctx, pg_region_state **dev_out) {
    if (!ctx || !dev_out) return PG_ERR_ARG;
    *dev_out = ctx->d_states;
    return PG_OK;
}

int pg_set_fit_tuning(pg_ctx *ctx, const pg_fit_tuning *t) {
    if (!ctx || !t) return PG_ERR_ARG;
    if (t->threads_per_cta && t->threads_per_cta != 128 && t->threads_per_cta != 256)
        return set_error(ctx, PG_ERR_ARG, "threads_per_cta must be 128 or 256");
    if (t->ctas_per_sm > 32) return set_error(ctx, PG_ERR_ARG, "ctas_per_sm must be <= 32");
    if (t->smem_samples > 13000) return set_error(ctx, PG_ERR_ARG, "smem_samples must be <= 13000");
    if (t->cluster_size > 16) return set_error(ctx, PG_ERR_ARG, "cluster_size must be <= 16");
    if (t->components_per_thread && t->components_per_thread != 8 && t->components_per_thread != 16)
        return set_error(ctx, PG_ERR_ARG, "components_per_thread must be 8 or 16");
    if (t->unroll > 2 && t->unroll != 4) return set_error(ctx, PG_ERR_ARG, "unroll must be 1, 2 or 4");
    if (t->unroll == 4 && t->threads_per_cta && t->threads_per_cta != 128)
        return set_error(ctx, PG_ERR_ARG, "unroll 4 needs 128 threads per CTA");
    if (t->stream_stages > 8) return set_error(ctx, PG_ERR_ARG, "stream_stages must be <= 8");
    ctx->tuning = *t;
    return PG_OK;
}

int pg_get_fit_tuning(const pg_ctx *ctx, pg_fit_tuning *t) {
    if (!ctx || !t) return PG_ERR_ARG;
    *t = ctx->tuning;
    return PG_OK;
}

int pg_sync_status(pg_ctx *ctx, void *stream) {
    if (!ctx) return PG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    int st = check_cuda(ctx, cudaStreamSynchronize(s), "stream sync");
    if (st) return st;
    uint32_t err = 0;
    st = check_cuda(ctx, cudaMemcpy(&err, ctx->d_counters + 2, sizeof(err), cudaMemcpyDeviceToHost), "error word");
    if (st) return st;
    if (err & PG_DEV_ERR_TIMEOUT) return set_error(ctx, PG_ERR_TIMEOUT, "a bounded device wait ran out");
    if (err & PG_DEV_ERR_BOUNDS) return set_error(ctx, PG_ERR_ARG, "a device index check failed");
    if (err & PG_DEV_ERR_NUMERIC) return set_error(ctx, PG_ERR_NUMERIC, "a fit produced a non-finite parameter");
    return PG_OK;
}

int pg_last_launch_count(const pg_ctx *ctx, uint32_t *count) {
    if (!ctx || !count) return PG_ERR_ARG;
    *count = ctx->last_launches;
    return PG_OK;
}

}  // extern "C"
