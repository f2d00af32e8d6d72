// pg_fit_graph.cu - the fit's autotuner and its CUDA-graph form.
//
// The autotuner times pg_fit_regions on the caller's samples for each
// candidate launch shape and keeps the fastest; the graph form captures one
// pg_fit_regions (ordering kernel + clustered persistent fit) so a guiding
// pass replays it with one launch call.
#include <float.h>
#include <string.h>

#include <vector>

#include "pg_internal.cuh"

struct pg_fit_graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    pg_ctx *ctx = nullptr;  // whose states a replay refits
};

namespace {

std::vector<pg_fit_tuning> default_grid() {
    // (CTAs per SM, components per thread, samples per trip, staged samples):
    // 3 and 4 CTAs per SM are the register-capped builds, 2 the unrestricted one.
    struct Shape {
        uint32_t cps, cpt, unroll, cap;
    };
    const Shape shapes[] = {{3, 16, 2, 4096}, {3, 16, 2, 3072}, {4, 16, 2, 3072}, {2, 16, 2, 6144}, {4, 8, 4, 3072}};
    std::vector<pg_fit_tuning> g;
    for (const Shape &sh : shapes)
        for (uint32_t cl : {1u, 2u, 4u})
            for (uint32_t large : {12288u, 24576u}) {
                if (cl == 1 && large != 12288u) continue;  // no cluster: the threshold is unused
                pg_fit_tuning t{};
                t.threads_per_cta = 128;
                t.ctas_per_sm = sh.cps;
                t.components_per_thread = sh.cpt;
                t.unroll = sh.unroll;
                t.smem_samples = sh.cap;
                t.cluster_size = cl;
                t.large_threshold = large;
                t.stream_stages = 2;
                g.push_back(t);
            }
    return g;
}

}  // namespace

extern "C" {

int pg_autotune_fit(pg_ctx *ctx, const float *dirw, const uint32_t *offsets, uint32_t n_regions, int mode,
                    const pg_fit_tuning *candidates, uint32_t n_candidates, pg_fit_tuning *best_out,
                    float *best_ms_out, void *stream) {
    using namespace pg;
    if (!ctx || !dirw || !offsets || (candidates && n_candidates == 0)) return PG_ERR_ARG;
    if (n_regions == 0 || n_regions > ctx->max_regions) return set_error(ctx, PG_ERR_ARG, "bad region count");
    cudaStream_t s = (cudaStream_t)stream;
    const std::vector<pg_fit_tuning> grid =
        candidates ? std::vector<pg_fit_tuning>(candidates, candidates + n_candidates) : default_grid();
    const pg_fit_tuning saved_tuning = ctx->tuning;
    const size_t state_bytes = sizeof(pg_region_state) * (size_t)n_regions;
    pg_region_state *saved = nullptr;
    if (int st = check_cuda(ctx, cudaMalloc(&saved, state_bytes), "autotune state copy")) return st;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int st = check_cuda(ctx, cudaEventCreate(&e0), "event");
    if (!st) st = check_cuda(ctx, cudaEventCreate(&e1), "event");
    if (!st) st = check_cuda(ctx, cudaMemcpyAsync(saved, ctx->d_states, state_bytes, cudaMemcpyDeviceToDevice, s),
                             "state save");
    float best_ms = FLT_MAX;
    pg_fit_tuning best = saved_tuning;
    for (size_t i = 0; !st && i < grid.size(); ++i) {
        if (pg_set_fit_tuning(ctx, &grid[i]) != PG_OK) continue;
        float total = 0.0f;
        bool ok = true;
        for (int rep = 0; rep < 3 && ok; ++rep) {  // first run warms up
            if (cudaMemcpyAsync(ctx->d_states, saved, state_bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
                st = set_error(ctx, PG_ERR_CUDA, "state restore");
                break;
            }
            cudaEventRecord(e0, s);
            ok = pg_fit_regions(ctx, dirw, offsets, n_regions, mode, s) == PG_OK;
            cudaEventRecord(e1, s);
            if (!ok) break;
            if (cudaEventSynchronize(e1) != cudaSuccess) {
                st = set_error(ctx, PG_ERR_CUDA, "autotune run");
                break;
            }
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0) total += ms;
        }
        if (!ok) {
            cudaGetLastError();  // a shape the device cannot launch: skip it
            continue;
        }
        if (!st && total / 2.0f < best_ms) {
            best_ms = total / 2.0f;
            best = grid[i];
        }
    }
    if (!st) st = check_cuda(ctx, cudaMemcpyAsync(ctx->d_states, saved, state_bytes, cudaMemcpyDeviceToDevice, s),
                             "state restore");
    if (!st) st = check_cuda(ctx, cudaStreamSynchronize(s), "autotune sync");
    if (!st && best_ms == FLT_MAX) st = set_error(ctx, PG_ERR_ARG, "no candidate tuning could be launched");
    ctx->tuning = st ? saved_tuning : best;
    if (!st) {
        if (best_out) *best_out = best;
        if (best_ms_out) *best_ms_out = best_ms;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(saved);
    // the error word may carry flags from the trial runs (e.g. numeric ones); clear it
    cudaMemset(ctx->d_counters + 2, 0, sizeof(uint32_t));
    return st;
}

int pg_fit_graph_create(pg_ctx *ctx, const float *dirw, const uint32_t *offsets, uint32_t n_regions, int mode,
                        void *stream, pg_fit_graph **out) {
    using namespace pg;
    if (!ctx || !out) return PG_ERR_ARG;
    if (!stream) return set_error(ctx, PG_ERR_ARG, "capture needs a non-default stream");
    cudaStream_t s = (cudaStream_t)stream;
    // the initial-mixture table may need an upload (and a synchronisation): do it before the capture
    if (int st = upload_init_table(ctx, s)) return st;
    if (int st = check_cuda(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed), "begin capture")) return st;
    const int fit = pg_fit_regions(ctx, dirw, offsets, n_regions, mode, stream);
    cudaGraph_t graph = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (fit != PG_OK) {
        if (graph) cudaGraphDestroy(graph);
        return fit;
    }
    if (ce != cudaSuccess || !graph) return set_error(ctx, PG_ERR_CUDA, "stream capture of the fit failed");
    pg_fit_graph *g = new pg_fit_graph();
    g->graph = graph;
    g->ctx = ctx;
    if (cudaGraphInstantiate(&g->exec, graph, 0) != cudaSuccess) {
        cudaGraphDestroy(graph);
        delete g;
        return set_error(ctx, PG_ERR_CUDA, "graph instantiation failed");
    }
    *out = g;
    return PG_OK;
}

int pg_fit_graph_launch(pg_fit_graph *g, void *stream) {
    if (!g || !g->exec) return PG_ERR_ARG;
    pg::guide_mark_stale(g->ctx);
    return cudaGraphLaunch(g->exec, (cudaStream_t)stream) == cudaSuccess
               ? PG_OK
               : pg::set_error(nullptr, PG_ERR_CUDA, "graph launch failed");
}

int pg_fit_graph_destroy(pg_fit_graph *g) {
    if (!g) return PG_OK;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return PG_OK;
}

}  // extern "C"
