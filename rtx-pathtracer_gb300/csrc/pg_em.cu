// pg_em.cu - host side of the batched EM fit (C ABI entry points), the
// largest-first region ordering and the log-likelihood evaluation kernel.
#include <algorithm>
#include <vector>

#include "pg_em_kernels.cuh"

namespace pg {

// Weighted log-likelihood of each region under its current mixture (FP32
// E-step arithmetic, compensated merge, FP64 result).
template <int KMAX, int NT>
__global__ void __launch_bounds__(NT) em_eval_kernel(EmArgs a) {
    constexpr int NW = NT / 32;
    __shared__ float s_c[5][KMAX];
    __shared__ float s_ll[NW];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (uint32_t r = blockIdx.x; r < a.n_regions; r += gridDim.x) {
        const pg_region_state *st = a.states + r;
        if (tid < KMAX) {
            const int c = tid;
            const float kl = st->kappa[c] * kLog2e;
            const float pn = st->weight[c] * st->norm[c];
            const float lw = (c < (int)st->k && pn > 0.0f) ? log2f(pn) : -INFINITY;
            s_c[0][c] = kl * st->mu_x[c];
            s_c[1][c] = kl * st->mu_y[c];
            s_c[2][c] = kl * st->mu_z[c];
            s_c[3][c] = lw - kl;
            s_c[4][c] = lw;
        }
        __syncthreads();
        const uint32_t b = a.offsets[r], e = a.offsets[r + 1];
        float ll = 0.0f;
        for (uint32_t n = b + tid; n < e; n += NT) {
            const float4 s = __ldg(a.dirw + n);
            float p = 0.0f;
#pragma unroll
            for (int c = 0; c < KMAX; ++c) {
                float t = fmaf(s_c[2][c], s.z, s_c[3][c]);
                t = fmaf(s_c[1][c], s.y, t);
                t = fmaf(s_c[0][c], s.x, t);
                p += ex2_approx(fminf(t, s_c[4][c]));
            }
            if (p > kPmmEps) ll = fmaf(s.w, lg2_approx(p), ll);
        }
        ll = warp_sum(ll);
        if (lane == 0) s_ll[warp] = ll;
        __syncthreads();
        if (tid == 0) {
            float h = 0.0f, cc = 0.0f;
            for (int w = 0; w < NW; ++w) neumaier_add(h, cc, s_ll[w]);
            a.ll_out[r] = ((double)h + (double)cc) * 0.6931471805599453;
        }
        __syncthreads();
    }
}

// Region ids into ctx->d_order, largest sample count first; the number of
// regions in size buckets at or above `large_threshold` into *n_large_out.
int order_regions(pg_ctx *ctx, const uint32_t *offsets, uint32_t n_regions, uint32_t large_threshold,
                  uint32_t *n_large_out, cudaStream_t s) {
    order_regions_kernel<128><<<1, 1024, 0, s>>>(offsets, n_regions, ctx->d_order, large_threshold, n_large_out);
    return check_cuda(ctx, cudaGetLastError(), "order_regions launch");
}

}  // namespace pg

using namespace pg;

extern "C" {

int pg_init_regions(pg_ctx *ctx, uint32_t n_regions, void *stream) {
    if (!ctx) return PG_ERR_ARG;
    if (n_regions > ctx->max_regions) return set_error(ctx, PG_ERR_ARG, "n_regions exceeds context capacity");
    if (n_regions == 0) return PG_OK;
    guide_mark_stale(ctx);
    // All-zero offsets: every region is empty, so only initialisation runs and
    // no sample is read (the sample pointer is never dereferenced).
    int st = pg_fit_regions(ctx, reinterpret_cast<const float *>(ctx->d_init), ctx->d_zero_offsets, n_regions,
                            PG_FIT_INIT, stream);
    // fresh mixtures start with fresh split/merge statistics (PMM_ExtraData{})
    if (!st && ctx->d_extras) st = extras_reset(ctx, 0, n_regions, (cudaStream_t)stream);
    return st;
}

}  // extern "C"

namespace pg {

// The fit of regions [first, first + n_regions): offsets points at region
// first's entry, the states written are first's onwards.
int fit_range(pg_ctx *ctx, const float *dirw, const uint32_t *offsets, uint32_t first, uint32_t n_regions, int mode,
              cudaStream_t s, const HostSamples *host) {
    ctx->last_launches = 0;
    if (n_regions == 0) return PG_OK;
    guide_mark_stale(ctx);
    int st = upload_init_table(ctx, s);
    if (st) return st;
    st = check_cuda(ctx, cudaMemsetAsync(ctx->d_counters, 0, sizeof(uint32_t) * 6, s), "queue reset");
    if (st) return st;
    const pg_fit_tuning &t = ctx->tuning;
    // Defaults: the best point of the tuning sweep on the 4096-region K=16
    // workload (pairs of CTAs share regions above 24576 samples, 4096 samples
    // staged per CTA in a two-stage ring when streamed, one thread per sample,
    // two samples per loop trip, three CTAs per SM).
    const uint32_t cluster = t.cluster_size ? t.cluster_size : 2u;
    const uint32_t cap = t.smem_samples ? t.smem_samples : 4096u;
    const uint32_t large_threshold =
        cluster > 1 ? (t.large_threshold ? t.large_threshold : 24576u) : 0xFFFFFFFFu;
    order_regions_kernel<128><<<1, 1024, 0, s>>>(offsets, n_regions, ctx->d_order, large_threshold, ctx->d_counters + 3,
                                                 ctx->d_states + first);
    st = check_cuda(ctx, cudaGetLastError(), "order_regions launch");
    if (st) return st;
    EmArgs args{};
    args.states = ctx->d_states + first;
    args.dirw = reinterpret_cast<const float4 *>(dirw);
    args.offsets = offsets;
    args.order = ctx->d_order;
    args.n_regions = n_regions;
    args.work_counter = ctx->d_counters;
    args.large_counter = ctx->d_counters + 1;
    args.error_word = ctx->d_counters + 2;
    args.n_large = ctx->d_counters + 3;
    args.init_table = ctx->d_init;
    args.cfg = ctx->cfg;
    args.mode = mode;
    args.ll_out = nullptr;
    args.smem_cap = cap;
    args.stages = t.stream_stages ? t.stream_stages : 2u;
    if (host)
        args.host = *host;
    else
        memset(&args.host, 0, sizeof args.host);
    const uint32_t K = ctx->cfg.num_initial_components;
    // The component count of an existing state is read from the state; size
    // for the widest case unless the mixtures are initialised here.
    const bool wide = (mode == PG_FIT_INIT) ? (K > 8) : true;
    st = wide ? launch_fit_k16(ctx, args, s, t, cluster) : launch_fit_k8(ctx, args, s, t, cluster);
    if (st) return st;
    ctx->last_launches = 2;
    return PG_OK;
}

}  // namespace pg

extern "C" {

int pg_fit_regions(pg_ctx *ctx, const float *dirw, const uint32_t *offsets, uint32_t n_regions, int mode,
                   void *stream) {
    if (!ctx) return PG_ERR_ARG;
    if (!dirw || !offsets) return set_error(ctx, PG_ERR_ARG, "null sample or offset pointer");
    if ((reinterpret_cast<uintptr_t>(dirw) & 15u) != 0) return set_error(ctx, PG_ERR_ARG, "dirw must be 16-byte aligned");
    if (n_regions > ctx->max_regions) return set_error(ctx, PG_ERR_ARG, "n_regions exceeds context capacity");
    if (mode != PG_FIT_INIT && mode != PG_FIT_CONTINUE && mode != PG_FIT_UPDATE)
        return set_error(ctx, PG_ERR_ARG, "unknown fit mode");
    return fit_range(ctx, dirw, offsets, 0, n_regions, mode, (cudaStream_t)stream);
}

int pg_fit_regions_host(pg_ctx *ctx, const float *dirw_host, const uint32_t *offsets_host, uint32_t n_regions,
                        int mode, void *stream) {
    if (!ctx) return PG_ERR_ARG;
    if (!dirw_host || !offsets_host) return set_error(ctx, PG_ERR_ARG, "null sample or offset pointer");
    if (n_regions > ctx->max_regions) return set_error(ctx, PG_ERR_ARG, "n_regions exceeds context capacity");
    if (mode != PG_FIT_INIT && mode != PG_FIT_CONTINUE && mode != PG_FIT_UPDATE)
        return set_error(ctx, PG_ERR_ARG, "unknown fit mode");
    ctx->last_launches = 0;
    if (n_regions == 0) return PG_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const uint64_t total = offsets_host[n_regions];
    // device copies of the samples and offsets, and the copy stream
    if (total > ctx->h2d_cap) {
        cudaFree(ctx->h2d_dirw);
        ctx->h2d_dirw = nullptr;
        ctx->h2d_cap = 0;
        if (int st = check_cuda(ctx, cudaMalloc(&ctx->h2d_dirw, sizeof(float4) * (total ? total : 1)), "host-fit samples"))
            return st;
        ctx->h2d_cap = total;
    }
    if (!ctx->h2d_offsets) {
        if (int st = check_cuda(ctx, cudaMalloc(&ctx->h2d_offsets, sizeof(uint32_t) * ((size_t)ctx->max_regions + 1)),
                                "host-fit offsets"))
            return st;
        int st = check_cuda(ctx, cudaStreamCreateWithFlags(&ctx->h2d_stream, cudaStreamNonBlocking), "copy stream");
        for (int i = 0; !st && i < 2; ++i)
            st = check_cuda(ctx, cudaEventCreateWithFlags(&ctx->h2d_events[i], cudaEventDisableTiming), "copy events");
        if (st) return st;
    }
    int st = check_cuda(ctx, cudaMemcpyAsync(ctx->h2d_offsets, offsets_host, sizeof(uint32_t) * (n_regions + 1),
                                             cudaMemcpyHostToDevice, s), "offsets upload");
    if (st) return st;
    // Page-locked samples are read by the fit itself: each CTA reads a region's
    // slice from host memory when it reaches the region, so the transfer follows
    // the fit's own order (largest regions first) and overlaps the rest of the
    // fit; slices above the staging capacity are copied once to the device
    // buffer, from which their iterations stream.
    cudaPointerAttributes pa{};
    const cudaError_t ae = cudaPointerGetAttributes(&pa, dirw_host);
    if (ae != cudaSuccess) (void)cudaGetLastError();
    if (ae == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer &&
        reinterpret_cast<uintptr_t>(pa.devicePointer) % 16u == 0) {  // 16-byte sample loads
        HostSamples hs;
        memset(&hs, 0, sizeof hs);
        hs.mapped = static_cast<const float4 *>(pa.devicePointer);
        hs.pulls = ctx->d_counters + 4;  // zeroed with the fit's queue counters
        return fit_range(ctx, reinterpret_cast<const float *>(ctx->h2d_dirw), ctx->h2d_offsets, 0, n_regions, mode,
                         s, &hs);
    }
    if (!ctx->h2d_ready) {
        st = check_cuda(ctx, cudaMalloc(&ctx->h2d_ready, sizeof(uint32_t) * kMaxArrivalChunks), "arrival flags");
        if (!st) st = check_cuda(ctx, cudaHostAlloc(&ctx->h2d_ones, sizeof(uint32_t) * kMaxArrivalChunks,
                                                    cudaHostAllocDefault),
                                 "arrival flag source");
        if (st) return st;
        for (uint32_t c = 0; c < kMaxArrivalChunks; ++c) ctx->h2d_ones[c] = 1u;
    }
    // Pageable samples travel in chunks cut at region boundaries, the chunks
    // holding the largest regions first (the fit starts with the largest), and
    // the fit runs from the start: each region waits for its chunk's flag, which
    // a 4-byte copy behind the chunk's copy sets.
    HostSamples arr;
    memset(&arr, 0, sizeof arr);
    std::vector<uint32_t> prio;
    {
        const uint32_t C = std::min<uint32_t>(kMaxArrivalChunks, n_regions);
        arr.start[0] = 0;
        uint32_t c = 0, biggest = 0;
        for (uint32_t r = 0; r < n_regions; ++r) {
            biggest = std::max(biggest, offsets_host[r + 1] - offsets_host[r]);
            const bool cut = (uint64_t)offsets_host[r + 1] * C >= (uint64_t)(c + 1) * total;
            if ((cut && c + 1 < C) || r + 1 == n_regions) {
                arr.start[++c] = offsets_host[r + 1];
                prio.push_back(biggest);
                biggest = 0;
            }
        }
        arr.n_chunks = c;
        arr.ready = ctx->h2d_ready;
    }
    std::vector<uint32_t> copy_order(arr.n_chunks);
    for (uint32_t c = 0; c < arr.n_chunks; ++c) copy_order[c] = c;
    std::stable_sort(copy_order.begin(), copy_order.end(), [&](uint32_t x, uint32_t y) { return prio[x] > prio[y]; });
    st = check_cuda(ctx, cudaMemsetAsync(ctx->h2d_ready, 0, sizeof(uint32_t) * kMaxArrivalChunks, s),
                    "arrival flags reset");
    // the copy stream starts after everything queued on the caller's stream
    // (an earlier fit may still read the sample buffer)
    if (!st) st = check_cuda(ctx, cudaEventRecord(ctx->h2d_events[1], s), "copy fork");
    if (!st) st = check_cuda(ctx, cudaStreamWaitEvent(ctx->h2d_stream, ctx->h2d_events[1], 0), "copy fork");
    for (uint32_t k = 0; !st && k < arr.n_chunks; ++k) {
        const uint32_t c = copy_order[k];
        const uint64_t n0 = arr.start[c], n1 = arr.start[c + 1];
        if (n1 > n0)
            st = check_cuda(ctx, cudaMemcpyAsync(ctx->h2d_dirw + n0, reinterpret_cast<const float4 *>(dirw_host) + n0,
                                                 sizeof(float4) * (n1 - n0), cudaMemcpyHostToDevice, ctx->h2d_stream),
                            "samples upload");
        if (!st)
            st = check_cuda(ctx, cudaMemcpyAsync(ctx->h2d_ready + c, ctx->h2d_ones + c, sizeof(uint32_t),
                                                 cudaMemcpyHostToDevice, ctx->h2d_stream),
                            "arrival flag");
    }
    if (!st) st = check_cuda(ctx, cudaEventRecord(ctx->h2d_events[0], ctx->h2d_stream), "copy event");
    if (st) return st;
    st = fit_range(ctx, reinterpret_cast<const float *>(ctx->h2d_dirw), ctx->h2d_offsets, 0, n_regions, mode, s, &arr);
    // work queued behind the fit also waits for every copy (a chunk no region waited on included)
    if (!st) st = check_cuda(ctx, cudaStreamWaitEvent(s, ctx->h2d_events[0], 0), "copy join");
    return st;
}

int pg_eval_loglik(pg_ctx *ctx, const float *dirw, const uint32_t *offsets, uint32_t n_regions, double *ll_out,
                   void *stream) {
    if (!ctx) return PG_ERR_ARG;
    if (!dirw || !offsets || !ll_out) return set_error(ctx, PG_ERR_ARG, "null pointer");
    if (n_regions > ctx->max_regions) return set_error(ctx, PG_ERR_ARG, "n_regions exceeds context capacity");
    if (n_regions == 0) return PG_OK;
    cudaStream_t s = (cudaStream_t)stream;
    EmArgs args{};
    args.states = ctx->d_states;
    args.dirw = reinterpret_cast<const float4 *>(dirw);
    args.offsets = offsets;
    args.n_regions = n_regions;
    args.ll_out = ll_out;
    const uint32_t grid = std::min<uint32_t>(n_regions, (uint32_t)ctx->sm_count * 8u);
    em_eval_kernel<16, 256><<<grid, 256, 0, s>>>(args);
    return check_cuda(ctx, cudaGetLastError(), "em_eval launch");
}

}  // extern "C"
