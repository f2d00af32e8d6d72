// pg_internal.cuh - shared declarations of the CUDA library (context, error
// reporting, small device helpers written as inline PTX).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "pathguide.h"

static_assert(sizeof(pg_region_state) == 704, "pg_region_state layout");
static_assert(sizeof(pg_directional_data) == 40, "DirectionalData layout");
static_assert(sizeof(pg_vmm_theta) == 720, "VMM_Theta layout");
static_assert(sizeof(pg_region_extra) == 400, "pg_region_extra layout");

// Device-side error word bits (ORed by kernels, read back by the host).
#define PG_DEV_ERR_TIMEOUT 1u   // a bounded wait ran out
#define PG_DEV_ERR_NUMERIC 2u   // non-finite parameter produced
#define PG_DEV_ERR_BOUNDS 4u    // an index check failed (access skipped)

struct pg_ctx {
    int device = 0;
    int sm_count = 0;
    pg_fit_config cfg{};
    pg_fit_tuning tuning{};
    uint32_t max_regions = 0;
    uint64_t max_samples = 0;
    pg_region_state *d_states = nullptr;
    uint32_t *d_order = nullptr;     // region ids, largest sample count first
    uint32_t *d_counters = nullptr;  // [0] fit work queue, [1] eval queue, [2] error word, ...
    float *d_init = nullptr;         // initial means x[16] y[16] z[16], initial r[16]
    uint32_t *d_zero_offsets = nullptr;  // max_regions+1 zeros (initialisation-only fits)
    uint32_t init_k = 0;             // K the table was computed for
    float init_kappa = -1.0f;
    uint32_t last_launches = 0;
    void *guide = nullptr;           // sort / parallax / distance scratch (pg_guide.cu)
    // pg_fit_regions_host: device copies of host samples (streamed slices of page-locked
    // samples, or every sample of pageable ones, filled on a copy stream)
    float4 *h2d_dirw = nullptr;
    uint64_t h2d_cap = 0;
    uint32_t *h2d_offsets = nullptr;
    cudaStream_t h2d_stream = nullptr;
    cudaEvent_t h2d_events[2] = {nullptr, nullptr};  // copy done, caller's stream fork
    uint32_t *h2d_ready = nullptr;                     // per chunk: its samples are in place (device)
    uint32_t *h2d_ones = nullptr;                      // page-locked source of the ready flags
    pg_region_extra *d_extras = nullptr;  // split/merge statistics per region (pg_splitmerge.cu)
    cudaStream_t sm_aux = nullptr;        // split/merge: the clustered launch runs beside the per-CTA one
    cudaEvent_t sm_fork = nullptr, sm_join = nullptr;
    pg_split_merge_config sm{};      // disabled unless pg_set_split_merge
    std::string last_error;
};

namespace pg {

int set_error(pg_ctx *ctx, int status, const std::string &msg);
int check_cuda(pg_ctx *ctx, cudaError_t e, const char *what);
int upload_init_table(pg_ctx *ctx, cudaStream_t s);
// Samples of a fit that start in host memory.  mapped non-null: page-locked
// host samples at this device address, read by each CTA as it reaches a region
// (slices above the staging capacity are first copied to the same offsets of
// the device sample buffer).  ready non-null: the samples are being copied to
// the device buffer in chunks; chunk c, samples [start[c], start[c + 1]) (region
// boundaries), is in place once ready[c] != 0.
constexpr uint32_t kMaxArrivalChunks = 16;
struct HostSamples {
    const float4 *mapped;
    uint32_t *pulls;  // mapped: [0] tickets handed out, [1] slices read (device counters, zeroed per fit)
    const uint32_t *ready;
    uint32_t n_chunks;
    uint32_t start[kMaxArrivalChunks + 1];
};
int fit_range(pg_ctx *ctx, const float *dirw, const uint32_t *offsets, uint32_t first, uint32_t n_regions, int mode,
              cudaStream_t s, const HostSamples *host = nullptr);
// region ids into ctx->d_order, largest sample count first; *n_large_out
// (device) = regions in size buckets at or above large_threshold
int order_regions(pg_ctx *ctx, const uint32_t *offsets, uint32_t n_regions, uint32_t large_threshold,
                  uint32_t *n_large_out, cudaStream_t s);
void guide_release(pg_ctx *ctx);
// The packed guide (VMM_Theta) is repacked from the states before the next
// guided render: called by every call that changes mixture states.
void guide_mark_stale(pg_ctx *ctx);
// split/merge statistics: allocated (zeroed) on first use, zeroed again when
// regions are initialised
int extras_ensure(pg_ctx *ctx, cudaStream_t s);
void extras_release(pg_ctx *ctx);
int extras_reset(pg_ctx *ctx, uint32_t first, uint32_t n, cudaStream_t s);

// What the renderer needs from a guiding context: the padded root box and
// split count of the region tree (point -> region by descent) and the packed
// VMM_Theta of every region.
struct GuideView {
    float root[6];
    uint32_t split_count;
    const int32_t *nodes;  // the region tree once a region was split (else null: complete tree)
    uint32_t n_regions;
    const pg_vmm_theta *vmm;
    int use_parallax;
};
int guide_view(pg_ctx *ctx, GuideView *out, cudaStream_t s);
// The packed-guide buffer and region boxes of a context, for guides computed
// elsewhere (the learned surrogate); guide_mark_written keeps what was written
// until the next pg_update or pg_set_regions.
struct GuideTarget {
    const float *aabbs;
    uint32_t n_regions;
    pg_vmm_theta *vmm;
};
int guide_target(pg_ctx *ctx, GuideTarget *out);
void guide_mark_written(pg_ctx *ctx);

constexpr float kLog2e = 1.4426950408889634f;
constexpr float kLn2 = 0.6931471805599453f;
constexpr float kInv4Pi = 0.0795774715459476679f;
constexpr float kTwoPi = 6.2831853071795865f;
constexpr float kPmmEps = 1.0e-8f;      // PMM_EPSILON (pmm.h:40)
constexpr float kVmfMinKappa = 1e-3f;   // VMF_MinKappa (VMFKernel.h:42)

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float lg2_approx(float x) {
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// mbarrier + 1-D TMA bulk copy (cp.async.bulk) helpers.
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_global() {
    asm volatile("fence.proxy.async.global;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void tma_bulk_g2s(void *smem_dst, const void *gmem_src, uint32_t bytes,
                                             uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(smem_dst)),
        "l"(gmem_src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait on an mbarrier phase: gives up after `max_cycles` SM clocks
// and reports PG_DEV_ERR_TIMEOUT instead of spinning forever.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t *err,
                                                  long long max_cycles = 4000000000LL) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > max_cycles) {
            atomicOr(err, PG_DEV_ERR_TIMEOUT);
            return false;
        }
    }
    return true;
}

// Neumaier compensated accumulation of x into (s, c).
__device__ __forceinline__ void neumaier_add(float &s, float &c, float x) {
    const float t = s + x;
    if (fabsf(s) >= fabsf(x))
        c += (s - t) + x;
    else
        c += (x - t) + s;
    s = t;
}

}  // namespace pg
