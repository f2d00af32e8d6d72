// pg_noalloc.cu - pg_fit_regions_noalloc: the batched EM fit for callers that
// cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: a renderer that
// hands out all device memory from its own arena and forbids other allocators
// (a second allocator fragments the arena and breaks its accounting), or a
// plugin host that gives the guiding step only the buffers it owns and no
// allocation rights of its own.  pg_ctx_create allocates the fit's
// scratch (work-queue counters, the largest-first region order and the initial
// mixture table), so those callers cannot use pg_fit_regions.  This entry point
// runs the same fit kernel with its scratch in one file-scope device array
// instead, and takes the mixture states as a caller-owned device buffer.
//
// The array holds at most PG_NOALLOC_MAX_REGIONS region ids.  Every GPU that
// loads the library keeps it (about 257 KB) until the process exits.  Every
// call shares it and it keeps the last call's contents; the counters that must
// start at zero are cleared on the caller's stream at the start of each call.
// Two calls whose work overlaps on the GPU (different streams, no ordering)
// race on the array and give wrong results: order them on one stream or with
// events.
//
// Nothing of a call goes through host memory: the initial mixture table
// travels as a kernel argument, and a bounded wait that ran out or a failed
// index check inside the fit is reported in the caller's states
// (PG_STATE_FIT_FAILED on every region of the call) by a last small kernel.
#include <atomic>

#include "pg_em_kernels.cuh"

namespace {

struct InitTable {
    float v[64];  // initial means x[16] y[16] z[16], initial mean cosines[16]
};

struct NoAllocScratch {
    uint32_t counters[64];                     // work queues, error word, cluster count
    float init_table[64];                      // initial means and mean cosines
    uint32_t order[PG_NOALLOC_MAX_REGIONS];    // region ids, largest first
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Device address of g_noalloc_scratch per device ordinal.  In host code the
// name g_noalloc_scratch is only a host-side stand-in for the symbol; the
// address kernels may use comes from cudaGetSymbolAddress with the device
// current, once per device.
constexpr int kMaxDevices = 64;
std::atomic<NoAllocScratch *> g_scratch_ptr[kMaxDevices];

int scratch_for_current_device(NoAllocScratch **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return PG_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return PG_ERR_ARG;
    NoAllocScratch *p = g_scratch_ptr[dev].load(std::memory_order_acquire);
    if (!p) {
        void *addr = nullptr;
        if (cudaGetSymbolAddress(&addr, g_noalloc_scratch) != cudaSuccess || !addr) return PG_ERR_CUDA;
        p = static_cast<NoAllocScratch *>(addr);
        g_scratch_ptr[dev].store(p, std::memory_order_release);
    }
    *out = p;
    return PG_OK;
}

// The initial mixture table of VMMFactory::initialize (VMMFactory.h:594-632) in
// the same arithmetic as the context path.
void initial_table(uint32_t K, float kap, float *t) {
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
}

// Clears the work counters and error word and stores the initial table; the
// table is a kernel argument, so the launch copies it and no host buffer has to
// outlive the call.
__global__ void noalloc_prepare_kernel(InitTable table, NoAllocScratch *scr) {
    const int t = threadIdx.x;
    if (t < 64) {
        scr->counters[t] = 0u;
        scr->init_table[t] = table.v[t];
    }
}

// Maps the fit's device error word into the states of the call: a wait that
// ran out or a failed index check leaves regions unfitted or partly fitted, so
// every region of the call is marked; a clean call clears the mark.
// Non-finite parameters are flagged per region by the fit itself.
__global__ void noalloc_finish_kernel(pg_region_state *states, uint32_t n_regions, const uint32_t *error_word) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_regions) return;
    const bool failed = (*error_word & (PG_DEV_ERR_TIMEOUT | PG_DEV_ERR_BOUNDS)) != 0u;
    const uint32_t f = states[r].flags;
    states[r].flags = failed ? (f | PG_STATE_FIT_FAILED) : (f & ~PG_STATE_FIT_FAILED);
}

// K <= 16: the register-capped build at three CTAs per SM (E-step constants in
// shared memory); K <= 8: the unrestricted build.
template <int KMAX, int MINB, bool SC>
int launch_noalloc(const pg::EmArgs &args, cudaStream_t s, uint32_t cluster, uint32_t smem_cap, int sm_count) {
    using namespace pg;
    constexpr int NT = 128;
    constexpr int CPT = KMAX;
    constexpr int U = 2;
    auto kern = em_fit_kernel<KMAX, NT, true, CPT, U, MINB, SC>;
    pg::EmArgs a = args;
    a.smem_cap = smem_cap;
    ring_shape(a, (uint32_t)NT * U);
    const size_t smem = fit_smem_bytes<KMAX, NT>(a.smem_cap);
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return PG_ERR_CUDA;
    cudaLaunchConfig_t lc = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    lc.blockDim = dim3(NT, 1, 1);
    lc.dynamicSmemBytes = smem;
    lc.stream = s;
    lc.attrs = attr;
    lc.numAttrs = 1;
    lc.gridDim = dim3(cluster * (uint32_t)sm_count, 1, 1);
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, kern, &lc) != cudaSuccess || nclusters < 1) return PG_ERR_CUDA;
    lc.gridDim = dim3((uint32_t)nclusters * cluster, 1, 1);
    return cudaLaunchKernelEx(&lc, kern, a) == cudaSuccess ? PG_OK : PG_ERR_CUDA;
}

}  // namespace

extern "C" int pg_fit_regions_noalloc(const pg_fit_config *cfg, pg_region_state *states, const float *dirw,
                                      const uint32_t *offsets, uint32_t n_regions, int mode, void *stream) {
    using namespace pg;
    if (!cfg || !states || !dirw || !offsets) return PG_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(dirw) & 15u) != 0) return PG_ERR_ARG;
    if (n_regions > PG_NOALLOC_MAX_REGIONS) return PG_ERR_NOMEM;
    if (mode != PG_FIT_INIT && mode != PG_FIT_CONTINUE && mode != PG_FIT_UPDATE) return PG_ERR_ARG;
    if (cfg->num_initial_components < 1 || cfg->num_initial_components > PG_MAX_COMPONENTS) return PG_ERR_ARG;
    if (!(cfg->max_kappa > 0.0f)) return PG_ERR_ARG;
    if (n_regions == 0) return PG_OK;
    NoAllocScratch *scr = nullptr;
    int st = scratch_for_current_device(&scr);
    if (st) return st;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return PG_ERR_CUDA;
    cudaStream_t s = (cudaStream_t)stream;
    // Work queues and the error word start at zero, the initial table is
    // rewritten (by value: no host buffer), and the order is rewritten below.
    InitTable table;
    initial_table(cfg->num_initial_components, cfg->init_kappa, table.v);
    noalloc_prepare_kernel<<<1, 64, 0, s>>>(table, scr);
    if (cudaGetLastError() != cudaSuccess) return PG_ERR_CUDA;
    const uint32_t cluster = 2u, cap = 4096u, large_threshold = 24576u;
    order_regions_kernel<128><<<1, 1024, 0, s>>>(offsets, n_regions, scr->order, large_threshold, scr->counters + 3,
                                                 states);
    if (cudaGetLastError() != cudaSuccess) return PG_ERR_CUDA;
    EmArgs args{};
    args.states = states;
    args.dirw = reinterpret_cast<const float4 *>(dirw);
    args.offsets = offsets;
    args.order = scr->order;
    args.n_regions = n_regions;
    args.work_counter = scr->counters;
    args.large_counter = scr->counters + 1;
    args.error_word = scr->counters + 2;
    args.n_large = scr->counters + 3;
    args.init_table = scr->init_table;
    args.cfg = *cfg;
    args.mode = mode;
    args.smem_cap = cap;
    args.ll_out = nullptr;
    args.stages = 2u;
    const bool wide = (mode == PG_FIT_INIT) ? (cfg->num_initial_components > 8) : true;
    st = wide ? launch_noalloc<16, 3, true>(args, s, cluster, cap, sms)
              : launch_noalloc<8, 0, false>(args, s, cluster, cap, sms);
    if (st) return st;
    noalloc_finish_kernel<<<(n_regions + 255) / 256, 256, 0, s>>>(states, n_regions, scr->counters + 2);
    return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ERR_CUDA;
}
