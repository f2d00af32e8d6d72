// pg_em_k8.cu - instantiations of the EM fit kernel for up to 8 components.
#include "pg_em_kernels.cuh"

namespace pg {

int launch_fit_k8(pg_ctx *ctx, const EmArgs &args, cudaStream_t s, const pg_fit_tuning &t, uint32_t cluster) {
    const uint32_t nt = t.threads_per_cta ? t.threads_per_cta : 128u;
    const uint32_t u = t.unroll ? t.unroll : 2u;
    const uint32_t cps = t.ctas_per_sm;
    if (nt == 256) return u == 2 ? launch_fit<8, 256, 8, 2>(ctx, args, s, cps, cluster)
                                 : launch_fit<8, 256, 8, 1>(ctx, args, s, cps, cluster);
    if (u == 4) return launch_fit<8, 128, 8, 4>(ctx, args, s, cps, cluster);
    return u == 2 ? launch_fit<8, 128, 8, 2>(ctx, args, s, cps, cluster)
                  : launch_fit<8, 128, 8, 1>(ctx, args, s, cps, cluster);
}

}  // namespace pg
