// pg_em_k16.cu - instantiations of the EM fit kernel for up to 16 components.
#include "pg_em_kernels.cuh"

namespace pg {

// Launch shapes: 128 or 256 threads; one thread per sample (16 components per
// thread) or a pair (8 each); 1, 2 or 4 samples per loop trip.  With 128
// threads, ctas_per_sm 3 and 4 select builds whose registers are capped so that
// as many CTAs fit on an SM; with one thread per sample those read the E-step
// constants from shared memory.
int launch_fit_k16(pg_ctx *ctx, const EmArgs &args, cudaStream_t s, const pg_fit_tuning &t, uint32_t cluster) {
    const uint32_t nt = t.threads_per_cta ? t.threads_per_cta : 128u;
    const uint32_t cpt = t.components_per_thread ? t.components_per_thread : 16u;
    const uint32_t u = t.unroll ? t.unroll : 2u;
    // Unset: the register-capped build at three CTAs per SM for the default shape.
    const uint32_t cps = t.ctas_per_sm ? t.ctas_per_sm : ((nt == 128 && cpt == 16 && u == 2) ? 3u : 0u);
    if (nt == 256) {
        if (cpt == 16) return u == 2 ? launch_fit<16, 256, 16, 2>(ctx, args, s, cps, cluster)
                                     : launch_fit<16, 256, 16, 1>(ctx, args, s, cps, cluster);
        return u == 2 ? launch_fit<16, 256, 8, 2>(ctx, args, s, cps, cluster)
                      : launch_fit<16, 256, 8, 1>(ctx, args, s, cps, cluster);
    }
    if (cpt == 16) {
        if (cps == 3 && u == 2) return launch_fit<16, 128, 16, 2, 3, true>(ctx, args, s, cps, cluster);
        if (cps == 4 && u == 2) return launch_fit<16, 128, 16, 2, 4, true>(ctx, args, s, cps, cluster);
        if (cps == 4 && u == 1) return launch_fit<16, 128, 16, 1, 4, true>(ctx, args, s, cps, cluster);
        if (u == 4) return launch_fit<16, 128, 16, 4>(ctx, args, s, cps, cluster);
        return u == 2 ? launch_fit<16, 128, 16, 2>(ctx, args, s, cps, cluster)
                      : launch_fit<16, 128, 16, 1>(ctx, args, s, cps, cluster);
    }
    if (u == 4) return cps == 4 ? launch_fit<16, 128, 8, 4, 4>(ctx, args, s, cps, cluster)
                                : launch_fit<16, 128, 8, 4>(ctx, args, s, cps, cluster);
    if (u == 2) return cps == 4 ? launch_fit<16, 128, 8, 2, 4>(ctx, args, s, cps, cluster)
                                : launch_fit<16, 128, 8, 2>(ctx, args, s, cps, cluster);
    return launch_fit<16, 128, 8, 1>(ctx, args, s, cps, cluster);
}

}  // namespace pg
