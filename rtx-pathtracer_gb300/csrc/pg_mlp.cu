// pg_mlp.cu - the learned guiding surrogate: a position -> vMF-mixture MLP
// trained on the tracer's guiding records, BF16 on the tensor cores with FP32
// accumulation (mma.sync m16n8k16), FP32 master weights and Adam.
//
// Model (restated in FP64 by oracle/mlp_oracle.py):
//   x = (p - lo) / (hi - lo); 112 inputs: sin/cos(2^k pi x_d) pairs for
//   k < 16 and the three axes (columns 2i, 2i+1 with d = i % 3, k = i / 3),
//   x at columns 96..98, zeros after; h1..h3 = relu(W h + b) with 64 units;
//   80 outputs = 16 components x {logit, m_x, m_y, m_z, log kappa};
//   q(d) = sum_j softmax(logit)_j vMF(d; m_j / |m_j|, exp(clamp(s_j)))
//   loss = sum_i w_i (-log q(d_i)) / sum_i w_i.
//
// One training step over a batch of B records:
//   k_fwd_bwd   one warp per 16 records: encoding, four layers, loss and its
//               output gradient, back through the layers; activations and
//               gradients go to a BF16 scratch (B x 1152 bytes, L2-resident
//               for B = 65536)
//   k_wgrad     weight gradients dW = D^T X as tensor-core GEMMs over the
//               batch (split over row blocks, one layer per grid row), bias
//               gradients by column sums; per-block partials
//   k_reduce_adam
//               partials -> gradient / sum(w) -> Adam -> FP32 masters and the
//               BF16 weight copy the next step reads (the loss and weight sums
//               are formed by the first weight-gradient block).
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "pg_internal.cuh"

namespace pg {
namespace mlp {

constexpr int NIN = 112, NH = 64, NOUT = 80, NC = 16;
constexpr int SIN = NIN + 8, SH = NH + 8;  // padded shared-memory row strides (bf16 elements)
constexpr float S_MIN = -4.0f, S_MAX = 9.0f;
constexpr int OW1 = 0, OB1 = OW1 + NH * NIN, OW2 = OB1 + NH, OB2 = OW2 + NH * NH, OW3 = OB2 + NH,
              OB3 = OW3 + NH * NH, OW4 = OB3 + NH, OB4 = OW4 + NOUT * NH, NPARAM = OB4 + NOUT;
static_assert(NPARAM == PG_MLP_PARAMS, "parameter count");
// bf16 weight copy: W1, W2, W3, W4 back to back (unpadded)
constexpr int WB1 = 0, WB2 = WB1 + NH * NIN, WB3 = WB2 + NH * NH, WB4 = WB3 + NH * NH, NWB = WB4 + NOUT * NH;
// scratch row layout (bf16 elements per record)
constexpr int RA0 = 0, RH1 = RA0 + NIN, RH2 = RH1 + NH, RH3 = RH2 + NH, RDO = RH3 + NH, RD3 = RDO + NOUT,
              RD2 = RD3 + NH, RD1 = RD2 + NH, RROW = RD1 + NH;  // 576 bf16 = 1152 bytes
constexpr int kWarps = 4, kRowsPerCta = 16 * kWarps;
constexpr float kPi = 3.14159265358979323846f;

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&v);
}
__device__ __forceinline__ uint32_t cat16(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

struct Shared {
    __nv_bfloat16 w1[NH * SIN];
    __nv_bfloat16 w2[NH * SH];
    __nv_bfloat16 w3[NH * SH];
    __nv_bfloat16 w4[NOUT * SH];
    float b[NH * 3 + NOUT];
    float o[kWarps][16][NOUT];
};

// acc = bias + A W^T for one layer (A: 16 x 16*KC in fragments, W: rows of K).
template <int KC, int NT>
__device__ __forceinline__ void layer_fwd(float (&acc)[NT][4], const uint32_t (&a)[KC][4], const __nv_bfloat16 *w,
                                          int stride, const float *bias, int g, int t) {
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
        const float b0 = bias[8 * nt + 2 * t], b1 = bias[8 * nt + 2 * t + 1];
        acc[nt][0] = b0;
        acc[nt][1] = b1;
        acc[nt][2] = b0;
        acc[nt][3] = b1;
    }
#pragma unroll
    for (int kc = 0; kc < KC; ++kc)
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            const __nv_bfloat16 *row = w + (8 * nt + g) * stride + 16 * kc + 2 * t;
            mma_bf16(acc[nt], a[kc], *reinterpret_cast<const uint32_t *>(row),
                     *reinterpret_cast<const uint32_t *>(row + 8));
        }
}

// acc = A W for the backward pass (A: 16 x 16*KC gradients over the layer's
// outputs, W: KC*16 rows of 8*NT inputs).
template <int KC, int NT>
__device__ __forceinline__ void layer_bwd(float (&acc)[NT][4], const uint32_t (&a)[KC][4], const __nv_bfloat16 *w,
                                          int stride, int g, int t) {
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
#pragma unroll
    for (int kc = 0; kc < KC; ++kc)
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            const int o0 = 16 * kc + 2 * t, i = 8 * nt + g;
            const uint32_t b0 = cat16(w[o0 * stride + i], w[(o0 + 1) * stride + i]);
            const uint32_t b1 = cat16(w[(o0 + 8) * stride + i], w[(o0 + 9) * stride + i]);
            mma_bf16(acc[nt], a[kc], b0, b1);
        }
}

// relu (or the relu mask for gradients), then the C fragments as the next
// MMA's A fragments.
__device__ __forceinline__ void relu_mask(float (&acc)[8][4], uint32_t &mask) {
    mask = 0;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const bool pos = acc[nt][i] > 0.0f;
            if (!pos) acc[nt][i] = 0.0f;
            mask |= (pos ? 1u : 0u) << (4 * nt + i);
        }
}
__device__ __forceinline__ void apply_mask(float (&acc)[8][4], uint32_t mask) {
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int i = 0; i < 4; ++i)
            if (!((mask >> (4 * nt + i)) & 1u)) acc[nt][i] = 0.0f;
}
__device__ __forceinline__ void to_afrag(const float (&acc)[8][4], uint32_t (&a)[4][4]) {
#pragma unroll
    for (int kc = 0; kc < 4; ++kc) {
        a[kc][0] = pack2(acc[2 * kc][0], acc[2 * kc][1]);
        a[kc][1] = pack2(acc[2 * kc][2], acc[2 * kc][3]);
        a[kc][2] = pack2(acc[2 * kc + 1][0], acc[2 * kc + 1][1]);
        a[kc][3] = pack2(acc[2 * kc + 1][2], acc[2 * kc + 1][3]);
    }
}
// A fragments of a 16 x 16*KC tile to rows of the scratch (row stride RROW).
template <int KC>
__device__ __forceinline__ void store_afrag(const uint32_t (&a)[KC][4], __nv_bfloat16 *rows, int col0, int g, int t) {
#pragma unroll
    for (int kc = 0; kc < KC; ++kc) {
        const int c = col0 + 16 * kc + 2 * t;
        *reinterpret_cast<uint32_t *>(rows + (size_t)g * RROW + c) = a[kc][0];
        *reinterpret_cast<uint32_t *>(rows + (size_t)(g + 8) * RROW + c) = a[kc][1];
        *reinterpret_cast<uint32_t *>(rows + (size_t)g * RROW + c + 8) = a[kc][2];
        *reinterpret_cast<uint32_t *>(rows + (size_t)(g + 8) * RROW + c + 8) = a[kc][3];
    }
}

// Fourier features of the columns (c, c+1) of one row.
__device__ __forceinline__ uint32_t enc_pair(const float x[3], int c) {
    if (c < 96) {
        const int i = c >> 1, d = i % 3, k = i / 3;
        float s, co;
        sincospif(ldexpf(x[d], k), &s, &co);
        return pack2(s, co);
    }
    if (c == 96) return pack2(x[0], x[1]);
    if (c == 98) return pack2(x[2], 0.0f);
    return 0u;
}

struct FwdArgs {
    const pg_directional_data *rec;  // training records (or NULL for inference)
    const float *pos;                // inference positions (3 floats each)
    uint32_t n;
    float lo[3], inv_ext[3];
    const __nv_bfloat16 *wb;         // bf16 weights
    const float *theta;              // fp32 masters (biases are read from here)
    __nv_bfloat16 *scratch;          // B x RROW (training)
    float *partials;                 // per-warp {sum w (-log q), sum w} (training)
    float *mix_out;                  // n x 80 mixture parameters (inference)
};

// kTrain: loss, gradients and scratch; otherwise mixture parameters.
template <bool kTrain>
__global__ void __launch_bounds__(32 * kWarps, 3) k_fwd_bwd(FwdArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Shared &S = *reinterpret_cast<Shared *>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    // weights to shared memory (padded rows)
    for (int i = tid; i < NH * NIN / 2; i += blockDim.x) {
        const int r = (2 * i) / NIN, c = (2 * i) % NIN;
        *reinterpret_cast<uint32_t *>(&S.w1[r * SIN + c]) = reinterpret_cast<const uint32_t *>(A.wb + WB1)[i];
    }
    for (int i = tid; i < NH * NH / 2; i += blockDim.x) {
        const int r = (2 * i) / NH, c = (2 * i) % NH;
        *reinterpret_cast<uint32_t *>(&S.w2[r * SH + c]) = reinterpret_cast<const uint32_t *>(A.wb + WB2)[i];
        *reinterpret_cast<uint32_t *>(&S.w3[r * SH + c]) = reinterpret_cast<const uint32_t *>(A.wb + WB3)[i];
    }
    for (int i = tid; i < NOUT * NH / 2; i += blockDim.x) {
        const int r = (2 * i) / NH, c = (2 * i) % NH;
        *reinterpret_cast<uint32_t *>(&S.w4[r * SH + c]) = reinterpret_cast<const uint32_t *>(A.wb + WB4)[i];
    }
    for (int i = tid; i < NH; i += blockDim.x) {
        S.b[i] = A.theta[OB1 + i];
        S.b[NH + i] = A.theta[OB2 + i];
        S.b[2 * NH + i] = A.theta[OB3 + i];
    }
    for (int i = tid; i < NOUT; i += blockDim.x) S.b[3 * NH + i] = A.theta[OB4 + i];
    __syncthreads();

    const uint32_t row0 = blockIdx.x * kRowsPerCta + warp * 16;
    // positions of this lane's two rows (g, g + 8); rows past n sit at the box corner with no weight
    float x[2][3];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const uint32_t r = row0 + g + 8 * h;
        float p[3] = {A.lo[0], A.lo[1], A.lo[2]};
        if (r < A.n) {
            if (kTrain) {
                p[0] = A.rec[r].position[0];
                p[1] = A.rec[r].position[1];
                p[2] = A.rec[r].position[2];
            } else {
                p[0] = A.pos[3 * (size_t)r];
                p[1] = A.pos[3 * (size_t)r + 1];
                p[2] = A.pos[3 * (size_t)r + 2];
            }
        }
        for (int d = 0; d < 3; ++d) x[h][d] = (p[d] - A.lo[d]) * A.inv_ext[d];
    }
    // layer 1 inputs: the encoding as A fragments
    uint32_t a0[7][4];
#pragma unroll
    for (int kc = 0; kc < 7; ++kc) {
        const int c = 16 * kc + 2 * t;
        a0[kc][0] = enc_pair(x[0], c);
        a0[kc][1] = enc_pair(x[1], c);
        a0[kc][2] = enc_pair(x[0], c + 8);
        a0[kc][3] = enc_pair(x[1], c + 8);
    }
    __nv_bfloat16 *rows = kTrain ? A.scratch + (size_t)row0 * RROW : nullptr;
    if (kTrain) store_afrag<7>(a0, rows, RA0, g, t);

    float acc[8][4];
    uint32_t m1, m2, m3;
    uint32_t h[4][4];
    layer_fwd<7, 8>(acc, a0, S.w1, SIN, S.b, g, t);
    relu_mask(acc, m1);
    to_afrag(acc, h);
    if (kTrain) store_afrag<4>(h, rows, RH1, g, t);
    layer_fwd<4, 8>(acc, h, S.w2, SH, S.b + NH, g, t);
    relu_mask(acc, m2);
    to_afrag(acc, h);
    if (kTrain) store_afrag<4>(h, rows, RH2, g, t);
    layer_fwd<4, 8>(acc, h, S.w3, SH, S.b + 2 * NH, g, t);
    relu_mask(acc, m3);
    to_afrag(acc, h);
    if (kTrain) store_afrag<4>(h, rows, RH3, g, t);
    {
        float out[10][4];
        layer_fwd<4, 10>(out, h, S.w4, SH, S.b + 3 * NH, g, t);
#pragma unroll
        for (int nt = 0; nt < 10; ++nt) {
            S.o[warp][g][8 * nt + 2 * t] = out[nt][0];
            S.o[warp][g][8 * nt + 2 * t + 1] = out[nt][1];
            S.o[warp][g + 8][8 * nt + 2 * t] = out[nt][2];
            S.o[warp][g + 8][8 * nt + 2 * t + 1] = out[nt][3];
        }
    }
    __syncwarp();

    // ---- mixture, loss and output gradient: two lanes per row, 8 components each
    {
        const int s = lane >> 1, half = lane & 1;
        const uint32_t r = row0 + s;
        float* o = S.o[warp][s];
        float d[3] = {0.0f, 0.0f, 1.0f}, w = 0.0f;
        if (kTrain && r < A.n) {
            const pg_directional_data &rc = A.rec[r];
            d[0] = rc.direction[0];
            d[1] = rc.direction[1];
            d[2] = rc.direction[2];
            w = rc.flags == PG_INVALID_REGION ? 0.0f : rc.weight;
            if (!(w > 0.0f) || !isfinite(w)) w = 0.0f;
        }
        // softmax normaliser of the logits
        float lmax = -INFINITY;
        for (int j = 8 * half; j < 8 * half + 8; ++j) lmax = fmaxf(lmax, o[5 * j]);
        lmax = fmaxf(lmax, __shfl_xor_sync(0xffffffffu, lmax, 1));
        float lsum = 0.0f;
        for (int j = 8 * half; j < 8 * half + 8; ++j) lsum += expf(o[5 * j] - lmax);
        lsum += __shfl_xor_sync(0xffffffffu, lsum, 1);
        const float lse = lmax + logf(lsum);
        float lp[8], kap[8], cs[8], mn[8], mu[8][3], sraw[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int j = 8 * half + q;
            const float mx = o[5 * j + 1], my = o[5 * j + 2], mz = o[5 * j + 3];
            mn[q] = sqrtf(mx * mx + my * my + mz * mz);
            const float inv = mn[q] > 0.0f ? 1.0f / mn[q] : 0.0f;
            mu[q][0] = mx * inv;
            mu[q][1] = my * inv;
            mu[q][2] = mz * inv;
            sraw[q] = o[5 * j + 4];
            kap[q] = expf(fminf(fmaxf(sraw[q], S_MIN), S_MAX));
            cs[q] = mu[q][0] * d[0] + mu[q][1] * d[1] + mu[q][2] * d[2];
            const float lognorm = logf(kap[q]) - logf(2.0f * kPi) - logf(-expm1f(-2.0f * kap[q]));
            lp[q] = (o[5 * j] - lse) + lognorm + kap[q] * (cs[q] - 1.0f);
        }
        if (!kTrain) {
            if (r < A.n) {
                float *mo = A.mix_out + (size_t)r * NOUT;
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int j = 8 * half + q;
                    mo[5 * j] = expf(o[5 * j] - lse);
                    mo[5 * j + 1] = mu[q][0];
                    mo[5 * j + 2] = mu[q][1];
                    mo[5 * j + 3] = mu[q][2];
                    mo[5 * j + 4] = kap[q];
                }
            }
        } else {
            float qmax = -INFINITY;
            for (int q = 0; q < 8; ++q) qmax = fmaxf(qmax, lp[q]);
            qmax = fmaxf(qmax, __shfl_xor_sync(0xffffffffu, qmax, 1));
            float qs = 0.0f;
            for (int q = 0; q < 8; ++q) qs += expf(lp[q] - qmax);
            qs += __shfl_xor_sync(0xffffffffu, qs, 1);
            const float logq = qmax + logf(qs);
            __syncwarp();
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int j = 8 * half + q;
                const float rr = expf(lp[q] - logq);  // responsibility
                const float pi = expf(o[5 * j] - lse);
                const float k = kap[q];
                const float f = mn[q] > 0.0f ? -w * rr * k / mn[q] : 0.0f;
                o[5 * j] = w * (pi - rr);
                o[5 * j + 1] = f * (d[0] - cs[q] * mu[q][0]);
                o[5 * j + 2] = f * (d[1] - cs[q] * mu[q][1]);
                o[5 * j + 3] = f * (d[2] - cs[q] * mu[q][2]);
                const bool inside = sraw[q] > S_MIN && sraw[q] < S_MAX;
                const float e = expf(-2.0f * k);
                const float tt = 2.0f * k * e / -expm1f(-2.0f * k);
                o[5 * j + 4] = inside ? -w * rr * (1.0f - tt + k * (cs[q] - 1.0f)) : 0.0f;
            }
            // loss partials: one lane per row
            float lw = half == 0 ? w * -logq : 0.0f, ww = half == 0 ? w : 0.0f;
            if (w == 0.0f) lw = 0.0f;
            for (int off = 16; off > 0; off >>= 1) {
                lw += __shfl_xor_sync(0xffffffffu, lw, off);
                ww += __shfl_xor_sync(0xffffffffu, ww, off);
            }
            if (lane == 0) {  // one slot per warp: the sums are deterministic
                A.partials[2 * (blockIdx.x * kWarps + warp)] = lw;
                A.partials[2 * (blockIdx.x * kWarps + warp) + 1] = ww;
            }
        }
    }
    if (!kTrain) return;
    __syncwarp();

    // ---- backward through the layers
    uint32_t dof[5][4];
#pragma unroll
    for (int kc = 0; kc < 5; ++kc) {
        const int c = 16 * kc + 2 * t;
        dof[kc][0] = pack2(S.o[warp][g][c], S.o[warp][g][c + 1]);
        dof[kc][1] = pack2(S.o[warp][g + 8][c], S.o[warp][g + 8][c + 1]);
        dof[kc][2] = pack2(S.o[warp][g][c + 8], S.o[warp][g][c + 9]);
        dof[kc][3] = pack2(S.o[warp][g + 8][c + 8], S.o[warp][g + 8][c + 9]);
    }
    store_afrag<5>(dof, rows, RDO, g, t);
    layer_bwd<5, 8>(acc, dof, S.w4, SH, g, t);
    apply_mask(acc, m3);
    to_afrag(acc, h);
    store_afrag<4>(h, rows, RD3, g, t);
    layer_bwd<4, 8>(acc, h, S.w3, SH, g, t);
    apply_mask(acc, m2);
    to_afrag(acc, h);
    store_afrag<4>(h, rows, RD2, g, t);
    layer_bwd<4, 8>(acc, h, S.w2, SH, g, t);
    apply_mask(acc, m1);
    to_afrag(acc, h);
    store_afrag<4>(h, rows, RD1, g, t);
}

// Weight gradients of one layer (blockIdx.y) over a block of rows:
// dW[o][i] = sum_r D[r][o] X[r][i] on the tensor cores (M = outputs,
// N = inputs, K = rows), db[o] = sum_r D[r][o].  Partials per row block.
struct WgradArgs {
    const __nv_bfloat16 *scratch;
    uint32_t rows;        // padded batch rows (multiple of 16)
    uint32_t rows_per_block;
    float *partials;      // gridDim.x x NPARAM
    const float *fwd_partials;  // per-warp {sum w (-log q), sum w} of the forward kernel
    uint32_t n_fwd_partials;
    double *scalars;      // their sums (written by block (0, 0))
};

// Block-wide sums of the forward kernel's per-warp partials (one block).
__device__ void sum_fwd_partials(const WgradArgs &A) {
    __shared__ double sl[32 * kWarps], sw[32 * kWarps];
    double l = 0.0, w = 0.0;
    for (uint32_t i = threadIdx.x; i < A.n_fwd_partials; i += blockDim.x) {
        l += A.fwd_partials[2 * i];
        w += A.fwd_partials[2 * i + 1];
    }
    sl[threadIdx.x] = l;
    sw[threadIdx.x] = w;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st) {
            sl[threadIdx.x] += sl[threadIdx.x + st];
            sw[threadIdx.x] += sw[threadIdx.x + st];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        A.scalars[0] = sl[0];
        A.scalars[1] = sw[0];
    }
}

template <int O, int I>
__device__ __forceinline__ void wgrad_layer(const WgradArgs &A, int dcol, int xcol, int wofs, int bofs) {
    constexpr int MT = O / 16, NT = I / 8;
    constexpr int MT_PER_WARP = (MT + kWarps - 1) / kWarps;
    __shared__ __align__(16) __nv_bfloat16 sd[16][NOUT + 8];
    __shared__ __align__(16) __nv_bfloat16 sx[16][NIN + 8];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    float acc[MT_PER_WARP][NT][4];
#pragma unroll
    for (int m = 0; m < MT_PER_WARP; ++m)
#pragma unroll
        for (int n = 0; n < NT; ++n) acc[m][n][0] = acc[m][n][1] = acc[m][n][2] = acc[m][n][3] = 0.0f;
    float bacc = 0.0f;
    const uint32_t r0 = blockIdx.x * A.rows_per_block;
    const uint32_t r1 = min(A.rows, r0 + A.rows_per_block);
    for (uint32_t rb = r0; rb < r1; rb += 16) {
        __syncthreads();
        for (int i = tid; i < 16 * O / 2; i += blockDim.x) {
            const int r = (2 * i) / O, c = (2 * i) % O;
            *reinterpret_cast<uint32_t *>(&sd[r][c]) =
                *reinterpret_cast<const uint32_t *>(A.scratch + (size_t)(rb + r) * RROW + dcol + c);
        }
        for (int i = tid; i < 16 * I / 2; i += blockDim.x) {
            const int r = (2 * i) / I, c = (2 * i) % I;
            *reinterpret_cast<uint32_t *>(&sx[r][c]) =
                *reinterpret_cast<const uint32_t *>(A.scratch + (size_t)(rb + r) * RROW + xcol + c);
        }
        __syncthreads();
        if (tid < O)
            for (int r = 0; r < 16; ++r) bacc += __bfloat162float(sd[r][tid]);
#pragma unroll
        for (int m = 0; m < MT_PER_WARP; ++m) {
            const int mt = warp + kWarps * m;
            if (mt >= MT) break;
            // A = D^T: rows o, columns r
            uint32_t a[4];
            const int o = 16 * mt + g;
            a[0] = cat16(sd[2 * t][o], sd[2 * t + 1][o]);
            a[1] = cat16(sd[2 * t][o + 8], sd[2 * t + 1][o + 8]);
            a[2] = cat16(sd[2 * t + 8][o], sd[2 * t + 9][o]);
            a[3] = cat16(sd[2 * t + 8][o + 8], sd[2 * t + 9][o + 8]);
#pragma unroll
            for (int n = 0; n < NT; ++n) {
                const int i = 8 * n + g;
                const uint32_t b0 = cat16(sx[2 * t][i], sx[2 * t + 1][i]);
                const uint32_t b1 = cat16(sx[2 * t + 8][i], sx[2 * t + 9][i]);
                mma_bf16(acc[m][n], a, b0, b1);
            }
        }
    }
    float *out = A.partials + (size_t)blockIdx.x * NPARAM;
#pragma unroll
    for (int m = 0; m < MT_PER_WARP; ++m) {
        const int mt = warp + kWarps * m;
        if (mt >= MT) break;
#pragma unroll
        for (int n = 0; n < NT; ++n) {
            const int o = 16 * mt + g, i = 8 * n + 2 * t;
            out[wofs + o * I + i] = acc[m][n][0];
            out[wofs + o * I + i + 1] = acc[m][n][1];
            out[wofs + (o + 8) * I + i] = acc[m][n][2];
            out[wofs + (o + 8) * I + i + 1] = acc[m][n][3];
        }
    }
    if (tid < O) out[bofs + tid] = bacc;
}

__global__ void __launch_bounds__(32 * kWarps) k_wgrad(WgradArgs A) {
    if (blockIdx.x == 0 && blockIdx.y == 0) sum_fwd_partials(A);
    switch (blockIdx.y) {
        case 0: wgrad_layer<NH, NIN>(A, RD1, RA0, OW1, OB1); break;
        case 1: wgrad_layer<NH, NH>(A, RD2, RH1, OW2, OB2); break;
        case 2: wgrad_layer<NH, NH>(A, RD3, RH2, OW3, OB3); break;
        default: wgrad_layer<NOUT, NH>(A, RDO, RH3, OW4, OB4); break;
    }
}

struct AdamArgs {
    const float *partials;
    uint32_t n_blocks;
    double *scalars;         // {sum w (-log q), sum w}
    const float *loss_partials;  // not null: the scalars are summed here from these
    uint32_t n_loss;             // (pairs), as k_tc_scalars sums them, and written
    float *theta, *m, *v;
    __nv_bfloat16 *wb;
    __nv_bfloat16 *img;      // the tensor-core kernel's weight image
    float *grad_out;         // gradient only (no update) when not null
    float lr, b1, b2, eps, c1, c2;  // c1 = 1 - b1^t, c2 = 1 - b2^t
};

// Index of weight p in the tensor-core kernel's BF16 image (rows = outputs,
// 8 x 8 core matrices; GEMM depth 128 for layer 1 and 80 for the others), or -1.
__host__ __device__ inline int tc_img_index(int p) {
    auto el = [](int r, int c, int kc) { return (((r >> 3) * kc + (c >> 3)) << 6) + ((r & 7) << 3) + (c & 7); };
    constexpr int i2 = NH * 128, i3 = i2 + NH * 80, i4 = i3 + NH * 80;
    if (p >= OW1 && p < OB1) return el((p - OW1) / NIN, (p - OW1) % NIN, 16);
    if (p >= OW2 && p < OB2) return i2 + el((p - OW2) / NH, (p - OW2) % NH, 10);
    if (p >= OW3 && p < OB3) return i3 + el((p - OW3) / NH, (p - OW3) % NH, 10);
    if (p >= OW4 && p < OB4) return i4 + el((p - OW4) / NH, (p - OW4) % NH, 10);
    return -1;
}

__device__ __forceinline__ int wb_index(int p) {
    if (p < OB1) return WB1 + (p - OW1);
    if (p >= OW2 && p < OB2) return WB2 + (p - OW2);
    if (p >= OW3 && p < OB3) return WB3 + (p - OW3);
    if (p >= OW4 && p < OB4) return WB4 + (p - OW4);
    return -1;
}

// 32 parameters per block of kAdamGroups warps: warp g sums the partials of
// blocks g, g + kAdamGroups, ... (coalesced rows, loads from all warps in
// flight), the groups' compensated sums are merged in a fixed order.
constexpr int kAdamGroups = 8;
__global__ void __launch_bounds__(32 * kAdamGroups) k_reduce_adam(AdamArgs A) {
    __shared__ float ps[kAdamGroups][32], pc[kAdamGroups][32];
    __shared__ double sl[1], sw[1];  // the batch's loss and weight sums
    // the next batch's training kernel may launch now; it waits for this grid
    // before it reads the weights
    asm volatile("griddepcontrol.launch_dependents;");
    const int lane = threadIdx.x & 31, grp = threadIdx.x >> 5;
    const int p = blockIdx.x * 32 + lane;
    if (A.loss_partials && grp == 0) {
        // The batch's loss and weight sums in k_tc_scalars' order, by one warp:
        // lane l holds that kernel's threads l + 32 k (k < 8), whose tree steps
        // 128, 64 and 32 stay in the lane and steps 16 .. 1 are shuffles.
        double l[8], w[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {  // the first element of each thread's sum (0 + x = x): loads in flight together
            const uint32_t i = lane + 32u * k;
            l[k] = i < A.n_loss ? (double)A.loss_partials[2 * i] : 0.0;
            w[k] = i < A.n_loss ? (double)A.loss_partials[2 * i + 1] : 0.0;
        }
        for (uint32_t i0 = 256u + lane; i0 < A.n_loss; i0 += 256u)  // more than 256 partials
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const uint32_t i = i0 + 32u * k;
                if (i < A.n_loss) {
                    l[k] += A.loss_partials[2 * i];
                    w[k] += A.loss_partials[2 * i + 1];
                }
            }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            l[k] += l[k + 4];
            w[k] += w[k + 4];
        }
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            l[k] += l[k + 2];
            w[k] += w[k + 2];
        }
        l[0] += l[1];
        w[0] += w[1];
        for (int st = 16; st > 0; st >>= 1) {
            const double lo = __shfl_down_sync(0xffffffffu, l[0], st), wo = __shfl_down_sync(0xffffffffu, w[0], st);
            if (lane < st) {
                l[0] += lo;
                w[0] += wo;
            }
        }
        if (lane == 0) {
            sl[0] = l[0];
            sw[0] = w[0];
            if (blockIdx.x == 0) {
                A.scalars[0] = l[0];
                A.scalars[1] = w[0];
            }
        }
    }
    {
        // this warp's partials, eight loads in flight, added in block order
        float s = 0.0f, c = 0.0f;
        if (p < NPARAM)
            for (uint32_t b0 = grp; b0 < A.n_blocks; b0 += 8u * kAdamGroups) {
                float v[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const uint32_t b = b0 + (uint32_t)k * kAdamGroups;
                    v[k] = b < A.n_blocks ? A.partials[(size_t)b * NPARAM + p] : 0.0f;
                }
#pragma unroll
                for (int k = 0; k < 8; ++k)
                    if (b0 + (uint32_t)k * kAdamGroups < A.n_blocks) neumaier_add(s, c, v[k]);
            }
        ps[grp][lane] = s;
        pc[grp][lane] = c;
    }
    __syncthreads();
    if (grp != 0 || p >= NPARAM) return;
    float s = 0.0f, c = 0.0f;
#pragma unroll
    for (int g = 0; g < kAdamGroups; ++g) {
        neumaier_add(s, c, ps[g][lane]);
        c += pc[g][lane];
    }
    const double W = A.loss_partials ? sw[0] : A.scalars[1];
    const float gr = W > 0.0 ? (float)((double)(s + c) / W) : 0.0f;
    if (A.grad_out) {
        A.grad_out[p] = gr;
        return;
    }
    const float m = A.b1 * A.m[p] + (1.0f - A.b1) * gr;
    const float v = A.b2 * A.v[p] + (1.0f - A.b2) * gr * gr;
    A.m[p] = m;
    A.v[p] = v;
    const float th = A.theta[p] - A.lr * (m / A.c1) / (sqrtf(v / A.c2) + A.eps);
    A.theta[p] = th;
    const int wi = wb_index(p);
    if (wi >= 0) A.wb[wi] = __float2bfloat16_rn(th);
    const int ii = tc_img_index(p);
    if (ii >= 0) A.img[ii] = __float2bfloat16_rn(th);
}

__global__ void k_theta_to_wb(const float *theta, __nv_bfloat16 *wb) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= NPARAM) return;
    const int wi = wb_index(p);
    if (wi >= 0) wb[wi] = __float2bfloat16_rn(theta[p]);
}

// ---- the training step on the 5th-generation tensor cores (tcgen05) --------
//
// k_train_tc: one persistent CTA per SM (TPR threads per record of a
// 128-record tile) runs a whole batch: encoding, the four layers forward, the
// loss and its output gradient, the three layers backward, and the weight
// gradients of its tiles accumulated in tensor memory across tiles - no
// scratch round trip through DRAM.  Every GEMM is a tcgen05.mma (BF16 operands
// from shared memory, FP32 accumulators in tensor memory) issued by one
// thread and completed through an mbarrier; the epilogues read tensor memory
// with tcgen05.ld (thread t of warp w <-> lane 32 w + t).
//
//   forward  l: D[128 rec x out]  = X_l (K-major) . W_l^T (K-major), then +b_l
//               (FP32), ReLU, BF16 -> X_{l+1}
//   backward l: D[128 rec x 64]   = dY_l (K-major) . W_l (MN-major)
//   weights  l: G_l[128 x out]   += X_l^T (MN-major) . dY_l (MN-major): rows
//               are the layer's inputs, a column of ones after them (its row
//               of G_l is the bias gradient) and zeros up to the GEMM depth.
//
// Operand tiles are stored as 8 x 8 core matrices (8 rows of 16 bytes):
// element (r, c) of a tile with KC column chunks at element
// ((r / 8) KC + c / 8) 64 + (r % 8) 8 + c % 8.  One buffer serves as a
// K-major operand (rows = M or N) and as an MN-major one (rows = K), with the
// descriptor's strides swapped: LBO is the byte stride between 8-wide units
// along K, SBO the stride between 8-wide units along M or N.
namespace tc {
constexpr int TILE = 128;                 // records per tile (the MMA's M)
constexpr int K1 = 128, KH = 80;          // GEMM depths: inputs, ones column, zeros
constexpr int KC1 = K1 / 8, KCH = KH / 8; // column chunks
// BF16 weight image (rows = outputs; input columns; the ones column's weight is
// zero - the FP32 bias is added in the epilogue)
constexpr int IW1 = 0, IW2 = IW1 + NH * K1, IW3 = IW2 + NH * KH, IW4 = IW3 + NH * KH, NIMG = IW4 + NOUT * KH;
// shared memory (bytes)
constexpr int SM_W = 0, SM_X1 = SM_W + NIMG * 2, SM_X2 = SM_X1 + TILE * K1 * 2, SM_X3 = SM_X2 + TILE * KH * 2,
              SM_X4 = SM_X3 + TILE * KH * 2, SM_DY = SM_X4 + TILE * KH * 2, SM_SLACK = SM_DY + TILE * KH * 2,
              SM_BIAS = SM_SLACK + 2048, SM_XCH = SM_BIAS + (3 * NH + NOUT) * 4,
              SM_REC = SM_XCH + 2 * 4 * TILE * 4, SM_X1B = (SM_REC + TILE * 40 + 127) / 128 * 128,
              SM_TOTAL = SM_X1B + TILE * K1 * 2;
// The weight GEMMs of layers 2-4 use M = 128 over 81 meaningful rows: rows 81..127
// read past the end of X_l (at most 767 bytes) into the next buffer or the slack.
static_assert(SM_X1 % 128 == 0 && SM_X1B % 128 == 0 && SM_TOTAL <= 227 * 1024, "shared memory layout");
// tensor-memory columns: layer accumulator, then the four weight-gradient blocks
constexpr uint32_t TM_ACT = 0, TM_G1 = 128, TM_G2 = 192, TM_G3 = 256, TM_G4 = 320, TM_COLS = 512;
constexpr int kTpr = 4;  // threads per record

__host__ __device__ constexpr int elem(int r, int c, int kc) {
    return (((r >> 3) * kc + (c >> 3)) << 6) + ((r & 7) << 3) + (c & 7);
}

static_assert(IW2 == NH * 128 && IW3 == IW2 + NH * 80 && IW4 == IW3 + NH * 80 && KC1 == 16 && KCH == 10,
              "tc_img_index uses this image layout");

// Shared-memory matrix descriptor: start, leading (K) and stride (M/N) byte
// offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, the
// operands' major-ness, N >> 3 and M >> 4.
__host__ __device__ constexpr uint32_t idesc(int M, int N, int a_mn, int b_mn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)a_mn << 15) | ((uint32_t)b_mn << 16) |
           ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(a), "l"(b), "r"(id), "r"(accumulate));
}
// One operand walk: start address, LBO, SBO, bytes to advance per K-step of 16.
struct Opnd {
    uint32_t addr, lbo, sbo, step;
};
// D (+)= A B over `steps` K-steps (one thread).
__device__ __forceinline__ void gemm(uint32_t d, Opnd a, Opnd b, int steps, uint32_t id, bool accumulate) {
    for (int k = 0; k < steps; ++k)
        mma(d, sdesc(a.addr + k * a.step, a.lbo, a.sbo), sdesc(b.addr + k * b.step, b.lbo, b.sbo), id,
            (accumulate || k > 0) ? 1u : 0u);
}
__device__ __forceinline__ void commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// 16 consecutive FP32 columns of this thread's tensor-memory lane
__device__ __forceinline__ void tld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}
__device__ __forceinline__ void tld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
// 4 consecutive FP32 columns of this thread's tensor-memory lane (column a multiple of 4)
__device__ __forceinline__ void tld4(uint32_t taddr, float *v) {
    uint32_t r0, r1, r2, r3;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(taddr));
    v[0] = __uint_as_float(r0);
    v[1] = __uint_as_float(r1);
    v[2] = __uint_as_float(r2);
    v[3] = __uint_as_float(r3);
}

struct TrainArgs {
    const pg_directional_data *rec;
    uint32_t n;
    float lo[3], inv_ext[3];
    const __nv_bfloat16 *wimg;  // NIMG
    const float *theta;         // FP32 masters (biases)
    float *partials;            // gridDim.x x NPARAM weight / bias gradient sums
    float *loss_partials;       // gridDim.x x {sum w (-log q), sum w}
    uint32_t *err;              // PG_DEV_ERR_TIMEOUT if a wait ran out
    const float *pos;           // inference: positions (3 floats each)
    float *mix_out;             // inference: n x 80 mixture parameters
};

// Waits for the MMAs committed to `bar` (phase `phase`), bounded.
__device__ __forceinline__ void mma_wait(uint64_t *bar, uint32_t &phase, uint32_t *err) {
    mbar_wait_bounded(bar, phase, err);
    phase ^= 1u;
    fence_after();
}

// Generic-proxy stores of the operands -> visible to the tensor cores; all
// threads' tensor-memory loads done; then thread 0 issues.
__device__ __forceinline__ void operands_ready() {
    fence_proxy_async_smem();
    fence_before();
    __syncthreads();
}

// Fourier features of columns (c, c + 1) as enc_pair, with the argument
// reduced exactly (2^k x minus the nearest even integer, |r| <= 1) and the fast
// sine / cosine of pi r (absolute error ~2^-21, far below the BF16 rounding
// of the features).
__device__ __forceinline__ uint32_t enc_pair_fast(const float x[3], int c) {
    if (c < 96) {
        const int i = c >> 1, d = i % 3, k = i / 3;
        const float y = ldexpf(d == 0 ? x[0] : (d == 1 ? x[1] : x[2]), k);  // selects: x stays in registers
        const float r = y - 2.0f * rintf(0.5f * y);
        float sn, cs;
        __sincosf(kPi * r, &sn, &cs);
        return pack2(sn, cs);
    }
    if (c == 96) return pack2(x[0], x[1]);
    if (c == 98) return pack2(x[2], 0.0f);
    return 0u;
}

// Hidden-layer epilogue for this thread's share of a record's 64 columns
// (NCOL from column c0): + bias, ReLU (mask bits kept), BF16 into the next
// layer's X; the last share also writes [1, 0...] and a zero chunk.
template <int NCOL>
__device__ __forceinline__ void hidden_epilogue(uint32_t tacc, int c0, const float *bias, __nv_bfloat16 *xn, int row,
                                                bool last, uint32_t &mask) {
    float v[NCOL / 16][16];
#pragma unroll
    for (int q = 0; q < NCOL / 16; ++q) tld16(tacc + c0 + 16 * q, v[q]);
    tld_wait();
    mask = 0u;
#pragma unroll
    for (int ch = 0; ch < NCOL / 8; ++ch) {
        uint32_t pk[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int c = 8 * ch + 2 * e;
            float a = v[c >> 4][c & 15] + bias[c0 + c], b = v[(c + 1) >> 4][(c + 1) & 15] + bias[c0 + c + 1];
            const bool pa = a > 0.0f, pb = b > 0.0f;
            a = pa ? a : 0.0f;
            b = pb ? b : 0.0f;
            mask |= ((pa ? 1u : 0u) << c) | ((pb ? 1u : 0u) << (c + 1));
            pk[e] = pack2(a, b);
        }
        *reinterpret_cast<uint4 *>(xn + elem(row, c0 + 8 * ch, KCH)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    }
    if (last) {
        *reinterpret_cast<uint4 *>(xn + elem(row, 64, KCH)) = make_uint4(pack2(1.0f, 0.0f), 0u, 0u, 0u);
        *reinterpret_cast<uint4 *>(xn + elem(row, 72, KCH)) = make_uint4(0u, 0u, 0u, 0u);
    }
}

// Backward epilogue for the same share: dH, ReLU mask, BF16 into dY.
template <int NCOL>
__device__ __forceinline__ void backward_epilogue(uint32_t tacc, int c0, uint32_t mask, __nv_bfloat16 *dy, int row) {
    float v[NCOL / 16][16];
#pragma unroll
    for (int q = 0; q < NCOL / 16; ++q) tld16(tacc + c0 + 16 * q, v[q]);
    tld_wait();
#pragma unroll
    for (int ch = 0; ch < NCOL / 8; ++ch) {
        uint32_t pk[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int c = 8 * ch + 2 * e;
            const float a = ((mask >> c) & 1u) ? v[c >> 4][c & 15] : 0.0f;
            const float b = ((mask >> (c + 1)) & 1u) ? v[(c + 1) >> 4][(c + 1) & 15] : 0.0f;
            pk[e] = pack2(a, b);
        }
        *reinterpret_cast<uint4 *>(dy + elem(row, c0 + 8 * ch, KCH)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    }
}

// Queues asynchronous 4-byte copies of tile `tile`'s inputs (its records, or
// its positions for inference) into shared memory: the copies of the next tile
// run while this one computes.  tile < number of tiles.
template <bool kInfer>
__device__ __forceinline__ void prefetch_tile(const TrainArgs &A, uint32_t tile, uint32_t *dst, int tid, int nt) {
    const uint32_t first = tile * TILE;
    const uint32_t nrec = min((uint32_t)TILE, A.n - first);
    const uint32_t words = nrec * (kInfer ? 3u : 10u);
    const uint32_t *src = kInfer ? reinterpret_cast<const uint32_t *>(A.pos + 3 * (size_t)first)
                                 : reinterpret_cast<const uint32_t *>(A.rec + first);
    for (uint32_t i = (uint32_t)tid; i < words; i += (uint32_t)nt)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst + i)), "l"(src + i) : "memory");
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// TPR threads per record: warps w, w + 4, ... share tensor-memory lanes
// 32 (w % 4) .. + 31, i.e. the same 32 records; share h = warp / 4 takes 64 / TPR
// of a layer's columns, 16 / TPR of the mixture components and every TPR-th
// encoding chunk.  The output layer's columns 5 j .. 5 j + 4 hold component
// j (logit, mean, log kappa): share h reads its components' 5 NC / TPR columns
// straight from tensor memory and writes their gradient into dY.
// kInfer: the forward pass only, writing each position's mixture parameters
// {pi, mu, kappa} per component (pg_mlp_infer).
template <int TPR, bool kInfer = false>
__global__ void __launch_bounds__(TILE * TPR, 1) k_train_tc(TrainArgs A) {
    constexpr int NT = TILE * TPR, HC = 64 / TPR, NCMP = NC / TPR;
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ uint32_t s_tmem;
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ float s_red[2 * NT / 32];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int rec = tid & (TILE - 1), h = tid / TILE;  // record within the tile, share
    // two X1 buffers: a tile's encoding is written while the tile before it runs its backward GEMMs
    __nv_bfloat16 *const sX1a = reinterpret_cast<__nv_bfloat16 *>(sm + SM_X1);
    __nv_bfloat16 *const sX1b = reinterpret_cast<__nv_bfloat16 *>(sm + SM_X1B);
    __nv_bfloat16 *sX2 = reinterpret_cast<__nv_bfloat16 *>(sm + SM_X2);
    __nv_bfloat16 *sX3 = reinterpret_cast<__nv_bfloat16 *>(sm + SM_X3);
    __nv_bfloat16 *sX4 = reinterpret_cast<__nv_bfloat16 *>(sm + SM_X4);
    __nv_bfloat16 *sDY = reinterpret_cast<__nv_bfloat16 *>(sm + SM_DY);
    float *sB = reinterpret_cast<float *>(sm + SM_BIAS);
    float *sXm = reinterpret_cast<float *>(sm + SM_XCH);   // [TPR][TILE] partial maxima
    float *sXs = sXm + TPR * TILE;                          // [TPR][TILE] partial sums
    uint32_t *sRec = reinterpret_cast<uint32_t *>(sm + SM_REC);  // the tile's records (10 words each)
    static_assert(sizeof(pg_directional_data) == 40, "record words");
    const uint32_t tiles = (A.n + TILE - 1) / TILE;
    // The first tile's inputs; then, when launched behind the previous batch's
    // update kernel (programmatic dependent launch), wait for its weights: the
    // records are not written by that kernel.
    if (blockIdx.x < tiles) prefetch_tile<kInfer>(A, blockIdx.x, sRec, tid, NT);
    asm volatile("griddepcontrol.wait;" ::: "memory");
    {
        const uint4 *src = reinterpret_cast<const uint4 *>(A.wimg);
        uint4 *dst = reinterpret_cast<uint4 *>(sm + SM_W);
        for (int i = tid; i < NIMG * 2 / 16; i += NT) dst[i] = src[i];
        uint4 *slack = reinterpret_cast<uint4 *>(sm + SM_SLACK);
        for (int i = tid; i < 2048 / 16; i += NT) slack[i] = make_uint4(0u, 0u, 0u, 0u);
        for (int i = tid; i < NH; i += NT) {
            sB[i] = A.theta[OB1 + i];
            sB[NH + i] = A.theta[OB2 + i];
            sB[2 * NH + i] = A.theta[OB3 + i];
        }
        for (int i = tid; i < NOUT; i += NT) sB[3 * NH + i] = A.theta[OB4 + i];
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                     "r"(TM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        mbar_init(&s_bar, 1);
        fence_mbar_init();
    }
    operands_ready();
    fence_after();
    const uint32_t tm = s_tmem;
    const uint32_t tl = tm + ((uint32_t)((warp & 3) * 32) << 16);  // this warp's lanes
    const uint32_t aW = smem_u32(sm + SM_W), aX1 = smem_u32(sX1a), aX1b = smem_u32(sX1b),
                   aX2 = smem_u32(sX2), aX3 = smem_u32(sX3),
                   aX4 = smem_u32(sX4), aDY = smem_u32(sDY);
    // operand walks (bytes): K-major tiles advance 2 chunks (256 B) per K-step of 16,
    // MN-major ones 2 row groups
    const Opnd fX2{aX2, 128, KCH * 128, 256}, fX3{aX3, 128, KCH * 128, 256},
        fX4{aX4, 128, KCH * 128, 256};
    const Opnd fW1{aW + IW1 * 2, 128, KC1 * 128, 256}, fW2{aW + IW2 * 2, 128, KCH * 128, 256},
        fW3{aW + IW3 * 2, 128, KCH * 128, 256}, fW4{aW + IW4 * 2, 128, KCH * 128, 256};
    const Opnd bDY{aDY, 128, KCH * 128, 256};
    const Opnd bW2{aW + IW2 * 2, KCH * 128, 128, 2 * KCH * 128}, bW3{aW + IW3 * 2, KCH * 128, 128, 2 * KCH * 128},
        bW4{aW + IW4 * 2, KCH * 128, 128, 2 * KCH * 128};
    const Opnd gX2{aX2, KCH * 128, 128, 2 * KCH * 128},
        gX3{aX3, KCH * 128, 128, 2 * KCH * 128}, gX4{aX4, KCH * 128, 128, 2 * KCH * 128};
    const Opnd gDY{aDY, KCH * 128, 128, 2 * KCH * 128};
    uint32_t phase = 0;
    float lsum = 0.0f, wsum = 0.0f;
    bool first = true;
    const int hc0 = h * HC;  // this share's hidden columns
    // encoding chunk ch of a record at x into the X1 tile dst: 112 features, the
    // ones column, zeros to 128 (this thread's chunks are h, h + TPR, ...)
    auto encode_chunk = [&](const float *xx, int ch, __nv_bfloat16 *dst) {
        const int c = 8 * ch;
        uint4 v;
        if (ch < 14)
            v = make_uint4(enc_pair_fast(xx, c), enc_pair_fast(xx, c + 2), enc_pair_fast(xx, c + 4),
                           enc_pair_fast(xx, c + 6));
        else
            v = make_uint4(ch == 14 ? pack2(1.0f, 0.0f) : 0u, 0u, 0u, 0u);
        *reinterpret_cast<uint4 *>(dst + elem(rec, c, KC1)) = v;
    };
    int xb = 0;            // this tile's X1 buffer
    bool encoded = false;  // this tile's X1 was written during the tile before
    for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint32_t r = tile * TILE + (uint32_t)rec;
        float x[3] = {0.0f, 0.0f, 0.0f}, d[3] = {0.0f, 0.0f, 1.0f}, w = 0.0f;
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        __syncthreads();  // the tile's inputs are in shared memory
        if (r < A.n) {
            if constexpr (kInfer) {
                const float *p = reinterpret_cast<const float *>(sRec) + 3 * rec;
                for (int k = 0; k < 3; ++k) x[k] = (p[k] - A.lo[k]) * A.inv_ext[k];
            } else {
                const float *rc = reinterpret_cast<const float *>(sRec) + 10 * rec;
                for (int k = 0; k < 3; ++k) {
                    x[k] = (rc[k] - A.lo[k]) * A.inv_ext[k];  // position
                    d[k] = rc[3 + k];                          // direction
                }
                const uint32_t flags = sRec[10 * rec + 9];
                w = flags == PG_INVALID_REGION ? 0.0f : rc[6];  // weight
                if (!(w > 0.0f) || !isfinite(w)) w = 0.0f;
            }
        }
        if (!encoded)
            for (int ch = h; ch < KC1; ch += TPR) encode_chunk(x, ch, xb ? sX1b : sX1a);
        uint32_t m1, m2, m3;
        // ---- forward
        operands_ready();  // also: every thread has read its record
        if (tile + gridDim.x < tiles) prefetch_tile<kInfer>(A, tile + gridDim.x, sRec, tid, NT);
        if (tid == 0) {
            fence_after();
            gemm(tm + TM_ACT, Opnd{xb ? aX1b : aX1, 128, KC1 * 128, 256}, fW1, K1 / 16, idesc(128, NH, 0, 0), false);
            commit(&s_bar);
        }
        mma_wait(&s_bar, phase, A.err);
        hidden_epilogue<HC>(tl + TM_ACT, hc0, sB, sX2, rec, h == TPR - 1, m1);
        operands_ready();
        if (tid == 0) {
            fence_after();
            gemm(tm + TM_ACT, fX2, fW2, KH / 16, idesc(128, NH, 0, 0), false);
            commit(&s_bar);
        }
        mma_wait(&s_bar, phase, A.err);
        hidden_epilogue<HC>(tl + TM_ACT, hc0, sB + NH, sX3, rec, h == TPR - 1, m2);
        operands_ready();
        if (tid == 0) {
            fence_after();
            gemm(tm + TM_ACT, fX3, fW3, KH / 16, idesc(128, NH, 0, 0), false);
            commit(&s_bar);
        }
        mma_wait(&s_bar, phase, A.err);
        hidden_epilogue<HC>(tl + TM_ACT, hc0, sB + 2 * NH, sX4, rec, h == TPR - 1, m3);
        operands_ready();
        if (tid == 0) {
            fence_after();
            gemm(tm + TM_ACT, fX4, fW4, KH / 16, idesc(128, NOUT, 0, 0), false);
            commit(&s_bar);
        }
        mma_wait(&s_bar, phase, A.err);
        // ---- mixture, loss and output gradient, from tensor memory (outputs + bias)
        static_assert((5 * NCMP) % 4 == 0 && (5 * NCMP) % 2 == 0, "share columns");
        const int j0 = h * NCMP;  // this share's components
        const int oc0 = 5 * j0;   // and their first output column
        float o[5 * NCMP];
#pragma unroll
        for (int q = 0; q < 5 * NCMP / 4; ++q) tld4(tl + TM_ACT + oc0 + 4 * q, &o[4 * q]);
        tld_wait();
#pragma unroll
        for (int c = 0; c < 5 * NCMP; ++c) o[c] += sB[3 * NH + oc0 + c];
        // Fast exponentials and logarithms (relative error ~1e-6): the loss and
        // gradient are sums over many records of terms that are rounded to
        // BF16 on the way back.
        float ml = -INFINITY;
#pragma unroll
        for (int q = 0; q < NCMP; ++q) ml = fmaxf(ml, o[5 * q]);
        float sl = 0.0f;
#pragma unroll
        for (int q = 0; q < NCMP; ++q) sl += __expf(o[5 * q] - ml);
        sXm[h * TILE + rec] = ml;
        sXs[h * TILE + rec] = sl;
        __syncthreads();
        float lmax = -INFINITY;
#pragma unroll
        for (int g = 0; g < TPR; ++g) lmax = fmaxf(lmax, sXm[g * TILE + rec]);
        float lsm = 0.0f;
#pragma unroll
        for (int g = 0; g < TPR; ++g) lsm += sXs[g * TILE + rec] * __expf(sXm[g * TILE + rec] - lmax);
        const float lse = lmax + __logf(lsm);
        if constexpr (kInfer) {
            if (r < A.n) {
                float *mo = A.mix_out + (size_t)r * NOUT;
#pragma unroll
                for (int q = 0; q < NCMP; ++q) {
                    const int j = j0 + q;
                    const float mx = o[5 * q + 1], my = o[5 * q + 2], mz = o[5 * q + 3];
                    const float mn = sqrtf(mx * mx + my * my + mz * mz);
                    const float inv = mn > 0.0f ? 1.0f / mn : 0.0f;
                    mo[5 * j] = __expf(o[5 * q] - lse);
                    mo[5 * j + 1] = mx * inv;
                    mo[5 * j + 2] = my * inv;
                    mo[5 * j + 3] = mz * inv;
                    mo[5 * j + 4] = __expf(fminf(fmaxf(o[5 * q + 4], S_MIN), S_MAX));
                }
            }
        } else {
            float lp[NCMP], kq[NCMP], csq[NCMP], mu[NCMP][3], fin[NCMP], pq[NCMP];
            uint32_t inside = 0u;  // bit q: log kappa strictly inside its clamp
    #pragma unroll
            for (int q = 0; q < NCMP; ++q) {
                const float mx = o[5 * q + 1], my = o[5 * q + 2], mz = o[5 * q + 3];
                pq[q] = __expf(o[5 * q] - lse);
                inside |= (o[5 * q + 4] > S_MIN && o[5 * q + 4] < S_MAX) ? 1u << q : 0u;
                const float mn = sqrtf(mx * mx + my * my + mz * mz);
                const float inv = mn > 0.0f ? 1.0f / mn : 0.0f;
                const float k = __expf(fminf(fmaxf(o[5 * q + 4], S_MIN), S_MAX));
                mu[q][0] = mx * inv;
                mu[q][1] = my * inv;
                mu[q][2] = mz * inv;
                const float cs = mu[q][0] * d[0] + mu[q][1] * d[1] + mu[q][2] * d[2];
                const float om = -expm1f(-2.0f * k);  // 1 - e^{-2k}
                const float lognorm = __logf(k) - __logf(2.0f * kPi) - __logf(om);
                lp[q] = (o[5 * q] - lse) + lognorm + k * (cs - 1.0f);
                kq[q] = k;
                csq[q] = cs;
                fin[q] = inv * k;  // kappa / |m|
            }
            float mq = -INFINITY;
    #pragma unroll
            for (int q = 0; q < NCMP; ++q) mq = fmaxf(mq, lp[q]);
            float sq = 0.0f;
    #pragma unroll
            for (int q = 0; q < NCMP; ++q) sq += __expf(lp[q] - mq);
            __syncthreads();  // everyone has read the logit maxima
            sXm[h * TILE + rec] = mq;
            sXs[h * TILE + rec] = sq;
            __syncthreads();
            float qmax = -INFINITY;
    #pragma unroll
            for (int g = 0; g < TPR; ++g) qmax = fmaxf(qmax, sXm[g * TILE + rec]);
            float qs = 0.0f;
    #pragma unroll
            for (int g = 0; g < TPR; ++g) qs += sXs[g * TILE + rec] * __expf(sXm[g * TILE + rec] - qmax);
            const float logq = qmax + __logf(qs);
            if (h == 0 && w > 0.0f) {
                lsum += w * -logq;
                wsum += w;
            }
            // the gradient of this share's outputs, BF16 pairs into dY
            float gq[5 * NCMP];
    #pragma unroll
            for (int q = 0; q < NCMP; ++q) {
                const float k = kq[q], cs = csq[q];
                const float rr = __expf(lp[q] - logq);  // responsibility
                const float pi = pq[q];
                const float f = -w * rr * fin[q];
                gq[5 * q] = w * (pi - rr);
                gq[5 * q + 1] = f * (d[0] - cs * mu[q][0]);
                gq[5 * q + 2] = f * (d[1] - cs * mu[q][1]);
                gq[5 * q + 3] = f * (d[2] - cs * mu[q][2]);
                const float e = __expf(-2.0f * k);
                const float tt = 2.0f * k * e / -expm1f(-2.0f * k);
                gq[5 * q + 4] = ((inside >> q) & 1u) ? -w * rr * (1.0f - tt + k * (cs - 1.0f)) : 0.0f;
            }
    #pragma unroll
            for (int c = 0; c < 5 * NCMP; c += 2)
                *reinterpret_cast<uint32_t *>(sDY + elem(rec, oc0 + c, KCH)) = pack2(gq[c], gq[c + 1]);
            // ---- backward: weight gradients of layer l and dH_{l-1} from one commit.
            // While each commit runs, the threads encode a quarter of the next
            // tile into the other X1 buffer (its records arrived during this tile).
            const uint32_t ntile = tile + gridDim.x;
            const bool has_next = ntile < tiles;
            __nv_bfloat16 *xn1 = xb ? sX1a : sX1b;  // the other X1 buffer
            asm volatile("cp.async.wait_group 0;" ::: "memory");  // the barrier below publishes them
            operands_ready();
            float xn[3] = {0.0f, 0.0f, 0.0f};
            if (has_next && ntile * TILE + (uint32_t)rec < A.n) {
                const float *rc = reinterpret_cast<const float *>(sRec) + 10 * rec;
                for (int k = 0; k < 3; ++k) xn[k] = (rc[k] - A.lo[k]) * A.inv_ext[k];
            }
            if (tid == 0) {
                fence_after();
                gemm(tm + TM_G4, gX4, gDY, TILE / 16, idesc(128, NOUT, 1, 1), !first);
                gemm(tm + TM_ACT, bDY, bW4, NOUT / 16, idesc(128, NH, 0, 1), false);
                commit(&s_bar);
            }
            if (has_next) encode_chunk(xn, h, xn1);
            mma_wait(&s_bar, phase, A.err);
            backward_epilogue<HC>(tl + TM_ACT, hc0, m3, sDY, rec);
            operands_ready();
            if (tid == 0) {
                fence_after();
                gemm(tm + TM_G3, gX3, gDY, TILE / 16, idesc(128, NH, 1, 1), !first);
                gemm(tm + TM_ACT, bDY, bW3, NH / 16, idesc(128, NH, 0, 1), false);
                commit(&s_bar);
            }
            if (has_next) encode_chunk(xn, h + TPR, xn1);
            mma_wait(&s_bar, phase, A.err);
            backward_epilogue<HC>(tl + TM_ACT, hc0, m2, sDY, rec);
            operands_ready();
            if (tid == 0) {
                fence_after();
                gemm(tm + TM_G2, gX2, gDY, TILE / 16, idesc(128, NH, 1, 1), !first);
                gemm(tm + TM_ACT, bDY, bW2, NH / 16, idesc(128, NH, 0, 1), false);
                commit(&s_bar);
            }
            if (has_next) encode_chunk(xn, h + 2 * TPR, xn1);
            mma_wait(&s_bar, phase, A.err);
            backward_epilogue<HC>(tl + TM_ACT, hc0, m1, sDY, rec);
            operands_ready();
            if (tid == 0) {
                fence_after();
                gemm(tm + TM_G1, Opnd{xb ? aX1b : aX1, KC1 * 128, 128, 2 * KC1 * 128}, gDY, TILE / 16,
                     idesc(128, NH, 1, 1), !first);
                commit(&s_bar);
            }
            if (has_next)
                for (int ch = h + 3 * TPR; ch < KC1; ch += TPR) encode_chunk(xn, ch, xn1);
            mma_wait(&s_bar, phase, A.err);
            first = false;
            encoded = has_next;
            xb ^= 1;
        }
    }
    if constexpr (!kInfer) {
        // ---- this CTA's gradient sums: lane = input row (bias row = the ones column);
        // column blocks h, h + TPR, ...
        float *out = A.partials + (size_t)blockIdx.x * NPARAM;
        const int i = rec;
        auto dump = [&](uint32_t tcol, int nout, int nin, int ow, int ob) {
            for (int c = 16 * h; c < nout; c += 16 * TPR) {
                float v[16];
                tld16(tl + tcol + c, v);
                tld_wait();
                if (first) {  // no tile: zero sums
    #pragma unroll
                    for (int j = 0; j < 16; ++j) v[j] = 0.0f;
                }
                if (i < nin) {
    #pragma unroll
                    for (int j = 0; j < 16; ++j) out[ow + (c + j) * nin + i] = v[j];
                } else if (i == nin) {
    #pragma unroll
                    for (int j = 0; j < 16; ++j) out[ob + c + j] = v[j];
                }
            }
        };
        dump(TM_G1, NH, NIN, OW1, OB1);
        dump(TM_G2, NH, NH, OW2, OB2);
        dump(TM_G3, NH, NH, OW3, OB3);
        dump(TM_G4, NOUT, NH, OW4, OB4);
        for (int off = 16; off > 0; off >>= 1) {
            lsum += __shfl_xor_sync(0xffffffffu, lsum, off);
            wsum += __shfl_xor_sync(0xffffffffu, wsum, off);
        }
        if (lane == 0) {
            s_red[2 * warp] = lsum;
            s_red[2 * warp + 1] = wsum;
        }
        fence_before();
        __syncthreads();
        if (tid == 0) {  // only share 0 (warps 0-3) carries loss sums
            A.loss_partials[2 * blockIdx.x] = (s_red[0] + s_red[2]) + (s_red[4] + s_red[6]);
            A.loss_partials[2 * blockIdx.x + 1] = (s_red[1] + s_red[3]) + (s_red[5] + s_red[7]);
        }
    } else {
        fence_before();
        __syncthreads();
    }
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm), "r"(TM_COLS));
    }
}

// Sums of the per-CTA loss partials (one block, deterministic order).
__global__ void k_tc_scalars(const float *lp, uint32_t n, double *scalars) {
    __shared__ double sl[256], sw[256];
    double l = 0.0, w = 0.0;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        l += lp[2 * i];
        w += lp[2 * i + 1];
    }
    sl[threadIdx.x] = l;
    sw[threadIdx.x] = w;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st) {
            sl[threadIdx.x] += sl[threadIdx.x + st];
            sw[threadIdx.x] += sw[threadIdx.x + st];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        scalars[0] = sl[0];
        scalars[1] = sw[0];
    }
}

__global__ void k_theta_to_img(const float *theta, __nv_bfloat16 *img) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= NPARAM) return;
    const int ii = tc_img_index(p);
    if (ii >= 0) img[ii] = __float2bfloat16_rn(theta[p]);
}
}  // namespace tc

// centres of the guide's region boxes
__global__ void k_region_centres(const float *aabbs, uint32_t n, float *pos) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    for (int i = 0; i < 3; ++i) pos[3 * r + i] = aabbs[6 * r + i] + 0.5f * (aabbs[6 * r + 3 + i] - aabbs[6 * r + i]);
}

// mixtures -> VMM_Theta (setK of guiding.glsl:23-30: norm and e^{-2k} from k)
__global__ void k_pack_guide(const float *mix, const float *pos, uint32_t n, pg_vmm_theta *out) {
    const uint32_t r = blockIdx.x;
    const int j = threadIdx.x;
    if (r >= n || j >= NC) return;
    const float *m = mix + (size_t)r * NOUT + 5 * j;
    pg_vmm_theta *v = out + r;
    pg_vmf_theta th;
    th.mu[0] = m[1];
    th.mu[1] = m[2];
    th.mu[2] = m[3];
    float k = m[4];
    k = k < kVmfMinKappa ? 0.0f : k;
    th.k = k;
    const double kd = (double)k;
    th.norm = k > 0.0f ? (float)(kd / (2.0 * 3.14159265358979323846 * (1.0 - exp(-2.0 * kd)))) : 0.0f;
    th.e_min2k = (float)exp(-2.0 * kd);
    th.distance = -1.0f;
    th.target[0] = th.target[1] = th.target[2] = 0.0f;
    v->thetas[j] = th;
    v->pi[j] = m[0];
    if (j == 0) {
        v->mean_position[0] = pos[3 * r];
        v->mean_position[1] = pos[3 * r + 1];
        v->mean_position[2] = pos[3 * r + 2];
        v->used_distributions = NC;
    }
}

// Mixture pdf of a packed VMM_Theta (guiding.glsl:32-60), parallax re-aiming
// toward each lobe's target when its distance is positive.
__device__ float vmm_theta_pdf(const pg_vmm_theta &v, const float d[3], const float x[3], int par) {
    float res = 0.0f;
    const int K = min(v.used_distributions, 16);
    for (int i = 0; i < K; ++i) {
        const pg_vmf_theta &t = v.thetas[i];
        float f;
        if (t.k == 0.0f) {
            f = 1.0f / (4.0f * kPi);
        } else {
            float mu[3] = {t.mu[0], t.mu[1], t.mu[2]};
            if (par && t.distance > 0.0f) {
                for (int c = 0; c < 3; ++c) mu[c] = t.target[c] - x[c];
                const float l = rsqrtf(mu[0] * mu[0] + mu[1] * mu[1] + mu[2] * mu[2]);
                for (int c = 0; c < 3; ++c) mu[c] *= l;
            }
            f = t.norm * expf(t.k * (mu[0] * d[0] + mu[1] * d[1] + mu[2] * d[2] - 1.0f));
        }
        res += v.pi[i] * f;
    }
    return res;
}

// per-region sums of w (-log q) under the context's and the network's mixtures
__global__ void k_judge_accumulate(const pg_directional_data *rec, uint64_t n, const pg_vmm_theta *fit,
                                   const pg_vmm_theta *net, uint32_t n_regions, int par, float *sums) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const pg_directional_data &r = rec[i];
        if (r.flags >= n_regions) continue;
        const float w = r.weight;
        if (!(w > 0.0f) || !isfinite(w)) continue;
        const float qf = fmaxf(vmm_theta_pdf(fit[r.flags], r.direction, r.position, par), 1e-30f);
        const float qn = fmaxf(vmm_theta_pdf(net[r.flags], r.direction, r.position, 0), 1e-30f);
        float *s = sums + 4 * (size_t)r.flags;
        atomicAdd(s, isfinite(qf) ? -w * logf(qf) : INFINITY);
        atomicAdd(s + 1, -w * logf(qn));
        atomicAdd(s + 2, w);
        atomicAdd(s + 3, 1.0f);
    }
}

__global__ void k_judge_select(const float *sums, const pg_vmm_theta *net, uint32_t n_regions, float min_records,
                               pg_vmm_theta *fit, uint32_t *switched) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_regions) return;
    const float *s = sums + 4 * (size_t)r;
    const bool better = s[1] < s[0] || (!isfinite(s[0]) && isfinite(s[1]));
    if (s[3] < min_records || !better) return;
    fit[r] = net[r];
    atomicAdd(switched, 1u);
}

// sum w (-log q) and sum w of records under a packed guide (double accumulators)
__global__ void k_guide_nll(const pg_directional_data *rec, uint64_t n, const pg_vmm_theta *vmm, uint32_t n_regions,
                            int par, double *out) {
    double l = 0.0, w = 0.0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const pg_directional_data &r = rec[i];
        if (r.flags >= n_regions || !(r.weight > 0.0f) || !isfinite(r.weight)) continue;
        const float q = fmaxf(vmm_theta_pdf(vmm[r.flags], r.direction, r.position, par), 1e-30f);
        l += -(double)r.weight * log((double)q);
        w += r.weight;
    }
    for (int o = 16; o > 0; o >>= 1) {
        l += __shfl_xor_sync(0xffffffffu, l, o);
        w += __shfl_xor_sync(0xffffffffu, w, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out, l);
        atomicAdd(out + 1, w);
    }
}

}  // namespace mlp
}  // namespace pg

using namespace pg;
using namespace pg::mlp;

struct pg_mlp {
    pg_mlp_config cfg{};
    int sm_count = 0;
    float *theta = nullptr, *m = nullptr, *v = nullptr;
    __nv_bfloat16 *wb = nullptr;
    __nv_bfloat16 *scratch = nullptr;
    float *fwd_partials = nullptr;   // 2 per forward CTA
    float *wg_partials = nullptr;    // per row block
    double *scalars = nullptr;       // per batch: {loss sum, weight sum}
    float *pos = nullptr;            // guide positions
    float *mix = nullptr;            // guide mixtures
    pg_vmm_theta *net_vmm = nullptr; // the network's packed mixtures at region centres
    float *judge = nullptr;          // per-region judge sums (4 floats)
    uint32_t *judge_count = nullptr;
    uint32_t cap_guide = 0;
    uint32_t cap_rows = 0;           // padded batch rows
    uint32_t cap_batches = 0;
    uint32_t wg_blocks = 0;
    uint32_t wg_used = 0;            // row blocks of the last weight-gradient launch
    uint32_t loss_pending = 0;       // loss partials of the last batch the update still sums
    uint32_t step = 0;
    size_t smem = 0;
    __nv_bfloat16 *img = nullptr;    // tensor-core kernel's weight image
    uint32_t *err = nullptr;         // device error word of the tensor-core kernel
    int path = PG_MLP_PATH_TCGEN05;
};

namespace {

int mlp_error(int st, const char *msg) { return set_error(nullptr, st, msg); }

FwdArgs fwd_args(const pg_mlp *M) {
    FwdArgs A{};
    for (int i = 0; i < 3; ++i) {
        A.lo[i] = M->cfg.scene_aabb[i];
        const float ext = M->cfg.scene_aabb[3 + i] - M->cfg.scene_aabb[i];
        A.inv_ext[i] = ext > 0.0f ? 1.0f / ext : 0.0f;
    }
    A.wb = M->wb;
    A.theta = M->theta;
    return A;
}

// forward + backward + weight gradients of one batch; leaves the partials and
// the batch's scalars in scalars[2 * slot]
int batch_gradients(pg_mlp *M, const pg_directional_data *rec, uint32_t n, uint32_t slot, cudaStream_t s,
                    bool scalars_now = true, bool after_update = false) {
    if (M->path == PG_MLP_PATH_TCGEN05) {
        const uint32_t tiles = (n + tc::TILE - 1) / tc::TILE;
        const uint32_t grid = std::min<uint32_t>(tiles, (uint32_t)M->sm_count);
        tc::TrainArgs T{};
        FwdArgs F = fwd_args(M);
        T.rec = rec;
        T.n = n;
        for (int i = 0; i < 3; ++i) {
            T.lo[i] = F.lo[i];
            T.inv_ext[i] = F.inv_ext[i];
        }
        T.wimg = M->img;
        T.theta = M->theta;
        T.partials = M->wg_partials;
        T.loss_partials = M->fwd_partials;
        T.err = M->err;
        // behind the previous batch's update kernel: a programmatic dependent
        // launch (the prologue and the first records overlap that kernel)
        cudaLaunchConfig_t lc = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        lc.gridDim = dim3(grid, 1, 1);
        lc.blockDim = dim3(tc::TILE * tc::kTpr, 1, 1);
        lc.dynamicSmemBytes = tc::SM_TOTAL;
        lc.stream = s;
        lc.attrs = at;
        lc.numAttrs = after_update ? 1 : 0;
        if (cudaLaunchKernelEx(&lc, tc::k_train_tc<tc::kTpr>, T) != cudaSuccess)
            return mlp_error(PG_ERR_CUDA, "surrogate gradient launch");
        // the batch's scalars: now, or summed by the update that follows (one launch fewer)
        M->loss_pending = scalars_now ? 0u : grid;
        if (scalars_now) tc::k_tc_scalars<<<1, 256, 0, s>>>(M->fwd_partials, grid, M->scalars + 2 * slot);
        if (cudaGetLastError() != cudaSuccess) return mlp_error(PG_ERR_CUDA, "surrogate gradient launch");
        M->wg_used = grid;
        return PG_OK;
    }
    const uint32_t ctas = (n + kRowsPerCta - 1) / kRowsPerCta;
    const uint32_t rows = ctas * kRowsPerCta;
    FwdArgs A = fwd_args(M);
    A.rec = rec;
    A.n = n;
    A.scratch = M->scratch;
    A.partials = M->fwd_partials;
    k_fwd_bwd<true><<<ctas, 32 * kWarps, M->smem, s>>>(A);
    WgradArgs W{};
    W.scratch = M->scratch;
    W.rows = rows;
    const uint32_t blocks = std::min<uint32_t>(M->wg_blocks, (rows + 15) / 16);
    W.rows_per_block = ((rows / 16 + blocks - 1) / blocks) * 16;
    const uint32_t used = (rows + W.rows_per_block - 1) / W.rows_per_block;
    W.partials = M->wg_partials;
    W.fwd_partials = M->fwd_partials;
    W.n_fwd_partials = ctas * kWarps;
    W.scalars = M->scalars + 2 * slot;
    k_wgrad<<<dim3(used, 4), 32 * kWarps, 0, s>>>(W);
    if (cudaGetLastError() != cudaSuccess) return mlp_error(PG_ERR_CUDA, "surrogate gradient launch");
    M->wg_used = used;
    return PG_OK;
}

int reduce_step(pg_mlp *M, uint32_t slot, float *grad_out, cudaStream_t s) {
    AdamArgs A{};
    A.partials = M->wg_partials;
    A.n_blocks = M->wg_used;
    A.scalars = M->scalars + 2 * slot;
    if (M->loss_pending) {
        A.loss_partials = M->fwd_partials;
        A.n_loss = M->loss_pending;
        M->loss_pending = 0;
    }
    A.theta = M->theta;
    A.m = M->m;
    A.v = M->v;
    A.wb = M->wb;
    A.img = M->img;
    A.grad_out = grad_out;
    if (!grad_out) {
        M->step += 1;
        A.lr = M->cfg.lr;
        A.b1 = M->cfg.beta1;
        A.b2 = M->cfg.beta2;
        A.eps = M->cfg.eps;
        A.c1 = (float)(1.0 - pow((double)M->cfg.beta1, (double)M->step));
        A.c2 = (float)(1.0 - pow((double)M->cfg.beta2, (double)M->step));
    }
    k_reduce_adam<<<(NPARAM + 31) / 32, 32 * kAdamGroups, 0, s>>>(A);
    return cudaGetLastError() == cudaSuccess ? PG_OK : mlp_error(PG_ERR_CUDA, "surrogate update launch");
}

// grows the batch scratch to `rows` padded rows and `batches` scalar slots
int ensure_capacity(pg_mlp *M, uint32_t rows, uint32_t batches) {
    if (rows > M->cap_rows) {
        cudaFree(M->scratch);
        cudaFree(M->fwd_partials);
        M->scratch = nullptr;
        M->fwd_partials = nullptr;
        if (cudaMalloc(&M->scratch, sizeof(__nv_bfloat16) * (size_t)rows * RROW) != cudaSuccess ||
            cudaMalloc(&M->fwd_partials, sizeof(float) * 2 * (rows / 16)) != cudaSuccess) {
            M->cap_rows = 0;
            return mlp_error(PG_ERR_NOMEM, "surrogate batch scratch: out of device memory");
        }
        M->cap_rows = rows;
    }
    if (batches > M->cap_batches) {
        cudaFree(M->scalars);
        M->scalars = nullptr;
        if (cudaMalloc(&M->scalars, sizeof(double) * 2 * batches) != cudaSuccess) {
            M->cap_batches = 0;
            return mlp_error(PG_ERR_NOMEM, "surrogate scalars: out of device memory");
        }
        M->cap_batches = batches;
    }
    return PG_OK;
}

// After a stream synchronisation: a bounded wait of the tensor-core kernel
// that ran out is reported (and the word cleared).
int check_device_error(pg_mlp *M) {
    uint32_t e = 0;
    if (cudaMemcpy(&e, M->err, sizeof e, cudaMemcpyDeviceToHost) != cudaSuccess)
        return mlp_error(PG_ERR_CUDA, "surrogate error word");
    if (e) {
        cudaMemset(M->err, 0, sizeof(uint32_t));
        return mlp_error(PG_ERR_TIMEOUT, "surrogate tensor-core kernel (training or inference): a bounded wait timed out");
    }
    return PG_OK;
}

uint32_t padded_rows(uint64_t n) { return (uint32_t)(((n + kRowsPerCta - 1) / kRowsPerCta) * kRowsPerCta); }

}  // namespace

extern "C" {

void pg_mlp_default_config(pg_mlp_config *out) {
    if (!out) return;
    memset(out, 0, sizeof *out);
    out->batch = 65536;
    out->lr = 1e-3f;
    out->beta1 = 0.9f;
    out->beta2 = 0.999f;
    out->eps = 1e-8f;
    out->seed = 1;
    for (int i = 0; i < 3; ++i) {
        out->scene_aabb[i] = 0.0f;
        out->scene_aabb[3 + i] = 1.0f;
    }
}

int pg_mlp_create(const pg_mlp_config *cfg, pg_mlp **out) {
    if (!cfg || !out) return PG_ERR_ARG;
    if (cfg->batch == 0 || cfg->batch > (1u << 22)) return mlp_error(PG_ERR_ARG, "batch must be in [1, 2^22]");
    for (int i = 0; i < 3; ++i)
        if (!(cfg->scene_aabb[3 + i] > cfg->scene_aabb[i])) return mlp_error(PG_ERR_ARG, "empty scene box");
    pg_mlp *M = new pg_mlp();
    M->cfg = *cfg;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&M->sm_count, cudaDevAttrMultiProcessorCount, dev);
    M->wg_blocks = std::max(1, M->sm_count);
    M->smem = sizeof(Shared);
    bool ok = cudaMalloc(&M->theta, sizeof(float) * NPARAM) == cudaSuccess &&
              cudaMalloc(&M->m, sizeof(float) * NPARAM) == cudaSuccess &&
              cudaMalloc(&M->v, sizeof(float) * NPARAM) == cudaSuccess &&
              cudaMalloc(&M->wb, sizeof(__nv_bfloat16) * NWB) == cudaSuccess &&
              cudaMalloc(&M->wg_partials, sizeof(float) * (size_t)M->wg_blocks * NPARAM) == cudaSuccess &&
              cudaMalloc(&M->img, sizeof(__nv_bfloat16) * tc::NIMG) == cudaSuccess &&
              cudaMemset(M->img, 0, sizeof(__nv_bfloat16) * tc::NIMG) == cudaSuccess &&
              cudaMalloc(&M->err, sizeof(uint32_t)) == cudaSuccess &&
              cudaMemset(M->err, 0, sizeof(uint32_t)) == cudaSuccess;
    ok = ok && cudaFuncSetAttribute(k_fwd_bwd<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)M->smem) ==
                   cudaSuccess &&
         cudaFuncSetAttribute(k_fwd_bwd<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)M->smem) ==
             cudaSuccess &&
         cudaFuncSetAttribute(tc::k_train_tc<tc::kTpr>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              tc::SM_TOTAL) == cudaSuccess &&
         cudaFuncSetAttribute(tc::k_train_tc<tc::kTpr, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              tc::SM_TOTAL) == cudaSuccess;
    if (!ok) {
        pg_mlp_destroy(M);
        return mlp_error(PG_ERR_CUDA, "surrogate allocation failed");
    }
    // initial weights: the same construction as the oracle's init_params
    // (He-uniform hidden layers from a seeded generator, small output layer,
    // log-kappa biases log 5, spherical-Fibonacci mean directions)
    std::vector<float> th(NPARAM, 0.0f);
    uint64_t st = 0x9E3779B97F4A7C15ull ^ ((uint64_t)cfg->seed * 0xBF58476D1CE4E5B9ull);
    auto uni = [&]() {  // splitmix64 -> [0, 1)
        uint64_t z = (st += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    auto fill = [&](int ofs, int rows, int cols, int fan_in, double scale) {
        const double lim = sqrt(6.0 / fan_in) * scale;
        for (int r = 0; r < rows; ++r)
            for (int c = 0; c < cols; ++c) th[ofs + r * cols + c] = (float)((2.0 * uni() - 1.0) * lim);
    };
    fill(OW1, NH, NIN, 99, 1.0);
    for (int r = 0; r < NH; ++r)
        for (int c = 99; c < NIN; ++c) th[OW1 + r * NIN + c] = 0.0f;
    fill(OW2, NH, NH, NH, 1.0);
    fill(OW3, NH, NH, NH, 1.0);
    fill(OW4, NOUT, NH, NH, 0.1);
    for (int j = 0; j < NC; ++j) {
        const double jj = j + 0.5, z = 1.0 - 2.0 * jj / NC, phi = 3.14159265358979323846 * (3.0 - sqrt(5.0)) * jj;
        const double rr = sqrt(1.0 - z * z);
        th[OB4 + 5 * j + 1] = (float)(rr * cos(phi));
        th[OB4 + 5 * j + 2] = (float)(rr * sin(phi));
        th[OB4 + 5 * j + 3] = (float)z;
        th[OB4 + 5 * j + 4] = (float)log(5.0);
    }
    *out = M;
    const int rc = pg_mlp_set_params(M, th.data());
    if (rc) {
        pg_mlp_destroy(M);
        *out = nullptr;
    }
    return rc;
}

int pg_mlp_destroy(pg_mlp *M) {
    if (!M) return PG_OK;
    cudaFree(M->theta);
    cudaFree(M->m);
    cudaFree(M->v);
    cudaFree(M->wb);
    cudaFree(M->scratch);
    cudaFree(M->fwd_partials);
    cudaFree(M->wg_partials);
    cudaFree(M->scalars);
    cudaFree(M->pos);
    cudaFree(M->mix);
    cudaFree(M->net_vmm);
    cudaFree(M->judge);
    cudaFree(M->judge_count);
    cudaFree(M->img);
    cudaFree(M->err);
    delete M;
    return PG_OK;
}

int pg_mlp_get_params(pg_mlp *M, float *host_out) {
    if (!M || !host_out) return PG_ERR_ARG;
    return cudaMemcpy(host_out, M->theta, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost) == cudaSuccess
               ? PG_OK
               : mlp_error(PG_ERR_CUDA, "parameter download");
}

int pg_mlp_set_params(pg_mlp *M, const float *host_in) {
    if (!M || !host_in) return PG_ERR_ARG;
    if (cudaMemcpy(M->theta, host_in, sizeof(float) * NPARAM, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(M->m, 0, sizeof(float) * NPARAM) != cudaSuccess ||
        cudaMemset(M->v, 0, sizeof(float) * NPARAM) != cudaSuccess)
        return mlp_error(PG_ERR_CUDA, "parameter upload");
    k_theta_to_wb<<<(NPARAM + 255) / 256, 256>>>(M->theta, M->wb);
    tc::k_theta_to_img<<<(NPARAM + 255) / 256, 256>>>(M->theta, M->img);
    if (cudaDeviceSynchronize() != cudaSuccess) return mlp_error(PG_ERR_CUDA, "weight conversion");
    M->step = 0;
    return PG_OK;
}

int pg_mlp_loss_grad(pg_mlp *M, const pg_directional_data *records, uint32_t n, float *grad_out, float *loss_out,
                     void *stream) {
    if (!M || (!records && n)) return PG_ERR_ARG;
    if (n == 0 || n > M->cfg.batch) return mlp_error(PG_ERR_ARG, "n must be in [1, batch]");
    cudaStream_t s = (cudaStream_t)stream;
    if (int st = ensure_capacity(M, padded_rows(n), 1)) return st;
    if (int st = batch_gradients(M, records, n, 0, s)) return st;
    if (grad_out)
        if (int st = reduce_step(M, 0, grad_out, s)) return st;
    if (loss_out) {
        double sc[2];
        if (cudaMemcpyAsync(sc, M->scalars, sizeof sc, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return mlp_error(PG_ERR_CUDA, "loss download");
        if (int st = check_device_error(M)) return st;
        *loss_out = sc[1] > 0.0 ? (float)(sc[0] / sc[1]) : 0.0f;
    }
    return PG_OK;
}

int pg_mlp_train(pg_mlp *M, const pg_directional_data *records, uint64_t n, float *loss_out, void *stream) {
    if (!M || (!records && n)) return PG_ERR_ARG;
    if (n == 0) return PG_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const uint64_t B = M->cfg.batch;
    const uint32_t batches = (uint32_t)((n + B - 1) / B);
    if (int st = ensure_capacity(M, padded_rows(std::min<uint64_t>(n, B)), batches)) return st;
    for (uint32_t b = 0; b < batches; ++b) {
        const uint64_t first = (uint64_t)b * B;
        const uint32_t cnt = (uint32_t)std::min<uint64_t>(B, n - first);
        if (int st = batch_gradients(M, records + first, cnt, b, s, false, b > 0)) return st;
        if (int st = reduce_step(M, b, nullptr, s)) return st;
    }
    if (loss_out) {
        std::vector<double> sc(2 * (size_t)batches);
        if (cudaMemcpyAsync(sc.data(), M->scalars, sizeof(double) * sc.size(), cudaMemcpyDeviceToHost, s) !=
                cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return mlp_error(PG_ERR_CUDA, "loss download");
        if (int st = check_device_error(M)) return st;
        double acc = 0.0;
        for (uint32_t b = 0; b < batches; ++b) acc += sc[2 * b + 1] > 0.0 ? sc[2 * b] / sc[2 * b + 1] : 0.0;
        *loss_out = (float)(acc / batches);
    }
    return PG_OK;
}

int pg_mlp_set_path(pg_mlp *M, int path) {
    if (!M || (path != PG_MLP_PATH_TCGEN05 && path != PG_MLP_PATH_WARP_MMA)) return PG_ERR_ARG;
    M->path = path;
    return PG_OK;
}

int pg_mlp_infer(pg_mlp *M, const float *positions, uint32_t n, float *mixtures_out, void *stream) {
    if (!M || (n && (!positions || !mixtures_out))) return PG_ERR_ARG;
    if (n == 0) return PG_OK;
    if (M->path == PG_MLP_PATH_TCGEN05) {
        const uint32_t tiles = (n + tc::TILE - 1) / tc::TILE;
        const uint32_t grid = std::min<uint32_t>(tiles, (uint32_t)M->sm_count);
        tc::TrainArgs T{};
        const FwdArgs F = fwd_args(M);
        for (int i = 0; i < 3; ++i) {
            T.lo[i] = F.lo[i];
            T.inv_ext[i] = F.inv_ext[i];
        }
        T.n = n;
        T.pos = positions;
        T.mix_out = mixtures_out;
        T.wimg = M->img;
        T.theta = M->theta;
        T.err = M->err;
        tc::k_train_tc<tc::kTpr, true><<<grid, tc::TILE * tc::kTpr, tc::SM_TOTAL, (cudaStream_t)stream>>>(T);
        return cudaGetLastError() == cudaSuccess ? PG_OK : mlp_error(PG_ERR_CUDA, "surrogate inference launch");
    }
    FwdArgs A = fwd_args(M);
    A.pos = positions;
    A.n = n;
    A.mix_out = mixtures_out;
    k_fwd_bwd<false><<<(n + kRowsPerCta - 1) / kRowsPerCta, 32 * kWarps, M->smem, (cudaStream_t)stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? PG_OK : mlp_error(PG_ERR_CUDA, "surrogate inference launch");
}

}  // extern "C"

namespace {
// the network's mixtures at the centres of the context's regions, packed into
// the context's guide (to_ctx) or into the surrogate's own buffer
int net_guide(pg_mlp *M, const GuideTarget &T, bool to_ctx, cudaStream_t s) {
    if (T.n_regions > M->cap_guide) {
        cudaFree(M->pos);
        cudaFree(M->mix);
        cudaFree(M->net_vmm);
        cudaFree(M->judge);
        M->pos = M->mix = M->judge = nullptr;
        M->net_vmm = nullptr;
        if (cudaMalloc(&M->pos, sizeof(float) * 3 * (size_t)T.n_regions) != cudaSuccess ||
            cudaMalloc(&M->mix, sizeof(float) * NOUT * (size_t)T.n_regions) != cudaSuccess ||
            cudaMalloc(&M->net_vmm, sizeof(pg_vmm_theta) * (size_t)T.n_regions) != cudaSuccess ||
            cudaMalloc(&M->judge, sizeof(float) * 4 * (size_t)T.n_regions) != cudaSuccess) {
            M->cap_guide = 0;
            return mlp_error(PG_ERR_NOMEM, "guide scratch: out of device memory");
        }
        M->cap_guide = T.n_regions;
    }
    k_region_centres<<<(T.n_regions + 255) / 256, 256, 0, s>>>(T.aabbs, T.n_regions, M->pos);
    if (int st = pg_mlp_infer(M, M->pos, T.n_regions, M->mix, s)) return st;
    // a tensor-core wait that ran out leaves mixtures unwritten: check before
    // they become a guide
    if (cudaStreamSynchronize(s) != cudaSuccess) return mlp_error(PG_ERR_CUDA, "surrogate inference");
    if (int st = check_device_error(M)) return st;
    k_pack_guide<<<T.n_regions, NC, 0, s>>>(M->mix, M->pos, T.n_regions, to_ctx ? T.vmm : M->net_vmm);
    return cudaGetLastError() == cudaSuccess ? PG_OK : mlp_error(PG_ERR_CUDA, "guide pack launch");
}
}  // namespace

extern "C" {

int pg_mlp_write_guide(pg_mlp *M, pg_ctx *guide, void *stream) {
    if (!M || !guide) return PG_ERR_ARG;
    GuideTarget T{};
    if (int st = guide_target(guide, &T)) return st;
    if (int st = net_guide(M, T, true, (cudaStream_t)stream)) return st;
    guide_mark_written(guide);
    return PG_OK;
}

int pg_mlp_judge_guide(pg_mlp *M, pg_ctx *guide, const pg_directional_data *records, uint64_t n,
                       uint32_t min_records, uint32_t *switched_out, void *stream) {
    if (!M || !guide || (!records && n)) return PG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    GuideView V{};
    if (int st = guide_view(guide, &V, s)) return st;  // brings the fit's packed mixtures up to date
    GuideTarget T{};
    if (int st = guide_target(guide, &T)) return st;
    if (int st = net_guide(M, T, false, s)) return st;
    if (!M->judge_count && cudaMalloc(&M->judge_count, sizeof(uint32_t)) != cudaSuccess)
        return mlp_error(PG_ERR_NOMEM, "judge counter");
    if (cudaMemsetAsync(M->judge, 0, sizeof(float) * 4 * (size_t)T.n_regions, s) != cudaSuccess ||
        cudaMemsetAsync(M->judge_count, 0, sizeof(uint32_t), s) != cudaSuccess)
        return mlp_error(PG_ERR_CUDA, "judge reset");
    if (n) {
        const uint32_t blocks = (uint32_t)std::min<uint64_t>((n + 255) / 256, (uint64_t)M->sm_count * 8);
        k_judge_accumulate<<<blocks, 256, 0, s>>>(records, n, T.vmm, M->net_vmm, T.n_regions, V.use_parallax,
                                                  M->judge);
    }
    k_judge_select<<<(T.n_regions + 255) / 256, 256, 0, s>>>(M->judge, M->net_vmm, T.n_regions,
                                                              (float)std::max(1u, min_records), T.vmm,
                                                              M->judge_count);
    if (cudaGetLastError() != cudaSuccess) return mlp_error(PG_ERR_CUDA, "judge launch");
    guide_mark_written(guide);
    if (switched_out) {
        if (cudaMemcpyAsync(switched_out, M->judge_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, s) !=
                cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return mlp_error(PG_ERR_CUDA, "judge count download");
    }
    return PG_OK;
}

int pg_guide_nll(pg_ctx *guide, const pg_directional_data *records, uint64_t n, double *nll_out, void *stream) {
    if (!guide || !nll_out || (!records && n)) return PG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    GuideView V{};
    if (int st = guide_view(guide, &V, s)) return st;
    double *acc = nullptr;
    if (cudaMalloc(&acc, 2 * sizeof(double)) != cudaSuccess) return mlp_error(PG_ERR_NOMEM, "nll accumulators");
    double h[2] = {0.0, 0.0};
    int st = PG_OK;
    if (cudaMemsetAsync(acc, 0, 2 * sizeof(double), s) != cudaSuccess) st = PG_ERR_CUDA;
    if (!st && n) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const uint32_t blocks = (uint32_t)std::min<uint64_t>((n + 255) / 256, (uint64_t)std::max(sms, 1) * 8);
        k_guide_nll<<<blocks, 256, 0, s>>>(records, n, V.vmm, V.n_regions, V.use_parallax, acc);
        if (cudaGetLastError() != cudaSuccess) st = PG_ERR_CUDA;
    }
    if (!st && (cudaMemcpyAsync(h, acc, sizeof h, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess))
        st = PG_ERR_CUDA;
    cudaFree(acc);
    if (st) return mlp_error(st, "guide NLL");
    *nll_out = h[1] > 0.0 ? h[0] / h[1] : 0.0;
    return PG_OK;
}

}  // extern "C"
