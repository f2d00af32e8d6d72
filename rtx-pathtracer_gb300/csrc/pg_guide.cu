// pg_guide.cu - the guiding steps around the fit, all device-resident:
//   * region tree (PathGuiding::createRegions, src/PathGuiding.cpp:81-104)
//   * stable bucket of the tracer's sample records by region
//     (SampleCollector::getSortedData, src/SampleCollector.cpp:76-131)
//   * parallax pre-pass (PathGuiding::preFit, src/PathGuiding.cpp:370-411)
//   * harmonic-mean lobe distances (the statistic of
//     external/guiding/incrementaldistance.h:57-107, PathGuiding::postFit :445-448)
//   * VMM_Theta packing (PathGuiding::pmmToVMM_Theta / syncPMMsToVMM_Thetas,
//     src/PathGuiding.cpp:53-69, 106-132)
//   * pg_update: the whole training pass (PathGuiding::update, :276-312).
//
// The sort is an LSD radix sort of 8-bit region-id digits over (id, index)
// pairs.  Each pass: per-tile digit histograms, a scan over (digit, tile),
// then a stable scatter whose in-tile ranks come from warp match masks in
// index order, so equal ids keep their original order (the reference's
// std::sort by flags leaves that order unspecified).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "pg_internal.cuh"

namespace pg {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;                          // keys per thread
constexpr int kSortTile = kSortThreads * kSortItems;    // 4096 keys per tile
constexpr int kScanThreads = 1024;

// Pass 0 input: the region id of each record (ids >= n_regions and INVALID
// become the sentinel n_regions, sorted last and dropped).
__global__ void sort_extract_keys(const pg_directional_data *rec, uint64_t n, uint32_t n_regions,
                                  uint32_t *keys, uint32_t *vals) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t f = rec[i].flags;
        keys[i] = f < n_regions ? f : n_regions;
        vals[i] = (uint32_t)i;
    }
}

__global__ void __launch_bounds__(kSortThreads) sort_histogram(const uint32_t *keys, uint32_t n, int shift,
                                                               uint32_t n_tiles, uint32_t *tile_counts) {
    __shared__ uint32_t h[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * (uint32_t)kSortTile;
    for (int j = 0; j < kSortItems; ++j) {
        const uint32_t idx = base + j * kSortThreads + threadIdx.x;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255u], 1u);
    }
    __syncthreads();
    // digit-major layout: counts[d * n_tiles + tile]
    for (int d = threadIdx.x; d < 256; d += blockDim.x) tile_counts[(size_t)d * n_tiles + blockIdx.x] = h[d];
}

// Exclusive scan of n values in place (three launches: chunk sums, scan of
// the sums in one CTA, rescan of each chunk with its offset).
__global__ void __launch_bounds__(kScanThreads) scan_chunk_sums(const uint32_t *v, uint32_t n, uint32_t *sums) {
    __shared__ uint32_t w[32];
    const uint32_t i = blockIdx.x * kScanThreads + threadIdx.x;
    uint32_t x = i < n ? v[i] : 0u;
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t y = w[threadIdx.x];
        for (int o = 16; o > 0; o >>= 1) y += __shfl_xor_sync(0xffffffffu, y, o);
        if (threadIdx.x == 0) sums[blockIdx.x] = y;
    }
}

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t x, uint32_t *total) {
    __shared__ uint32_t w[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = x;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) w[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        uint32_t v = lane < nw ? w[lane] : 0u;
        uint32_t vi = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, vi, o);
            if (lane >= o) vi += y;
        }
        if (lane < nw) w[lane] = vi - v;
        if (lane == nw - 1) *total = vi;
    }
    __syncthreads();
    const uint32_t r = w[warp] + incl - x;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kScanThreads) scan_sums_single(uint32_t *sums, uint32_t n) {
    __shared__ uint32_t carry, tot;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < n; base += kScanThreads) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t x = i < n ? sums[i] : 0u;
        const uint32_t e = block_exclusive_scan(x, &tot);
        if (i < n) sums[i] = carry + e;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kScanThreads) scan_chunks_apply(uint32_t *v, uint32_t n, const uint32_t *sums) {
    __shared__ uint32_t tot;
    const uint32_t i = blockIdx.x * kScanThreads + threadIdx.x;
    const uint32_t x = i < n ? v[i] : 0u;
    const uint32_t e = block_exclusive_scan(x, &tot);
    if (i < n) v[i] = sums[blockIdx.x] + e;
}

// Stable scatter of one digit pass.  Warp w of the tile owns keys
// [base + w*512, base + (w+1)*512) in 16 groups of 32 consecutive keys; ranks
// follow index order within the group (match masks), then across groups, then
// across warps, so the scatter is stable.
__global__ void __launch_bounds__(kSortThreads) sort_scatter(const uint32_t *keys_in, const uint32_t *vals_in,
                                                             uint32_t n, int shift, uint32_t n_tiles,
                                                             const uint32_t *tile_offsets, uint32_t *keys_out,
                                                             uint32_t *vals_out) {
    constexpr int NW = kSortThreads / 32;
    __shared__ uint32_t wcount[NW][256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int d = lane; d < 256; d += 32) wcount[warp][d] = 0;
    __syncwarp();
    const uint32_t base = blockIdx.x * (uint32_t)kSortTile + (uint32_t)warp * 32u * kSortItems;
    uint32_t k[kSortItems], v[kSortItems], pos[kSortItems];
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
        const uint32_t idx = base + j * 32 + lane;
        const bool ok = idx < n;
        k[j] = ok ? keys_in[idx] : 0xFFFFFFFFu;
        v[j] = ok ? vals_in[idx] : 0u;
        const int d = ok ? (int)((k[j] >> shift) & 255u) : -1;
        const unsigned m = __match_any_sync(0xffffffffu, d);
        const unsigned lt = m & ((1u << lane) - 1u);
        const uint32_t before = (d >= 0) ? wcount[warp][d] : 0u;
        pos[j] = before + __popc(lt);
        __syncwarp();
        if (d >= 0 && lt == 0) wcount[warp][d] = before + __popc(m);
        __syncwarp();
    }
    __syncthreads();
    // per digit: warps' exclusive prefix (warp order = index order)
    for (int d = threadIdx.x; d < 256; d += blockDim.x) {
        uint32_t acc = tile_offsets[(size_t)d * n_tiles + blockIdx.x];
        for (int w = 0; w < NW; ++w) {
            const uint32_t c = wcount[w][d];
            wcount[w][d] = acc;
            acc += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
        const uint32_t idx = base + j * 32 + lane;
        if (idx < n) {
            const uint32_t d = (k[j] >> shift) & 255u;
            const uint32_t dst = wcount[warp][d] + pos[j];
            keys_out[dst] = k[j];
            vals_out[dst] = v[j];
        }
    }
}

// offsets[r] = first sorted position with key >= r (r = 0..n_regions).
__global__ void sort_offsets(const uint32_t *keys, uint32_t n, uint32_t n_regions, uint32_t *offsets) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r <= n_regions; r += gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = n;
        while (lo < hi) {
            const uint32_t mid = lo + (hi - lo) / 2;
            if (keys[mid] < r)
                lo = mid + 1;
            else
                hi = mid;
        }
        offsets[r] = lo;
    }
}

// Gathers the sorted records (valid ones only).
__global__ void gather_records(const pg_directional_data *rec, const uint32_t *order, const uint32_t *offsets,
                               uint32_t n_regions, pg_directional_data *out) {
    const uint32_t n = offsets[n_regions];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = rec[order[i]];
}

// ---------------------------------------------------------------------------
// Parallax pre-pass, distances, reposition, packing
// ---------------------------------------------------------------------------

// PathGuiding::preFit (src/PathGuiding.cpp:370-402) for every sorted sample:
// the region's parallax mean is its box centre; a sample with distance > 0 is
// re-aimed from the mean at the point it saw, others get distance +inf.
// Reads the records through the sort order (gather) and writes the fit's
// float4 {direction, weight} and the re-centred distance.
// The sample count is n_valid, or *n_valid_dev when given (the sort's valid
// count, which only the device knows); records with an out-of-range region id
// are written with zero weight.
// pdf (may be null): the records' sampling pdf, for the split/merge statistics.
__global__ void prefit_parallax_kernel(const pg_directional_data *rec, const uint32_t *order, uint32_t n_valid,
                                       const uint32_t *n_valid_dev, uint32_t n_regions, const float *means,
                                       int use_parallax, float4 *dirw, float *dist, float *pdf) {
    const uint32_t n = n_valid_dev ? *n_valid_dev : n_valid;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const pg_directional_data d = rec[order ? order[i] : i];
        float dx = d.direction[0], dy = d.direction[1], dz = d.direction[2];
        float t = d.distance;
        if (pdf) pdf[i] = d.pdf;
        if (d.flags >= n_regions) {
            dirw[i] = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
            dist[i] = INFINITY;
            continue;
        }
        if (use_parallax) {
            const float *m = means + 3 * (size_t)d.flags;
            if (d.distance > 0.0f) {
                const float nx = __fsub_rn(__fadd_rn(d.position[0], __fmul_rn(d.distance, dx)), m[0]);
                const float ny = __fsub_rn(__fadd_rn(d.position[1], __fmul_rn(d.distance, dy)), m[1]);
                const float nz = __fsub_rn(__fadd_rn(d.position[2], __fmul_rn(d.distance, dz)), m[2]);
                const float l2 = __fadd_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)), __fmul_rn(nz, nz));
                const float l = __fsqrt_rn(l2);
                const float inv = __fdiv_rn(1.0f, l);
                dx = __fmul_rn(nx, inv);
                dy = __fmul_rn(ny, inv);
                dz = __fmul_rn(nz, inv);
                t = l;
            } else {
                t = INFINITY;
            }
        }
        dirw[i] = make_float4(dx, dy, dz, d.weight);
        dist[i] = t;
    }
}

// Per region: record the previous parallax mean, set the new one (box centre,
// src/PathGuiding.cpp:380-383) and, after the first fit, re-aim the lobes with a
// finite distance at the new mean (IncrementalDistance::reposition,
// external/guiding/incrementaldistance.h:109-131).
__global__ void parallax_means_kernel(pg_region_state *states, const float *aabbs, const uint32_t *offsets,
                                      uint32_t n_regions, int reposition, float *means_out) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_regions) return;
    pg_region_state *s = states + r;
    const float *b = aabbs + 6 * (size_t)r;
    float m[3];
    for (int i = 0; i < 3; ++i) {
        m[i] = __fadd_rn(b[i], __fmul_rn(0.5f, __fsub_rn(b[3 + i], b[i])));
        means_out[3 * (size_t)r + i] = m[i];
    }
    // regions without samples in this pass are left alone (PathGuiding::update
    // calls updateRegion only for non-empty ranges, src/PathGuiding.cpp:281-288)
    if (offsets && offsets[r + 1] == offsets[r]) return;
    for (int i = 0; i < 3; ++i) {
        s->last_parallax_mean[i] = s->parallax_mean[i];
        s->parallax_mean[i] = m[i];
    }
    if (!reposition) return;
    const float d0 = __fsub_rn(s->last_parallax_mean[0], m[0]);
    const float d1 = __fsub_rn(s->last_parallax_mean[1], m[1]);
    const float d2 = __fsub_rn(s->last_parallax_mean[2], m[2]);
    for (uint32_t c = 0; c < s->k && c < 16; ++c) {
        const float dist = s->distance[c];
        if (isinf(dist) || s->dist_sum_w[c] <= 0.0f) continue;
        const float x = __fadd_rn(__fmul_rn(s->mu_x[c], dist), d0);
        const float y = __fadd_rn(__fmul_rn(s->mu_y[c], dist), d1);
        const float z = __fadd_rn(__fmul_rn(s->mu_z[c], dist), d2);
        const float l = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
        s->distance[c] = l;
        s->mu_x[c] = __fdiv_rn(x, l);
        s->mu_y[c] = __fdiv_rn(y, l);
        s->mu_z[c] = __fdiv_rn(z, l);
    }
}

// Harmonic-mean distance per lobe, weighted by w * gamma_k * pdf_k over the
// samples with distance > 0 (the statistic of incrementaldistance.h:57-107),
// merged with the previous estimate.  The samples are cut into work items of
// at most kDistChunk samples of one region, so a large region is spread over
// many CTAs: distance_items_kernel numbers the items (region-major),
// distance_partial_kernel sums each item's 32 statistics, and
// distance_finalize_kernel adds a region's items in item order (Neumaier) and
// updates the lobes - deterministic whatever the launch shape.
constexpr uint32_t kDistChunk = 2048;
constexpr int kDistThreads = 64;

// item_offsets[r] = first work item of region r (empty regions have none);
// item_offsets[n_regions] = the item count.  One CTA.
// item_region[i] = the region of work item i (items beyond cap_items are not
// written; the partial kernel then reports the overflow).
__global__ void __launch_bounds__(kScanThreads) distance_items_kernel(const uint32_t *offsets, uint32_t n_regions,
                                                                      uint32_t *item_offsets, uint32_t *item_region,
                                                                      uint64_t cap_items) {
    __shared__ uint32_t carry, tot;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < n_regions; base += kScanThreads) {
        const uint32_t r = base + threadIdx.x;
        const uint32_t n = r < n_regions ? offsets[r + 1] - offsets[r] : 0u;
        const uint32_t cnt = (n + kDistChunk - 1) / kDistChunk;
        const uint32_t e = block_exclusive_scan(cnt, &tot);
        if (r < n_regions) {
            item_offsets[r] = carry + e;
            for (uint32_t i = carry + e; i < carry + e + cnt && i < cap_items; ++i) item_region[i] = r;
        }
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) item_offsets[n_regions] = carry;
}

// Per work item: the sums over its samples of a_k = w gamma_k pdf_k and
// a_k / t.  With e_k = pi_k pdf_k (one ex2 per lobe; the exponent
// kl (mu.d - 1) + log2(norm) is clamped at log2(norm), cos <= 1) and
// p = sum_k e_k: a_k = (w / p) e_k^2 / pi_k.  partial[item] = {sum a[16],
// sum a / t[16]}.  More items than the scratch holds: nothing is written and
// PG_DEV_ERR_BOUNDS is reported.
__global__ void __launch_bounds__(kDistThreads) distance_partial_kernel(const pg_region_state *states,
                                                                        const float4 *dirw, const float *dist,
                                                                        const uint32_t *offsets, uint32_t n_regions,
                                                                        const uint32_t *item_offsets,
                                                                        const uint32_t *item_region, float *partial,
                                                                        uint64_t cap_items, uint32_t *error_word) {
    constexpr int NW = kDistThreads / 32;
    // component constants as pairs (component 2j in .x, 2j + 1 in .y): the
    // per-sample arithmetic runs on packed FP32x2 instructions
    __shared__ float2 c_ax[8], c_ay[8], c_az[8], c_c0[8], c_cm[8], c_lk[8], c_ipi[8];
    __shared__ float red[NW][32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t n_items = item_offsets[n_regions];
    if (n_items > cap_items) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(error_word, PG_DEV_ERR_BOUNDS);
        return;
    }
    for (uint32_t item = blockIdx.x; item < n_items; item += gridDim.x) {
        const uint32_t r = item_region[item];
        const pg_region_state *s = states + r;
        if (tid < 16) {
            const int c = tid;
            const uint32_t K = min(s->k, 16u);
            const bool on = c < (int)K && s->norm[c] > 0.0f && s->weight[c] > 0.0f;
            const float kl = s->kappa[c] * kLog2e;
            const float ln = on ? log2f(s->norm[c]) : -INFINITY;
            float *ax = reinterpret_cast<float *>(c_ax), *ay = reinterpret_cast<float *>(c_ay),
                  *az = reinterpret_cast<float *>(c_az), *c0 = reinterpret_cast<float *>(c_c0),
                  *cm = reinterpret_cast<float *>(c_cm), *lk = reinterpret_cast<float *>(c_lk),
                  *ipi = reinterpret_cast<float *>(c_ipi);
            ax[c] = kl * s->mu_x[c];
            ay[c] = kl * s->mu_y[c];
            az[c] = kl * s->mu_z[c];
            c0[c] = ln - kl;
            cm[c] = ln;
            lk[c] = on ? log2f(s->weight[c]) : -INFINITY;
            ipi[c] = on ? 1.0f / s->weight[c] : 0.0f;
        }
        __syncthreads();
        float2 bw[8], bwd[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) bw[j] = bwd[j] = make_float2(0.0f, 0.0f);
        const uint32_t b = offsets[r] + (item - item_offsets[r]) * kDistChunk;
        const uint32_t e = min(offsets[r + 1], b + kDistChunk);
        // the next sample's distance and direction load while this one computes
        uint32_t i = b + tid;
        float t_nx = i < e ? dist[i] : 0.0f;
        float4 d_nx = i < e ? dirw[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        for (; i < e; i += kDistThreads) {
            const float t = t_nx;
            const float4 d = d_nx;
            if (i + kDistThreads < e) {
                t_nx = dist[i + kDistThreads];
                d_nx = dirw[i + kDistThreads];
            }
            if (!(t > 0.0f)) continue;
            const float2 dx2 = make_float2(d.x, d.x), dy2 = make_float2(d.y, d.y), dz2 = make_float2(d.z, d.z);
            float2 ek[8];
            float p = 0.0f;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                float2 a = __ffma2_rn(c_az[j], dz2, c_c0[j]);
                a = __ffma2_rn(c_ay[j], dy2, a);
                a = __ffma2_rn(c_ax[j], dx2, a);
                const float2 m = c_cm[j], l = c_lk[j];
                ek[j].x = ex2_approx(fminf(a.x, m.x) + l.x);
                ek[j].y = ex2_approx(fminf(a.y, m.y) + l.y);
                p += ek[j].x;
                p += ek[j].y;
            }
            if (!(p > kPmmEps)) continue;
            const float sc = d.w / p;
            const float it = 1.0f / t;
            const float2 sc2 = make_float2(sc, sc), it2 = make_float2(it, it);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const float2 a = __fmul2_rn(__fmul2_rn(__fmul2_rn(ek[j], ek[j]), c_ipi[j]), sc2);
                bw[j] = __fadd2_rn(bw[j], a);
                bwd[j] = __ffma2_rn(a, it2, bwd[j]);
            }
        }
#pragma unroll
        for (int c = 0; c < 16; ++c) {
            float x = (c & 1) ? bw[c >> 1].y : bw[c >> 1].x, y = (c & 1) ? bwd[c >> 1].y : bwd[c >> 1].x;
            for (int o = 16; o > 0; o >>= 1) {
                x += __shfl_xor_sync(0xffffffffu, x, o);
                y += __shfl_xor_sync(0xffffffffu, y, o);
            }
            if (lane == 0) {
                red[warp][c] = x;
                red[warp][16 + c] = y;
            }
        }
        __syncthreads();
        if (tid < 32) {
            float h = 0.f, l = 0.f;
            for (int w = 0; w < NW; ++w) neumaier_add(h, l, red[w][tid]);
            partial[(size_t)item * 32 + tid] = h + l;
        }
        __syncthreads();
    }
}

// One warp per region: the items' sums added in item order, then the
// harmonic-mean update of every lane of the active 4-lane groups, as the
// reference's SIMD update does.  Regions without samples are not updated
// (postFit runs only for non-empty regions, src/PathGuiding.cpp:281-288): an
// empty batch would turn the initial infinite distance into 0/0.
__global__ void distance_finalize_kernel(pg_region_state *states, const uint32_t *item_offsets, uint32_t n_regions,
                                         const float *partial, uint64_t cap_items) {
    const uint32_t r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= n_regions || item_offsets[n_regions] > cap_items) return;
    const uint32_t i0 = item_offsets[r], i1 = item_offsets[r + 1];
    if (i0 == i1) return;
    float h = 0.f, l = 0.f;
    for (uint32_t it = i0; it < i1; ++it) neumaier_add(h, l, partial[(size_t)it * 32 + lane]);
    const float sum = h + l;
    const float wd = __shfl_down_sync(0xffffffffu, sum, 16);  // lane c: the sum of a_c / t
    pg_region_state *s = states + r;
    const uint32_t K = min(s->k, 16u);
    if (lane < 16 && lane < (int)((K + 3u) & ~3u)) {
        const int c = lane;
        const float old_w = s->dist_sum_w[c];
        const float new_w = old_w + sum;
        s->distance[c] = new_w / (old_w / s->distance[c] + wd);
        s->dist_sum_w[c] = new_w;
    }
}

// PathGuiding::pmmToVMM_Theta + syncPMMsToVMM_Thetas; norm and e^{-2k} of
// VMF_Theta::setK are evaluated in double as the reference does.
__global__ void pack_vmm_theta_kernel(const pg_region_state *states, uint32_t n_regions, int use_parallax,
                                      pg_vmm_theta *out) {
    const uint32_t r = blockIdx.x;
    const int c = threadIdx.x;  // 16 threads
    if (r >= n_regions || c >= 16) return;
    const pg_region_state *s = states + r;
    pg_vmm_theta *v = out + r;
    const uint32_t K = min(s->k, 16u);
    pg_vmf_theta th;
    th.mu[0] = th.mu[1] = th.mu[2] = 0.0f;
    th.k = 0.0f;
    th.norm = 0.0f;
    th.e_min2k = 0.0f;
    th.distance = -1.0f;
    th.target[0] = th.target[1] = th.target[2] = 0.0f;
    float pi = 0.0f;
    if (c < (int)K) {
        pi = s->weight[c];
        th.mu[0] = s->mu_x[c];
        th.mu[1] = s->mu_y[c];
        th.mu[2] = s->mu_z[c];
        float k = s->kappa[c];
        k = k < kVmfMinKappa ? 0.0f : k;
        th.k = k;
        const double kd = (double)k;
        th.norm = (float)(kd / (2.0 * 3.14159265358979323846 * (1.0 - exp(-2.0 * kd))));
        th.e_min2k = (float)exp(-2.0 * kd);
    }
    if (use_parallax) {
        float dd = s->distance[c];
        dd = (dd == INFINITY) ? -1.0f : dd;
        th.distance = dd;
        for (int i = 0; i < 3; ++i) th.target[i] = __fadd_rn(s->parallax_mean[i], __fmul_rn(dd, th.mu[i]));
    }
    v->thetas[c] = th;
    v->pi[c] = pi;
    if (c == 0) {
        for (int i = 0; i < 3; ++i) v->mean_position[i] = use_parallax ? s->parallax_mean[i] : 0.0f;
        v->used_distributions = (int32_t)K;
    }
}

// PathGuiding::update's split check and splitRegion (src/PathGuiding.cpp:290-348)
// over regions [0, R), one CTA: regions above the threshold are ranked in
// region order by a block scan, the k-th becomes region R + k and takes nodes
// n_nodes + 2k, n_nodes + 2k + 1.  out = {new region count, new node count}.
__global__ void __launch_bounds__(1024) split_regions_kernel(pg_region_state *states, pg_region_extra *extras,
                                                             float *aabbs, int32_t *nodes, uint32_t *leaf_of,
                                                             uint32_t R, uint32_t n_nodes, uint32_t cap, float thr,
                                                             uint32_t *out) {
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t base;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (tid == 0) base = 0;
    __syncthreads();
    for (uint32_t c0 = 0; c0 < R; c0 += 1024u) {
        const uint32_t r = c0 + tid;
        const bool flag = r < R && states[r].num_samples > thr;
        const uint32_t bal = __ballot_sync(0xffffffffu, flag);
        if (lane == 0) warp_tot[warp] = __popc(bal);
        __syncthreads();
        uint32_t before = 0, total = 0;
        for (uint32_t w = 0; w < 32u; ++w) {
            const uint32_t t = warp_tot[w];
            before += w < warp ? t : 0u;
            total += t;
        }
        const uint32_t rank = base + before + __popc(bal & ((1u << lane) - 1u));
        if (flag && R + rank < cap) {
            const uint32_t nr = R + rank, a = n_nodes + 2u * rank;
            pg_region_state &st = states[r];
            st.num_samples = __fmul_rn(st.num_samples, 0.25f);  // decayTerm
            st.sample_weight = __fmul_rn(st.sample_weight, 0.25f);
            states[nr] = st;
            if (extras) extras[nr] = extras[r];
            // Aabb::splitAabb (src/Shapes.h:32-46): the lower half stays, the upper half is new
            float *b = aabbs + 6 * (size_t)r, *c = aabbs + 6 * (size_t)nr;
            float size[3];
            for (int i = 0; i < 3; ++i) size[i] = __fsub_rn(b[3 + i], b[i]);
            const int ax = size[0] > size[1] ? (size[0] > size[2] ? 0 : 2) : (size[1] > size[2] ? 1 : 2);
            for (int i = 0; i < 6; ++i) c[i] = b[i];
            const float half = __fmul_rn(0.5f, size[ax]);
            b[3 + ax] = __fsub_rn(b[3 + ax], half);
            c[ax] = __fadd_rn(c[ax], half);
            const uint32_t leaf = leaf_of[r];
            nodes[leaf] = (int32_t)a;
            nodes[a] = -(int32_t)r - 1;
            nodes[a + 1] = -(int32_t)nr - 1;
            leaf_of[r] = a;
            leaf_of[nr] = a + 1;
        }
        __syncthreads();
        if (tid == 0) base += total;
        __syncthreads();
    }
    if (tid == 0) {
        const uint32_t room = cap > R ? cap - R : 0u;
        const uint32_t n = base < room ? base : room;
        out[0] = R + n;
        out[1] = n_nodes + 2u * n;
    }
}

// ---------------------------------------------------------------------------
// Host helpers
// ---------------------------------------------------------------------------

// Region boxes: Aabb::addEpsilon then split_count rounds of midpoint splits
// along the largest axis, breadth first (src/Shapes.h:32-53,
// src/PathGuiding.cpp:81-104), in the reference's float arithmetic.
void region_boxes(uint32_t split_count, const float a[6], std::vector<float> &out) {
    float mn[3], mx[3];
    for (int i = 0; i < 3; ++i) {
        const float ext = a[3 + i] - a[i];
        const float cen = a[i] + 0.5f * ext;
        mn[i] = cen - 0.50001f * ext;
        mx[i] = cen + 0.50001f * ext;
    }
    std::vector<float> cur = {mn[0], mn[1], mn[2], mx[0], mx[1], mx[2]};
    for (uint32_t s = 0; s < split_count; ++s) {
        std::vector<float> nxt;
        nxt.reserve(cur.size() * 2);
        for (size_t b = 0; b < cur.size() / 6; ++b) {
            const float *bx = &cur[6 * b];
            float size[3];
            for (int i = 0; i < 3; ++i) size[i] = bx[3 + i] - bx[i];
            const int axis = size[0] > size[1] ? (size[0] > size[2] ? 0 : 2) : (size[1] > size[2] ? 1 : 2);
            float L[6], R[6];
            memcpy(L, bx, sizeof L);
            memcpy(R, bx, sizeof R);
            L[3 + axis] -= 0.5f * size[axis];
            R[axis] += 0.5f * size[axis];
            nxt.insert(nxt.end(), L, L + 6);
            nxt.insert(nxt.end(), R, R + 6);
        }
        cur.swap(nxt);
    }
    out.swap(cur);
}

}  // namespace pg

using namespace pg;

namespace pg {

// Scratch of the sort and of the guiding pass, grown on demand and owned by the context.
struct GuideScratch {
    uint32_t *keys[2] = {nullptr, nullptr};
    uint32_t *vals[2] = {nullptr, nullptr};
    uint32_t *tile_counts = nullptr;
    uint32_t *scan_sums = nullptr;
    uint64_t cap_n = 0;
    uint64_t cap_tiles = 0;
    float4 *dirw = nullptr;
    float *dist = nullptr;
    float *pdf = nullptr;
    uint32_t *offsets = nullptr;
    uint32_t *order = nullptr;
    float *means = nullptr;
    float *aabbs = nullptr;
    uint32_t n_regions = 0;
    uint32_t split_count = 0;
    uint64_t cap_samples = 0;
    bool fitted = false;
    pg_vmm_theta *vmm = nullptr;   // packed mixtures for the renderer
    bool vmm_fresh = false;
    float root[6] = {0, 0, 0, 0, 0, 0};
    // region tree (2 n - 1 nodes; see pg_get_region_tree) and each region's leaf
    int32_t *nodes = nullptr;
    uint32_t *leaf_of = nullptr;
    uint32_t n_nodes = 0;
    bool tree_split = false;       // a region was split: the renderer descends the node array
    uint32_t *split_out = nullptr; // device: new region and node counts
    pg_region_split_config rs{};
    // distance pass: work-item offsets per region and the items' partial sums
    uint32_t *dist_items = nullptr;
    uint32_t *dist_item_region = nullptr;  // per work item: its region
    float *dist_partial = nullptr;
    uint32_t cap_dist_regions = 0;
    uint64_t cap_dist_items = 0;
};

static GuideScratch &guide(pg_ctx *ctx) {
    if (!ctx->guide) ctx->guide = new GuideScratch();
    return *static_cast<GuideScratch *>(ctx->guide);
}

void guide_release(pg_ctx *ctx) {
    if (!ctx || !ctx->guide) return;
    GuideScratch &g = *static_cast<GuideScratch *>(ctx->guide);
    cudaFree(g.pdf);
    for (int i = 0; i < 2; ++i) {
        cudaFree(g.keys[i]);
        cudaFree(g.vals[i]);
    }
    cudaFree(g.tile_counts);
    cudaFree(g.scan_sums);
    cudaFree(g.dirw);
    cudaFree(g.dist);
    cudaFree(g.offsets);
    cudaFree(g.order);
    cudaFree(g.means);
    cudaFree(g.aabbs);
    cudaFree(g.vmm);
    cudaFree(g.nodes);
    cudaFree(g.leaf_of);
    cudaFree(g.split_out);
    cudaFree(g.dist_items);
    cudaFree(g.dist_item_region);
    cudaFree(g.dist_partial);
    delete static_cast<GuideScratch *>(ctx->guide);
    ctx->guide = nullptr;
}

}  // namespace pg

static int ensure_sort_capacity(pg_ctx *ctx, uint64_t n) {
    GuideScratch &g = guide(ctx);
    const uint64_t tiles = (n + kSortTile - 1) / kSortTile;
    if (n > g.cap_n) {
        for (int i = 0; i < 2; ++i) {
            cudaFree(g.keys[i]);
            cudaFree(g.vals[i]);
            g.keys[i] = g.vals[i] = nullptr;
        }
        for (int i = 0; i < 2; ++i) {
            int st = check_cuda(ctx, cudaMalloc(&g.keys[i], sizeof(uint32_t) * n), "sort keys");
            if (!st) st = check_cuda(ctx, cudaMalloc(&g.vals[i], sizeof(uint32_t) * n), "sort values");
            if (st) return st;
        }
        g.cap_n = n;
    }
    if (tiles > g.cap_tiles) {
        cudaFree(g.tile_counts);
        cudaFree(g.scan_sums);
        g.tile_counts = g.scan_sums = nullptr;
        const uint64_t cnt = 256 * tiles;
        int st = check_cuda(ctx, cudaMalloc(&g.tile_counts, sizeof(uint32_t) * cnt), "sort tile counts");
        if (!st)
            st = check_cuda(ctx, cudaMalloc(&g.scan_sums, sizeof(uint32_t) * ((cnt + kScanThreads - 1) / kScanThreads + 1)),
                            "sort scan sums");
        if (st) return st;
        g.cap_tiles = tiles;
    }
    return PG_OK;
}

static void exclusive_scan(uint32_t *v, uint32_t n, uint32_t *sums, cudaStream_t s) {
    const uint32_t chunks = (n + kScanThreads - 1) / kScanThreads;
    scan_chunk_sums<<<chunks, kScanThreads, 0, s>>>(v, n, sums);
    scan_sums_single<<<1, kScanThreads, 0, s>>>(sums, chunks);
    scan_chunks_apply<<<chunks, kScanThreads, 0, s>>>(v, n, sums);
}

// The distance pass: the work items, their partial sums, the per-region
// update.  The scratch holds the items of as many samples as the larger of the
// context's max_samples and the largest record set sorted so far; more
// samples than that are reported as PG_DEV_ERR_BOUNDS and leave the distances
// untouched.
static int update_distances(pg_ctx *ctx, const float4 *dirw, const float *dist, const uint32_t *offsets,
                            uint32_t n_regions, cudaStream_t s) {
    GuideScratch &g = guide(ctx);
    const uint64_t max_samples = std::max<uint64_t>(ctx->max_samples, g.cap_n);
    const uint64_t items = max_samples / kDistChunk + n_regions + 1;
    if (n_regions + 1 > g.cap_dist_regions) {
        cudaFree(g.dist_items);
        g.dist_items = nullptr;
        if (int st = check_cuda(ctx, cudaMalloc(&g.dist_items, sizeof(uint32_t) * (n_regions + 1)), "distance items"))
            return st;
        g.cap_dist_regions = n_regions + 1;
    }
    if (items > g.cap_dist_items) {
        cudaFree(g.dist_partial);
        cudaFree(g.dist_item_region);
        g.dist_partial = nullptr;
        g.dist_item_region = nullptr;
        g.cap_dist_items = 0;
        if (int st = check_cuda(ctx, cudaMalloc(&g.dist_partial, sizeof(float) * 32 * items), "distance sums"))
            return st;
        if (int st = check_cuda(ctx, cudaMalloc(&g.dist_item_region, sizeof(uint32_t) * items), "distance items"))
            return st;
        g.cap_dist_items = items;
    }
    distance_items_kernel<<<1, kScanThreads, 0, s>>>(offsets, n_regions, g.dist_items, g.dist_item_region,
                                                     g.cap_dist_items);
    // persistent: as many CTAs as are resident (each thread sums 32 samples of
    // an item; several items in flight per SM hide the per-item latency)
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, distance_partial_kernel, kDistThreads, 0) !=
            cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    const uint32_t grid = (uint32_t)std::min<uint64_t>(items, (uint64_t)ctx->sm_count * (uint64_t)per_sm);
    distance_partial_kernel<<<grid, kDistThreads, 0, s>>>(ctx->d_states, dirw, dist, offsets, n_regions,
                                                          g.dist_items, g.dist_item_region, g.dist_partial,
                                                          g.cap_dist_items,
                                                          ctx->d_counters + 2);
    distance_finalize_kernel<<<(n_regions + 7) / 8, 256, 0, s>>>(ctx->d_states, g.dist_items, n_regions,
                                                                  g.dist_partial, g.cap_dist_items);
    return check_cuda(ctx, cudaGetLastError(), "distance launch");
}

// Sorts the (region id, index) pairs of n records; leaves the sorted indices in
// *order_out (a scratch buffer) and the region offsets in offsets (device).
static int sort_records(pg_ctx *ctx, const pg_directional_data *rec, uint64_t n, uint32_t n_regions,
                        uint32_t *offsets, uint32_t **order_out, cudaStream_t s) {
    if (n > 0xFFFFFFFFull - kSortTile) return set_error(ctx, PG_ERR_ARG, "too many sample records");
    int st = ensure_sort_capacity(ctx, n ? n : 1);
    if (st) return st;
    GuideScratch &g = guide(ctx);
    const uint32_t nn = (uint32_t)n;
    const uint32_t tiles = (nn + kSortTile - 1) / kSortTile;
    if (nn > 0) {
        sort_extract_keys<<<std::min<uint32_t>((nn + 255) / 256, 8192u), 256, 0, s>>>(rec, n, n_regions, g.keys[0],
                                                                                     g.vals[0]);
        int passes = 0;
        for (uint32_t m = n_regions; m > 0; m >>= 8) ++passes;  // digits of the sentinel n_regions
        int cur = 0;
        for (int p = 0; p < passes; ++p) {
            const int shift = 8 * p;
            sort_histogram<<<tiles, kSortThreads, 0, s>>>(g.keys[cur], nn, shift, tiles, g.tile_counts);
            exclusive_scan(g.tile_counts, 256u * tiles, g.scan_sums, s);
            sort_scatter<<<tiles, kSortThreads, 0, s>>>(g.keys[cur], g.vals[cur], nn, shift, tiles, g.tile_counts,
                                                        g.keys[cur ^ 1], g.vals[cur ^ 1]);
            cur ^= 1;
        }
        sort_offsets<<<(n_regions + 256) / 256, 256, 0, s>>>(g.keys[cur], nn, n_regions, offsets);
        *order_out = g.vals[cur];
    } else {
        st = check_cuda(ctx, cudaMemsetAsync(offsets, 0, sizeof(uint32_t) * (n_regions + 1), s), "offsets");
        if (st) return st;
        *order_out = g.vals[0];
    }
    return check_cuda(ctx, cudaGetLastError(), "sort launch");
}

namespace pg {
int guide_target(pg_ctx *ctx, GuideTarget *out) {
    GuideScratch &g = guide(ctx);
    if (!g.aabbs || !g.vmm || g.n_regions == 0) return set_error(ctx, PG_ERR_STATE, "pg_set_regions must run first");
    out->aabbs = g.aabbs;
    out->n_regions = g.n_regions;
    out->vmm = g.vmm;
    return PG_OK;
}

void guide_mark_written(pg_ctx *ctx) { guide(ctx).vmm_fresh = true; }
void guide_mark_stale(pg_ctx *ctx) {
    if (ctx && ctx->guide) static_cast<GuideScratch *>(ctx->guide)->vmm_fresh = false;
}

int guide_view(pg_ctx *ctx, GuideView *out, cudaStream_t s) {
    GuideScratch &g = guide(ctx);
    if (!g.aabbs || !g.vmm) return set_error(ctx, PG_ERR_STATE, "pg_set_regions must run before guided rendering");
    if (!g.vmm_fresh) {
        int st = pg_pack_vmm_theta(ctx, g.n_regions, g.vmm, s);
        if (st) return st;
        g.vmm_fresh = true;
    }
    for (int i = 0; i < 6; ++i) out->root[i] = g.root[i];
    out->split_count = g.split_count;
    out->nodes = g.tree_split ? g.nodes : nullptr;
    out->n_regions = g.n_regions;
    out->vmm = g.vmm;
    out->use_parallax = ctx->cfg.use_parallax ? 1 : 0;
    return PG_OK;
}
}  // namespace pg

extern "C" {

int pg_set_regions(pg_ctx *ctx, uint32_t split_count, const float scene_aabb[6], void *stream) {
    if (!ctx || !scene_aabb) return PG_ERR_ARG;
    if (split_count > 24) return set_error(ctx, PG_ERR_ARG, "split_count must be <= 24");
    const uint32_t n = 1u << split_count;
    if (n > ctx->max_regions) return set_error(ctx, PG_ERR_ARG, "2^split_count exceeds the context's regions");
    GuideScratch &g = guide(ctx);
    std::vector<float> boxes;
    region_boxes(split_count, scene_aabb, boxes);
    cudaStream_t s = (cudaStream_t)stream;
    // boxes, means, packed mixtures and the tree for the context's capacity:
    // regions may be split later (pg_split_regions)
    const uint32_t cap = ctx->max_regions;
    if (!g.aabbs) {
        int st = check_cuda(ctx, cudaMalloc(&g.aabbs, sizeof(float) * 6 * cap), "region boxes");
        if (!st) st = check_cuda(ctx, cudaMalloc(&g.means, sizeof(float) * 3 * cap), "region means");
        if (!st) st = check_cuda(ctx, cudaMalloc(&g.nodes, sizeof(int32_t) * (2 * (size_t)cap)), "region tree");
        if (!st) st = check_cuda(ctx, cudaMalloc(&g.leaf_of, sizeof(uint32_t) * cap), "region leaves");
        if (!st) st = check_cuda(ctx, cudaMalloc(&g.split_out, sizeof(uint32_t) * 2), "split counts");
        if (st) return st;
    }
    // the complete tree in breadth-first order: inner node k has children 2k+1, 2k+2
    std::vector<int32_t> nodes(2 * (size_t)n - 1);
    std::vector<uint32_t> leaf_of(n);
    for (uint32_t k = 0; k + 1 < n; ++k) nodes[k] = (int32_t)(2 * k + 1);
    for (uint32_t r = 0; r < n; ++r) {
        nodes[n - 1 + r] = -(int32_t)r - 1;
        leaf_of[r] = n - 1 + r;
    }
    g.n_regions = n;
    g.n_nodes = 2 * n - 1;
    g.tree_split = false;
    g.split_count = split_count;
    g.fitted = false;
    g.vmm_fresh = false;
    for (int i = 0; i < 3; ++i) {  // Aabb::addEpsilon (src/Shapes.h:48-53)
        const float ext = scene_aabb[3 + i] - scene_aabb[i];
        const float cen = scene_aabb[i] + 0.5f * ext;
        g.root[i] = cen - 0.50001f * ext;
        g.root[3 + i] = cen + 0.50001f * ext;
    }
    if (!g.vmm) {
        int st0 = check_cuda(ctx, cudaMalloc(&g.vmm, sizeof(pg_vmm_theta) * cap), "packed mixtures");
        if (st0) return st0;
    }
    int st = check_cuda(ctx, cudaMemcpyAsync(g.aabbs, boxes.data(), sizeof(float) * 6 * n, cudaMemcpyHostToDevice, s),
                        "region boxes upload");
    if (!st)
        st = check_cuda(ctx, cudaMemcpyAsync(g.nodes, nodes.data(), sizeof(int32_t) * nodes.size(),
                                             cudaMemcpyHostToDevice, s), "region tree upload");
    if (!st)
        st = check_cuda(ctx, cudaMemcpyAsync(g.leaf_of, leaf_of.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, s),
                        "region leaves upload");
    if (!st) st = check_cuda(ctx, cudaStreamSynchronize(s), "region boxes sync");
    if (st) return st;
    return pg_init_regions(ctx, n, stream);
}


int pg_region_count(const pg_ctx *ctx, uint32_t *out) {
    if (!ctx || !out) return PG_ERR_ARG;
    *out = ctx->guide ? static_cast<const GuideScratch *>(ctx->guide)->n_regions : 0u;
    return PG_OK;
}

int pg_get_region_aabbs(pg_ctx *ctx, float *host_out, uint32_t count) {
    if (!ctx || !host_out) return PG_ERR_ARG;
    GuideScratch &g = guide(ctx);
    if (!g.aabbs || count > g.n_regions) return set_error(ctx, PG_ERR_STATE, "regions not set");
    return check_cuda(ctx, cudaMemcpy(host_out, g.aabbs, sizeof(float) * 6 * count, cudaMemcpyDeviceToHost),
                      "region boxes download");
}

int pg_region_aabbs_device(pg_ctx *ctx, const float **dev_out) {
    if (!ctx || !dev_out) return PG_ERR_ARG;
    GuideScratch &g = guide(ctx);
    *dev_out = g.aabbs;
    return g.aabbs ? PG_OK : set_error(ctx, PG_ERR_STATE, "regions not set");
}

int pg_sort_samples(pg_ctx *ctx, const pg_directional_data *records, uint64_t n_records, uint32_t n_regions,
                    pg_directional_data *sorted_out, uint32_t *offsets_out, void *stream) {
    if (!ctx || (!records && n_records) || !offsets_out) return PG_ERR_ARG;
    if (n_regions == 0 || n_regions >= 0xFFFFFF00u) return set_error(ctx, PG_ERR_ARG, "bad region count");
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t *order = nullptr;
    int st = sort_records(ctx, records, n_records, n_regions, offsets_out, &order, s);
    if (st) return st;
    if (sorted_out && n_records) {
        gather_records<<<std::min<uint64_t>((n_records + 255) / 256, 8192u), 256, 0, s>>>(records, order, offsets_out,
                                                                                         n_regions, sorted_out);
        st = check_cuda(ctx, cudaGetLastError(), "gather launch");
    }
    return st;
}

int pg_prefit_parallax(pg_ctx *ctx, const pg_directional_data *sorted, const uint32_t *offsets, uint32_t n_regions,
                       uint64_t n_valid, float *dirw_out, float *dist_out, void *stream) {
    if (!ctx || !offsets || !dirw_out || !dist_out || (!sorted && n_valid)) return PG_ERR_ARG;
    GuideScratch &g = guide(ctx);
    if (ctx->cfg.use_parallax && (!g.aabbs || n_regions > g.n_regions))
        return set_error(ctx, PG_ERR_STATE, "pg_set_regions must run before the parallax pre-pass");
    cudaStream_t s = (cudaStream_t)stream;
    if (ctx->cfg.use_parallax) {
        parallax_means_kernel<<<(n_regions + 127) / 128, 128, 0, s>>>(ctx->d_states, g.aabbs, offsets, n_regions,
                                                                       g.fitted ? 1 : 0, g.means);
    }
    if (n_valid)
        prefit_parallax_kernel<<<std::min<uint64_t>((n_valid + 255) / 256, 16384u), 256, 0, s>>>(
            sorted, nullptr, (uint32_t)n_valid, nullptr, n_regions, g.means, ctx->cfg.use_parallax ? 1 : 0,
            reinterpret_cast<float4 *>(dirw_out), dist_out, nullptr);
    return check_cuda(ctx, cudaGetLastError(), "prefit launch");
}

int pg_update_distances(pg_ctx *ctx, const float *dirw, const float *dist, const uint32_t *offsets,
                        uint32_t n_regions, void *stream) {
    if (!ctx || !dirw || !dist || !offsets) return PG_ERR_ARG;
    if (n_regions > ctx->max_regions) return set_error(ctx, PG_ERR_ARG, "n_regions exceeds context capacity");
    if (n_regions == 0) return PG_OK;
    return update_distances(ctx, reinterpret_cast<const float4 *>(dirw), dist, offsets, n_regions,
                            (cudaStream_t)stream);
}

int pg_pack_vmm_theta(pg_ctx *ctx, uint32_t n_regions, pg_vmm_theta *out, void *stream) {
    if (!ctx || !out) return PG_ERR_ARG;
    if (n_regions > ctx->max_regions) return set_error(ctx, PG_ERR_ARG, "n_regions exceeds context capacity");
    if (n_regions == 0) return PG_OK;
    pack_vmm_theta_kernel<<<n_regions, 16, 0, (cudaStream_t)stream>>>(ctx->d_states, n_regions,
                                                                       ctx->cfg.use_parallax ? 1 : 0, out);
    return check_cuda(ctx, cudaGetLastError(), "pack launch");
}

int pg_update(pg_ctx *ctx, const pg_directional_data *records, uint64_t n_records, pg_vmm_theta *vmm_out,
              void *stream) {
    if (!ctx || (!records && n_records)) return PG_ERR_ARG;
    GuideScratch &g = guide(ctx);
    if (!g.aabbs || g.n_regions == 0) return set_error(ctx, PG_ERR_STATE, "pg_set_regions must run before pg_update");
    const uint32_t R = g.n_regions;
    cudaStream_t s = (cudaStream_t)stream;
    if (n_records > g.cap_samples || !g.dirw) {
        cudaFree(g.dirw);
        cudaFree(g.dist);
        cudaFree(g.pdf);
        g.dirw = nullptr;
        g.dist = nullptr;
        g.pdf = nullptr;
        const uint64_t cap = std::max<uint64_t>(n_records, 1);
        int st = check_cuda(ctx, cudaMalloc(&g.dirw, sizeof(float4) * cap), "fit samples");
        if (!st) st = check_cuda(ctx, cudaMalloc(&g.dist, sizeof(float) * cap), "fit distances");
        if (!st) st = check_cuda(ctx, cudaMalloc(&g.pdf, sizeof(float) * cap), "sample pdfs");
        if (st) return st;
        g.cap_samples = cap;
    }
    if (!g.offsets) {
        int st = check_cuda(ctx, cudaMalloc(&g.offsets, sizeof(uint32_t) * ((size_t)ctx->max_regions + 1)), "offsets");
        if (st) return st;
    }
    // 1. bucket by region (SampleCollector::getSortedData)
    uint32_t *order = nullptr;
    int st = sort_records(ctx, records, n_records, R, g.offsets, &order, s);
    if (st) return st;
    // 2. parallax pre-pass (PathGuiding::preFit), gathering through the sort order
    const int par = ctx->cfg.use_parallax ? 1 : 0;
    if (par)
        parallax_means_kernel<<<(R + 127) / 128, 128, 0, s>>>(ctx->d_states, g.aabbs, g.offsets, R, g.fitted ? 1 : 0,
                                                              g.means);
    if (n_records)
        prefit_parallax_kernel<<<std::min<uint64_t>((n_records + 255) / 256, 16384u), 256, 0, s>>>(
            records, order, (uint32_t)n_records, g.offsets + R, R, g.means, par, g.dirw, g.dist, g.pdf);
    st = check_cuda(ctx, cudaGetLastError(), "prefit launch");
    if (st) return st;
    // Records past the valid count (invalid slots) are never read by the fit:
    // offsets[R] bounds every region.
    // 3. fit (VMMFactory::fit on the first pass, updateFit afterwards)
    st = pg_fit_regions(ctx, reinterpret_cast<const float *>(g.dirw), g.offsets, R,
                        g.fitted ? PG_FIT_UPDATE : PG_FIT_CONTINUE, stream);
    if (st) return st;
    // 3b. split and merge of components (PathGuiding::postFit, before the distances)
    if (ctx->sm.enabled) {
        st = pg_split_merge(ctx, reinterpret_cast<const float *>(g.dirw), g.pdf, g.offsets, R, stream);
        if (st) return st;
    }
    // 4. parallax distances (PathGuiding::postFit)
    if (par) {
        st = pg_update_distances(ctx, reinterpret_cast<const float *>(g.dirw), g.dist, g.offsets, R, stream);
        if (st) return st;
    }
    g.fitted = true;
    // 5. the split check of PathGuiding::update (src/PathGuiding.cpp:290-300)
    uint32_t R_out = R;
    if (g.rs.enabled) {
        st = pg_split_regions(ctx, &R_out, stream);
        if (st) return st;
    }
    // 6. VMM_Theta for the tracer (the context's copy, and the caller's if asked)
    st = pg_pack_vmm_theta(ctx, R_out, g.vmm, stream);
    if (st) return st;
    g.vmm_fresh = true;
    if (vmm_out) st = check_cuda(ctx, cudaMemcpyAsync(vmm_out, g.vmm, sizeof(pg_vmm_theta) * R_out,
                                                      cudaMemcpyDeviceToDevice, s), "VMM_Theta copy");
    return st;
}

void pg_default_region_split_config(pg_region_split_config *out) {
    if (!out) return;
    out->enabled = 1;
    out->samples_for_region_split = 10000.0f;
}

int pg_set_region_split(pg_ctx *ctx, const pg_region_split_config *cfg) {
    if (!ctx || !cfg) return PG_ERR_ARG;
    guide(ctx).rs = *cfg;
    return PG_OK;
}

int pg_split_regions(pg_ctx *ctx, uint32_t *n_regions_out, void *stream) {
    if (!ctx) return PG_ERR_ARG;
    GuideScratch &g = guide(ctx);
    if (!g.aabbs || g.n_regions == 0) return set_error(ctx, PG_ERR_STATE, "pg_set_regions must run first");
    cudaStream_t s = (cudaStream_t)stream;
    const float thr = g.rs.samples_for_region_split > 0.0f ? g.rs.samples_for_region_split : 10000.0f;
    split_regions_kernel<<<1, 1024, 0, s>>>(ctx->d_states, ctx->d_extras, g.aabbs, g.nodes, g.leaf_of, g.n_regions,
                                            g.n_nodes, ctx->max_regions, thr, g.split_out);
    int st = check_cuda(ctx, cudaGetLastError(), "region split launch");
    uint32_t h[2] = {0, 0};
    if (!st)
        st = check_cuda(ctx, cudaMemcpyAsync(h, g.split_out, sizeof h, cudaMemcpyDeviceToHost, s), "split counts");
    if (!st) st = check_cuda(ctx, cudaStreamSynchronize(s), "region split sync");
    if (st) return st;
    if (h[0] != g.n_regions) {
        g.n_regions = h[0];
        g.n_nodes = h[1];
        g.tree_split = true;
        g.vmm_fresh = false;
    }
    if (n_regions_out) *n_regions_out = g.n_regions;
    return PG_OK;
}

int pg_get_region_tree(pg_ctx *ctx, int32_t *host_nodes, uint32_t capacity, uint32_t *n_nodes_out) {
    if (!ctx || (!host_nodes && capacity)) return PG_ERR_ARG;
    GuideScratch &g = guide(ctx);
    if (!g.nodes || g.n_regions == 0) return set_error(ctx, PG_ERR_STATE, "pg_set_regions must run first");
    if (n_nodes_out) *n_nodes_out = g.n_nodes;
    if (!host_nodes) return PG_OK;
    if (capacity < g.n_nodes) return set_error(ctx, PG_ERR_ARG, "capacity below the node count");
    return check_cuda(ctx, cudaMemcpy(host_nodes, g.nodes, sizeof(int32_t) * g.n_nodes, cudaMemcpyDeviceToHost),
                      "region tree download");
}

}  // extern "C"
