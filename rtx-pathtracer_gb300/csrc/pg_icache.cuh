// pg_icache.cuh - the irradiance cache of the wavefront tracer: its state,
// queries, request queue, commit and grid (included by pg_trace.cu before the
// render state; the hemisphere paths are in pg_icache_paths.cuh).
//
// The reference keeps the cache as spheres in a ray-tracing acceleration
// structure and queries it with a zero-length ray whose any-hit shader
// weighs every sphere containing the point (raytrace.irradiance.rint:11-21,
// raytrace.irradiance.rahit:18-51).  Here the entries sit in one device array
// and a uniform 32^3 grid over the scene box lists, per cell and in entry
// order, the entries whose sphere box overlaps the cell; a query walks its
// point's cell.
//
// New entries and updates (createIrradianceCache / updateIrradianceCache,
// raytrace.rgen:1334-1421) are queued while a sample pass renders and computed
// after it, before the next pass - the reference computes them at the end of
// its frame and makes them visible with the acceleration-structure update
// after the frame (src/RayTracingApp.cpp:115-120); one pass of the library is
// one frame of the reference at one sample per pixel.  calculateCacheData's
// 20 x 10 stratified hemisphere paths (raytrace.rgen:1231-1316) run one thread
// per stratum (k_ic_paths), one warp per request sums them into irradiance,
// harmonic mean distance and the two gradients (k_ic_reduce), and the results
// are written in request order - by pixel, then bounce, whatever order the
// requests were queued in - so a render repeats bit for bit.
#pragma once

namespace pg {

constexpr int kIcN = 20;                   // azimuthal strata (calculateCacheData: N)
constexpr int kIcM = 10;                   // polar strata (M)
constexpr int kIcSamples = kIcN * kIcM;
constexpr int kIcGrid = 32;                // grid cells per axis
constexpr uint32_t kIcCells = kIcGrid * kIcGrid * kIcGrid;
constexpr int kIcMaxFollow = 10;           // maxFollowDiscrete of calculateCacheData
constexpr uint32_t kIcMaxNewPerPixel = 5;  // MAX_NEW_IRRADIANCE_ENTRIES (raytrace.rgen:65)
constexpr uint32_t kIcUpdateBounce = 255;  // bounce field of an update request
constexpr uint32_t kIcSalt = 0x1c0ffee1u;  // seed salt of the cache's random numbers

// A queued request: a new entry at (o, n) (target -1) or an update of an
// entry (target >= 0 once assigned; -2: nothing to do).  pixel (the
// requesting path's stream: its pixel for a camera path) / bounce / pass name
// its random numbers and its place in the commit order.
struct IcRequest {
    float o[3], n[3];
    int32_t target;
    uint32_t pixel, bounce, pass;
    uint32_t slot;  // entry a new one is written to (assigned after its paths)
};

// What a request's paths yield, before the entry is written.
struct IcResult {
    float color[3], rot[3], trans[3];
    float harmonic_r;  // < 0: nothing was hit in the hemisphere
};

struct DevIc {
    pg_ic_entry *entries;
    const uint32_t *cell_start;  // kIcCells + 1 (the last one: total references)
    const uint32_t *cell_refs;
    uint32_t cap_refs;
    float lo[3], inv_cell[3];
    float a, min_radius, create_prob, update_prob, grad_max;
    int use_gradients, visibility, on_glossy;
    uint32_t num_nee;            // light samples averaged per vertex of an entry's paths (>= 1)
    int query, grow;             // what this render call does: query; create and update
    IcRequest *requests;
    uint32_t req_cap, capacity;
    uint32_t *created;           // per pixel: new-entry requests of this pass
    uint32_t *state;             // [0] requests queued, [1] round-robin update position, [2] entries,
                                 // [3] new entries written this pass
};

__host__ __device__ __forceinline__ uint32_t ic_stream(uint32_t pixel, uint32_t bounce, uint32_t pass) {
    return fmix32(pixel * 256u + bounce + fmix32(pass ^ 0x9e3779b9u));
}
__device__ __forceinline__ uint64_t ic_key(const IcRequest &r) { return ((uint64_t)r.pixel << 8) | r.bounce; }

// isICCapable (raytrace.rgen:806-813) for a vertex that is not an emitter
// (the library's paths end at emitters): diffuse surfaces, and any other
// non-discrete one when the cache is used on glossy surfaces too.
__device__ __forceinline__ bool ic_capable(const DevIc &ic, const pg_material &m) {
    if (m.type == PG_MAT_DIFFUSE) return true;
    return ic.on_glossy && !is_delta(m);
}

// approxDiffuse (raytrace.rgen:815-828): the Lambertian part the cached
// irradiance is multiplied by - the diffuse reflectance / pi, a rough
// conductor's Fresnel term / pi; GGX (no counterpart in the reference) its
// tint / pi.
__device__ __forceinline__ V approx_diffuse(const pg_material &m, V n, V wi) {
    if (m.type == PG_MAT_BECKMANN) {
        const float F = fresnel_conductor(dot3(wi, n), m.eta, m.k) * (1.0f / kPi);
        return mk(F, F, F);
    }
    return mul(mk(m.albedo[0], m.albedo[1], m.albedo[2]), 1.0f / kPi);
}

// One entry's share of a query at (p, n): the sphere test of
// raytrace.irradiance.rint:13-20, then irradianceWeight, the threshold, the
// visibility test and the (gradient-corrected) value of
// raytrace.irradiance.rahit:18-51.
__device__ __forceinline__ bool ic_contribution(const DevIc &ic, const pg_ic_entry &e, V p, V n, V &wval,
                                                float &w) {
    const V c = mk(e.center[0], e.center[1], e.center[2]);
    const V oc = sub(p, c);
    const float dist = sqrtf(dot3(oc, oc));
    if (!(dist <= e.radius)) return false;
    const V en = mk(e.normal[0], e.normal[1], e.normal[2]);
    w = 1.0f / (dist / e.harmonic_r + sqrtf(1.0f - dot3(n, en)));
    if (isnan(w) || isinf(w)) w = 1000000.0f;
    if (w <= 1.0f / ic.a) return false;
    if (ic.visibility && !(-0.001f <= dot3(oc, mul(add(n, en), 0.5f)))) return false;
    const V col = mk(e.color[0], e.color[1], e.color[2]);
    if (ic.use_gradients) {
        const float E = sqrtf(dot3(col, col));
        const V dir = E != 0.0f ? mul(col, 1.0f / E) : mk(0, 0, 0);
        const V rg = mk(e.rot_grad[0], e.rot_grad[1], e.rot_grad[2]);
        const V tg = mk(e.trans_grad[0], e.trans_grad[1], e.trans_grad[2]);
        wval = mul(dir, w * (E + dot3(cross3(en, n), rg) + dot3(oc, tg)));
    } else {
        wval = mul(col, w);
    }
    return true;
}

__device__ __forceinline__ int ic_cell_coord(float x, float lo, float inv) {
    const float f = floorf((x - lo) * inv);
    return f >= 0.0f ? (f < (float)kIcGrid ? (int)f : kIcGrid - 1) : 0;  // NaN: cell 0
}

// queryIrradianceCache (raytrace.rgen:748-773): the weighted mean of the
// entries around p; false when none applies.
__device__ __forceinline__ bool ic_query(const DevIc &ic, V p, V n, V &E) {
    const int cx = ic_cell_coord(p.x, ic.lo[0], ic.inv_cell[0]);
    const int cy = ic_cell_coord(p.y, ic.lo[1], ic.inv_cell[1]);
    const int cz = ic_cell_coord(p.z, ic.lo[2], ic.inv_cell[2]);
    const uint32_t cell = ((uint32_t)cz * kIcGrid + (uint32_t)cy) * kIcGrid + (uint32_t)cx;
    const uint32_t b = ic.cell_start[cell], e = min(ic.cell_start[cell + 1], ic.cap_refs);
    V sum = mk(0, 0, 0);
    float total = 0.0f;
    for (uint32_t i = b; i < e; ++i) {
        V wv;
        float w;
        if (ic_contribution(ic, ic.entries[ic.cell_refs[i]], p, n, wv, w)) {
            sum = add(sum, wv);
            total += w;
        }
    }
    if (!(total > 0.0f)) return false;
    E = mul(sum, 1.0f / total);
    return true;
}

__device__ __forceinline__ void ic_push(const DevIc &ic, V o, V n, int32_t target, uint32_t pixel, uint32_t bounce,
                                        uint32_t pass) {
    const uint32_t q = atomicAdd(&ic.state[0], 1u);
    if (q >= ic.req_cap) return;
    IcRequest r;
    r.o[0] = o.x;
    r.o[1] = o.y;
    r.o[2] = o.z;
    r.n[0] = n.x;
    r.n[1] = n.y;
    r.n[2] = n.z;
    r.target = target;
    r.pixel = pixel;
    r.bounce = bounce;
    r.pass = pass;
    r.slot = 0xFFFFFFFFu;
    ic.requests[q] = r;
}

// The number of queued requests i with sel(i) whose key is below `key`,
// counted by the CTA through shared-memory tiles of keys (every thread of
// the CTA takes part; `active` threads use the count).
constexpr uint32_t kIcRankTile = 512;
template <class Sel>
__device__ __forceinline__ uint32_t ic_rank(const DevIc &ic, uint32_t n_req, uint64_t key, bool active, Sel sel) {
    __shared__ uint64_t tk[kIcRankTile];
    uint32_t rank = 0;
    for (uint32_t base = 0; base < n_req; base += kIcRankTile) {
        __syncthreads();
        for (uint32_t j = threadIdx.x; j < kIcRankTile; j += blockDim.x) {
            const uint32_t i = base + j;
            tk[j] = (i < n_req && sel(i)) ? ic_key(ic.requests[i]) : ~0ull;
        }
        __syncthreads();
        if (active) {
            const uint32_t m = min(kIcRankTile, n_req - base);
            for (uint32_t j = 0; j < m; ++j) rank += tk[j] < key ? 1u : 0u;
        }
    }
    return rank;
}

// Update requests take their entries in request order from the round-robin
// position (updateIrradianceCache, raytrace.rgen:1334-1345: the position
// advances by one per request, and a request that finds it past the last
// entry sets it back to 0 and updates nothing).  An entry that an earlier
// request of the same pass already updates is skipped.  One thread per
// request (the grid covers req_cap); ranks by counting, O(requests^2).
__global__ void __launch_bounds__(128) k_ic_assign(DevIc ic) {
    const uint32_t n_req = min(ic.state[0], ic.req_cap);
    if (blockIdx.x * blockDim.x >= n_req) return;  // the whole CTA
    const uint32_t n = ic.state[2], start = ic.state[1];
    const uint32_t first = n > start ? n - start : 0u;  // requests before the first reset
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = q < n_req && ic.requests[q].bounce == kIcUpdateBounce;
    const uint64_t key = active ? ic_key(ic.requests[q]) : 0ull;
    const uint32_t rank = ic_rank(ic, n_req, key, active,
                                  [&](uint32_t i) { return ic.requests[i].bounce == kIcUpdateBounce; });
    if (!active) return;
    IcRequest &rq = ic.requests[q];
    int32_t target = -2;
    if (rank < first) {
        target = (int32_t)(start + rank);
    } else if (n > 0) {
        const uint32_t r = rank - first, pos = r % (n + 1u);
        const uint32_t t = pos - 1u;
        // pos 0: the reset; a second cycle, or an entry of the first stretch: already updated
        if (pos != 0 && r < n + 1u && (first == 0 || t < start)) target = (int32_t)t;
    }
    if (target >= 0) {
        const pg_ic_entry &e = ic.entries[target];
        if (e.num_updates < 1u) {
            target = -2;
        } else {
            for (int c = 0; c < 3; ++c) {
                rq.o[c] = e.center[c];
                rq.n[c] = e.normal[c];
            }
        }
    }
    rq.target = target;
}

// New entries take consecutive slots after the existing ones in request
// order, counting only requests whose hemisphere saw something
// (createIrradianceCache, raytrace.rgen:1383-1421).  One thread per request.
__global__ void __launch_bounds__(128) k_ic_slots(DevIc ic, const IcResult *res) {
    const uint32_t n_req = min(ic.state[0], ic.req_cap);
    if (blockIdx.x * blockDim.x >= n_req) return;  // the whole CTA
    const uint32_t n = ic.state[2];
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    auto creates = [&](uint32_t i) { return ic.requests[i].target == -1 && res[i].harmonic_r >= 0.0f; };
    const bool active = q < n_req && creates(q);
    const uint64_t key = active ? ic_key(ic.requests[q]) : 0ull;
    const uint32_t rank = ic_rank(ic, n_req, key, active, creates);
    if (!active) return;
    const uint32_t slot = n + rank;
    if (slot < ic.capacity) {
        ic.requests[q].slot = slot;
        atomicAdd(&ic.state[3], 1u);
    }
}

// clampGradients (raytrace.rgen:1318-1329).
__device__ __forceinline__ void ic_clamp(float g[3], float mx) {
    const float l = sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
    if (l > mx)
        for (int c = 0; c < 3; ++c) g[c] *= mx / l;
}

// A new entry as createIrradianceCache writes it (raytrace.rgen:1403-1420).
__device__ __forceinline__ void ic_make_entry(const DevIc &ic, const float o[3], const float nr[3], const IcResult &r,
                                              pg_ic_entry &e) {
    float rot[3] = {r.rot[0], r.rot[1], r.rot[2]}, tr[3] = {r.trans[0], r.trans[1], r.trans[2]};
    ic_clamp(rot, ic.grad_max);
    ic_clamp(tr, ic.grad_max);
    const float hr = fmaxf(r.harmonic_r, ic.min_radius);
    for (int c = 0; c < 3; ++c) {
        e.center[c] = o[c];
        e.normal[c] = nr[c];
        e.color[c] = r.color[c];
        e.rot_grad[c] = rot[c];
        e.trans_grad[c] = tr[c];
    }
    e.harmonic_r = hr;
    e.radius = ic.a * hr;
    e.num_updates = 1;
}

// Writes the entries: new ones, and updates as the rest of
// updateIrradianceCache does (the running mean with weight
// min(n / (n + 1), 0.95) on the old values, raytrace.rgen:1347-1380).
__global__ void __launch_bounds__(128) k_ic_commit(DevIc ic, const IcResult *res) {
    const uint32_t n_req = min(ic.state[0], ic.req_cap);
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n_req; q += gridDim.x * blockDim.x) {
        const IcRequest rq = ic.requests[q];
        const IcResult r = res[q];
        if (rq.target == -1) {
            if (rq.slot == 0xFFFFFFFFu) continue;
            pg_ic_entry e;
            ic_make_entry(ic, rq.o, rq.n, r, e);
            ic.entries[rq.slot] = e;
        } else if (rq.target >= 0) {
            pg_ic_entry e = ic.entries[rq.target];
            const float a = fminf((float)e.num_updates / (float)(e.num_updates + 1u), 0.95f);
            float rot[3], tr[3];
            for (int c = 0; c < 3; ++c) {
                e.color[c] = r.color[c] * (1.0f - a) + e.color[c] * a;
                rot[c] = r.rot[c] * (1.0f - a) + e.rot_grad[c] * a;
                tr[c] = r.trans[c] * (1.0f - a) + e.trans_grad[c] * a;
            }
            ic_clamp(rot, ic.grad_max);
            ic_clamp(tr, ic.grad_max);
            for (int c = 0; c < 3; ++c) {
                e.rot_grad[c] = rot[c];
                e.trans_grad[c] = tr[c];
            }
            float hr = r.harmonic_r > 0.0f ? r.harmonic_r * (1.0f - a) + e.harmonic_r * a : e.harmonic_r;
            hr = fmaxf(hr, ic.min_radius);
            e.harmonic_r = hr;
            e.radius = ic.a * hr;
            e.num_updates += 1u;
            ic.entries[rq.target] = e;
        }
    }
}

// After the commit: the entry count, the round-robin position after this
// pass's update requests, an empty queue.
__global__ void k_ic_finish(DevIc ic) {
    const uint32_t n_req = min(ic.state[0], ic.req_cap);
    uint32_t updates = 0;
    for (uint32_t q = 0; q < n_req; ++q) updates += ic.requests[q].bounce == kIcUpdateBounce ? 1u : 0u;
    const uint32_t n = ic.state[2], start = ic.state[1];
    uint32_t next = start;
    if (updates > 0) {
        const uint32_t first = n > start ? n - start : 0u;
        next = updates <= first ? start + updates : (updates - first - 1u) % (n + 1u);
    }
    ic.state[1] = next;
    ic.state[2] = min(n + ic.state[3], ic.capacity);
    ic.state[0] = 0;
    ic.state[3] = 0;
}

// Grid build: the cell range of an entry's sphere box.
__device__ __forceinline__ void ic_cell_range(const DevIc &ic, const pg_ic_entry &e, int lo[3], int hi[3]) {
    for (int c = 0; c < 3; ++c) {
        lo[c] = ic_cell_coord(e.center[c] - e.radius, ic.lo[c], ic.inv_cell[c]);
        hi[c] = ic_cell_coord(e.center[c] + e.radius, ic.lo[c], ic.inv_cell[c]);
    }
}
// One thread per (entry, z) slab of cells: an entry's box (it can cover
// thousands of cells) spreads over up to 32 threads.
__global__ void __launch_bounds__(128) k_ic_grid_count(DevIc ic, uint32_t *count) {
    const uint32_t n = ic.state[2];
    const uint64_t slabs = (uint64_t)n * kIcGrid;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < slabs;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t i = (uint32_t)(t / kIcGrid);
        const int z = (int)(t % kIcGrid);
        int lo[3], hi[3];
        ic_cell_range(ic, ic.entries[i], lo, hi);
        if (z < lo[2] || z > hi[2]) continue;
        for (int y = lo[1]; y <= hi[1]; ++y)
            for (int x = lo[0]; x <= hi[0]; ++x) atomicAdd(&count[(z * kIcGrid + y) * kIcGrid + x], 1u);
    }
}
// Exclusive scan of the cell counts into start, one CTA of 32 warps: warp w
// scans cells [1024 w, 1024 (w + 1)) in coalesced 32-cell chunks;
// start[kIcCells] is the total.
__global__ void __launch_bounds__(1024) k_ic_grid_scan(const uint32_t *count, uint32_t *start) {
    constexpr uint32_t per_warp = kIcCells / 32;
    __shared__ uint32_t wsum[32];
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t *c = count + w * per_warp;
    uint32_t tot = 0;
    for (uint32_t k = lane; k < per_warp; k += 32) tot += c[k];
    for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
    if (lane == 0) wsum[w] = tot;
    __syncthreads();
    uint32_t base = 0;
    for (uint32_t k = 0; k < w; ++k) base += wsum[k];
    for (uint32_t k0 = 0; k0 < per_warp; k0 += 32) {
        const uint32_t v = c[k0 + lane];
        uint32_t inc = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= (uint32_t)o) inc += u;
        }
        start[w * per_warp + k0 + lane] = base + inc - v;
        base += __shfl_sync(0xffffffffu, inc, 31);
    }
    if (threadIdx.x == 1023) start[kIcCells] = base;
}
__global__ void __launch_bounds__(128) k_ic_grid_fill(DevIc ic, const uint32_t *start, uint32_t *fill,
                                                      uint32_t *refs) {
    const uint32_t n = ic.state[2];
    const uint64_t slabs = (uint64_t)n * kIcGrid;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < slabs;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t i = (uint32_t)(t / kIcGrid);
        const int z = (int)(t % kIcGrid);
        int lo[3], hi[3];
        ic_cell_range(ic, ic.entries[i], lo, hi);
        if (z < lo[2] || z > hi[2]) continue;
        for (int y = lo[1]; y <= hi[1]; ++y)
            for (int x = lo[0]; x <= hi[0]; ++x) {
                const uint32_t cc = (z * kIcGrid + y) * kIcGrid + x;
                const uint32_t slot = start[cc] + atomicAdd(&fill[cc], 1u);
                if (slot < ic.cap_refs) refs[slot] = i;
            }
    }
}
// Each cell's list in entry order (insertion sort; lists are short), so a
// query sums its entries in a fixed order.
__global__ void __launch_bounds__(128) k_ic_grid_sort(const uint32_t *start, uint32_t *refs, uint32_t cap_refs) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= kIcCells) return;
    const uint32_t b = min(start[c], cap_refs), e = min(start[c + 1], cap_refs);
    for (uint32_t i = b + 1; i < e; ++i) {
        const uint32_t v = refs[i];
        uint32_t k = i;
        while (k > b && refs[k - 1] > v) {
            refs[k] = refs[k - 1];
            --k;
        }
        refs[k] = v;
    }
}

// Probe input: public requests to queue entries.
__global__ void k_ic_load_requests(const pg_ic_request *in, uint32_t n, IcRequest *out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const pg_ic_request r = in[i];
    IcRequest q;
    for (int c = 0; c < 3; ++c) {
        q.o[c] = r.position[c];
        q.n[c] = r.normal[c];
    }
    q.target = -1;
    q.pixel = r.pixel;
    q.bounce = r.bounce;
    q.pass = r.pass;
    q.slot = 0xFFFFFFFFu;
    out[i] = q;
}

// Probe: cache queries at given points.
__global__ void k_ic_query_probe(DevIc ic, const float *pos, const float *nrm, uint32_t n, float *rgb,
                                 uint32_t *found) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    V E = mk(0, 0, 0);
    const bool f = ic_query(ic, mk(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]),
                            mk(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]), E);
    rgb[3 * i] = E.x;
    rgb[3 * i + 1] = E.y;
    rgb[3 * i + 2] = E.z;
    found[i] = f ? 1u : 0u;
}

}  // namespace pg
