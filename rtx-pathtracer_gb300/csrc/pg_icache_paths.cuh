// pg_icache_paths.cuh - the irradiance cache's hemisphere paths
// (calculateCacheData, raytrace.rgen:1231-1316) and their sums; included by
// pg_trace.cu after the render state, next-event estimation and the
// continuation sampler, which the paths share with the renderer.  The cache
// itself, its queries and its commit are in pg_icache.cuh.
#pragma once

namespace pg {

// The surface a ray hit: position, geometric and shading normal, side, and
// the material with the texture applied to its diffuse reflectance
// (raytrace.rchit:16-58 with the face normal, as the renderer shades).
__device__ __forceinline__ void surface_at(const DevRender &R, const pg_hit &h, V o, V d, V &x, V &ng, V &n,
                                           bool &front, pg_material &m) {
    x = add(o, mul(d, h.t));
    uint32_t mat_id;
    if (h.prim & PG_SPHERE_BIT) {
        const pg_sphere &sp = R.S.spheres[h.prim & ~PG_SPHERE_BIT];
        ng = mul(sub(x, mk(sp.center[0], sp.center[1], sp.center[2])), 1.0f / sp.radius);
        mat_id = sp.material;
    } else {
        const uint32_t t = h.prim;
        const V v0 = ld3(R.pos, R.idx[3 * t]), v1 = ld3(R.pos, R.idx[3 * t + 1]), v2 = ld3(R.pos, R.idx[3 * t + 2]);
        ng = nrm(cross3(sub(v1, v0), sub(v2, v0)));
        mat_id = R.tri_mat[t];
    }
    m = R.mats[mat_id];
    if (m.texture > 0 && !(h.prim & PG_SPHERE_BIT) && (m.type == PG_MAT_DIFFUSE || m.type == PG_MAT_PHONG)) {
        float tc[3];
        tex_rgb(R.S, h.prim, (uint32_t)m.texture - 1u, h.u, h.v, tc);
        for (int c = 0; c < 3; ++c) m.albedo[c] *= tc[c];
    }
    front = dot3(d, ng) < 0.0f;
    n = front ? ng : mul(ng, -1.0f);
}

// Direct light at x from one light sample and its shadow ray - the expected
// value of multipleNEE with one sample (raytrace.rgen:601-731, 871-877), by
// light sampling alone: the cache's paths take no light by continuation.
__device__ __forceinline__ V ic_direct(const DevRender &R, const pg_material &m, V x, V n, V wi, float ul, float u1,
                                       float u2) {
    if (R.n_lights == 0 || is_delta(m)) return mk(0, 0, 0);
    NeeSample ns;
    if (!nee_sample(R, m, x, n, wi, ul, u1, u2, ns)) return mk(0, 0, 0);
    const float o[3] = {x.x, x.y, x.z}, d[3] = {ns.wl.x, ns.wl.y, ns.wl.z};
    if (trace_any(R.S, o, d, kTMin, ns.tmax)) return mk(0, 0, 0);
    return mul(ns.fLe, 1.0f / ns.pl);
}

__device__ __forceinline__ V ic_dir_world(float theta, float phi, V n) {
    return to_world(mk(sinf(theta) * cosf(phi), sinf(theta) * sinf(phi), cosf(theta)), n);
}

// The stratum jitters of a request: one per azimuthal stratum k (its M polar
// strata share it, as calculateCacheData draws phi once per k) and one per
// stratum (k, j).
__device__ __forceinline__ float ic_phi(uint32_t seed, uint32_t stream, int k) {
    return 2.0f * kPi * ((float)k + rnd(seed, stream, (uint32_t)(k * kIcM), 0)) / (float)kIcN;
}
__device__ __forceinline__ float ic_theta(uint32_t seed, uint32_t stream, int k, int j) {
    return asinf(sqrtf(((float)j + rnd(seed, stream, (uint32_t)(k * kIcM + j), 1)) / (float)kIcM));
}

// One stratum of calculateCacheData: raytrace() with maxDepth 1 (two
// non-discrete vertices at most), no light taken at the first hit or after a
// non-discrete vertex, next-event estimation at every non-discrete vertex,
// the cache queried there (useIC) and never grown, discrete vertices followed
// up to ten more times (raytrace.rgen:992-1226 with the arguments of :1265).
// Returns the radiance; first_t is the first hit's distance (tMax on a miss).
__device__ V ic_stratum_path(const DevRender &R, uint32_t seed, uint32_t stream, int s, V o, V n0, float &first_t) {
    const int k = s / kIcM, j = s % kIcM;
    V d = ic_dir_world(ic_theta(seed, stream, k, j), ic_phi(seed, stream, k), n0);
    V L = mk(0, 0, 0), thr = mk(1, 1, 1);
    first_t = kTMax;
    bool add_next = false;
    int depth = 0, follow_count = 0;
    for (;;) {
        ++depth;
        const uint32_t dim = 2u + 16u * (uint32_t)depth;
        const float of[3] = {o.x, o.y, o.z}, df[3] = {d.x, d.y, d.z};
        pg_hit h;
        if (!trace_closest(R.S, of, df, kTMin, kTMax, h)) {
            if (add_next && R.env) L = add(L, hmul(thr, env_radiance(R, d)));
            break;
        }
        if (depth == 1) first_t = h.t;
        V x, ng, n;
        bool front;
        pg_material m;
        surface_at(R, h, o, d, x, ng, n, front, m);
        if (m.type == PG_MAT_LIGHT) {
            if (add_next && (front || (h.prim & PG_SPHERE_BIT) == 0))
                L = add(L, hmul(thr, mk(m.emission[0], m.emission[1], m.emission[2])));
            break;
        }
        const V wi = mul(d, -1.0f);
        const bool follow = is_delta(m);
        if (follow) {
            add_next = true;
            ++follow_count;  // depth >= maxDepth (1) always holds
        } else {
            add_next = false;
            // multipleNEE (raytrace.rgen:871-877): the mean of irradianceNumNEE light
            // samples; sample q > 0 draws from the stratum's stream at index s + 256 q
            V direct = ic_direct(R, m, x, n, wi, rnd(seed, stream, (uint32_t)s, dim),
                                 rnd(seed, stream, (uint32_t)s, dim + 1), rnd(seed, stream, (uint32_t)s, dim + 2));
            if (R.ic.num_nee > 1) {
                for (uint32_t q = 1; q < R.ic.num_nee; ++q) {
                    const uint32_t sq = (uint32_t)s + 256u * q;
                    direct = add(direct, ic_direct(R, m, x, n, wi, rnd(seed, stream, sq, dim),
                                                   rnd(seed, stream, sq, dim + 1), rnd(seed, stream, sq, dim + 2)));
                }
                direct = mul(direct, 1.0f / (float)R.ic.num_nee);
            }
            V E;
            if (R.ic.query && ic_capable(R.ic, m) && ic_query(R.ic, x, n, E)) {
                L = add(L, hmul(thr, add(hmul(approx_diffuse(m, n, wi), E), direct)));
                break;
            }
            L = add(L, hmul(thr, direct));
        }
        // loop condition of raytrace(): depth <= 1 || (follow && followCount <= 10)
        if (!(depth <= 1 || (follow && follow_count <= kIcMaxFollow))) break;
        const bool gm = R.guiding && guided_material(m, R.rp.flags);
        const pg_vmm_theta *mix = nullptr;
        if (gm) {
            const uint32_t reg = region_of(R.guide, x);
            if (reg != PG_INVALID_REGION) mix = &R.guide.vmm[reg];
        }
        const Continuation c = continue_path(m, d, n, front, x, gm, mix, R.guide.use_parallax, R.rp.guiding_prob,
                                             rnd(seed, stream, (uint32_t)s, dim + 3),
                                             rnd(seed, stream, (uint32_t)s, dim + 4),
                                             rnd(seed, stream, (uint32_t)s, dim + 5),
                                             rnd(seed, stream, (uint32_t)s, dim + 6),
                                             [&] { return rnd(seed, stream, (uint32_t)s, dim + 7); });
        if (!(c.pdf > 0.0f && maxc(c.tc) > 0.0f)) break;
        thr = hmul(thr, c.tc);
        o = x;
        d = c.wo;
    }
    return L;
}

// All strata of the queued requests, one thread each (grid-stride over
// requests x 200).  out: radiance and first-hit distance per stratum.
__global__ void __launch_bounds__(128) k_ic_paths(DevRender R, float4 *out) {
    const uint32_t n_req = min(R.ic.state[0], R.ic.req_cap);
    const uint32_t seed = R.rp.seed ^ kIcSalt;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n_req * (uint32_t)kIcSamples;
         t += gridDim.x * blockDim.x) {
        const uint32_t q = t / kIcSamples, s = t % kIcSamples;
        const IcRequest rq = R.ic.requests[q];
        if (rq.target < -1) continue;
        float r;
        const V L = ic_stratum_path(R, seed, ic_stream(rq.pixel, rq.bounce, rq.pass), (int)s,
                                    mk(rq.o[0], rq.o[1], rq.o[2]), mk(rq.n[0], rq.n[1], rq.n[2]), r);
        out[t] = make_float4(L.x, L.y, L.z, r);
    }
}

// calculateCacheData's sums (raytrace.rgen:1244-1315) over one request's
// strata: one warp per request, lanes over strata, then a butterfly sum.  The
// translation gradient takes the differences with the previous polar stratum
// (j - 1) and the previous azimuthal one (k - 1).
__device__ __forceinline__ void ic_reduce_one(uint32_t seed, const IcRequest &rq, const float4 *S, int lane,
                                              IcResult &out) {
    const uint32_t stream = ic_stream(rq.pixel, rq.bounce, rq.pass);
    const V n0 = mk(rq.n[0], rq.n[1], rq.n[2]);
    float acc[11];  // radiance 3, rotation 3, translation 3, inverse distances, hits
    for (int i = 0; i < 11; ++i) acc[i] = 0.0f;
    for (int s = lane; s < kIcSamples; s += 32) {
        const int k = s / kIcM, j = s % kIcM;
        const float phi = ic_phi(seed, stream, k);
        const float theta = ic_theta(seed, stream, k, j);
        const float4 v = S[s];
        const float L = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z), r = v.w;
        acc[0] += v.x;
        acc[1] += v.y;
        acc[2] += v.z;
        if (r < kTMax) {
            acc[9] += 1.0f / r;
            acc[10] += 1.0f;
        }
        float tt = tanf(theta);
        if (isinf(tt) || isnan(tt)) tt = 0.0f;
        const V vk = ic_dir_world(0.5f * kPi, phi + 0.5f * kPi, n0);
        acc[3] -= tt * L * vk.x;
        acc[4] -= tt * L * vk.y;
        acc[5] -= tt * L * vk.z;
        const float th_prev = asinf(sqrtf((float)j / (float)kIcM));
        const float th_next = asinf(sqrtf((float)(j + 1) / (float)kIcM));
        if (j > 0) {
            const float4 pj = S[s - 1];
            const float Lp = sqrtf(pj.x * pj.x + pj.y * pj.y + pj.z * pj.z);
            const V uk = ic_dir_world(0.5f * kPi, phi, n0);
            const float cp = cosf(th_prev);
            const float f = 2.0f * kPi / (float)kIcN * sinf(th_prev) * cp * cp / fminf(r, pj.w) * (L - Lp);
            acc[6] += uk.x * f;
            acc[7] += uk.y * f;
            acc[8] += uk.z * f;
        }
        if (k > 0) {
            const float4 pk = S[s - kIcM];
            const float Lp = sqrtf(pk.x * pk.x + pk.y * pk.y + pk.z * pk.z);
            const V pvk = ic_dir_world(0.5f * kPi, 2.0f * kPi * (float)k / (float)kIcN + 0.5f * kPi, n0);
            const float f = (sinf(th_next) - sinf(th_prev)) / fminf(r, pk.w) * (L - Lp);
            acc[6] += pvk.x * f;
            acc[7] += pvk.y * f;
            acc[8] += pvk.z * f;
        }
    }
    for (int i = 0; i < 11; ++i)
        for (int o = 16; o > 0; o >>= 1) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], o);
    const float nf = kPi / (float)(kIcM * kIcN);
    for (int c = 0; c < 3; ++c) {
        out.color[c] = nf * acc[c];
        out.rot[c] = nf * acc[3 + c];
        out.trans[c] = acc[6 + c];
    }
    out.harmonic_r = (acc[9] == 0.0f || acc[10] == 0.0f) ? -1.0f : 1.0f / (acc[9] / acc[10]);
}
__global__ void __launch_bounds__(128) k_ic_reduce(DevRender R, const float4 *smp, IcResult *res) {
    const uint32_t n_req = min(R.ic.state[0], R.ic.req_cap);
    const int lane = threadIdx.x & 31;
    const uint32_t seed = R.rp.seed ^ kIcSalt;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < n_req; q += (gridDim.x * blockDim.x) >> 5) {
        const IcRequest rq = R.ic.requests[q];
        if (rq.target < -1) continue;  // warp-uniform
        IcResult out;
        ic_reduce_one(seed, rq, smp + (size_t)q * kIcSamples, lane, out);
        if (lane == 0) res[q] = out;
    }
}

// Probe: the entries computed at given points (calculateCacheData with the
// streams of the given requests), without touching the cache; one warp per
// request after the strata of all of them.
__global__ void __launch_bounds__(128) k_ic_compute_probe_reduce(DevRender R, const float4 *smp, uint32_t n,
                                                                 pg_ic_entry *out) {
    const int lane = threadIdx.x & 31;
    const uint32_t seed = R.rp.seed ^ kIcSalt;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < n; q += (gridDim.x * blockDim.x) >> 5) {
        const IcRequest rq = R.ic.requests[q];
        IcResult r;
        ic_reduce_one(seed, rq, smp + (size_t)q * kIcSamples, lane, r);
        if (lane == 0) {
            pg_ic_entry e;
            ic_make_entry(R.ic, rq.o, rq.n, r, e);
            if (r.harmonic_r < 0.0f) {
                e.harmonic_r = r.harmonic_r;  // nothing hit: no entry would be made
                e.radius = 0.0f;
                e.num_updates = 0;
            }
            out[q] = e;
        }
    }
}

}  // namespace pg
