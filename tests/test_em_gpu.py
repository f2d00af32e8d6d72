"""GPU parity of the batched EM fit (pg_fit_regions) through the C ABI.

Tolerances, GPU vs the FP64 oracle (GPU_TOL): the GPU E-step evaluates the
exponent kappa log2(e) mu.d + log2(pi norm) - kappa log2(e) with three FP32 FMAs
whose intermediates are of size kappa log2(e), so each responsibility carries a
relative error up to ~2.4e-7 kappa (plus 2^-22 from ex2); the reference's own
FP32 cos(theta) rounding is ~1.2e-7 kappa.  These per-sample errors average
out in the sufficient statistics; GPU_TOL bounds what is left after 20 EM
iterations.  GPU vs the reference itself uses the FP64-vs-reference bound
REF_TOL of test_oracle.py (lightpmm's fastexp dominates).
"""
from __future__ import annotations

import numpy as np
import pytest

from test_oracle import FIT_SETS, REF_TOL, assert_params_close, cfg_from, mu_angle

pytestmark = pytest.mark.gpu

GPU_TOL = {"weight_rtol": 5e-4, "kappa_rtol": 1e-3, "r_atol": 1e-4, "mu_angle": 5e-4,
           "ll_rtol": 2e-5, "ll_per_weight": 2e-5}


def run_fit(cuda, pkg, cfg, dirw, offsets, mode=None, states=None, tuning=None, ctx=None):
    torch = cuda
    abi = pkg.abi
    R = len(offsets) - 1
    own = ctx is None
    if own:
        ctx = pkg.FitContext(cfg, max_regions=max(R, 1))
    if tuning:
        ctx.set_tuning(**tuning)
    if states is not None:
        ctx.set_states(states)
    d = torch.from_numpy(np.ascontiguousarray(dirw, dtype=np.float32)).cuda()
    o = torch.from_numpy(np.asarray(offsets, dtype=np.uint32).view(np.int32)).cuda()
    ctx.fit(d, o, R, abi.PG_FIT_INIT if mode is None else mode)
    ctx.sync()
    st = ctx.states(R)
    ll = torch.zeros(R, dtype=torch.float64, device="cuda")
    ctx.eval_loglik(d, o, R, ll)
    ctx.sync()
    out = (st, ll.cpu().numpy())
    if own:
        ctx.close()
    return out


def ll_close(got, want, dirw, offsets, tol):
    sw = np.array([dirw[offsets[r]:offsets[r + 1], 3].astype(np.float64).sum() for r in range(len(offsets) - 1)])
    d = np.abs(got - want)
    bound = tol["ll_per_weight"] * sw + tol["ll_rtol"] * np.abs(want) + 1e-4
    assert np.all(d <= bound), f"log-likelihood off by {d.max():.3g}"


@pytest.mark.parametrize("name", FIT_SETS)
def test_fit_matches_fp64_oracle(name, cuda, pkg, golden, oracle, abi):
    g = golden(name)
    cfg = cfg_from(abi, g["cfg"])
    K = cfg.num_initial_components
    mode = abi.PG_FIT_UPDATE if "states_in" in g else abi.PG_FIT_INIT
    st, ll = run_fit(cuda, pkg, cfg, g["dirw"], g["offsets"], mode=mode, states=g.get("states_in"))
    want, want_ll = oracle.fit(cfg, g["dirw"], g["offsets"], states=g.get("states_in"), mode=mode, f64=True)
    np.testing.assert_array_equal(st["iters_last"], want["iters_last"])
    np.testing.assert_array_equal(st["total_num_samples"], want["total_num_samples"])
    fitted = want["iters_last"] > 0
    assert_params_close(st, want, K, GPU_TOL, fitted)
    np.testing.assert_allclose(st["sample_weight"], want["sample_weight"], rtol=1e-5)
    ll_close(ll, oracle.eval_ll(g["dirw"], g["offsets"], st), g["dirw"], g["offsets"], GPU_TOL)
    ll_close(ll, want_ll, g["dirw"], g["offsets"], REF_TOL)


@pytest.mark.parametrize("name", FIT_SETS)
def test_fit_within_stated_tolerance_of_reference(name, cuda, pkg, golden, abi):
    g = golden(name)
    cfg = cfg_from(abi, g["cfg"])
    K = cfg.num_initial_components
    mode = abi.PG_FIT_UPDATE if "states_in" in g else abi.PG_FIT_INIT
    st, ll = run_fit(cuda, pkg, cfg, g["dirw"], g["offsets"], mode=mode, states=g.get("states_in"))
    ref = g["states"]
    np.testing.assert_array_equal(st["iters_last"], ref["iters_last"])
    assert_params_close(st, ref, K, REF_TOL, ref["iters_last"] > 0)
    ll_close(ll, g["ll_final"].astype(np.float64), g["dirw"], g["offsets"], REF_TOL)


@pytest.mark.parametrize("K", [8, 16])
@pytest.mark.parametrize("tuning", [{}, {"components_per_thread": 16}, {"unroll": 2}, {"threads_per_cta": 256},
                                    {"threads_per_cta": 256, "components_per_thread": 16, "unroll": 2},
                                    {"smem_samples": 256}, {"cluster_size": 1}, {"cluster_size": 2},
                                    {"cluster_size": 16}, {"cluster_size": 4, "smem_samples": 512},
                                    {"unroll": 4}, {"stream_stages": 1}, {"stream_stages": 3, "smem_samples": 2048},
                                    {"unroll": 4, "stream_stages": 8, "smem_samples": 4096},
                                    {"ctas_per_sm": 3, "smem_samples": 3072, "stream_stages": 2},
                                    {"ctas_per_sm": 4, "unroll": 1, "smem_samples": 2048},
                                    {"ctas_per_sm": 4, "components_per_thread": 8, "unroll": 4,
                                     "smem_samples": 2048}])
def test_uneven_batch_and_launch_shapes(K, tuning, cuda, pkg, oracle, abi, workloads):
    """Uneven regions (64..20000 samples): resident and streamed staging, regions
    shared by a cluster of 2..16 CTAs and regions fitted by one CTA."""
    w = workloads.fit_batched(seed=11, n_regions=24, median=1500, sigma=1.2, lo=64, hi=20000)
    cfg = abi.forced_iterations(20, num_initial_components=K)
    st, ll = run_fit(cuda, pkg, cfg, w["dirw"], w["offsets"], tuning=tuning)
    want, _ = oracle.fit(cfg, w["dirw"], w["offsets"], f64=True)
    assert_params_close(st, want, K, GPU_TOL, want["iters_last"] > 0)
    ll_close(ll, oracle.eval_ll(w["dirw"], w["offsets"], st), w["dirw"], w["offsets"], GPU_TOL)


@pytest.mark.parametrize("K,unroll", [(8, 2), (16, 2), (16, 4)])
def test_streamed_ring_equals_resident_slices(K, unroll, cuda, pkg, abi, workloads):
    """Slices larger than the staging capacity stream from L2 through a ring of
    TMA-filled stages.  Each stage holds a whole number of E-step trips, so every
    thread meets the same samples in the same order as when the whole slice is
    resident: the fitted states are bit-identical for any stage count.  The
    convergence test is on, so regions stop at different iterations with ring
    copies still in flight (drained before the next region)."""
    w = workloads.fit_batched(seed=5, n_regions=40, median=3000, sigma=1.0, lo=64, hi=20000)
    cfg = abi.default_fit_config(num_initial_components=K)
    base = {"cluster_size": 2, "large_threshold": 4096, "unroll": unroll}
    want, _ = run_fit(cuda, pkg, cfg, w["dirw"], w["offsets"], tuning={**base, "smem_samples": 12288})
    iters = want["iters_last"]
    assert len(np.unique(iters[iters > 0])) > 1  # regions stop at different iterations
    for ns in (1, 2, 3, 4, 8):
        got, _ = run_fit(cuda, pkg, cfg, w["dirw"], w["offsets"],
                         tuning={**base, "smem_samples": 2048, "stream_stages": ns})
        assert got.tobytes() == want.tobytes(), f"{ns} stages"


def test_shared_constants_equal_register_constants(cuda, pkg, abi, workloads):
    """The register-capped builds read the E-step constants from shared memory;
    the arithmetic and its order are those of the register build, so the fitted
    states are bit-identical."""
    w = workloads.fit_batched(seed=6, n_regions=30, median=2500, sigma=1.0, lo=64, hi=20000)
    cfg = abi.default_fit_config(num_initial_components=16)
    base = {"cluster_size": 2, "smem_samples": 3072, "stream_stages": 2}
    want, _ = run_fit(cuda, pkg, cfg, w["dirw"], w["offsets"], tuning={**base, "unroll": 2})
    for extra in ({"ctas_per_sm": 3, "unroll": 2}, {"ctas_per_sm": 4, "unroll": 2}):
        got, _ = run_fit(cuda, pkg, cfg, w["dirw"], w["offsets"], tuning={**base, **extra})
        assert got.tobytes() == want.tobytes(), extra


def test_fit_is_deterministic(cuda, pkg, abi, workloads):
    w = workloads.fit_batched(seed=4, n_regions=16, median=1200, sigma=1.0, lo=64, hi=9000)
    cfg = abi.forced_iterations(20, num_initial_components=16)
    a, _ = run_fit(cuda, pkg, cfg, w["dirw"], w["offsets"])
    b, _ = run_fit(cuda, pkg, cfg, w["dirw"], w["offsets"])
    assert a.tobytes() == b.tobytes()


def test_init_regions_matches_oracle(cuda, pkg, oracle, abi):
    cfg = abi.default_fit_config(num_initial_components=12)
    ctx = pkg.FitContext(cfg, max_regions=5)
    ctx.init_regions(5)
    ctx.sync()
    got = ctx.states(5)
    want = oracle.init_states(cfg, 5, exact=True)
    for f in ("weight", "mu_x", "mu_y", "mu_z", "kappa"):
        np.testing.assert_array_equal(got[f], want[f])
    np.testing.assert_allclose(got["norm"], want["norm"], rtol=2e-6)
    np.testing.assert_allclose(got["r"], want["r"], rtol=1e-6)
    assert np.all(np.isinf(got["distance"]))
    ctx.close()


def test_edge_cases(cuda, pkg, oracle, abi):
    """Empty regions, too few samples, one repeated direction (kappa clamps at
    maxKappa), zero-weight samples."""
    rng = np.random.default_rng(3)
    d = rng.normal(size=(3000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    same = np.tile(np.array([[0.0, 0.6, 0.8]]), (500, 1))
    counts = [0, 16, 17, 500, 1000, 0]
    dirs = np.concatenate([d[:16], d[16:33], same, d[33:1033]])
    w = np.ones(len(dirs))
    w[-1000:-500] = 0.0
    dirw = np.concatenate([dirs, w[:, None]], axis=1).astype(np.float32)
    offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint32)
    cfg = abi.forced_iterations(15, num_initial_components=8)
    st, _ = run_fit(cuda, pkg, cfg, dirw, offsets)
    want, _ = oracle.fit(cfg, dirw, offsets, f64=True)
    np.testing.assert_array_equal(st["iters_last"], [0, 0, 15, 15, 15, 0])
    np.testing.assert_array_equal(st["iters_last"], want["iters_last"])
    assert np.all(np.isfinite(st["kappa"])) and np.all(np.isfinite(st["weight"]))
    # one repeated direction: the mean-cosine prior r n/(n+1) (VMMFactory.h:415-420),
    # n = N pi, bounds kappa near n; the GPU lands where the oracle does
    top = np.argmax(want["weight"][3, :8])
    np.testing.assert_allclose(st["kappa"][3, top], want["kappa"][3, top], rtol=2e-3)
    assert st["kappa"][3, top] > 100.0
    assert_params_close(st, want, 8, GPU_TOL, np.array([False, False, True, False, True, False]))


def test_nonfinite_samples_are_reported(cuda, pkg, abi):
    torch = cuda
    dirw = np.tile(np.array([[0.0, 0.0, 1.0, 1.0]], dtype=np.float32), (400, 1))
    dirw[5, 0] = np.nan
    offsets = np.array([0, 200, 400], dtype=np.uint32)
    cfg = abi.forced_iterations(5, num_initial_components=8)
    ctx = pkg.FitContext(cfg, max_regions=2)
    d = torch.from_numpy(dirw).cuda()
    o = torch.from_numpy(offsets.view(np.int32)).cuda()
    ctx.fit(d, o, 2, abi.PG_FIT_INIT)
    with pytest.raises(pkg.PathGuideError) as e:
        ctx.sync()
    assert e.value.status == abi.PG_ERR_NUMERIC
    st = ctx.states(2)
    assert st["flags"][0] & 2 and not (st["flags"][1] & 2)
    ctx.close()


def test_argument_errors(cuda, pkg, abi):
    torch = cuda
    ctx = pkg.FitContext(abi.default_fit_config(), max_regions=4)
    d = torch.zeros(64, dtype=torch.float32, device="cuda")
    o = torch.zeros(8, dtype=torch.int32, device="cuda")
    with pytest.raises(pkg.PathGuideError) as e:
        ctx.fit(d, o, 5)  # more regions than the context holds
    assert e.value.status == abi.PG_ERR_ARG
    with pytest.raises(pkg.PathGuideError):
        ctx.fit(d.data_ptr() + 4, o, 2)  # misaligned float4 array
    with pytest.raises(pkg.PathGuideError):
        ctx.fit(d, o, 2, mode=7)
    ctx.close()



def test_fit_from_host_memory_with_empty_regions(cuda, pkg, abi, workloads):
    """Host-fed fits with empty regions between full ones, and with every region
    empty: page-locked (read by the fit) and pageable (copied in chunks) samples
    give the device fit's states bit for bit."""
    torch = cuda
    w = workloads.fit_batched(seed=31, n_regions=120, median=3000, sigma=1.0, lo=64, hi=30000)
    counts = np.diff(w["offsets"].astype(np.int64))
    counts[::3] = 0  # every third region empty
    counts[-1] = 0
    keep = np.concatenate([np.arange(w["offsets"][r], w["offsets"][r] + counts[r]) for r in range(len(counts))])
    dirw = np.ascontiguousarray(w["dirw"][keep], dtype=np.float32)
    offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint32)
    R = len(counts)
    cfg = abi.forced_iterations(20, num_initial_components=16)
    for dw, off in ((dirw, offsets), (np.zeros((0, 4), np.float32), np.zeros(R + 1, np.uint32))):
        a = pkg.FitContext(cfg, max_regions=R)
        d = torch.from_numpy(dw.reshape(-1, 4) if dw.size else np.zeros((1, 4), np.float32)).cuda()
        o = torch.from_numpy(off.view(np.int32)).cuda()
        a.fit(d, o, R, abi.PG_FIT_INIT)
        a.sync()
        want = a.states(R)
        for host in (torch.from_numpy(dw.reshape(-1) if dw.size else np.zeros(4, np.float32)).pin_memory(),
                     np.ascontiguousarray(dw.reshape(-1) if dw.size else np.zeros(4, np.float32))):
            b = pkg.FitContext(cfg, max_regions=R)
            b.fit_host(host, torch.from_numpy(off.view(np.int32)).pin_memory(), R, abi.PG_FIT_INIT)
            b.sync()
            assert want.tobytes() == b.states(R).tobytes()
            b.close()
        a.close()

@pytest.mark.parametrize("mode", ["init", "update", "forced16"])
def test_fit_from_host_memory_equals_device_fit(mode, cuda, pkg, abi, workloads):
    """pg_fit_regions_host (the fit from host memory) gives the same states,
    bit for bit, as pg_fit_regions on device copies of the samples: page-locked
    samples read by the fit itself (resident slices, streamed slices above the
    staging capacity, cluster slices; early stops in the converged modes),
    a page-locked view that starts inside its allocation, and pageable samples
    copied in chunks."""
    torch = cuda
    w = workloads.fit_batched(seed=12, n_regions=300, median=3000, sigma=1.0, lo=64, hi=40000)
    R = len(w["offsets"]) - 1
    if mode == "forced16":
        cfg = abi.forced_iterations(20, num_initial_components=16)
    else:
        cfg = abi.default_fit_config(num_initial_components=8)
    m = abi.PG_FIT_UPDATE if mode == "update" else abi.PG_FIT_INIT
    start = None
    if mode == "update":
        start, _ = run_fit(cuda, pkg, cfg, w["dirw"], w["offsets"])
    a_ctx = pkg.FitContext(cfg, max_regions=R)
    b_ctx = pkg.FitContext(cfg, max_regions=R)
    if start is not None:
        a_ctx.set_states(start)
        b_ctx.set_states(start)
    d = torch.from_numpy(np.ascontiguousarray(w["dirw"], dtype=np.float32)).cuda()
    o = torch.from_numpy(w["offsets"].astype(np.uint32).view(np.int32)).cuda()
    a_ctx.fit(d, o, R, m)
    dirw_h = torch.from_numpy(np.ascontiguousarray(w["dirw"], dtype=np.float32)).pin_memory()
    offs_h = torch.from_numpy(w["offsets"].astype(np.uint32).view(np.int32)).pin_memory()
    b_ctx.fit_host(dirw_h, offs_h, R, m)
    a_ctx.sync()
    b_ctx.sync()
    assert a_ctx.states(R).tobytes() == b_ctx.states(R).tobytes()
    # pageable numpy buffers work too
    c_ctx = pkg.FitContext(cfg, max_regions=R)
    if start is not None:
        c_ctx.set_states(start)
    c_ctx.fit_host(np.ascontiguousarray(w["dirw"], dtype=np.float32), w["offsets"].astype(np.uint32), R, m)
    c_ctx.sync()
    assert a_ctx.states(R).tobytes() == c_ctx.states(R).tobytes()
    # a page-locked view 16 bytes into its allocation, and one 4 bytes in (not
    # aligned for 16-byte loads: copied instead)
    for shift in (4, 1):
        e_ctx = pkg.FitContext(cfg, max_regions=R)
        if start is not None:
            e_ctx.set_states(start)
        flat = np.ascontiguousarray(w["dirw"], dtype=np.float32).reshape(-1)
        big = torch.zeros(flat.size + 8, dtype=torch.float32).pin_memory()
        big[shift:shift + flat.size] = torch.from_numpy(flat)
        e_ctx.fit_host(big[shift:shift + flat.size], offs_h, R, m)
        e_ctx.sync()
        assert a_ctx.states(R).tobytes() == e_ctx.states(R).tobytes(), shift
        e_ctx.close()
