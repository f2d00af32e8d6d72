"""GPU parity of the guiding steps around the fit, through the C ABI:
sample bucketing (SampleCollector::getSortedData), region tree, parallax
pre-pass, lobe distances, VMM_Theta packing and the whole PathGuiding::update
pass, each against the oracle (oracle/pg_oracle.c) on the same inputs.

Exactness: bucketing, region boxes and the parallax pre-pass are integer or
single-rounding FP32 work and must be bit-exact.  Distances accumulate in FP32
on the GPU and FP64 in the oracle (rtol 2e-4; the reference itself, in FP32
with its fast exp, is within 2e-3 of the oracle - see test_oracle.py).
"""
from __future__ import annotations

import numpy as np
import pytest

from test_em_gpu import GPU_TOL
from test_oracle import REF_TOL, assert_params_close

pytestmark = pytest.mark.gpu


def dev(torch, arr):
    a = np.ascontiguousarray(arr)
    return torch.from_numpy(a.view(np.uint8).reshape(-1).copy()).cuda()


def host(t, dtype):
    return np.frombuffer(t.cpu().numpy().tobytes(), dtype=dtype).copy()


def records_in_regions(workloads, oracle, split_count, scene, seed, median=600, miss=0.1, invalid=0.1):
    boxes = oracle.region_aabbs(split_count, scene)
    R = boxes.shape[0]
    rng = np.random.default_rng(seed)
    counts = workloads.region_counts_lognormal(rng, R, median, 1.0, 0, 20000)
    w = workloads.mixture_samples(rng, counts, 1, 4, 3.0, 600.0, 1.0, region_boxes=boxes,
                                  dist_range=(0.05, 30.0), miss_frac=miss)
    rec = w["records"]
    # interleave as a tracer writes them (pixel order), with invalid slots
    perm = rng.permutation(rec.shape[0])
    rec = rec[perm]
    bad = rng.random(rec.shape[0]) < invalid
    rec["flags"][bad] = 0xFFFFFFFF
    rec["flags"][rng.random(rec.shape[0]) < 0.01] = R + 3  # out-of-range ids are dropped too
    return rec, boxes


@pytest.mark.parametrize("n,R", [(0, 7), (1, 1), (4095, 3), (70000, 300), (200000, 4096)])
def test_sort_samples_matches_stable_bucketing(n, R, cuda, pkg, abi, oracle, workloads):
    torch = cuda
    rng = np.random.default_rng(n + R)
    rec = np.zeros(n, dtype=workloads.RECORD_DTYPE)
    rec["flags"] = rng.integers(0, R, size=n)
    rec["flags"][rng.random(n) < 0.15] = 0xFFFFFFFF
    rec["weight"] = np.arange(n, dtype=np.float32)
    rec["direction"] = rng.normal(size=(n, 3))
    want, want_off = oracle.sort_samples(rec, R)
    ctx = pkg.FitContext(abi.default_fit_config(), max_regions=max(R, 1))
    d_rec = dev(torch, rec)
    d_sorted = torch.zeros(max(n, 1) * 40, dtype=torch.uint8, device="cuda")
    d_off = torch.zeros(R + 1, dtype=torch.int32, device="cuda")
    ctx.sort_samples(d_rec, n, R, d_sorted, d_off)
    ctx.sync()
    off = d_off.cpu().numpy().view(np.uint32)
    np.testing.assert_array_equal(off, want_off)
    got = host(d_sorted, workloads.RECORD_DTYPE)[:off[-1]]
    assert got.tobytes() == want.tobytes()
    ctx.close()


def test_region_tree_matches_oracle(cuda, pkg, abi, oracle):
    scene = np.array([-2.0, 0.0, -1.0, 3.0, 2.5, 4.0], dtype=np.float32)
    ctx = pkg.FitContext(abi.default_fit_config(), max_regions=1024)
    for splits in (0, 1, 5, 10):
        ctx.set_regions(splits, scene)
        assert ctx.region_count() == 1 << splits
        np.testing.assert_array_equal(ctx.region_aabbs(), oracle.region_aabbs(splits, scene))
    ctx.close()


def test_prefit_parallax_matches_oracle(cuda, pkg, abi, oracle, workloads):
    torch = cuda
    scene = np.array([0.0, 0.0, 0.0, 4.0, 2.0, 3.0], dtype=np.float32)
    rec, boxes = records_in_regions(workloads, oracle, 4, scene, seed=9)
    R = boxes.shape[0]
    srt, off = oracle.sort_samples(rec, R)
    means = boxes[:, :3] + np.float32(0.5) * (boxes[:, 3:] - boxes[:, :3])
    want_dirw, want_dist = oracle.prefit_parallax(srt, off, means)
    ctx = pkg.FitContext(abi.default_fit_config(), max_regions=R)
    ctx.set_regions(4, scene)
    n = srt.shape[0]
    d_dirw = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    d_dist = torch.zeros(n, dtype=torch.float32, device="cuda")
    d_off = torch.from_numpy(off.view(np.int32)).cuda()
    ctx.prefit_parallax(dev(torch, srt), d_off, R, n, d_dirw, d_dist)
    ctx.sync()
    np.testing.assert_array_equal(d_dirw.cpu().numpy(), want_dirw)
    np.testing.assert_array_equal(d_dist.cpu().numpy(), want_dist)
    st = ctx.states(R)
    busy = np.diff(off.astype(np.int64)) > 0
    np.testing.assert_array_equal(st["parallax_mean"][busy], means[busy])
    np.testing.assert_array_equal(st["parallax_mean"][~busy], 0.0)  # empty regions keep their state
    ctx.close()


def test_update_distances_matches_oracle_and_reference(cuda, pkg, abi, oracle, golden):
    torch = cuda
    g = golden("distances_k8")
    R = len(g["offsets"]) - 1
    ctx = pkg.FitContext(abi.default_fit_config(), max_regions=R)
    ctx.set_states(g["states_in"])
    d_off = torch.from_numpy(g["offsets"].view(np.int32)).cuda()
    d_dist = torch.from_numpy(g["dist"]).cuda()
    for dirw, ref in ((g["dirw"], g["states1"]), (g["dirw2"], g["states2"])):
        before = ctx.states(R)
        ctx.update_distances(torch.from_numpy(dirw).cuda(), d_dist, d_off, R)
        ctx.sync()
        got = ctx.states(R)
        want = oracle.update_distances(dirw, g["dist"], g["offsets"], before)
        fin = np.isfinite(want["distance"][:, :8])
        assert np.array_equal(fin, np.isfinite(got["distance"][:, :8]))
        np.testing.assert_allclose(got["distance"][:, :8][fin], want["distance"][:, :8][fin], rtol=2e-4)
        np.testing.assert_allclose(got["dist_sum_w"][:, :8], want["dist_sum_w"][:, :8], rtol=2e-4, atol=1e-30)
        fr = np.isfinite(ref["distance"][:, :8])
        np.testing.assert_allclose(got["distance"][:, :8][fr], ref["distance"][:, :8][fr], rtol=2e-3)
    ctx.close()


def test_pack_vmm_theta_matches_oracle(cuda, pkg, abi, oracle, golden):
    torch = cuda
    g = golden("fit_forced_k16")
    st = g["states"].copy()
    rng = np.random.default_rng(1)
    st["distance"] = np.where(rng.random(st["distance"].shape) < 0.5, np.inf,
                              rng.uniform(0.1, 9.0, size=st["distance"].shape)).astype(np.float32)
    st["parallax_mean"] = rng.normal(size=(st.shape[0], 3)).astype(np.float32)
    st["kappa"][0, 3] = 0.0005  # below VMF_MinKappa: packed as 0
    R = st.shape[0]
    ctx = pkg.FitContext(abi.default_fit_config(), max_regions=R)
    ctx.set_states(st)
    out = torch.zeros(R * 720, dtype=torch.uint8, device="cuda")
    ctx.pack_vmm_theta(R, out)
    ctx.sync()
    got = host(out, abi.VMM_THETA_DTYPE)
    want = oracle.pack_vmm_theta(st, use_parallax=True)
    for f in ("pi", "mean_position", "used_distributions"):
        np.testing.assert_array_equal(got[f], want[f])
    for f in ("mu", "k", "distance", "target", "e_min2k"):
        np.testing.assert_array_equal(got["thetas"][f], want["thetas"][f])
    np.testing.assert_allclose(got["thetas"]["norm"], want["thetas"]["norm"], rtol=1e-7, equal_nan=True)
    ctx.close()


def oracle_update(oracle, abi, cfg, rec, boxes, states, first):
    """PathGuiding::update restated with the oracle: bucket, pre-fit, fit, distances, pack."""
    R = boxes.shape[0]
    srt, off = oracle.sort_samples(rec, R)
    means = boxes[:, :3] + np.float32(0.5) * (boxes[:, 3:] - boxes[:, :3])
    st = states.copy()
    busy = np.diff(off.astype(np.int64)) > 0  # empty regions are not updated (PathGuiding.cpp:281-288)
    st["last_parallax_mean"][busy] = st["parallax_mean"][busy]
    st["parallax_mean"][busy] = means[busy]
    if not first:
        for r in np.where(busy)[0]:
            st[r] = oracle.reposition(st[r], st["last_parallax_mean"][r] - means[r])
    dirw, dist = oracle.prefit_parallax(srt, off, means)
    st, _ = oracle.fit(cfg, dirw, off, states=st, mode=abi.PG_FIT_CONTINUE if first else abi.PG_FIT_UPDATE)
    st = oracle.update_distances(dirw, dist, off, st)
    return st, oracle.pack_vmm_theta(st, use_parallax=True)


def test_guiding_pass_matches_oracle(cuda, pkg, abi, oracle, workloads):
    torch = cuda
    scene = np.array([-1.0, -1.0, -1.0, 1.0, 1.0, 1.0], dtype=np.float32)
    cfg = abi.default_fit_config(num_initial_components=8)
    ctx = pkg.FitContext(cfg, max_regions=64)
    ctx.set_regions(5, scene)
    R = ctx.region_count()
    boxes = ctx.region_aabbs()
    want_states = ctx.states(R)
    for p in range(3):
        rec, _ = records_in_regions(workloads, oracle, 5, scene, seed=100 + p, median=900)
        vmm = torch.zeros(R * 720, dtype=torch.uint8, device="cuda")
        ctx.update(dev(torch, rec), rec.shape[0], vmm)
        ctx.sync()
        got = ctx.states(R)
        want_states, want_vmm = oracle_update(oracle, abi, cfg, rec, boxes, want_states, first=(p == 0))
        np.testing.assert_array_equal(got["iters_last"], want_states["iters_last"])
        np.testing.assert_array_equal(got["total_num_samples"], want_states["total_num_samples"])
        fitted = want_states["iters_last"] > 0
        assert_params_close(got, want_states, 8, GPU_TOL, fitted)
        fin = np.isfinite(want_states["distance"][:, :8])
        np.testing.assert_allclose(got["distance"][:, :8][fin], want_states["distance"][:, :8][fin], rtol=2e-3)
        v = host(vmm, abi.VMM_THETA_DTYPE)
        np.testing.assert_array_equal(v["used_distributions"], 8)
        np.testing.assert_allclose(v["pi"], want_vmm["pi"], rtol=GPU_TOL["weight_rtol"], atol=1e-7)
        want_states = got  # continue both from the GPU state, as PathGuiding keeps one state
    ctx.close()


def test_update_requires_regions(cuda, pkg, abi):
    torch = cuda
    ctx = pkg.FitContext(abi.default_fit_config(), max_regions=8)
    with pytest.raises(pkg.PathGuideError) as e:
        ctx.update(torch.zeros(40, dtype=torch.uint8, device="cuda"), 1)
    assert e.value.status == abi.PG_ERR_STATE
    ctx.close()


def test_region_first_seen_in_a_later_pass(cuda, pkg, abi, oracle, workloads):
    """A region empty in the first pass and filled in a later one is fitted
    from its initial mixture (no prior statistics), never NaN; regions that
    stay empty keep their state untouched."""
    torch = cuda
    scene = np.array([-1.0, -1.0, -1.0, 1.0, 1.0, 1.0], dtype=np.float32)
    cfg = abi.default_fit_config(num_initial_components=8)
    ctx = pkg.FitContext(cfg, max_regions=8)
    ctx.set_regions(3, scene)
    R = ctx.region_count()
    rec, _ = records_in_regions(workloads, oracle, 3, scene, seed=5, median=900, invalid=0.0)
    rec["flags"][rec["flags"] >= R] = 0
    first = rec[rec["flags"] < 4]           # pass 0: regions 0-3 only
    ctx.update(dev(torch, first), first.shape[0])
    ctx.sync()
    s0 = ctx.states(R)
    assert (s0["total_num_samples"][4:] == 0).all()
    ctx.update(dev(torch, rec[rec["flags"] != 7]), int((rec["flags"] != 7).sum()))  # pass 1: all but region 7
    ctx.sync()                              # raises PG_ERR_NUMERIC on a non-finite parameter
    s1 = ctx.states(R)
    K = 8
    for f in ("weight", "mu_x", "mu_y", "mu_z", "kappa"):
        assert np.isfinite(s1[f][:, :K]).all(), f
    assert (s1["total_num_samples"][4:7] > 0).all()
    for f in s0.dtype.names:                 # region 7 untouched
        np.testing.assert_array_equal(s1[f][7], s0[f][7])
    # the later-first region matches a fresh fit (continue mode) of its samples
    want, _ = oracle.fit(cfg, *_dirw_offsets(oracle, rec[(rec["flags"] >= 4) & (rec["flags"] < 7)], 3, s0, R),
                         mode=abi.PG_FIT_UPDATE)
    assert_params_close(s1[4:7], want[4:7], K, GPU_TOL, want["iters_last"][4:7] > 0)
    ctx.close()


def _dirw_offsets(oracle, rec, split_count, states, R):
    """Oracle inputs of one update pass: bucketed float4 samples seen from the
    region centres (the first pass of these regions: no reposition)."""
    srt, off = oracle.sort_samples(rec, R)
    boxes = oracle.region_aabbs(split_count, np.array([-1.0, -1.0, -1.0, 1.0, 1.0, 1.0], dtype=np.float32))
    means = boxes[:, :3] + np.float32(0.5) * (boxes[:, 3:] - boxes[:, :3])
    dirw, _ = oracle.prefit_parallax(srt, off, means)
    return dirw, off, states
