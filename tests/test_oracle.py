"""CPU tests: the oracle against the reference's own outputs (golden fixtures).

The golden fixtures were produced by the reference's lightpmm fit compiled in
place (tests/golden/make_golden.py).  The FP32 restatement in oracle/ must
reproduce them bit for bit on the machine that made them (x86-64; on other
ISAs libm may differ in the last ulp, so a tight tolerance applies there).  The
FP64 oracle differs from the reference only through lightpmm's exp
approximation (max relative error 6.1e-5, measured below), amplified by the EM
iterations; the tolerances FP64-vs-reference are stated in REF_TOL.
"""
from __future__ import annotations

import platform

import numpy as np
import pytest

FIELDS = ("weight", "mu_x", "mu_y", "mu_z", "kappa", "r", "norm", "e_min2k")
EXACT_ISA = platform.machine() in ("x86_64", "AMD64")

# FP64 (exact exp) vs the reference (lightpmm fastexp), after up to 20 EM iterations.
REF_TOL = {"weight_rtol": 2e-3, "kappa_rtol": 2e-3, "r_atol": 3e-4, "mu_angle": 2e-3,
           "ll_per_weight": 2e-4, "ll_rtol": 1e-3}


def cfg_from(abi, c):
    return abi.FitConfig(int(c[0]), int(c[1]), float(c[2]), int(c[3]), float(c[4]), float(c[5]),
                         float(c[6]), float(c[7]), float(c[8]), int(c[9]))


def mu_angle(a, b):
    ma = np.stack([a["mu_x"], a["mu_y"], a["mu_z"]], -1).astype(np.float64)
    mb = np.stack([b["mu_x"], b["mu_y"], b["mu_z"]], -1).astype(np.float64)
    with np.errstate(invalid="ignore", divide="ignore"):  # unused components may hold zero vectors
        c = (ma * mb).sum(-1) / np.linalg.norm(ma, axis=-1) / np.linalg.norm(mb, axis=-1)
    return np.arccos(np.clip(c, -1.0, 1.0))


def assert_params_close(got, ref, K, tol, fitted):
    for f, key in (("weight", "weight_rtol"), ("kappa", "kappa_rtol")):
        a, b = got[f][fitted, :K], ref[f][fitted, :K]
        err = np.abs(a - b) / np.maximum(np.abs(b), 1e-6)
        assert err.max() <= tol[key], f"{f}: max rel err {err.max():.3g} > {tol[key]}"
    err = np.abs(got["r"][fitted, :K] - ref["r"][fitted, :K]).max()
    assert err <= tol["r_atol"], f"r: max abs err {err:.3g}"
    ang = mu_angle(got[fitted], ref[fitted])[:, :K].max()
    assert ang <= tol["mu_angle"], f"mu: max angle {ang:.3g} rad"


FIT_SETS = ["fit_forced_k8", "fit_forced_k16", "fit_forced_k5", "fit_converge_k8", "fit_update_k8"]


@pytest.mark.parametrize("name", FIT_SETS)
def test_port_reproduces_reference_fit(name, golden, oracle, abi):
    g = golden(name)
    cfg = cfg_from(abi, g["cfg"])
    K = cfg.num_initial_components
    mode = abi.PG_FIT_UPDATE if "states_in" in g else abi.PG_FIT_INIT
    st, ll = oracle.fit(cfg, g["dirw"], g["offsets"], states=g.get("states_in"), mode=mode, f64=False)
    ref = g["states"]
    assert np.array_equal(st["iters_last"], ref["iters_last"])
    assert np.array_equal(st["total_num_samples"], ref["total_num_samples"])
    for f in FIELDS:
        if EXACT_ISA:
            assert np.array_equal(st[f][:, :K], ref[f][:, :K]), f"{name}: {f} not bit-exact"
        else:
            np.testing.assert_allclose(st[f][:, :K], ref[f][:, :K], rtol=2e-5, atol=1e-6)
    if EXACT_ISA:
        assert np.array_equal(st["sample_weight"], ref["sample_weight"])
        assert np.array_equal(ll, g["ll_final"])


@pytest.mark.parametrize("name", FIT_SETS)
def test_fp64_oracle_within_stated_tolerance_of_reference(name, golden, oracle, abi):
    g = golden(name)
    cfg = cfg_from(abi, g["cfg"])
    K = cfg.num_initial_components
    mode = abi.PG_FIT_UPDATE if "states_in" in g else abi.PG_FIT_INIT
    st, ll = oracle.fit(cfg, g["dirw"], g["offsets"], states=g.get("states_in"), mode=mode, f64=True)
    ref = g["states"]
    np.testing.assert_array_equal(st["iters_last"], ref["iters_last"])
    fitted = ref["iters_last"] > 0
    assert_params_close(st, ref, K, REF_TOL, fitted)
    counts = np.diff(g["offsets"].astype(np.int64))
    sw = np.array([g["dirw"][g["offsets"][r]:g["offsets"][r + 1], 3].sum() for r in range(len(counts))])
    d = np.abs(ll - g["ll_final"].astype(np.float64))
    assert np.all(d <= REF_TOL["ll_per_weight"] * sw + REF_TOL["ll_rtol"] * np.abs(ll) + 1e-3)


def test_unfitted_regions_keep_initial_mixture(golden, oracle, abi):
    """Regions with N <= 2K samples are not fitted (VMMFactory.h:175-177)."""
    g = golden("fit_forced_k8")
    counts = np.diff(g["offsets"].astype(np.int64))
    st, _ = oracle.fit(cfg_from(abi, g["cfg"]), g["dirw"], g["offsets"], f64=True)
    init = oracle.init_states(cfg_from(abi, g["cfg"]), 1)[0]
    for r in np.nonzero(counts <= 16)[0]:
        assert st["iters_last"][r] == 0 and st["total_num_samples"][r] == 0
        np.testing.assert_array_equal(st["weight"][r], init["weight"])
        np.testing.assert_array_equal(st["mu_z"][r], init["mu_z"])


def test_fastexp_port_matches_reference(golden, oracle):
    g = golden("fastexp")
    np.testing.assert_array_equal(oracle.fastexp(g["x"]), g["y"])
    x = g["x"].astype(np.float64)
    ok = x > -87.0
    rel = np.abs(g["y"][ok] / np.exp(x[ok]) - 1.0)
    assert rel.max() < 6.2e-5  # the error that sets REF_TOL


def test_distance_statistic_within_tolerance_of_reference(golden, oracle):
    g = golden("distances_k8")
    d1 = oracle.update_distances(g["dirw"], g["dist"], g["offsets"], g["states_in"])
    d2 = oracle.update_distances(g["dirw2"], g["dist"], g["offsets"], d1)
    for got, ref in ((d1, g["states1"]), (d2, g["states2"])):
        fin = np.isfinite(ref["distance"][:, :8])
        assert np.array_equal(fin, np.isfinite(got["distance"][:, :8]))
        np.testing.assert_allclose(got["distance"][:, :8][fin], ref["distance"][:, :8][fin], rtol=2e-3)
        np.testing.assert_allclose(got["dist_sum_w"][:, :8], ref["dist_sum_w"][:, :8], rtol=2e-3, atol=1e-30)


def test_reposition_matches_reference(golden, oracle):
    g = golden("reposition_k8")
    got = oracle.reposition(g["state_in"][0], g["delta"])
    ref = g["state_out"][0]
    for f in ("distance", "mu_x", "mu_y", "mu_z"):
        np.testing.assert_array_equal(got[f][:8], ref[f][:8])


def test_initial_mixture_matches_reference(golden, oracle, abi):
    """VMMFactory::initialize: the port's state equals the reference's initial PMM."""
    from oracle.oracle import ReferenceFit
    if not ReferenceFit.available():
        pytest.skip("reference harness not built on this machine")
    ref = ReferenceFit()
    for K in (1, 5, 8, 16):
        cfg = abi.default_fit_config(num_initial_components=K)
        a = ref.init_states(cfg, 1)[0]
        b = oracle.init_states(cfg, 1, exact=False)[0]
        for f in FIELDS:
            assert np.array_equal(a[f][:K], b[f][:K]), (K, f)


def test_region_tree(oracle):
    box = np.array([-1.0, 0.0, -2.0, 3.0, 1.0, 2.0], dtype=np.float32)
    for splits in (0, 1, 3, 6):
        b = oracle.region_aabbs(splits, box)
        assert b.shape == (1 << splits, 6)
        assert np.all(b[:, 3:] > b[:, :3])
        vol = np.prod(b[:, 3:] - b[:, :3], axis=1).sum()
        np.testing.assert_allclose(vol, np.prod((box[3:] - box[:3]) * 1.00002), rtol=1e-4)
    # Aabb::splitAabb picks the largest axis; on a tie of x and z it takes z
    b1 = oracle.region_aabbs(1, box)
    assert abs(b1[0, 5] - b1[1, 2]) < 1e-6 and b1[0, 3] == b1[1, 3]
    box2 = np.array([0.0, 0.0, 0.0, 5.0, 1.0, 2.0], dtype=np.float32)
    b2 = oracle.region_aabbs(1, box2)
    assert abs(b2[0, 3] - b2[1, 0]) < 1e-6 and b2[0, 5] == b2[1, 5]


def test_sort_samples_buckets_stably(oracle, workloads):
    rng = np.random.default_rng(5)
    rec = np.zeros(5000, dtype=workloads.RECORD_DTYPE)
    rec["flags"] = rng.integers(0, 9, size=5000)
    rec["flags"][rng.random(5000) < 0.2] = 0xFFFFFFFF
    rec["weight"] = np.arange(5000, dtype=np.float32)
    s, off = oracle.sort_samples(rec, 9)
    valid = rec[rec["flags"] != 0xFFFFFFFF]
    assert s.shape[0] == valid.shape[0] == off[-1]
    for r in range(9):
        seg = s[off[r]:off[r + 1]]
        assert np.all(seg["flags"] == r)
        assert np.all(np.diff(seg["weight"]) > 0)  # stable


def test_prefit_parallax_geometry(oracle, workloads):
    rng = np.random.default_rng(2)
    w = workloads.mixture_samples(rng, np.array([50, 70]), 1, 3, 2.0, 100.0, 1.0,
                                  dist_range=(0.5, 20.0), miss_frac=0.2)
    means = np.array([[0.5, 0.5, 0.5], [0.2, 0.4, 0.9]], dtype=np.float32)
    dirw, dist = oracle.prefit_parallax(w["records"], w["offsets"], means)
    rec = w["records"]
    region = rec["flags"]
    hit = rec["distance"] > 0
    assert np.all(np.isinf(dist[~hit]))
    np.testing.assert_allclose(np.linalg.norm(dirw[:, :3], axis=1), 1.0, atol=1e-6)
    target = rec["position"] + rec["distance"][:, None] * rec["direction"]
    recon = means[region] + dist[:, None] * dirw[:, :3]
    np.testing.assert_allclose(recon[hit], target[hit], atol=2e-5 * (1 + np.abs(target[hit]).max()))
    np.testing.assert_array_equal(dirw[~hit, :3], rec["direction"][~hit])


def test_pack_vmm_theta_layout(oracle, golden):
    g = golden("fit_forced_k8")
    st = g["states"].copy()
    st["distance"][:] = np.inf
    st["distance"][:, 0] = 2.5
    st["parallax_mean"] = [1.0, 2.0, 3.0]
    v = oracle.pack_vmm_theta(st, use_parallax=True)
    assert np.all(v["used_distributions"] == 8)
    np.testing.assert_array_equal(v["pi"][:, :8], st["weight"][:, :8])
    assert np.all(v["thetas"]["distance"][:, 1:] == -1.0)
    assert np.all(v["thetas"]["distance"][:, 0] == 2.5)
    np.testing.assert_allclose(v["thetas"]["target"][:, 0, 0], 1.0 + 2.5 * st["mu_x"][:, 0], rtol=1e-6)
