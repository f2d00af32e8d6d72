"""Parity at the benchmark sizes.

- The CPU-runnable configuration (64 regions x 16384 samples, K = 8, 20 EM
  iterations): every region of the GPU fit against the FP64 oracle.
- The batched configuration (4096 regions, lognormal sizes up to 262144,
  K = 16, 20 iterations, 13.9 M samples): the GPU fits all regions in one
  launch; the FP64 oracle refits a sample of 192 regions that includes the
  largest ones (regions are independent, so the subset is exact), and
  size-independent properties hold for all regions: weights sum to one, means
  are unit vectors, kappa lies in [0, maxKappa], the sample counts add up.
"""
from __future__ import annotations

import numpy as np
import pytest

from test_em_gpu import GPU_TOL
from test_oracle import assert_params_close

pytestmark = pytest.mark.gpu


def _fit_gpu(torch, pkg, abi, cfg, w):
    R = len(w["offsets"]) - 1
    ctx = pkg.FitContext(cfg, max_regions=R)
    d = torch.from_numpy(np.ascontiguousarray(w["dirw"], dtype=np.float32)).cuda()
    o = torch.from_numpy(np.asarray(w["offsets"], dtype=np.uint32).view(np.int32)).cuda()
    ctx.fit(d, o, R, abi.PG_FIT_INIT)
    ctx.sync()
    st = ctx.states(R)
    ctx.close()
    return st


def test_cpu_runnable_configuration(cuda, pkg, abi, workloads, oracle):
    w = workloads.fit_plain()
    cfg = abi.forced_iterations(20, num_initial_components=8)
    st = _fit_gpu(cuda, pkg, abi, cfg, w)
    want, _ = oracle.fit(cfg, w["dirw"], w["offsets"], f64=True)
    np.testing.assert_array_equal(st["iters_last"], want["iters_last"])
    assert_params_close(st, want, 8, GPU_TOL, want["iters_last"] > 0)


def test_batched_configuration(cuda, pkg, abi, workloads, oracle):
    w = workloads.fit_batched(seed=3)
    K = 16
    cfg = abi.forced_iterations(20, num_initial_components=K)
    st = _fit_gpu(cuda, pkg, abi, cfg, w)
    offsets = w["offsets"].astype(np.int64)
    counts = np.diff(offsets)
    R = counts.size
    fitted = counts > 2 * K
    # size-independent properties over all regions
    np.testing.assert_allclose(st["weight"][:, :K].sum(1), 1.0, atol=2e-5)
    mu = np.stack([st["mu_x"][:, :K], st["mu_y"][:, :K], st["mu_z"][:, :K]], -1)
    np.testing.assert_allclose(np.linalg.norm(mu, axis=-1), 1.0, atol=1e-5)
    assert (st["kappa"][:, :K] >= 0).all() and (st["kappa"][:, :K] <= cfg.max_kappa).all()
    np.testing.assert_array_equal(st["total_num_samples"][fitted], counts[fitted])
    assert (st["iters_last"][fitted] == 20).all()
    # exact subset parity: the 64 largest regions and 128 others
    rng = np.random.default_rng(0)
    largest = np.argsort(counts)[-64:]
    rest = rng.choice(np.setdiff1d(np.arange(R), largest), size=128, replace=False)
    pick = np.sort(np.concatenate([largest, rest]))
    sub_dirw = np.concatenate([w["dirw"][offsets[r]:offsets[r + 1]] for r in pick])
    sub_off = np.concatenate([[0], np.cumsum(counts[pick])]).astype(np.uint32)
    want, _ = oracle.fit(cfg, sub_dirw, sub_off, f64=True)
    got = st[pick]
    np.testing.assert_array_equal(got["iters_last"], want["iters_last"])
    assert_params_close(got, want, K, GPU_TOL, want["iters_last"] > 0)
