"""pg_fit_regions_noalloc: the fit for callers that cannot allocate device memory.

Renderers that hand out all device memory from their own arena (a second
allocator would fragment it), and plugin hosts that give the guiding step only
its own buffers and no right to allocate, cannot let the library call
cudaMalloc.  This entry point runs the same fit with its scratch in a static
device array of the library and the mixture states in a buffer the caller owns.
The test calls it through the C ABI twice in a row (the second call reuses the
scratch left by the first) and checks both results against the context-based
pg_fit_regions, within the GPU tolerance of the fit tests, then runs a stepwise
update (PG_FIT_UPDATE) from those states on both paths and compares again.  It
runs last (file name) so that a failure here stops a run only after every other
test has run.
"""
from __future__ import annotations

import numpy as np
import pytest

from test_em_gpu import GPU_TOL, run_fit
from test_oracle import assert_params_close

pytestmark = pytest.mark.gpu


def _noalloc_fit(cuda, pkg, abi, cfg, d, o, R, mode=None, states=None):
    torch = cuda
    if states is None:
        buf = torch.zeros(R * abi.STATE_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    else:
        buf = torch.from_numpy(np.frombuffer(states.tobytes(), dtype=np.uint8).copy()).cuda()
    st = pkg.fit_regions_noalloc(cfg, buf, d, o, R, abi.PG_FIT_INIT if mode is None else mode)
    assert st == abi.PG_OK, pkg.status_string(st)
    torch.cuda.synchronize()
    return np.frombuffer(buf.cpu().numpy().tobytes(), dtype=abi.STATE_DTYPE).copy()


def test_noalloc_fit_matches_context_fit_on_consecutive_calls(cuda, pkg, abi, workloads):
    torch = cuda
    # uneven regions, some above 24576 samples so the cluster-shared path runs too
    w = workloads.fit_batched(seed=21, n_regions=40, median=1500, sigma=1.3, lo=64, hi=30000)
    R = len(w["offsets"]) - 1
    assert (np.diff(w["offsets"]) > 24576).any()
    d = torch.from_numpy(w["dirw"]).cuda()
    o = torch.from_numpy(w["offsets"].view(np.int32)).cuda()
    for K in (16, 8):  # two consecutive calls with different mixtures over the same scratch
        cfg = abi.forced_iterations(20, num_initial_components=K)
        want, _ = run_fit(cuda, pkg, cfg, w["dirw"], w["offsets"])
        got = _noalloc_fit(cuda, pkg, abi, cfg, d, o, R)
        np.testing.assert_array_equal(got["iters_last"], want["iters_last"])
        np.testing.assert_array_equal(got["total_num_samples"], want["total_num_samples"])
        assert_params_close(got, want, K, GPU_TOL, want["iters_last"] > 0)
        assert not (got["flags"] & (abi.PG_STATE_FIT_FAILED | abi.PG_STATE_NONFINITE)).any()
        got2 = _noalloc_fit(cuda, pkg, abi, cfg, d, o, R)
        assert_params_close(got2, want, K, GPU_TOL, want["iters_last"] > 0)


def test_noalloc_update_matches_context_update(cuda, pkg, abi, workloads):
    """The stepwise update (always the 16-component build) from the states of a
    first fit, on new samples: the allocation-free path against the context's."""
    torch = cuda
    w1 = workloads.fit_batched(seed=31, n_regions=24, median=1200, sigma=1.2, lo=64, hi=28000)
    w2 = workloads.fit_batched(seed=32, n_regions=24, median=1200, sigma=1.2, lo=64, hi=28000)
    R = len(w1["offsets"]) - 1
    cfg = abi.forced_iterations(10, num_initial_components=8)
    first, _ = run_fit(cuda, pkg, cfg, w1["dirw"], w1["offsets"])
    want, _ = run_fit(cuda, pkg, cfg, w2["dirw"], w2["offsets"], mode=abi.PG_FIT_UPDATE, states=first)
    d = torch.from_numpy(w2["dirw"]).cuda()
    o = torch.from_numpy(w2["offsets"].view(np.int32)).cuda()
    for _ in range(2):
        got = _noalloc_fit(cuda, pkg, abi, cfg, d, o, R, mode=abi.PG_FIT_UPDATE, states=first)
        np.testing.assert_array_equal(got["iters_last"], want["iters_last"])
        np.testing.assert_array_equal(got["total_num_samples"], want["total_num_samples"])
        assert_params_close(got, want, 8, GPU_TOL, want["iters_last"] > 0)
        assert not (got["flags"] & abi.PG_STATE_FIT_FAILED).any()


def test_noalloc_rejects_too_many_regions(cuda, pkg, abi):
    torch = cuda
    d = torch.zeros(16, dtype=torch.float32, device="cuda")
    o = torch.zeros(8, dtype=torch.int32, device="cuda")
    cfg = abi.default_fit_config()
    st = pkg.fit_regions_noalloc(cfg, d, d, o, pkg.NOALLOC_MAX_REGIONS + 1)
    assert st == abi.PG_ERR_NOMEM
