"""The fit's autotuner (pg_autotune_fit) and CUDA-graph form
(pg_fit_graph_*): the tuner picks a launch shape from its grid and leaves the
mixture states as it found them; a captured fit replays bit-identically to a
direct pg_fit_regions with the same tuning, also after the caller refills the
captured buffers with new samples."""
from __future__ import annotations

import numpy as np
import pytest

from test_em_gpu import GPU_TOL
from test_oracle import assert_params_close

pytestmark = pytest.mark.gpu


def _upload(torch, w):
    d = torch.from_numpy(np.ascontiguousarray(w["dirw"], dtype=np.float32)).cuda()
    o = torch.from_numpy(np.asarray(w["offsets"], dtype=np.uint32).view(np.int32)).cuda()
    return d, o


def test_autotune_keeps_states_and_picks_a_grid_point(cuda, pkg, abi, workloads, oracle):
    torch = cuda
    # the uneven workload every launch shape is checked on (test_em_gpu.py)
    w = workloads.fit_batched(seed=11, n_regions=24, median=1500, sigma=1.2, lo=64, hi=20000)
    R = len(w["offsets"]) - 1
    cfg = abi.forced_iterations(20, num_initial_components=16)
    ctx = pkg.FitContext(cfg, max_regions=R)
    d, o = _upload(torch, w)
    ctx.fit(d, o, R, abi.PG_FIT_INIT)
    ctx.sync()
    before = ctx.states(R)
    s = torch.cuda.Stream()
    best, ms = ctx.autotune(d, o, R, abi.PG_FIT_UPDATE, stream=s)
    assert ms > 0 and best.threads_per_cta == 128 and best.components_per_thread in (8, 16)
    assert best.cluster_size in (1, 2, 4, 8, 16) and best.smem_samples in (3072, 6144)
    after = ctx.states(R)
    assert before.tobytes() == after.tobytes()
    # the tuned shape fits as well as any other
    ctx.fit(d, o, R, abi.PG_FIT_INIT)
    ctx.sync()
    want, _ = oracle.fit(cfg, w["dirw"], w["offsets"], f64=True)
    assert_params_close(ctx.states(R), want, 16, GPU_TOL, want["iters_last"] > 0)
    # explicit candidates, one of which the device cannot take (cluster of 16 with 256 threads is fine;
    # an invalid CTA size is rejected and skipped)
    cands = [abi.FitTuning(threads_per_cta=192), abi.FitTuning(cluster_size=2, smem_samples=3072)]
    best2, _ = ctx.autotune(d, o, R, abi.PG_FIT_INIT, candidates=cands, stream=s)
    assert best2.cluster_size == 2 and best2.smem_samples == 3072
    ctx.close()


def test_captured_fit_replays_like_a_direct_fit(cuda, pkg, abi, workloads):
    torch = cuda
    w1 = workloads.fit_batched(seed=5, n_regions=64, median=1500, sigma=1.0, lo=64, hi=20000)
    # a second sample set with the same region sizes (the captured offsets stay valid): axes permuted
    dirw2 = np.ascontiguousarray(w1["dirw"][:, [1, 2, 0, 3]])
    R = 64
    cfg = abi.forced_iterations(20, num_initial_components=16)
    s = torch.cuda.Stream()
    d, o = _upload(torch, w1)
    direct = pkg.FitContext(cfg, max_regions=R)
    direct.fit(d, o, R, abi.PG_FIT_INIT, stream=s)
    direct.sync(s)
    want1 = direct.states(R)
    ctx = pkg.FitContext(cfg, max_regions=R)
    g = ctx.capture_fit(d, o, R, abi.PG_FIT_INIT, stream=s)
    g.launch(s)
    ctx.sync(s)
    assert ctx.states(R).tobytes() == want1.tobytes()
    g.launch(s)  # replays are repeatable
    ctx.sync(s)
    assert ctx.states(R).tobytes() == want1.tobytes()
    # refill the captured sample buffer, replay, compare with a direct fit of the new samples
    d.copy_(torch.from_numpy(np.ascontiguousarray(dirw2, dtype=np.float32)).cuda())
    g.launch(s)
    ctx.sync(s)
    direct.fit(d, o, R, abi.PG_FIT_INIT, stream=s)
    direct.sync(s)
    assert ctx.states(R).tobytes() == direct.states(R).tobytes()
    g.close()
    ctx.close()
    direct.close()


def test_capture_needs_a_stream(cuda, pkg, abi, workloads):
    torch = cuda
    w = workloads.fit_batched(seed=5, n_regions=8, median=500, sigma=1.0, lo=64, hi=2000)
    ctx = pkg.FitContext(abi.default_fit_config(), max_regions=8)
    d, o = _upload(torch, w)
    with pytest.raises(pkg.PathGuideError) as e:
        ctx.capture_fit(d, o, 8, abi.PG_FIT_INIT, stream=None)
    assert e.value.status == abi.PG_ERR_ARG
    ctx.close()
