"""GPU parity of adaptive region splitting (PathGuiding::update's split check
and splitRegion, src/PathGuiding.cpp:290-348) through the C ABI, against the
oracle (oracle/pg_oracle.c: pgo_split_regions, pgo_region_of).

The split itself is exact work (a comparison, two multiplications by 0.25,
copies, one midpoint): states, statistics, boxes and the tree are compared bit
for bit; fits around it to the GPU fit's tolerance (GPU_TOL)."""
from __future__ import annotations

import numpy as np
import pytest

from test_em_gpu import GPU_TOL
from test_guide_gpu import dev, host, oracle_update
from test_oracle import assert_params_close
from test_regions import SCENE, split_fixture
from test_trace_gpu import assert_same_seed_parity, render_gpu, tracer  # noqa: F401 (fixture)

pytestmark = pytest.mark.gpu


def test_split_regions_matches_oracle(cuda, pkg, abi, oracle):
    st, ex, boxes, nodes, leaf = split_fixture(oracle, abi, split_count=3, seed=4)
    R, cap = st.shape[0], 64
    ctx = pkg.FitContext(abi.default_fit_config(), max_regions=cap)
    ctx.set_regions(3, SCENE)
    ctx.set_split_merge(abi.default_split_merge_config())
    ctx.set_states(st)
    ctx.set_extras(ex)
    ctx.set_region_split(abi.default_region_split_config())
    n = ctx.split_regions()
    s2, e2, b2, n2, _, _ = oracle.split_regions(cap, 10000.0, st, ex, boxes, nodes, leaf, 2 * R - 1)
    assert n == s2.shape[0] > R
    assert ctx.states(n).tobytes() == s2.tobytes()
    assert ctx.extras(n).tobytes() == e2.tobytes()
    np.testing.assert_array_equal(ctx.region_aabbs(), b2)
    np.testing.assert_array_equal(ctx.region_tree(), n2)
    # a second check splits nothing more (the halves were decayed below the threshold)
    assert ctx.split_regions() == n
    ctx.close()


def test_split_regions_stops_at_capacity(cuda, pkg, abi, oracle):
    st, ex, boxes, nodes, leaf = split_fixture(oracle, abi, split_count=3, seed=4)
    R = st.shape[0]
    ctx = pkg.FitContext(abi.default_fit_config(), max_regions=R + 1)
    ctx.set_regions(3, SCENE)
    ctx.set_states(st)
    ctx.set_region_split(abi.default_region_split_config())
    assert ctx.split_regions() == R + 1
    s2, _, b2, n2, _, _ = oracle.split_regions(R + 1, 10000.0, st, None, boxes, nodes, leaf, 2 * R - 1)
    assert ctx.states(R + 1).tobytes() == s2.tobytes()
    np.testing.assert_array_equal(ctx.region_tree(), n2)
    ctx.close()


def records_in_boxes(workloads, boxes, seed, median):
    rng = np.random.default_rng(seed)
    R = boxes.shape[0]
    counts = workloads.region_counts_lognormal(rng, R, median, 0.5, 50, 20000)
    w = workloads.mixture_samples(rng, counts, 1, 4, 3.0, 600.0, 1.0, region_boxes=boxes.astype(np.float64),
                                  dist_range=(0.05, 30.0), miss_frac=0.1)
    rec = w["records"][rng.permutation(int(counts.sum()))]
    rec["flags"][rng.random(rec.shape[0]) < 0.1] = 0xFFFFFFFF
    return rec


def test_update_with_region_splits_matches_oracle(cuda, pkg, abi, oracle, workloads):
    """Three update passes with region splitting on: the region count, tree,
    boxes and sample counts exact, mixtures to the fit tolerance."""
    torch = cuda
    cfg = abi.default_fit_config(num_initial_components=8)
    cap, thr = 64, 2500.0
    ctx = pkg.FitContext(cfg, max_regions=cap)
    ctx.set_regions(2, SCENE)
    ctx.set_region_split(abi.default_region_split_config(samples_for_region_split=thr))
    want = ctx.states(4)
    boxes = ctx.region_aabbs()
    nodes, leaf = oracle.complete_tree(2)
    nn = 7
    grew = False
    for p in range(3):
        rec = records_in_boxes(workloads, boxes, seed=70 + p, median=2000)
        R = boxes.shape[0]
        vmm = torch.zeros(cap * 720, dtype=torch.uint8, device="cuda")
        ctx.update(dev(torch, rec), rec.shape[0], vmm)
        ctx.sync()
        want, _ = oracle_update(oracle, abi, cfg, rec, boxes, want, first=(p == 0))
        want, _, boxes, nodes, leaf, nn = oracle.split_regions(cap, thr, want, None, boxes, nodes, leaf, nn)
        n = ctx.region_count()
        assert n == want.shape[0], f"pass {p}: {n} regions vs {want.shape[0]}"
        grew |= n > R
        np.testing.assert_array_equal(ctx.region_tree(), nodes)
        np.testing.assert_array_equal(ctx.region_aabbs(), boxes)
        got = ctx.states(n)
        np.testing.assert_array_equal(got["num_samples"], want["num_samples"])
        np.testing.assert_array_equal(got["total_num_samples"], want["total_num_samples"])
        fitted = want["iters_last"] > 0
        assert_params_close(got, want, 8, GPU_TOL, fitted)
        v = np.frombuffer(vmm.cpu().numpy()[: n * 720].tobytes(), dtype=abi.VMM_THETA_DTYPE)
        np.testing.assert_array_equal(v["used_distributions"], got["k"].astype(np.int32))
    assert grew
    ctx.close()


def test_tracer_finds_split_regions(cuda, pkg, abi, tracer):
    """After region splits the tracer descends the node array: every recorded
    sample carries the region the oracle's descent finds for its position, and
    a guided render keeps same-seed parity with the FP64 renderer."""
    torch = cuda
    sc = pkg.Scene.cornell(48, 32, ico_level=4)
    i = sc.info()
    P = i.camera.width * i.camera.height
    ctx = pkg.FitContext(abi.default_fit_config(), max_regions=512)
    ctx.set_regions(4, np.array(i.aabb, dtype=np.float32))
    ctx.set_region_split(abi.default_region_split_config(samples_for_region_split=200.0))
    rec = torch.zeros(P * 16 * 40, dtype=torch.uint8, device="cuda")
    for p in range(2):
        render_gpu(torch, sc, abi.render_params(spp=8, max_depth=8, seed=1 + p, record_samples=1,
                                                use_guiding=1 if p else 0), guide=ctx, records=rec)
        ctx.update(rec, P * 16)
    ctx.sync()
    n = ctx.region_count()
    assert n > 16
    nodes = ctx.region_tree()
    boxes = ctx.region_aabbs()
    root = np.concatenate([boxes[:, :3].min(0), boxes[:, 3:].max(0)]).astype(np.float32)
    render_gpu(torch, sc, abi.render_params(spp=2, max_depth=8, seed=9, record_samples=1, use_guiding=1),
               guide=ctx, records=rec)
    from oracle.oracle import Oracle
    r = host(rec, np.dtype([("position", "<f4", (3,)), ("direction", "<f4", (3,)), ("weight", "<f4"),
                            ("pdf", "<f4"), ("distance", "<f4"), ("flags", "<u4")]))
    v = r[r["flags"] != 0xFFFFFFFF]
    assert v.shape[0] > 1000
    sel = v[:: max(1, v.shape[0] // 3000)]
    want = Oracle().region_of(root, nodes, sel["position"])
    np.testing.assert_array_equal(sel["flags"], want)
    # same-seed guided render against the FP64 renderer descending the same tree
    vmm = torch.zeros(n * 720, dtype=torch.uint8, device="cuda")
    ctx.pack_vmm_theta(n, vmm)
    torch.cuda.synchronize()
    guide = {"vmm": vmm.cpu().numpy(), "root": root, "split_count": 0, "nodes": nodes,
             "use_parallax": int(abi.default_fit_config().use_parallax)}
    params = abi.render_params(spp=4, max_depth=8, seed=17, use_guiding=1, guiding_prob=0.5)
    got, _ = render_gpu(torch, sc, params, guide=ctx)
    want_img = tracer.render(sc.export(), params, guide=guide)
    assert_same_seed_parity(got, want_img, "guided cornell, split regions")
    ctx.close()
