"""The GPU irradiance cache against the reference's own cache functions
(compiled as C++ into tests/golden/ic_ref.npz by
tests/golden/make_ic_golden.py) and the numpy restatement
(oracle/ic_oracle.py):

  * queries (pg_ic_query): the found flag exactly, the value within FP32
    rounding, with and without gradients and the visibility test;
  * calculateCacheData (pg_ic_compute): the mean colour, harmonic distance
    and gradients of 4096 runs per point within 5 standard errors of the
    reference's 1024, with an empty cache and with a cache the paths query;
  * the estimator with a fixed cache (PG_RENDER_IRRADIANCE_CACHE |
    PG_RENDER_IC_FROZEN): block means of 8 parts within 6 standard
    deviations, image means within 1 %;
  * a cache grown while rendering: entries exactly what pg_ic_compute makes
    for the request's stream, updates exactly the restated running mean in
    round robin, and two renders from the same start give the same cache
    bit for bit.
"""
from __future__ import annotations

import numpy as np
import pytest

import ic_scenes as S
from conftest import GOLDEN
from oracle import ic_oracle
from test_trace_gpu import render_gpu

pytestmark = pytest.mark.gpu
FLAGS = [(g, v) for g in (0, 1) for v in (0, 1)]


@pytest.fixture(scope="module")
def fixture():
    return np.load(GOLDEN / "ic_ref.npz")


def _compare_fields(got, want, rtol, atol, what):
    for name in ic_oracle.ENTRY_FIELDS:
        a, b = np.asarray(got[name], np.float64), np.asarray(want[name], np.float64)
        assert np.allclose(a, b, rtol=rtol, atol=atol), f"{what}: {name} {a} vs {b}"


@pytest.mark.parametrize("grads,vis", FLAGS)
def test_query_matches_reference(grads, vis, fixture, cuda, pkg, abi):
    sc = S.cornell()
    e = fixture["query__entries"]
    # the entries lie in [-1, 1]^3, the grid spans the scene box [0, 1]^3: points outside it use the border cells
    sc.set_irradiance_cache(capacity=S.IC_CAPACITY, a=S.IC_A, use_gradients=grads, visibility_check=vis,
                            create_prob=0.0, update_prob=0.0)
    sc.set_irradiance_cache_entries(e)
    rgb, found = sc.ic_query(fixture["query__pos"], fixture["query__nrm"])
    want_f = fixture[f"query__found_g{grads}_v{vis}"].astype(bool)
    want = fixture[f"query__rgb_g{grads}_v{vis}"]
    assert np.array_equal(found.astype(bool), want_f), f"{(found.astype(bool) != want_f).sum()} found flags differ"
    err = np.abs(rgb - want) / np.maximum(np.abs(want), 1e-3)
    assert err.max() < 2e-5, err.max()
    sc.close()


def _gpu_compute(sc, abi, points, normals, runs, seed=1):
    req = np.zeros(len(points) * runs, dtype=abi.IC_REQUEST_DTYPE)
    req["position"] = np.repeat(points, runs, axis=0)
    req["normal"] = np.repeat(normals, runs, axis=0)
    req["pixel"] = np.tile(np.arange(runs, dtype=np.uint32), len(points))
    req["bounce"] = 0
    req["pass"] = np.repeat(np.arange(len(points), dtype=np.uint32), runs)
    params = abi.render_params(spp=1, max_depth=S.PATH_LENGTH, seed=seed, use_nee=1, use_mis=1)
    return sc.ic_compute(params, req).reshape(len(points), runs)


@pytest.mark.parametrize("cache", ["empty", "cache", "empty_nee3"])
def test_compute_matches_reference(cache, fixture, cuda, pkg, abi):
    """calculateCacheData: the GPU's entries against the reference's over many
    runs (empty_nee3: three light samples per vertex, irradianceNumNEE 3)."""
    sc = S.cornell()
    sc.set_irradiance_cache(capacity=S.IC_CAPACITY, a=S.IC_A, create_prob=0.0, update_prob=0.0,
                            num_nee=3 if cache == "empty_nee3" else 1)
    if cache == "cache":
        sc.set_irradiance_cache_entries(fixture["render__entries"])
    runs = 4096
    got = _gpu_compute(sc, abi, fixture["compute_points"], fixture["compute_normals"], runs)
    ref = fixture[f"compute__{cache}"]  # (points, runs, 10)
    g = np.concatenate([got["color"], got["rot_grad"], got["trans_grad"], got["harmonic_r"][..., None]], axis=-1)
    gm, gs = g.mean(1), g.std(1, ddof=1) / np.sqrt(runs)
    rm, rs = ref.mean(1), ref.std(1, ddof=1) / np.sqrt(ref.shape[1])
    z = np.abs(gm - rm) / np.sqrt(gs ** 2 + rs ** 2 + 1e-12)
    names = ["r", "g", "b", "rot_x", "rot_y", "rot_z", "trans_x", "trans_y", "trans_z", "harmonic_r"]
    worst = np.unravel_index(np.argmax(z), z.shape)
    assert z.max() < 5.0, (f"point {worst[0]} {names[worst[1]]}: |z| {z.max():.2f} "
                           f"(gpu {gm[worst]:.5f} ref {rm[worst]:.5f})")
    # every hemisphere of the box's walls sees something
    assert (got["num_updates"] == 1).all() and (got["harmonic_r"] > 0).all()
    sc.close()


def test_frozen_cache_render_matches_reference(fixture, cuda, pkg, abi):
    import estimator_scenes as E
    torch = cuda
    sc = S.cornell()
    sc.set_irradiance_cache(capacity=S.IC_CAPACITY, a=S.IC_A, create_prob=0.0, update_prob=0.0)
    sc.set_irradiance_cache_entries(fixture["render__entries"])
    parts = []
    for p in range(S.PARTS):
        params = abi.render_params(spp=S.SPP, max_depth=S.PATH_LENGTH, seed=2000 + p, use_nee=1, use_mis=1,
                                   flags=abi.PG_RENDER_IRRADIANCE_CACHE | abi.PG_RENDER_IC_FROZEN)
        img, _ = render_gpu(torch, sc, params)
        parts.append(S.blocks(img / S.SPP))
    z, ratio, ok = E.compare_blocks(fixture["render__blocks"], np.stack(parts))
    assert ok, f"block |z| {z:.2f}, mean ratio {ratio:.4f}"
    # the cache is unchanged by a frozen render
    assert len(sc.irradiance_cache()) == len(fixture["render__entries"])
    sc.close()


def _one_pixel_camera(sc, abi, origin, target):
    cam = sc.info().camera
    cam.width, cam.height = 1, 1
    cam.origin[:] = origin
    cam.target[:] = target
    cam.vfov_deg = 0.01  # the pixel jitter spans the whole view of a one-pixel image
    sc.set_camera(cam)


def test_created_entry_is_the_computed_one(cuda, pkg, abi):
    """One pixel, paths of two segments: the only vertex that can ask for an
    entry is the camera's hit (bounce 0); the entry the pass writes is what
    pg_ic_compute makes for that request's stream."""
    torch = cuda
    sc = S.cornell()
    _one_pixel_camera(sc, abi, [0.5, 0.5, 2.35], [0.2, 0.0, 0.8])  # the floor
    sc.set_irradiance_cache(capacity=64, a=0.2, create_prob=1.0, update_prob=0.0)
    params = abi.render_params(spp=1, max_depth=2, seed=77, use_nee=1, use_mis=1,
                               flags=abi.PG_RENDER_IRRADIANCE_CACHE)
    render_gpu(torch, sc, params)
    got = sc.irradiance_cache()
    assert len(got) == 1
    req = np.zeros(1, dtype=abi.IC_REQUEST_DTYPE)
    req["position"], req["normal"] = got["center"], got["normal"]
    req["pixel"], req["bounce"], req["pass"] = 0, 0, 0
    # computed against the cache the pass saw: an empty one
    sc2 = S.cornell()
    sc2.set_irradiance_cache(capacity=64, a=0.2, create_prob=1.0, update_prob=0.0)
    want = sc2.ic_compute(params, req)
    sc2.close()
    _compare_fields(got, want, 0.0, 0.0, "created entry")
    assert abs(got["normal"][0][1] - 1.0) < 1e-6 and abs(got["center"][0][1]) < 1e-5  # on the floor, facing up
    sc.close()


def test_updates_follow_the_running_mean_in_round_robin(cuda, pkg, abi, tmp_path):
    """Inside the closed sphere every update computes colour 0, zero gradients
    and harmonic distance 2; one update per pass (one pixel, update_prob 1)
    walks the three entries in round robin, skipping a pass at the reset."""
    torch = cuda
    sc = S.sphere_scene(tmp_path)
    sc.set_irradiance_cache(capacity=8, a=0.2, min_radius=0.1, gradients_max_length=5.0, create_prob=0.0,
                            update_prob=1.0)
    old = S.sphere_entries()
    sc.set_irradiance_cache_entries(old)
    passes = 6
    params = abi.render_params(spp=passes, max_depth=3, seed=5, use_nee=1, use_mis=1,
                               flags=abi.PG_RENDER_IRRADIANCE_CACHE)
    render_gpu(torch, sc, params)
    got = sc.irradiance_cache()
    targets, _ = ic_oracle.update_targets(passes, 0, 3)
    assert targets == [0, 1, 2, -1, 0, 1]
    want = old.copy()
    for t in targets:
        if t >= 0:
            want[t] = ic_oracle.updated_entry(want[t], np.zeros(3), np.zeros(3), np.zeros(3), 2.0, 0.2, 0.1, 5.0)
    _compare_fields(got, want, 2e-6, 1e-7, "updated entries")
    sc.close()


def test_grown_cache_is_repeatable_and_well_formed(cuda, pkg, abi):
    torch = cuda
    caches = []
    for _ in range(2):
        sc = S.cornell()
        sc.set_irradiance_cache(capacity=2000, a=0.3, create_prob=0.02, update_prob=0.01)
        params = abi.render_params(spp=32, max_depth=8, seed=3, use_nee=1, use_mis=1,
                                   flags=abi.PG_RENDER_IRRADIANCE_CACHE)
        img, _ = render_gpu(torch, sc, params)
        assert np.isfinite(img).all() and img.mean() > 0
        caches.append(sc.irradiance_cache())
        sc.close()
    a, b = caches
    assert 50 < len(a) <= 2000
    assert a.tobytes() == b.tobytes()
    box = (a["center"] >= -1e-4).all() and (a["center"] <= 1 + 1e-4).all()
    assert box
    assert (a["num_updates"] >= 1).all()
    hr = np.maximum(a["harmonic_r"], 0.1)
    assert np.allclose(a["harmonic_r"], hr) and np.allclose(a["radius"], np.float32(0.3) * a["harmonic_r"])
    assert np.allclose(np.linalg.norm(a["normal"], axis=1), 1.0, atol=1e-5)
    assert (np.linalg.norm(a["rot_grad"], axis=1) <= 5.0 + 1e-4).all()
    assert (np.linalg.norm(a["trans_grad"], axis=1) <= 5.0 + 1e-4).all()
    assert (a["num_updates"] > 1).any()  # some entries were updated


def _adrrs_setup(torch, fixture, abi, split, s=S.ADRRS_S):
    """The Cornell box of the estimator comparison with the reference-made
    cache and the fixture's pixel estimate (the reference's plain estimator)."""
    sc = S.cornell()
    sc.set_irradiance_cache(capacity=S.IC_CAPACITY, a=S.IC_A, create_prob=0.0, update_prob=0.0)
    sc.set_irradiance_cache_entries(fixture["render__entries"])
    est = torch.from_numpy(np.ascontiguousarray(fixture["adrrs__estimate"], dtype=np.float32).reshape(-1)).cuda()
    sc.set_adrrs(est, s=s, split=bool(split))
    return sc, est


@pytest.mark.parametrize("split", [0, 1])
def test_adrrs_render_converges_to_reference_adrrs(split, fixture, cuda, pkg, abi):
    """The ADRRS image converges to the reference's own estimator with ADRRS
    (its weight windows, roulette and split paths, in the fixture) - with
    splitting also to the plain estimator, since roulette and splitting then
    change only the noise.  Without splitting the reference's rule is biased:
    a path the window would split in two keeps its whole throughput while one
    kept single is divided by q (raytrace.rgen:1094-1101); the library keeps
    that rule."""
    torch = cuda
    sc, est = _adrrs_setup(torch, fixture, abi, split)
    parts = []
    for p in range(S.PARTS):
        params = abi.render_params(spp=S.SPP, max_depth=S.PATH_LENGTH, seed=3000 + p, use_nee=1, use_mis=1,
                                   flags=abi.PG_RENDER_ADRRS)
        img, _ = render_gpu(torch, sc, params)
        parts.append(S.blocks(img / S.SPP))
    got = np.stack(parts)
    import estimator_scenes as E
    z, ratio, ok = E.compare_blocks(fixture[f"adrrs__blocks_split{split}"], got)
    assert ok, f"split {split}: block |z| {z:.2f}, mean ratio {ratio:.4f} against the reference's ADRRS"
    if split:
        plain = np.load(GOLDEN / "estimator_ref.npz")["cornell_mis__blocks"]
        z, ratio, ok = E.compare_blocks(plain, got)
        assert ok, f"block |z| {z:.2f}, mean ratio {ratio:.4f} against the plain estimator"
    sc.close()


def test_adrrs_roulette_and_splitting_change_the_work(fixture, cuda, pkg, abi):
    torch = cuda
    rays = {}
    for name, flags, split, s in (("plain", 0, 0, 1.5), ("rr", abi.PG_RENDER_ADRRS, 0, 1.5),
                                  ("split", abi.PG_RENDER_ADRRS, 1, 1.5)):
        sc, est = _adrrs_setup(torch, fixture, abi, split, s)
        params = abi.render_params(spp=64, max_depth=S.PATH_LENGTH, seed=7, use_nee=1, use_mis=1, flags=flags)
        _, st = render_gpu(torch, sc, params)
        rays[name] = st.extension_rays
        sc.close()
    # with a narrow window roulette ends paths early, and splitting adds copies to the same decisions
    assert rays["rr"] < 0.95 * rays["plain"], rays
    assert rays["split"] > rays["rr"], rays


def test_adrrs_rejects_missing_estimate_and_recording_with_splits(cuda, pkg, abi):
    torch = cuda
    sc = S.cornell()
    sc.set_irradiance_cache(capacity=16, create_prob=0.0, update_prob=0.0)
    img = torch.zeros(S.W * S.H * 3, dtype=torch.float32, device="cuda")
    with pytest.raises(pkg.PathGuideError):
        sc.render(abi.render_params(spp=1, max_depth=4, flags=abi.PG_RENDER_ADRRS), img)
    est = torch.ones(S.W * S.H * 3, dtype=torch.float32, device="cuda")
    sc.set_adrrs(est, s=5.0, split=True)
    rec = torch.zeros(S.W * S.H * 16 * 10, dtype=torch.float32, device="cuda")
    ctx = pkg.FitContext(abi.default_fit_config(), max_regions=8)
    ctx.set_regions(2, np.array(sc.info().aabb, dtype=np.float32))
    with pytest.raises(pkg.PathGuideError):
        sc.render(abi.render_params(spp=1, max_depth=4, record_samples=1, flags=abi.PG_RENDER_ADRRS), img,
                  guide=ctx, records_dev=rec)
    ctx.close()
    sc.close()
