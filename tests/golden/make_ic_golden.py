"""Generates tests/golden/ic_ref.npz: the reference's own irradiance-cache
functions - queryIrradianceCache with the cache's intersection and any-hit
shaders, calculateCacheData, createIrradianceCache and raytrace() with the
cache (shaders/raytrace.rgen, shaders/raytrace.irradiance.r*) compiled as host
C++ by oracle/build_glsl_ref.py - on seeded inputs, for the GPU cache to match
(tests/test_icache_gpu.py) and the numpy restatement to be pinned against
(tests/test_icache.py).

  * query__*: 200 random entries, 4000 random points and normals; the
    reference's colour and found flag with and without gradients and the
    visibility test;
  * compute__*: calculateCacheData at six surface points of the Cornell box,
    COMPUTE_RUNS runs each (random states 1..), with an empty cache and with
    the cache of render__entries, and with an empty cache and three light
    samples per vertex (irradianceNumNEE 3, compute__empty_nee3);
  * render__*: a cache of entries createIrradianceCache made at surface
    points the camera sees and their next bounce, and the reference's
    estimator querying it (no entries made while rendering): PARTS parts of
    SPP samples per pixel as 4 x 4 block means;
  * adrrs__*: the reference's estimator with ADRRS over that cache (its
    weight windows, roulette and split paths as main() runs them), against
    an estimate the plain estimator rendered, with and without splitting.

Run from the repository root:

    python tests/golden/make_ic_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import __graft_entry__ as entry  # noqa: E402

pkg = entry.load_package()
abi = pkg.abi

from oracle import build_glsl_ref  # noqa: E402
from oracle.glsl_ref import GlslRef, ic_config  # noqa: E402
from ic_scenes import (ADRRS_S, COMPUTE_POINTS, COMPUTE_RUNS, ESTIMATE_SPP, IC_A, IC_CAPACITY, PATH_LENGTH,  # noqa: E402
                       PARTS, SPP, blocks, query_case, surface_points, cornell)

OUT = Path(__file__).resolve().parent / "ic_ref.npz"


def main(out: Path = OUT):
    build_glsl_ref.build_glsl_ref()
    g = GlslRef()
    arrays = {}
    # function-level queries
    entries, pos, nrm = query_case()
    arrays["query__entries"], arrays["query__pos"], arrays["query__nrm"] = entries, pos, nrm
    for grads in (0, 1):
        for vis in (0, 1):
            g.ic_set(entries, ic_config(IC_CAPACITY, a=IC_A, use_gradients=grads, visibility_check=vis))
            rgb, found = g.ic_query(pos, nrm)
            arrays[f"query__rgb_g{grads}_v{vis}"] = rgb
            arrays[f"query__found_g{grads}_v{vis}"] = found
    # a cache made by createIrradianceCache at points the camera and one bounce see
    sc = cornell()
    exp = sc.export()
    sp, sn = surface_points(exp, 400, seed=11)
    g.ic_set(np.zeros(0, dtype=abi.IC_ENTRY_DTYPE), ic_config(IC_CAPACITY, a=IC_A))
    for i in range(len(sp)):
        g.ic_create_update(exp, sp[i], sn[i], updates=0, seed=1 + i)
    cache, _ = g.ic_get(abi.IC_ENTRY_DTYPE)
    arrays["render__entries"] = cache
    print(f"cache: {len(cache)} entries of {len(sp)} requests")
    # calculateCacheData at fixed points, empty cache and that cache
    cp = np.array([p for p, _ in COMPUTE_POINTS], dtype=np.float32)
    cn = np.array([n for _, n in COMPUTE_POINTS], dtype=np.float32)
    pos_r = np.repeat(cp, COMPUTE_RUNS, axis=0)
    nrm_r = np.repeat(cn, COMPUTE_RUNS, axis=0)
    seeds = np.tile(np.arange(1, COMPUTE_RUNS + 1, dtype=np.uint32), len(cp))
    empty = np.zeros(0, dtype=abi.IC_ENTRY_DTYPE)
    for name, ent, nee in (("empty", empty, 0), ("cache", cache, 0), ("empty_nee3", empty, 3)):
        g.ic_set(ent, ic_config(IC_CAPACITY, a=IC_A, num_nee=nee))
        res = g.ic_compute(exp, pos_r, nrm_r, seeds).reshape(len(cp), COMPUTE_RUNS, 10)
        arrays[f"compute__{name}"] = res
        print(name, np.round(res.mean(1)[:, [0, 1, 2, 9]], 4))
    # the estimator with that cache
    g.ic_set(cache, ic_config(IC_CAPACITY, a=IC_A))
    res = []
    for p in range(PARTS):
        img = g.render(exp, path_length=PATH_LENGTH, spp=SPP, frame_seed=p + 1, use_nee=True, use_mis=True,
                       use_ic=True) / SPP
        res.append(blocks(img).astype(np.float32))
    arrays["render__blocks"] = np.stack(res)
    b = arrays["render__blocks"]
    print(f"render: mean {b.mean():.5f}, part spread {b.mean(axis=(1, 2, 3)).std() / b.mean():.4f}")
    # ADRRS with that cache against an estimate of the plain estimator, with
    # and without splitting
    est = (g.render(exp, path_length=PATH_LENGTH, spp=ESTIMATE_SPP, frame_seed=777, use_nee=True, use_mis=True)
           / ESTIMATE_SPP).astype(np.float32)
    arrays["adrrs__estimate"] = est
    for split in (0, 1):
        res = []
        for p in range(PARTS):
            img = g.render(exp, path_length=PATH_LENGTH, spp=SPP, frame_seed=100 + p, use_nee=True, use_mis=True,
                           adrrs={"estimate": est, "s": ADRRS_S, "split": split}) / SPP
            res.append(blocks(img).astype(np.float32))
        arrays[f"adrrs__blocks_split{split}"] = np.stack(res)
        b = arrays[f"adrrs__blocks_split{split}"]
        print(f"adrrs split {split}: mean {b.mean():.5f}, part spread {b.mean(axis=(1, 2, 3)).std() / b.mean():.4f}")
    sc.close()
    np.savez_compressed(out, compute_points=cp, compute_normals=cn, **arrays)
    print(out)


if __name__ == "__main__":
    main()
