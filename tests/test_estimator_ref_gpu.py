"""The GPU path tracer converges to the reference's own estimator
(raytrace(), nextEventEstimation(), sampleLights(), getNewDirection() and the
hit / miss shaders of shaders/raytrace*.r*, compiled as host C++ and rendered
on the CPU into tests/golden/estimator_ref.npz by
tests/golden/make_estimator_golden.py).

The two estimators pair next-event estimation with BSDF sampling differently
(the reference traces an extra BSDF ray inside nextEventEstimation,
raytrace.rgen:665-729; the library weights the continuation ray) and draw
different random numbers, so they are compared in expectation: 8 parts of
2048 samples per pixel on each side, 4 x 4 block means within 6 standard
deviations of the parts' spread and image means within 1 %.  Cases: the
Cornell box with its glass sphere (NEE + MIS, BSDF sampling only), the
Phong / conductor / Beckmann / mirror scene (NEE + MIS, NEE only, with an
environment map), and the Cornell box guided by fixed region mixtures with
the reference's rule (every non-discrete material guided).
"""
from __future__ import annotations

import numpy as np
import pytest

import estimator_scenes as E
from conftest import GOLDEN
from test_trace_gpu import render_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fixture():
    return np.load(GOLDEN / "estimator_ref.npz")


@pytest.mark.parametrize("case", sorted(E.CASES))
def test_gpu_converges_to_reference_estimator(case, fixture, cuda, pkg, abi):
    torch = cuda
    scene, nee, mis, guided = E.CASES[case]
    sc = E.make_scene(scene)
    ctx = None
    flags = 0
    if guided:
        ctx = pkg.FitContext(abi.default_fit_config(use_parallax=1), max_regions=1 << E.GUIDE_SPLITS)
        ctx.set_regions(E.GUIDE_SPLITS, np.array(sc.info().aabb, dtype=np.float32))
        ctx.set_states(fixture[f"{case}__states"])
        flags = abi.PG_RENDER_GUIDE_ALMOST_DISCRETE
    parts = []
    for p in range(E.PARTS):
        params = abi.render_params(spp=E.SPP, max_depth=E.PATH_LENGTH, seed=1000 + p, use_nee=nee, use_mis=mis,
                                   use_guiding=int(guided), guiding_prob=0.5, flags=flags)
        img, _ = render_gpu(torch, sc, params, guide=ctx)
        parts.append(E.blocks(img.reshape(E.H, E.W, 3) / E.SPP))
    z, ratio, ok = E.compare_blocks(fixture[f"{case}__blocks"], np.stack(parts))
    if ctx is not None:
        ctx.close()
    sc.close()
    assert ok, f"{case}: block |z| {z:.2f}, mean ratio {ratio:.4f}"
