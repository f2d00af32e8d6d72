"""The reference's own lightpmm fit on hosts where its vectorclass back end
cannot build (oracle/build_oracle.py, oracle/vcl_shim/).

On x86-64 with the reference tree both builds exist: the one with the
reference's vectorclass (SSE) and the one with the project's portable
stand-in, compiled from the staged copies of the reference's headers as the
Arm host compiles them.  They must fit identically; the region-parallel entry
point must equal the serial one."""
from __future__ import annotations

import numpy as np
import pytest


def _fitters():
    from oracle import build_oracle
    if build_oracle.build_reference() is None:
        pytest.skip("no reference lightpmm build on this host")
    from oracle.oracle import ReferenceFit
    port = build_oracle.HERE / "_ref" / "liblightpmm_ref_portable.so"
    if not port.exists():
        pytest.skip("only one reference build on this host")
    return ReferenceFit(), ReferenceFit(port)


FIELDS = ("weight", "mu_x", "mu_y", "mu_z", "kappa", "r", "iters_last", "total_num_samples")


@pytest.mark.parametrize("K,iters,converge", [(8, 20, False), (16, 10, False), (8, 100, True)])
def test_portable_build_fits_as_the_vectorclass_build(K, iters, converge, abi, workloads):
    sse, portable = _fitters()
    w = workloads.fit_batched(seed=11, n_regions=48, median=900, sigma=1.0, lo=64, hi=6000)
    cfg = abi.default_fit_config(num_initial_components=K, max_itr=iters) if converge else \
        abi.forced_iterations(iters, num_initial_components=K)
    a, _ = sse.fit(cfg, w["dirw"], w["offsets"])
    b, _ = portable.fit(cfg, w["dirw"], w["offsets"])
    for f in FIELDS:
        assert np.array_equal(a[f][..., :K] if a[f].ndim > 1 else a[f], b[f][..., :K] if b[f].ndim > 1 else b[f]), f


def test_region_parallel_fit_equals_serial(abi, workloads):
    sse, _ = _fitters()
    w = workloads.fit_batched(seed=12, n_regions=40, median=700, sigma=1.0, lo=64, hi=5000)
    cfg = abi.forced_iterations(10, num_initial_components=8)
    a, _ = sse.fit(cfg, w["dirw"], w["offsets"])
    b, _ = sse.fit(cfg, w["dirw"], w["offsets"], threads=4)
    for f in FIELDS:
        assert np.array_equal(a[f], b[f]), f
