"""The GPU renderer's own shading and recording functions (the device
functions k_shade and k_shadow call, run through pg_probe_shading /
pg_probe_records) against the reference's shader functions compiled as host
C++ (tests/golden/shader_ref.npz; tests/golden/make_shader_golden.py):

* evalBsdf / pdfBSDF, sampleBSDF, fresnel, fresnelConductor
  (raytrace.rgen:145-332, 483-599);
* VMM and sampleVMM (guiding.glsl:32-96), with and without parallax;
* getNewDirection and the throughput change evalBsdf / pdf
  (raytrace.rgen:923-960, 1176), guided and unguided, with the reference's
  rule of guiding every non-discrete material;
* toWorld (transform.glsl:7-38);
* updateSamples / commitSamples over recorded paths (raytrace.rgen:973-990).

Each case replays the random numbers the reference function drew.  The
comparison rules and tolerances are in tests/shader_cmp.py.
"""
from __future__ import annotations

import numpy as np
import pytest

from shader_cmp import compare, compare_records

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fixture():
    return np.load(GOLDEN / "shader_ref.npz")


def test_gpu_shading_functions_match_reference(cuda, pkg, fixture):
    got = pkg.probe_shading(fixture["mats"], fixture["vmms"], fixture["probes"]).astype(np.float64)
    report, failures = compare(fixture, got)
    assert not failures, "\n".join(failures[:20])
    for name in ("fresnel", "eval", "sample_dir", "vmm_pdf", "vmm_sample", "continue_dir", "continue_tc"):
        assert report[name][0] > 100, name


def test_gpu_probe_rejects_bad_indices(cuda, pkg, abi, fixture):
    p = fixture["probes"][:4].copy()
    p["op"] = abi.PG_PROBE_BSDF_EVAL
    p["material"] = [0, 99, 0, 0]
    got = pkg.probe_shading(fixture["mats"], fixture["vmms"], p)
    assert np.isnan(got[1]).all() and np.isfinite(got[[0, 2, 3]]).all()


def test_gpu_sample_recording_matches_reference(cuda, pkg, fixture):
    w, f, c = pkg.probe_records(fixture["rec_events"], fixture["rec_offsets"])
    worst, failures = compare_records(fixture, w, f, c)
    assert not failures, "\n".join(failures[:10])
    assert c.sum() > 500
