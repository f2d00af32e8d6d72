"""The split/merge fixtures (tests/golden/splitmerge_*.npz) against the
reference's PathGuiding::postFit restated around its own lightpmm classes
(oracle/lightpmm_harness.cpp, lpmm_ref_postfit), and their invariants.

The fixtures are regenerated bit for bit where the reference harness is built
(x86 with the reference tree); the invariants hold everywhere.
"""
from __future__ import annotations

import numpy as np
import pytest

SETS = ["splitmerge_default", "splitmerge_eager"]


def sm_from(abi, v):
    return abi.SplitMergeConfig(int(v[0]), int(v[1]), int(v[2]), int(v[3]), float(v[4]), float(v[5]))


@pytest.mark.parametrize("name", SETS)
def test_fixture_invariants(name, golden, abi):
    g = golden(name)
    sm = sm_from(abi, g["sm"])
    since = np.zeros(len(g["offsets0"]) - 1)
    changed = 0
    for p in range(int(g["passes"])):
        st, ex, fitted = g[f"states{p}"], g[f"extras{p}"], g[f"fitted{p}"]
        counts = np.diff(g[f"offsets{p}"].astype(np.int64))
        K = st["k"].astype(np.int64)
        assert np.all((K >= 1) & (K <= 16))
        for r in range(K.shape[0]):
            w = st["weight"][r]
            assert np.isfinite(w).all() and abs(w[:K[r]].sum() - 1.0) < 1e-4
            assert np.all(w[K[r]:] == 0.0)
            mu = np.stack([st["mu_x"][r, :K[r]], st["mu_y"][r, :K[r]], st["mu_z"][r, :K[r]]], -1)
            np.testing.assert_allclose(np.linalg.norm(mu, axis=-1), 1.0, atol=1e-4)
        # samplesSinceLastMerge counts samples and resets when the merge ran
        since = np.where(counts > 0, since + counts, since)
        merged = since > sm.min_samples_for_merging
        since[merged] = 0
        np.testing.assert_array_equal(ex["samples_since_merge"], since.astype(np.float32))
        changed += int(np.sum(st["k"] != fitted["k"]))
        # regions without samples are untouched
        empty = counts == 0
        assert st[empty].tobytes() == fitted[empty].tobytes()
    assert changed > 0  # the sequences do split and merge


@pytest.mark.parametrize("name", SETS)
def test_reference_postfit_reproduces_fixture(name, golden, abi):
    from oracle.oracle import ReferenceFit
    if not ReferenceFit.available():
        pytest.skip("reference harness not built on this machine")
    from test_oracle import cfg_from
    g = golden(name)
    ref = ReferenceFit()
    cfg, sm = cfg_from(abi, g["cfg"]), sm_from(abi, g["sm"])
    for p in range(int(g["passes"])):
        st, ex = ref.postfit(cfg, sm, g[f"dirw{p}"], g[f"pdf{p}"], None, g[f"offsets{p}"], g[f"fitted{p}"],
                             g[f"extras_in{p}"])
        assert st.tobytes() == g[f"states{p}"].tobytes(), p
        assert ex.tobytes() == g[f"extras{p}"].tobytes(), p


def test_disabled_postfit_leaves_mixture(golden, abi):
    from oracle.oracle import ReferenceFit
    if not ReferenceFit.available():
        pytest.skip("reference harness not built on this machine")
    from test_oracle import cfg_from
    g = golden("splitmerge_eager")
    ref = ReferenceFit()
    sm = abi.default_split_merge_config(enabled=0)
    st, ex = ref.postfit(cfg_from(abi, g["cfg"]), sm, g["dirw1"], g["pdf1"], None, g["offsets1"], g["fitted1"],
                         g["extras_in1"])
    assert st.tobytes() == g["fitted1"].tobytes()


def test_update_fixture_invariants(golden):
    g = golden("splitmerge_update")
    R = 1 << int(g["split_count"])
    seen = set()
    for p in range(int(g["passes"])):
        st, ex = g[f"states{p}"], g[f"extras{p}"]
        assert st.shape[0] == R and ex.shape[0] == R
        ids = g[f"records{p}"]["flags"]
        busy = np.isin(np.arange(R), ids[ids < R])
        for r in range(R):
            k = int(st["k"][r])
            seen.add(k)
            assert 1 <= k <= 16 and abs(st["weight"][r, :k].sum() - 1.0) < 1e-4
            if not busy[r]:
                assert st["total_num_samples"][r] == 0
    assert seen - {8}  # components were split or merged
