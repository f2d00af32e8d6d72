"""The irradiance cache's numpy restatement (oracle/ic_oracle.py) pinned
against the reference's own cache functions: the committed fixture of
queryIrradianceCache with the cache's intersection and any-hit shaders
(tests/golden/ic_ref.npz, made by tests/golden/make_ic_golden.py) and, where
the reference tree is present, the reference's functions compiled as C++
(oracle/build_glsl_ref.py) - queries, createIrradianceCache and
updateIrradianceCache's running mean and round-robin entry choice."""
from __future__ import annotations

import numpy as np
import pytest

import ic_scenes as S
from conftest import GOLDEN
from oracle import ic_oracle

FLAGS = [(g, v) for g in (0, 1) for v in (0, 1)]


@pytest.fixture(scope="module")
def fixture():
    return np.load(GOLDEN / "ic_ref.npz")


def _glslref():
    from oracle.glsl_ref import GlslRef, available
    if not available():
        pytest.skip("the reference's shader functions are not built here")
    return GlslRef()


@pytest.mark.parametrize("grads,vis", FLAGS)
def test_oracle_query_matches_fixture(fixture, grads, vis):
    rgb, found = ic_oracle.query(fixture["query__entries"], fixture["query__pos"], fixture["query__nrm"], S.IC_A,
                                 grads, vis)
    want_f = fixture[f"query__found_g{grads}_v{vis}"].astype(bool)
    want = fixture[f"query__rgb_g{grads}_v{vis}"]
    assert want_f.sum() > 200 and (~want_f).sum() > 200
    assert np.array_equal(found, want_f)
    err = np.abs(rgb - want) / np.maximum(np.abs(want), 1e-3)
    assert err.max() < 1e-5, err.max()


def test_oracle_query_matches_reference_functions():
    g = _glslref()
    from oracle.glsl_ref import ic_config
    e, p, q = S.query_case(n_entries=120, n_points=1500, seed=21)
    for grads, vis in FLAGS:
        g.ic_set(e, ic_config(S.IC_CAPACITY, a=S.IC_A, use_gradients=grads, visibility_check=vis))
        want, want_f = g.ic_query(p, q)
        rgb, found = ic_oracle.query(e, p, q, S.IC_A, grads, vis)
        assert np.array_equal(found, want_f.astype(bool))
        assert (np.abs(rgb - want) / np.maximum(np.abs(want), 1e-3)).max() < 1e-5


def test_oracle_commit_rules_match_reference(abi, tmp_path):
    """In the closed sphere, calculateCacheData at the centre returns colour 0,
    zero gradients and harmonic distance 2; the reference's
    updateIrradianceCache and createIrradianceCache then write exactly what
    the restated rules predict, and walk the entries in round robin."""
    g = _glslref()
    from oracle.glsl_ref import ic_config
    sc = S.sphere_scene(tmp_path)
    exp = sc.export()
    old = S.sphere_entries()
    cfg = ic_config(8, a=0.2, min_radius=0.1, gradients_max_length=5.0)
    g.ic_set(old, cfg)
    n_upd = 5
    made = g.ic_create_update(exp, np.zeros(3, np.float32), np.array([0, 0, 1], np.float32), updates=n_upd, seed=9)
    assert made == 1
    got, nxt = g.ic_get(abi.IC_ENTRY_DTYPE)
    # the new entry first (createIrradianceCache), then the updates in round robin over the four entries
    new = ic_oracle.new_entry(np.zeros(3), [0, 0, 1], np.zeros(3), np.zeros(3), np.zeros(3), 2.0, 0.2, 0.1, 5.0,
                              abi.IC_ENTRY_DTYPE)
    want = np.concatenate([old, new[None]])
    targets, want_next = ic_oracle.update_targets(n_upd, 0, 4)
    assert targets == [0, 1, 2, 3, -1] and nxt == want_next == 0
    for t in targets:
        if t >= 0:
            want[t] = ic_oracle.updated_entry(want[t], np.zeros(3), np.zeros(3), np.zeros(3), 2.0, 0.2, 0.1, 5.0)
    assert len(got) == 4
    for name in ic_oracle.ENTRY_FIELDS:
        a, b = got[name].astype(np.float64), want[name].astype(np.float64)
        assert np.allclose(a, b, rtol=2e-6, atol=1e-7), (name, a, b)
    # clamping took effect: the second entry's rotation gradient (length 10 * 5/6) was scaled to 5
    assert abs(np.linalg.norm(got["rot_grad"][1]) - 5.0) < 1e-5
    sc.close()


def test_update_targets_restatement():
    assert ic_oracle.update_targets(4, 1, 3) == ([1, 2, -1, 0], 1)
    assert ic_oracle.update_targets(3, 5, 3) == ([-1, 0, 1], 2)
    assert ic_oracle.update_targets(2, 0, 0) == ([-1, -1], 0)
