"""Region splitting (PathGuiding::update's split check and splitRegion,
src/PathGuiding.cpp:290-348) in the oracle: the region tree, its lookup and
the split semantics the GPU is checked against."""
from __future__ import annotations

import numpy as np


SCENE = np.array([-1.0, -0.5, -2.0, 3.0, 1.5, 2.0], dtype=np.float32)


def root_box(oracle):
    b = oracle.region_aabbs(0, SCENE)
    return b[0]


def test_complete_tree_lookup_matches_region_boxes(oracle):
    for split_count in (0, 1, 4, 7):
        boxes = oracle.region_aabbs(split_count, SCENE)
        nodes, _ = oracle.complete_tree(split_count)
        rng = np.random.default_rng(split_count)
        pts = root_box(oracle)[:3] + rng.random((400, 3)) * (root_box(oracle)[3:] - root_box(oracle)[:3])
        pts = pts.astype(np.float32)
        ids = oracle.region_of(root_box(oracle), nodes, pts)
        ok = ids != 0xFFFFFFFF
        assert ok.mean() > 0.99
        b = boxes[ids[ok]]
        assert ((pts[ok] >= b[:, :3]) & (pts[ok] <= b[:, 3:])).all()


def split_fixture(oracle, abi, split_count=3, seed=0):
    R = 1 << split_count
    rng = np.random.default_rng(seed)
    st = oracle.init_states(abi.default_fit_config(), R)
    st["num_samples"] = rng.choice([500.0, 9000.0, 10000.0, 12000.0, 40000.0], size=R).astype(np.float32)
    st["sample_weight"] = rng.uniform(1.0, 100.0, size=R).astype(np.float32)
    ex = np.zeros(R, dtype=abi.EXTRA_DTYPE)
    ex["chi2_div"] = rng.random((R, 16)).astype(np.float32)
    boxes = oracle.region_aabbs(split_count, SCENE)
    nodes, leaf = oracle.complete_tree(split_count)
    return st, ex, boxes, nodes, leaf


def test_split_semantics(oracle, abi):
    st, ex, boxes, nodes, leaf = split_fixture(oracle, abi)
    R = st.shape[0]
    big = np.nonzero(st["num_samples"] > 10000.0)[0]
    s2, e2, b2, n2, l2, nn = oracle.split_regions(64, 10000.0, st, ex, boxes, nodes, leaf, 2 * R - 1)
    assert s2.shape[0] == R + big.size and nn == 2 * s2.shape[0] - 1
    for k, r in enumerate(big):  # new regions in region order
        nr = R + k
        assert s2["num_samples"][r] == st["num_samples"][r] * np.float32(0.25)
        assert s2["sample_weight"][r] == st["sample_weight"][r] * np.float32(0.25)
        assert s2[nr].tobytes() == s2[r].tobytes() and e2[nr].tobytes() == e2[r].tobytes()
        # the two halves tile the parent box along its largest axis
        lo, hi = boxes[r, :3], boxes[r, 3:]
        sz = hi - lo  # Aabb::splitAabb's axis rule (ties go to the later axis)
        ax = (0 if sz[0] > sz[2] else 2) if sz[0] > sz[1] else (1 if sz[1] > sz[2] else 2)
        assert b2[r, 3 + ax] < hi[ax] and b2[nr, ax] > lo[ax]
        np.testing.assert_allclose(b2[r, 3 + ax], b2[nr, ax])
        assert b2[r, ax] == lo[ax] and b2[nr, 3 + ax] == hi[ax]
    small = np.setdiff1d(np.arange(R), big)
    assert s2[small].tobytes() == st[small].tobytes()
    # every point of a new region's box finds it in the tree
    rng = np.random.default_rng(9)
    for r in range(s2.shape[0]):
        p = (b2[r, :3] + (0.1 + 0.8 * rng.random((20, 3))) * (b2[r, 3:] - b2[r, :3])).astype(np.float32)
        assert (oracle.region_of(root_box(oracle), n2, p) == r).all()


def test_split_stops_at_capacity(oracle, abi):
    st, ex, boxes, nodes, leaf = split_fixture(oracle, abi)
    R = st.shape[0]
    big = np.nonzero(st["num_samples"] > 10000.0)[0]
    assert big.size >= 2
    s2, _, _, _, _, nn = oracle.split_regions(R + 1, 10000.0, st, ex, boxes, nodes, leaf, 2 * R - 1)
    assert s2.shape[0] == R + 1 and nn == 2 * R + 1
    assert s2["num_samples"][big[0]] == st["num_samples"][big[0]] * np.float32(0.25)
    assert s2["num_samples"][big[1]] == st["num_samples"][big[1]]  # no room left
