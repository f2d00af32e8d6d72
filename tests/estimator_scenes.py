"""Scenes and cases of the estimator comparison (tests/golden/make_estimator_golden.py
makes the reference side, tests/test_estimator_ref_gpu.py and
tests/test_estimator_ref.py the library side): 32 x 24 images, paths of at
most 16 segments, 8 parts of 2048 samples per pixel compared as 4 x 4 block
means."""
from __future__ import annotations

import tempfile
from pathlib import Path

import numpy as np

import __graft_entry__ as entry

pkg = entry.load_package()
abi = pkg.abi

W, H = 32, 24
PATH_LENGTH = 16
PARTS, SPP = 8, 2048
GUIDE_SPLITS = 6


def blocks(img: np.ndarray) -> np.ndarray:
    h, w = img.shape[:2]
    return img.reshape(h // 4, 4, w // 4, 4, 3).mean(axis=(1, 3))


def materials_scene(with_env: bool):
    from test_exr import sky
    from test_scene import MITSUBA, QUAD_OBJ
    d = Path(tempfile.mkdtemp())
    (d / "quad.obj").write_text(QUAD_OBJ)
    (d / "scene.xml").write_text(MITSUBA)
    sc = pkg.Scene.load(d / "scene.xml", W, H)
    if with_env:
        sc.set_envmap(sky())
    return sc


def cornell():
    return pkg.Scene.cornell(W, H, ico_level=3)


def guide_states(sc, split_count: int, seed: int = 5):
    """Region mixtures of four lobes: one towards the light from the region's
    centre (with a parallax distance), three random; valid lightpmm states."""
    rng = np.random.default_rng(seed)
    info = sc.info()
    aabb = np.array(info.aabb, dtype=np.float32)
    from oracle.oracle import Oracle
    boxes = Oracle().region_aabbs(split_count, aabb)
    R = boxes.shape[0]
    exp = sc.export()
    light = [t for t in range(len(exp["tri_mat"])) if exp["mats"][exp["tri_mat"][t]]["type"] == abi.PG_MAT_LIGHT]
    lc = exp["pos"].reshape(-1, 3)[exp["idx"].reshape(-1, 3)[light].reshape(-1)].mean(axis=0)
    st = np.zeros(R, dtype=abi.STATE_DTYPE)
    for r in range(R):
        c = 0.5 * (boxes[r, :3] + boxes[r, 3:])
        to_light = lc - c
        dist = float(np.linalg.norm(to_light))
        mus = [to_light / dist] + [v / np.linalg.norm(v) for v in rng.normal(size=(3, 3))]
        kap = [20.0] + list(np.exp(rng.uniform(0.0, np.log(200.0), 3)))
        w = np.array([0.5] + list(rng.uniform(0.1, 1.0, 3)))
        w /= w.sum()
        s = st[r]
        s["k"] = 4
        s["flags"] = abi.PG_STATE_FITTED
        s["parallax_mean"] = c
        s["last_parallax_mean"] = c
        s["distance"][:] = np.inf
        for k in range(4):
            kk = np.float32(kap[k])
            s["weight"][k] = w[k]
            s["mu_x"][k], s["mu_y"][k], s["mu_z"][k] = mus[k]
            s["kappa"][k] = kk
            s["r"][k] = np.float32(1.0 / np.tanh(np.float64(kk)) - 1.0 / np.float64(kk))
            s["norm"][k] = np.float32(kk / (2 * np.pi * (1 - np.exp(-2 * np.float64(kk)))))
            s["e_min2k"][k] = np.float32(np.exp(-2 * np.float64(kk)))
        s["distance"][0] = dist
        s["dist_sum_w"][0] = 1.0
    root = np.concatenate([boxes[:, :3].min(0), boxes[:, 3:].max(0)])
    return st, root


CASES = {
    # name: (scene, use_nee, use_mis, guided)
    "cornell_mis": ("cornell", 1, 1, False),
    "cornell_bsdf": ("cornell", 0, 0, False),
    "materials_mis": ("materials", 1, 1, False),
    "materials_nee": ("materials", 1, 0, False),
    "materials_env_mis": ("materials_env", 1, 1, False),
    "cornell_guided": ("cornell", 1, 1, True),
}


def make_scene(name):
    return {"cornell": cornell, "materials": lambda: materials_scene(False),
            "materials_env": lambda: materials_scene(True)}[name]()




def compare_blocks(ref_parts: np.ndarray, got_parts: np.ndarray, z_max: float = 6.0, mean_tol: float = 0.01):
    """Block means of two sets of independent parts: the largest |z| of the
    difference against the spread of the parts, and the ratio of image means."""
    rm, gm = ref_parts.mean(0), got_parts.mean(0)
    rs = ref_parts.std(0, ddof=1) / np.sqrt(ref_parts.shape[0])
    gs = got_parts.std(0, ddof=1) / np.sqrt(got_parts.shape[0])
    z = np.abs(gm - rm) / np.sqrt(rs ** 2 + gs ** 2 + (1e-4 * rm.mean()) ** 2)
    ratio = gm.mean() / rm.mean()
    return float(z.max()), float(ratio), bool(z.max() < z_max and abs(ratio - 1.0) < mean_tol)
