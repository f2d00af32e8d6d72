"""Inputs of the irradiance-cache comparisons (tests/golden/make_ic_golden.py
makes the reference side, tests/test_icache.py and tests/test_icache_gpu.py
the library side)."""
from __future__ import annotations

import numpy as np

import __graft_entry__ as entry

pkg = entry.load_package()
abi = pkg.abi

W, H = 32, 24
PATH_LENGTH = 16
PARTS, SPP = 8, 1024
IC_A = 0.5          # irradianceA: larger spheres than the default 0.2, so most paths meet the cache
IC_CAPACITY = 4096
COMPUTE_RUNS = 1024
ESTIMATE_SPP = 256  # the ADRRS estimate: the plain estimator's mean
ADRRS_S = 5.0       # adrrsS
# (point, normal) on the Cornell box's diffuse walls: left, right, back, ceiling, floor (twice)
COMPUTE_POINTS = [
    ((0.0, 0.5, 0.5), (1.0, 0.0, 0.0)),
    ((1.0, 0.3, 0.6), (-1.0, 0.0, 0.0)),
    ((0.5, 0.5, 0.0), (0.0, 0.0, 1.0)),
    ((0.3, 1.0, 0.3), (0.0, -1.0, 0.0)),
    ((0.15, 0.0, 0.85), (0.0, 1.0, 0.0)),
    ((0.8, 0.0, 0.2), (0.0, 1.0, 0.0)),
]


def cornell():
    return pkg.Scene.cornell(W, H, ico_level=3)


def blocks(img: np.ndarray) -> np.ndarray:
    h, w = img.shape[:2]
    return img.reshape(h // 4, 4, w // 4, 4, 3).mean(axis=(1, 3))


def query_case(n_entries: int = 200, n_points: int = 4000, seed: int = 3):
    """Random entries in [-1, 1]^3 and query points, the points kept only where
    every containment, weight-threshold and visibility decision is clear by a
    relative 1e-4 in FP64 (so FP32 rounding cannot flip one)."""
    rng = np.random.default_rng(seed)
    e = np.zeros(n_entries, dtype=abi.IC_ENTRY_DTYPE)
    e["center"] = rng.uniform(-1, 1, (n_entries, 3))
    nr = rng.normal(size=(n_entries, 3))
    e["normal"] = nr / np.linalg.norm(nr, axis=1, keepdims=True)
    e["harmonic_r"] = rng.uniform(0.3, 2.0, n_entries)
    e["radius"] = IC_A * e["harmonic_r"]
    e["color"] = rng.uniform(0, 2, (n_entries, 3))
    e["num_updates"] = rng.integers(1, 30, n_entries)
    e["rot_grad"] = rng.normal(size=(n_entries, 3)) * 0.5
    e["trans_grad"] = rng.normal(size=(n_entries, 3)) * 0.5
    m = 3 * n_points
    p = rng.uniform(-1.2, 1.2, (m, 3))
    q = rng.normal(size=(m, 3))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    p, q = p.astype(np.float32).astype(np.float64), q.astype(np.float32).astype(np.float64)
    keep = np.ones(m, dtype=bool)
    for x in e:
        c, en = x["center"].astype(np.float64), x["normal"].astype(np.float64)
        oc = p - c
        d = np.linalg.norm(oc, axis=1)
        r = float(x["radius"])
        keep &= np.abs(d - r) > 1e-4 * r
        with np.errstate(divide="ignore"):
            w = 1.0 / (d / float(x["harmonic_r"]) + np.sqrt(np.maximum(1.0 - (q * en).sum(1), 0.0)))
        keep &= np.abs(w * IC_A - 1.0) > 1e-4
        keep &= np.abs((oc * (q + en) / 2).sum(1) + 0.001) > 1e-5
    idx = np.where(keep)[0][:n_points]
    return e, p[idx].astype(np.float32), q[idx].astype(np.float32)


def surface_points(exp: dict, n: int, seed: int):
    """n diffuse surface points with their normals facing the ray: first hits
    of camera rays through random image positions, then the hits of one
    cosine-distributed bounce from them (the points a render queries)."""
    from oracle.oracle import TraceOracle
    rng = np.random.default_rng(seed)
    tr = TraceOracle()
    cam = exp["info"].camera
    o = np.array(cam.origin[:], dtype=np.float64)
    f = np.array(cam.target[:], dtype=np.float64) - o
    f /= np.linalg.norm(f)
    r = np.cross(f, np.array(cam.up[:], dtype=np.float64))
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    th = np.tan(np.radians(cam.vfov_deg) / 2)
    asp = cam.width / cam.height
    pos = exp["pos"].reshape(-1, 3).astype(np.float64)
    idx = exp["idx"].reshape(-1, 3)
    mats = exp["mats"]

    def trace(org, dirs):
        rays = np.zeros(len(dirs), dtype=abi.RAY_DTYPE)
        rays["org"], rays["dir"], rays["tmin"], rays["tmax"] = org, dirs, 1e-3, 1e6
        h = tr.closest(exp, rays)
        out_p, out_n, ok = [], [], []
        for k in range(len(dirs)):
            t, prim = float(h["t"][k]), int(h["prim"][k])
            if prim == 0xFFFFFFFF or prim & 0x80000000:
                ok.append(False)
                out_p.append(np.zeros(3))
                out_n.append(np.zeros(3))
                continue
            v = pos[idx[prim]]
            ng = np.cross(v[1] - v[0], v[2] - v[0])
            ng /= np.linalg.norm(ng)
            if ng @ dirs[k] > 0:
                ng = -ng
            good = mats[exp["tri_mat"][prim]]["type"] == abi.PG_MAT_DIFFUSE
            ok.append(bool(good))
            out_p.append((org[k] if org.ndim == 2 else org) + t * dirs[k])
            out_n.append(ng)
        return np.array(out_p), np.array(out_n), np.array(ok)

    sx = (2 * rng.uniform(0, 1, 2 * n) - 1) * th * asp
    sy = (1 - 2 * rng.uniform(0, 1, 2 * n)) * th
    d = f[None] + sx[:, None] * r[None] + sy[:, None] * u[None]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    p1, n1, ok1 = trace(o, d)
    p1, n1 = p1[ok1], n1[ok1]
    # cosine bounce
    a, b = rng.uniform(0, 1, len(p1)), rng.uniform(0, 1, len(p1))
    loc = np.stack([np.sqrt(a) * np.cos(2 * np.pi * b), np.sqrt(a) * np.sin(2 * np.pi * b), np.sqrt(1 - a)], 1)
    tx = np.cross(n1, np.where(np.abs(n1[:, :1]) > 0.9, [[0, 1, 0]], [[1, 0, 0]]))
    tx /= np.linalg.norm(tx, axis=1, keepdims=True)
    ty = np.cross(n1, tx)
    d2 = loc[:, :1] * tx + loc[:, 1:2] * ty + loc[:, 2:] * n1
    p2, n2, ok2 = trace(p1, d2)
    h = n // 2
    pts = np.concatenate([p1[:h], p2[ok2][:n - h]])
    nrm = np.concatenate([n1[:h], n2[ok2][:n - h]])
    return pts.astype(np.float32), nrm.astype(np.float32)


SPHERE_XML = """<?xml version="1.0" encoding="utf-8"?>
<scene version="0.5.0">
  <sensor type="perspective">
    <float name="fov" value="40"/>
    <transform name="toWorld"><lookAt origin="0, 0, 0" target="0, 0, -1" up="0, 1, 0"/></transform>
  </sensor>
  <shape type="sphere">
    <point name="center" x="0" y="0" z="0"/>
    <float name="radius" value="2"/>
    <bsdf type="diffuse"><rgb name="reflectance" value="0.5, 0.5, 0.5"/></bsdf>
  </shape>
  <shape type="sphere">
    <point name="center" x="10" y="0" z="0"/>
    <float name="radius" value="0.5"/>
    <emitter type="area"><rgb name="radiance" value="1, 1, 1"/></emitter>
  </shape>
</scene>
"""


def sphere_scene(tmp_path, width=1, height=1):
    """A diffuse sphere of radius 2 around the camera and a light outside it:
    every hemisphere path from inside sees no light (radiance 0) and every
    path from the centre hits the wall at distance 2, so calculateCacheData
    returns colour 0, zero gradients and harmonic distance 2 there."""
    (tmp_path / "sphere.xml").write_text(SPHERE_XML)
    return pkg.Scene.load(tmp_path / "sphere.xml", width, height)


def sphere_entries():
    """Three entries at the sphere's centre with given values."""
    e = np.zeros(3, dtype=abi.IC_ENTRY_DTYPE)
    e["center"] = 0.0
    e["normal"] = [[0, 0, 1], [0, 1, 0], [1, 0, 0]]
    e["harmonic_r"] = [0.5, 3.0, 0.05]
    e["radius"] = 0.2 * e["harmonic_r"]
    e["color"] = [[1.0, 2.0, 3.0], [0.5, 0.25, 0.125], [4.0, 0.0, 1.0]]
    e["num_updates"] = [1, 5, 40]
    e["rot_grad"] = [[1, 0, 0], [0, 6, 8], [0.1, 0.2, 0.3]]
    e["trans_grad"] = [[0, 0, 0.5], [3, 4, 0], [-7, 0, 0]]
    return e
