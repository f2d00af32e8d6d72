"""TEST INFRASTRUCTURE: a numpy restatement of the reference's irradiance
cache arithmetic, the checker of the library's cache kernels.

  * query(): queryIrradianceCache (shaders/raytrace.rgen:748-773) over the
    cache spheres - the intersection shader's containment test
    (shaders/raytrace.irradiance.rint:13-20) and the any-hit shader's weight,
    threshold, visibility test and gradient-corrected value
    (shaders/raytrace.irradiance.rahit:18-51) - in FP32, summed in entry order;
  * new_entry() / updated_entry(): what createIrradianceCache and
    updateIrradianceCache write from calculateCacheData's results
    (shaders/raytrace.rgen:1318-1421), clampGradients included;
  * update_targets(): the round-robin entry choice of updateIrradianceCache
    (:1335-1345) for update requests taken in order.

Pinned against the reference's own shader functions compiled as C++
(oracle/build_glsl_ref.py; tests/test_icache.py) and the committed fixture
tests/golden/ic_ref.npz.  Nothing in the library imports this module.
"""
from __future__ import annotations

import numpy as np

F = np.float32
ENTRY_FIELDS = ("center", "radius", "normal", "harmonic_r", "color", "num_updates", "rot_grad", "trans_grad")


def query(entries: np.ndarray, pos: np.ndarray, nrm: np.ndarray, a: float, use_gradients: bool = False,
          visibility_check: bool = False):
    """(rgb (n, 3) float32, found (n,) bool) at points pos with normals nrm."""
    pos = np.asarray(pos, dtype=F)
    nrm = np.asarray(nrm, dtype=F)
    n = len(pos)
    vsum = np.zeros((n, 3), dtype=F)
    wsum = np.zeros(n, dtype=F)
    inv_a = F(1.0) / F(a)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        for e in entries:
            c = e["center"].astype(F)
            en = e["normal"].astype(F)
            oc = pos - c
            dist = np.sqrt((oc * oc).sum(1, dtype=F)).astype(F)
            inside = dist <= F(e["radius"])
            w = (F(1.0) / (dist / F(e["harmonic_r"]) + np.sqrt(F(1.0) - (nrm * en).sum(1, dtype=F)))).astype(F)
            w = np.where(np.isnan(w) | np.isinf(w), F(1000000.0), w).astype(F)
            ok = inside & ~(w <= inv_a)
            if visibility_check:
                ok &= F(-0.001) <= (oc * ((nrm + en) / F(2.0))).sum(1, dtype=F)
            col = e["color"].astype(F)
            if use_gradients:
                E = F(np.sqrt((col * col).sum(dtype=F)))
                d = col / E if E != 0 else np.zeros(3, dtype=F)
                rot = np.cross(en, nrm).astype(F)
                val = (E + (rot * e["rot_grad"].astype(F)).sum(1, dtype=F) +
                       (oc * e["trans_grad"].astype(F)).sum(1, dtype=F)).astype(F)
                contrib = (w * val)[:, None] * d[None, :]
            else:
                contrib = w[:, None] * col[None, :]
            vsum = np.where(ok[:, None], vsum + contrib.astype(F), vsum).astype(F)
            wsum = np.where(ok, wsum + w, wsum).astype(F)
        found = wsum > 0
        rgb = np.where(found[:, None], vsum / np.where(found, wsum, F(1.0))[:, None], F(0.0)).astype(F)
    return rgb, found


def clamp_gradient(g: np.ndarray, max_length: float) -> np.ndarray:
    """clampGradients (raytrace.rgen:1318-1329) for one gradient."""
    g = np.asarray(g, dtype=F)
    ln = F(np.sqrt((g * g).sum(dtype=F)))
    return (g * (F(max_length) / ln)).astype(F) if ln > F(max_length) else g


def new_entry(pos, nrm, color, rot, trans, harmonic_r, a, min_radius, max_length, dtype):
    """The entry createIrradianceCache writes (raytrace.rgen:1383-1421); None
    where calculateCacheData saw nothing (harmonic_r < 0)."""
    if harmonic_r < 0:
        return None
    e = np.zeros((), dtype=dtype)
    hr = max(F(harmonic_r), F(min_radius))
    e["center"], e["normal"], e["color"] = pos, nrm, color
    e["rot_grad"] = clamp_gradient(rot, max_length)
    e["trans_grad"] = clamp_gradient(trans, max_length)
    e["harmonic_r"] = hr
    e["radius"] = F(a) * hr
    e["num_updates"] = 1
    return e


def updated_entry(old, color, rot, trans, harmonic_r, a, min_radius, max_length):
    """updateIrradianceCache's new values (raytrace.rgen:1347-1380): the
    running mean with weight min(n / (n + 1), 0.95) on the old values."""
    e = old.copy()
    n = int(old["num_updates"])
    w = min(F(n) / F(n + 1), F(0.95))
    mix = lambda x, y: (np.asarray(x, dtype=F) * (F(1.0) - w) + np.asarray(y, dtype=F) * w).astype(F)
    e["color"] = mix(color, old["color"])
    e["rot_grad"] = clamp_gradient(mix(rot, old["rot_grad"]), max_length)
    e["trans_grad"] = clamp_gradient(mix(trans, old["trans_grad"]), max_length)
    hr = mix(harmonic_r, old["harmonic_r"]) if harmonic_r > 0 else F(old["harmonic_r"])
    hr = max(F(hr), F(min_radius))
    e["harmonic_r"] = hr
    e["radius"] = F(a) * hr
    e["num_updates"] = n + 1
    return e


def update_targets(n_requests: int, start: int, n_entries: int):
    """Entries hit by n_requests update requests taken in order from
    round-robin position `start` (-1: the request finds the position past the
    last entry, resets it and updates nothing), and the position after."""
    out, nxt = [], start
    for _ in range(n_requests):
        k = nxt
        nxt += 1
        if k >= n_entries:
            nxt = 0
            out.append(-1)
        else:
            out.append(k)
    return out, nxt
