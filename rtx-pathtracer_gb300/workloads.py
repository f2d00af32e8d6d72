"""Seeded synthetic guiding-sample workloads.

The reference publishes no sample dump for its guiding fit, so the fit is
measured and checked on seeded synthetic samples with the shapes of the two
fit workloads it is quoted on:

* ``fit_plain``: 64 regions x 16384 samples, drawn from a 4-lobe von
  Mises-Fisher ground truth per region (kappa log-uniform in [5, 500], lobe
  means uniform on the sphere, lobe weights Dirichlet(1)), sample weights
  lognormal(0, 1), positions uniform in the region's unit box, pdf 1,
  distance 1.  Fitted with K=8 for 20 iterations.
* ``fit_batched``: 4096 regions whose sample counts are lognormal with
  median 2048 and sigma 1.0, clipped to [64, 262144]; 1-6 ground-truth lobes
  (kappa log-uniform in [2, 2000]); weights lognormal(0, 1.5); positions
  uniform in the region box; distances log-uniform in [0.1, 100] with 10%
  misses (distance 0, i.e. +inf after the parallax pre-pass).  Fitted with
  K=16, parallax on.

Samples are returned in the two layouts the library consumes: 40-byte
``DirectionalData`` records (external/lightpmm/include/pmm/DirectionalData.h:44-101)
and the fit's packed float4 {direction.xyz, weight}.
"""
from __future__ import annotations

import numpy as np

RECORD_DTYPE = np.dtype(
    [("position", "<f4", (3,)), ("direction", "<f4", (3,)), ("weight", "<f4"),
     ("pdf", "<f4"), ("distance", "<f4"), ("flags", "<u4")]
)
assert RECORD_DTYPE.itemsize == 40


def _frame(mu: np.ndarray):
    """Orthonormal tangent frame around unit vectors mu (n, 3)."""
    a = np.where(np.abs(mu[:, :1]) > 0.9, np.array([[0.0, 1.0, 0.0]]), np.array([[1.0, 0.0, 0.0]]))
    t = np.cross(mu, a)
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    b = np.cross(mu, t)
    return t, b


def sample_vmf(rng: np.random.Generator, mu: np.ndarray, kappa: np.ndarray) -> np.ndarray:
    """One vMF draw per row (mu (n,3) unit, kappa (n,)), inverse-CDF in float64."""
    n = mu.shape[0]
    u = rng.random(n)
    phi = 2.0 * np.pi * rng.random(n)
    # cos(theta) = 1 + log(u + (1-u) e^{-2 kappa}) / kappa
    w = 1.0 + np.log(u + (1.0 - u) * np.exp(-2.0 * kappa)) / kappa
    w = np.clip(w, -1.0, 1.0)
    s = np.sqrt(np.maximum(0.0, 1.0 - w * w))
    t, b = _frame(mu)
    d = (s * np.cos(phi))[:, None] * t + (s * np.sin(phi))[:, None] * b + w[:, None] * mu
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return d


def _uniform_sphere(rng: np.random.Generator, n: int) -> np.ndarray:
    z = 2.0 * rng.random(n) - 1.0
    phi = 2.0 * np.pi * rng.random(n)
    s = np.sqrt(1.0 - z * z)
    return np.stack([s * np.cos(phi), s * np.sin(phi), z], axis=1)


def region_counts_lognormal(rng, n_regions, median, sigma, lo, hi):
    c = np.exp(np.log(median) + sigma * rng.standard_normal(n_regions))
    return np.clip(np.rint(c), lo, hi).astype(np.int64)


def mixture_samples(rng, counts, lobes_lo, lobes_hi, kappa_lo, kappa_hi, w_sigma,
                    region_boxes=None, dist_range=None, miss_frac=0.0):
    """Draw samples for every region from its own random vMF mixture.

    Returns a dict with ``records`` (structured, 40 B each, flags = region id),
    ``dirw`` (float32 (N, 4)), ``offsets`` (uint32 (R+1,)) and the ground truth.
    """
    counts = np.asarray(counts, dtype=np.int64)
    R = counts.shape[0]
    n_lobes = rng.integers(lobes_lo, lobes_hi + 1, size=R)
    L = int(n_lobes.max())
    lobe_mu = _uniform_sphere(rng, R * L).reshape(R, L, 3)
    lobe_kappa = np.exp(rng.uniform(np.log(kappa_lo), np.log(kappa_hi), size=(R, L)))
    lobe_w = rng.gamma(1.0, size=(R, L))
    lobe_w *= (np.arange(L)[None, :] < n_lobes[:, None])
    lobe_w /= lobe_w.sum(axis=1, keepdims=True)
    N = int(counts.sum())
    region = np.repeat(np.arange(R), counts)
    cdf = np.cumsum(lobe_w, axis=1)
    u = rng.random(N)
    lobe = (u[:, None] > cdf[region]).sum(axis=1)
    lobe = np.minimum(lobe, n_lobes[region] - 1)
    d = sample_vmf(rng, lobe_mu[region, lobe], lobe_kappa[region, lobe])
    w = np.exp(w_sigma * rng.standard_normal(N))
    if region_boxes is None:
        lo = np.zeros((R, 3))
        hi = np.ones((R, 3))
    else:
        lo = region_boxes[:, :3].astype(np.float64)
        hi = region_boxes[:, 3:].astype(np.float64)
    pos = lo[region] + rng.random((N, 3)) * (hi - lo)[region]
    if dist_range is None:
        dist = np.ones(N)
    else:
        dist = np.exp(rng.uniform(np.log(dist_range[0]), np.log(dist_range[1]), size=N))
        if miss_frac > 0:
            dist[rng.random(N) < miss_frac] = 0.0
    rec = np.zeros(N, dtype=RECORD_DTYPE)
    rec["position"] = pos
    rec["direction"] = d
    rec["weight"] = w
    rec["pdf"] = 1.0
    rec["distance"] = dist
    rec["flags"] = region.astype(np.uint32)
    dirw = np.empty((N, 4), dtype=np.float32)
    dirw[:, :3] = rec["direction"]
    dirw[:, 3] = rec["weight"]
    offsets = np.zeros(R + 1, dtype=np.uint32)
    offsets[1:] = np.cumsum(counts)
    return {"records": rec, "dirw": dirw, "offsets": offsets, "n_lobes": n_lobes,
            "lobe_mu": lobe_mu, "lobe_kappa": lobe_kappa, "lobe_w": lobe_w}


def fit_plain(seed: int = 1, n_regions: int = 64, n_per_region: int = 16384):
    """The 64-region x 16384-sample K=8 fit workload (scaled down by arguments for tests)."""
    rng = np.random.default_rng(seed)
    counts = np.full(n_regions, n_per_region, dtype=np.int64)
    return mixture_samples(rng, counts, 4, 4, 5.0, 500.0, 1.0)


def fit_batched(seed: int = 3, n_regions: int = 4096, median: float = 2048.0, sigma: float = 1.0,
                lo: int = 64, hi: int = 262144, region_boxes=None):
    """The 4096-region uneven K=16 parallax fit workload (scaled by arguments for tests)."""
    rng = np.random.default_rng(seed)
    counts = region_counts_lognormal(rng, n_regions, median, sigma, lo, hi)
    return mixture_samples(rng, counts, 1, 6, 2.0, 2000.0, 1.5, region_boxes=region_boxes,
                           dist_range=(0.1, 100.0), miss_frac=0.1)


def surrogate_records(seed: int = 5, n: int = 1 << 22, box=(-2.0, -1.0, -1.5, 2.0, 3.0, 1.5), lights=4,
                      kappa: float = 50.0) -> np.ndarray:
    """Training records for the learned surrogate: positions uniform in the
    box, each direction drawn from a vMF (kappa) around the direction to one
    of `lights` seeded point lights (picked per record), weights
    lognormal(0, 1).  Returns a RECORD_DTYPE array (flags 0)."""
    rng = np.random.default_rng(seed)
    box = np.asarray(box, dtype=np.float64)
    lo, hi = box[:3], box[3:]
    pos = lo + (hi - lo) * rng.random((n, 3))
    lp = lo + (hi - lo) * rng.random((lights, 3))
    pick = rng.integers(0, lights, n)
    mu = lp[pick] - pos
    mu /= np.maximum(np.linalg.norm(mu, axis=1, keepdims=True), 1e-12)
    d = sample_vmf(rng, mu, np.full(n, kappa))
    rec = np.zeros(n, dtype=RECORD_DTYPE)
    rec["position"] = pos
    rec["direction"] = d
    rec["weight"] = rng.lognormal(0.0, 1.0, n)
    rec["pdf"] = 1.0
    rec["distance"] = np.linalg.norm(lp[pick] - pos, axis=1)
    return rec
