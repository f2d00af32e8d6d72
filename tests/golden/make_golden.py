"""Generates the golden fixtures of the guiding fit from the reference itself.

Runs the reference's vendored lightpmm fit and its parallax-distance statistic
(compiled in place into oracle/_ref/liblightpmm_ref.so by
oracle/build_oracle.py) on small seeded synthetic sample sets and stores inputs
and outputs as .npz files next to this script.  Needs the reference tree, so it
runs where that tree is mounted; the fixtures it writes are committed.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle import build_oracle  # noqa: E402
from oracle.oracle import ReferenceFit, abi  # noqa: E402

spec = importlib.util.spec_from_file_location("wl", ROOT / "rtx-pathtracer_gb300" / "workloads.py")
wl = importlib.util.module_from_spec(spec)
spec.loader.exec_module(wl)

# region sample counts: empty, too few to fit (<= 2K), small, medium, large
COUNTS = np.array([0, 12, 40, 300, 1500, 3100, 64, 2500], dtype=np.int64)


def cfg_dict(cfg):
    return {f: getattr(cfg, f) for f, _ in cfg._fields_}


def save(name, **arrays):
    out = {}
    for k, v in arrays.items():
        if isinstance(v, np.ndarray) and v.dtype.names:
            out[k] = v.view(np.uint8).reshape(v.shape[0], -1)
            out[k + "__dtype"] = np.array(str(v.dtype.descr))
        else:
            out[k] = v
    np.savez_compressed(HERE / f"{name}.npz", **out)


def main():
    build_oracle.build_reference(force=True)
    ref = ReferenceFit()
    rng = np.random.default_rng(20240601)
    w = wl.mixture_samples(rng, COUNTS, 1, 5, 3.0, 800.0, 1.0, dist_range=(0.2, 50.0), miss_frac=0.1)
    dirw, offsets = w["dirw"], w["offsets"]
    dist = w["records"]["distance"].astype(np.float32)
    dist[dist <= 0] = np.inf  # misses, as the parallax pre-pass leaves them
    for K in (8, 16, 5):
        cfg = abi.forced_iterations(20, num_initial_components=K)
        st, ll = ref.fit(cfg, dirw, offsets)
        save(f"fit_forced_k{K}", dirw=dirw, offsets=offsets, states=st, ll_final=ll,
             cfg=np.array(list(cfg_dict(cfg).values()), dtype=np.float64))
    cfg = abi.default_fit_config(num_initial_components=8)
    st, ll = ref.fit(cfg, dirw, offsets)
    save("fit_converge_k8", dirw=dirw, offsets=offsets, states=st, ll_final=ll,
         cfg=np.array(list(cfg_dict(cfg).values()), dtype=np.float64))
    # a second pass with new samples of the same regions (stepwise EM, updateFit)
    w2 = wl.mixture_samples(np.random.default_rng(77), COUNTS, 1, 5, 3.0, 800.0, 1.0)
    st2, ll2 = ref.fit(cfg, w2["dirw"], offsets, states=st, mode=abi.PG_FIT_UPDATE)
    save("fit_update_k8", dirw=w2["dirw"], offsets=offsets, states_in=st, states=st2, ll_final=ll2,
         cfg=np.array(list(cfg_dict(cfg).values()), dtype=np.float64))
    # parallax distance statistic over the fitted mixtures, two passes
    d1 = ref.update_distances(dirw, dist, offsets, st)
    d2 = ref.update_distances(w2["dirw"], dist, offsets, d1)
    save("distances_k8", dirw=dirw, dirw2=w2["dirw"], dist=dist, offsets=offsets, states_in=st,
         states1=d1, states2=d2)
    # reposition of the lobes with finite distance (region 5)
    moved = ref.reposition(d1[5], np.array([0.3, -0.2, 0.5], dtype=np.float32))
    save("reposition_k8", state_in=d1[5:6], state_out=np.array([moved]), delta=np.array([0.3, -0.2, 0.5],
                                                                                          dtype=np.float32))
    # lightpmm's exp approximation on a grid
    x = np.concatenate([np.linspace(-130.0, 0.0, 4001), -np.logspace(-6, 1, 200)]).astype(np.float32)
    save("fastexp", x=x, y=ref.fastexp(x))
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
