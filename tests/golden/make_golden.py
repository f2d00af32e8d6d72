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
    make_splitmerge(ref)
    make_update_splitmerge(ref)
    print("golden fixtures written to", HERE)


# Split/merge sequences: region sample counts per pass, the split/merge knobs
# and the number of passes.  "default" uses the reference's knobs
# (src/PathGuiding.h:124-129); "eager" lowers the sample thresholds so small
# regions merge, split and refit within a few passes.
SPLITMERGE = {
    "default": (np.array([0, 40, 700, 2800, 4500, 8500, 1500], dtype=np.int64), {}, 3),
    "eager": (np.array([0, 30, 300, 800, 1500, 2500, 600], dtype=np.int64),
              {"min_samples_for_merging": 2048, "min_samples_for_splitting": 1024,
               "min_samples_for_post_split_fitting": 1024}, 4),
}


def make_splitmerge(ref):
    """PathGuiding::update over several passes (fit, then postFit with split
    and merge) on samples of fixed per-region mixtures; stores every pass's
    samples, the fitted states that enter postFit and what postFit returns."""
    for name, (counts, knobs, passes) in SPLITMERGE.items():
        rng = np.random.default_rng(4242 if name == "default" else 5151)
        w = wl.mixture_samples(rng, counts * passes, 1, 6, 2.0, 2000.0, 1.0)
        R = counts.shape[0]
        cfg = abi.default_fit_config(num_initial_components=8)
        sm = abi.default_split_merge_config(**knobs)
        st = ref.init_states(cfg, R)
        ex = np.zeros(R, dtype=abi.EXTRA_DTYPE)
        big = w["offsets"].astype(np.int64)
        out = {"cfg": np.array(list(cfg_dict(cfg).values()), dtype=np.float64),
               "sm": np.array(list(cfg_dict(sm).values()), dtype=np.float64), "passes": np.array(passes)}
        for p in range(passes):
            idx = np.concatenate([np.arange(big[r] + p * counts[r], big[r] + (p + 1) * counts[r]) for r in range(R)])
            dirw = np.ascontiguousarray(w["dirw"][idx])
            offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint32)
            pdf = (rng.uniform(0.5, 2.0, dirw.shape[0]) / (4.0 * np.pi)).astype(np.float32)
            st, _ = ref.fit(cfg, dirw, offsets, states=st, mode=abi.PG_FIT_CONTINUE if p == 0 else abi.PG_FIT_UPDATE)
            fitted, ex_in = st.copy(), ex.copy()
            st, ex = ref.postfit(cfg, sm, dirw, pdf, None, offsets, st, ex)
            out.update({f"dirw{p}": dirw, f"pdf{p}": pdf, f"offsets{p}": offsets, f"fitted{p}": fitted,
                        f"extras_in{p}": ex_in, f"states{p}": st.copy(), f"extras{p}": ex.copy()})
            print(name, "pass", p, "K", st["k"].tolist(), "since", ex["samples_since_merge"].tolist())
        save(f"splitmerge_{name}", **out)


def make_update_splitmerge(ref):
    """Whole PathGuiding::update passes with splitAndMerge on: the tracer's
    records in, per pass the reference's states and split/merge statistics
    out.  Bucketing, region centres, reposition and the parallax pre-pass are
    the oracle's (pinned against the reference by the other fixtures); fit and
    postFit (merge, statistics, split, distances) are the reference's."""
    build_oracle.build_oracle()
    from oracle.oracle import Oracle  # noqa: E402
    orc = Oracle()
    split_count, passes = 3, 3
    scene = np.array([-1.0, -1.0, -1.0, 1.0, 1.0, 1.0], dtype=np.float32)
    boxes = orc.region_aabbs(split_count, scene)
    R = boxes.shape[0]
    means = boxes[:, :3] + np.float32(0.5) * (boxes[:, 3:] - boxes[:, :3])
    rng = np.random.default_rng(8080)
    counts = wl.region_counts_lognormal(rng, R, 700, 1.0, 0, 6000)
    counts[2] = 0  # a region that never has samples
    w = wl.mixture_samples(rng, counts * passes, 1, 5, 3.0, 600.0, 1.0, region_boxes=boxes,
                           dist_range=(0.05, 30.0), miss_frac=0.1)
    cfg = abi.default_fit_config(num_initial_components=8)
    sm = abi.default_split_merge_config(min_samples_for_merging=1536, min_samples_for_splitting=768,
                                        min_samples_for_post_split_fitting=768)
    st = ref.init_states(cfg, R)
    st["distance"][:] = np.inf
    ex = np.zeros(R, dtype=abi.EXTRA_DTYPE)
    big = w["offsets"].astype(np.int64)
    out = {"cfg": np.array(list(cfg_dict(cfg).values()), dtype=np.float64),
           "sm": np.array(list(cfg_dict(sm).values()), dtype=np.float64), "passes": np.array(passes),
           "split_count": np.array(split_count), "scene": scene}
    for p in range(passes):
        idx = np.concatenate([np.arange(big[r] + p * counts[r], big[r] + (p + 1) * counts[r]) for r in range(R)])
        rec = w["records"][idx].copy()
        rec["pdf"] = (rng.uniform(0.5, 2.0, rec.shape[0]) / (4.0 * np.pi)).astype(np.float32)
        rec = rec[rng.permutation(rec.shape[0])]
        rec["flags"][rng.random(rec.shape[0]) < 0.1] = 0xFFFFFFFF  # invalid slots
        srt, off = orc.sort_samples(rec, R)
        busy = np.diff(off.astype(np.int64)) > 0
        st["last_parallax_mean"][busy] = st["parallax_mean"][busy]
        st["parallax_mean"][busy] = means[busy]
        if p > 0:
            for r in np.nonzero(busy)[0]:
                st[r] = ref.reposition(st[r], st["last_parallax_mean"][r] - means[r])
        dirw, dist = orc.prefit_parallax(srt, off, means)
        st, _ = ref.fit(cfg, dirw, off, states=st, mode=abi.PG_FIT_CONTINUE if p == 0 else abi.PG_FIT_UPDATE)
        st, ex = ref.postfit(cfg, sm, dirw, srt["pdf"], dist, off, st, ex)
        out.update({f"records{p}": rec, f"states{p}": st.copy(), f"extras{p}": ex.copy()})
        print("update pass", p, "K", st["k"].tolist())
    save("splitmerge_update", **out)


if __name__ == "__main__":
    if sys.argv[1:] == ["splitmerge"]:
        build_oracle.build_reference(force=False)
        make_splitmerge(ReferenceFit())
        make_update_splitmerge(ReferenceFit())
    else:
        main()
