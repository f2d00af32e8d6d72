"""Comparison rules between the library's shading functions (GPU probes or
the FP64 oracle) and the reference's shader functions compiled as C++
(tests/golden/shader_ref.npz, made by tests/golden/make_shader_golden.py).

Results are pg_shading_result rows: v[0:3] a direction or value, v[3] a pdf,
v[4:7] a throughput change.  Tolerances are relative (with a small absolute
floor) for values and pdfs, and in radians for directions; they cover FP32
rounding of the reference's single-precision arithmetic (pow with exponent
300 and exp(kappa (mu.d - 1)) with kappa up to 2000 amplify it most).

Differences by design, and how they are compared:
  * Discrete materials (dielectric, mirror, conductor): the reference's
    getNewDirection returns the choice probability (Fresnel F or 1 - F, or 1)
    and evalBsdf divides it out again; the library returns pdf 1 with the
    same throughput change.  Only direction and throughput change compare.
  * The rough conductor's pdfBSDF does not check the side of the sampled
    direction (raytrace.rgen:284-294): below the surface it is positive while
    evalBsdf is 0 there (G1 returns 0), so the reference continues a path
    with zero throughput; the library gives pdf 0 and ends it.  Such cases
    compare as "no contribution" on both sides.
  * A contribution below 1e-20 (the FP64 oracle keeps values that underflow
    to 0 in FP32) counts as none.
"""
from __future__ import annotations

import numpy as np

DISCRETE_TYPES = (1, 2, 5)  # PG_MAT_SPECULAR, PG_MAT_DIELECTRIC, PG_MAT_CONDUCTOR

TOL = {
    "fresnel": 2e-5, "fresnel_conductor": 2e-5, "eval": 5e-5, "sample_pdf": 3e-4,
    "vmm_pdf": 4e-4, "continue": 4e-4, "angle": 3e-5, "vmm_angle": 3e-5, "weight_window": 1e-5,
}


def _angle(a, b):
    c = np.sum(a * b, 1) / np.maximum(np.linalg.norm(a, axis=1) * np.linalg.norm(b, axis=1), 1e-30)
    return np.arccos(np.clip(c, -1.0, 1.0))


def _rel(a, b, floor=1e-6):
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


def compare(fx, got, tol=TOL, scale=1.0):
    """Returns {family: (count, worst error, bound)} and a list of failures.
    fx: the fixture (npz); got: (n, 8) results for fx['probes']."""
    want, tags, probes, mats = fx["want"], fx["tags"], fx["probes"], fx["mats"]
    report, failures = {}, []

    def check(name, err, bound, idx):
        worst = float(err.max()) if err.size else 0.0
        report[name] = (int(err.size), worst, bound * scale)
        bad = np.where(~(err <= bound * scale))[0]
        for i in bad[:5]:
            failures.append(f"{name}: case {int(idx[i])} error {float(err[i]):.3g} > {bound * scale:.3g} "
                            f"(got {got[idx[i], :7]}, want {want[idx[i], :7]})")

    fam = np.array([t.split("_")[0] if not t.startswith(("fresnel", "vmm", "to_world", "weight_window",
                                                          "approx_diffuse")) else t for t in tags])
    for name in ("fresnel", "fresnel_conductor", "vmm_pdf"):
        idx = np.where(fam == name)[0]
        check(name, _rel(got[idx, 0], want[idx, 0]), tol[name], idx)
    idx = np.where(fam == "eval")[0]
    check("eval", np.max(_rel(got[idx, :4], want[idx, :4]), axis=1), tol["eval"], idx)
    # ADRRS weight window: the number of paths exactly, q to FP32 rounding
    idx = np.where(fam == "weight_window")[0]
    check("weight_window_n", np.abs(got[idx, 1] - want[idx, 1]), 0.0, idx)
    check("weight_window_q", _rel(got[idx, 0], want[idx, 0]), tol["weight_window"], idx)
    idx = np.where(fam == "approx_diffuse")[0]
    check("approx_diffuse", np.max(_rel(got[idx, :3], want[idx, :3]), axis=1), tol["fresnel_conductor"], idx)
    idx = np.where(fam == "to_world")[0]
    check("to_world", _angle(got[idx, :3], want[idx, :3]), tol["angle"], idx)
    idx = np.where(fam == "vmm_sample")[0]
    check("vmm_sample", _angle(got[idx, :3], want[idx, :3]), tol["vmm_angle"], idx)

    # sampleBSDF: direction always; pdf where the direction is above the surface
    idx = np.where(fam == "sample")[0]
    check("sample_dir", _angle(got[idx, :3], want[idx, :3]), tol["angle"], idx)
    above = np.sum(probes["n"][idx] * want[idx, :3], 1) > 0
    check("sample_pdf", _rel(got[idx[above], 3], want[idx[above], 3]), tol["sample_pdf"], idx[above])
    below = idx[~above]
    check("sample_pdf_below", np.abs(got[below, 3]), 0.0, below)

    # getNewDirection + throughput change
    idx = np.where(fam == "continue")[0]
    mtype = mats["type"][probes["material"][idx]]
    live_w = (want[idx, 3] > 0) & (np.max(np.abs(want[idx, 4:7]), 1) > 1e-20)
    live_g = (got[idx, 3] > 0) & (np.max(np.abs(got[idx, 4:7]), 1) > 1e-20)
    check("continue_alive", (live_w != live_g).astype(np.float64), 0.0, idx)
    both = live_w & live_g
    check("continue_dir", _angle(got[idx[both], :3], want[idx[both], :3]), tol["angle"], idx[both])
    check("continue_tc", np.max(_rel(got[idx[both], 4:7], want[idx[both], 4:7]), 1), tol["continue"], idx[both])
    smooth = both & ~np.isin(mtype, DISCRETE_TYPES)
    check("continue_pdf", _rel(got[idx[smooth], 3], want[idx[smooth], 3]), tol["continue"], idx[smooth])
    return report, failures


def compare_records(fx, weights, flags, counts, tol=2e-6):
    """The committed weights and flags of every replayed path."""
    off, sw = fx["rec_slot_offsets"], fx["rec_want"]
    failures = []
    worst = 0.0
    for p in range(len(off) - 1):
        w = sw[off[p]:off[p + 1]]
        n = len(w)
        if counts[p] != n:
            failures.append(f"path {p}: {counts[p]} records, want {n}")
            continue
        ww, wf = w[:, 0], w[:, 1].view(np.uint32)
        valid = wf != 0xFFFFFFFF
        if not np.array_equal(flags[p, :n], wf):
            failures.append(f"path {p}: flags {flags[p, :n]} want {wf}")
        if valid.any():
            e = _rel(weights[p, :n][valid], ww[valid], 1e-30)
            worst = max(worst, float(e.max()))
            if not (e <= tol).all():
                failures.append(f"path {p}: weights {weights[p, :n]} want {ww}")
    return worst, failures
