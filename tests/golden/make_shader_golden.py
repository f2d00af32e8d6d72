"""Generates tests/golden/shader_ref.npz: the reference's shader functions
(shaders/raytrace.rgen, guiding.glsl, random.glsl, transform.glsl compiled as
host C++ by oracle/build_glsl_ref.py) evaluated on seeded inputs.

Every case is stored as a pg_probe_shading record (include/pathguide.h) with
the random numbers the reference function drew, in the order the library's
functions take them, and the reference's result (`want`, 8 floats laid out as
pg_shading_result).  The GPU test (tests/test_shader_ref_gpu.py) and the
oracle test (tests/test_shader_ref.py) replay the records through the
library and compare.  Run from the repository root:

    python tests/golden/make_shader_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import __graft_entry__ as entry  # noqa: E402

abi = entry.load_package().abi

from oracle import build_glsl_ref  # noqa: E402
from oracle.glsl_ref import GlslRef, ref_material  # noqa: E402

OUT = Path(__file__).resolve().parent / "shader_ref.npz"


def materials() -> np.ndarray:
    M = abi.MATERIAL_DTYPE
    rows = []

    def mat(t, albedo=(0, 0, 0), roughness=0.0, ior=1.0, specular=(0, 0, 0), exponent=0.0, eta=0.0, k=0.0):
        r = np.zeros(1, M)[0]
        r["type"], r["albedo"], r["roughness"], r["ior"] = t, albedo, roughness, ior
        r["specular"], r["exponent"], r["eta"], r["k"] = specular, exponent, eta, k
        rows.append(r)

    mat(0, albedo=(0.7, 0.5, 0.3))                                               # 0 diffuse
    mat(4, albedo=(0.5, 0.4, 0.3), specular=(0.3, 0.3, 0.3), exponent=20.0)      # 1 Phong
    mat(4, albedo=(0.2, 0.2, 0.2), specular=(0.6, 0.5, 0.4), exponent=300.0)     # 2 Phong, almost discrete
    mat(4, albedo=(0.6, 0.6, 0.6), specular=(0.1, 0.1, 0.1), exponent=1.0)       # 3 Phong, broad lobe
    mat(7, roughness=0.5, eta=0.2, k=3.0)                                        # 4 Beckmann
    mat(7, roughness=0.12, eta=1.1, k=2.2)                                       # 5 Beckmann, almost discrete
    mat(2, albedo=(1.0, 1.0, 1.0), ior=1.5)                                      # 6 dielectric
    mat(5, eta=0.2, k=3.0)                                                       # 7 conductor
    mat(1, albedo=(0.9, 0.8, 0.7))                                               # 8 mirror
    return np.array(rows, dtype=M)


def unit(rng, n):
    v = rng.normal(size=(n, 3))
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)


def hemi(rng, normals, lo=0.02):
    out = np.zeros_like(normals)
    for i, n in enumerate(normals):
        while True:
            v = unit(rng, 1)[0]
            c = float(v @ n)
            if abs(c) > lo:
                out[i] = v if c > 0 else -v
                break
    return out


def mixtures(rng, count=12) -> np.ndarray:
    V = np.zeros(count, abi.VMM_THETA_DTYPE)
    for i in range(count):
        K = int(rng.integers(1, 17))
        pi = rng.gamma(1.0, size=K)
        pi /= pi.sum()
        mus = unit(rng, K)
        kap = np.exp(rng.uniform(np.log(0.5), np.log(2000.0), size=K)).astype(np.float32)
        V[i]["used_distributions"] = K
        V[i]["pi"][:K] = pi
        V[i]["mean_position"] = rng.uniform(-1, 1, 3)
        for j in range(K):
            t = V[i]["thetas"][j]
            k = np.float32(kap[j])
            t["mu"] = mus[j]
            t["k"] = k
            t["norm"] = np.float32(k / (2 * np.pi * (1 - np.exp(-2 * np.float64(k)))))
            t["e_min2k"] = np.float32(np.exp(-2 * np.float64(k)))
            if rng.random() < 0.6:
                t["distance"] = np.float32(rng.uniform(0.2, 5.0))
                t["target"] = V[i]["mean_position"] + t["distance"] * mus[j]
            else:
                t["distance"] = -1.0
    return V


def main(out: Path = OUT):
    build_glsl_ref.build_glsl_ref()
    g = GlslRef()
    rng = np.random.default_rng(20241204)
    mats = materials()
    refm = [ref_material(m) for m in mats]
    vmms = mixtures(rng)
    P = abi.PROBE_DTYPE
    probes, want, tags = [], [], []

    def add(p, w, tag):
        probes.append(p)
        want.append(np.asarray(w, dtype=np.float64))
        tags.append(tag)

    def base(op, material=0, vmm=0, flags=0):
        p = np.zeros(1, P)[0]
        p["op"], p["material"], p["vmm"], p["flags"] = op, material, vmm, flags
        return p

    # fresnel (raytrace.rgen:145-160), fresnelConductor (:163-175)
    for _ in range(300):
        p = base(abi.PG_PROBE_FRESNEL)
        p["a"], p["b"] = rng.uniform(0.4, 2.5), rng.uniform(0.0, 1.0)
        add(p, [g.fresnel(float(p["a"]), float(p["b"]))] + [0] * 7, "fresnel")
    for _ in range(300):
        p = base(abi.PG_PROBE_FRESNEL_CONDUCTOR)
        p["a"], p["b"], p["c"] = rng.uniform(-1, 1), rng.uniform(0.05, 3.0), rng.uniform(0.0, 6.0)
        add(p, [g.fresnel_conductor(float(p["a"]), float(p["b"]), float(p["c"]))] + [0] * 7, "fresnel_conductor")

    # evalBsdf / pdfBSDF of the non-discrete materials (both sides of the reflection)
    for mi in (0, 1, 2, 3, 4, 5):
        ns = unit(rng, 200)
        wis, wos = hemi(rng, ns, 0.05), hemi(rng, ns, 0.05)
        for n, wi, wo in zip(ns, wis, wos):
            p = base(abi.PG_PROBE_BSDF_EVAL, mi, flags=abi.PROBE_FRONT)
            p["n"], p["wi"], p["wo"] = n, wi, wo
            f, pdf = g.eval_bsdf(refm[mi], n, wi, wo, True)
            add(p, list(f) + [pdf, 0, 0, 0, 0], f"eval_{mi}")

    # sampleBSDF of the non-discrete materials: the numbers it drew, in the
    # library's order (ul: Phong lobe choice; u1, u2: the warp)
    for mi in (0, 1, 2, 3, 4, 5):
        ns = unit(rng, 200)
        wis = hemi(rng, ns, 0.05)
        for n, wi in zip(ns, wis):
            state = int(rng.integers(0, 2**32))
            d, pdf, drawn = g.sample_bsdf(refm[mi], wi, n, True, state)
            p = base(abi.PG_PROBE_BSDF_SAMPLE, mi, flags=abi.PROBE_FRONT)
            p["n"], p["wi"] = n, wi
            if len(drawn) == 3:
                p["u"][1:4] = drawn
            else:
                p["u"][2:4] = drawn
            add(p, list(d) + [pdf, 0, 0, 0, 0], f"sample_{mi}")

    # VMM pdf (guiding.glsl:53-60), with and without parallax re-aiming
    for vi in range(len(vmms)):
        for par in (0, 1):
            for wo, x in zip(unit(rng, 40), rng.uniform(-1.5, 1.5, size=(40, 3)).astype(np.float32)):
                p = base(abi.PG_PROBE_VMM_PDF, vmm=vi, flags=abi.PROBE_PARALLAX * par)
                p["wo"], p["x"] = wo, x
                add(p, [g.vmm_pdf(vmms[vi:vi + 1], wo, x, par)] + [0] * 7, "vmm_pdf")
        # also close to each lobe's mean, where the pdf is large
        for j in range(int(vmms[vi]["used_distributions"])):
            mu = vmms[vi]["thetas"][j]["mu"]
            wo = mu + rng.normal(scale=0.02, size=3).astype(np.float32)
            wo = (wo / np.linalg.norm(wo)).astype(np.float32)
            p = base(abi.PG_PROBE_VMM_PDF, vmm=vi)
            p["wo"] = wo
            add(p, [g.vmm_pdf(vmms[vi:vi + 1], wo, np.zeros(3), 0)] + [0] * 7, "vmm_pdf")

    # sampleVMM (guiding.glsl:62-96): lobe choice, then the cosine inversion
    for vi in range(len(vmms)):
        for par in (0, 1):
            for x in rng.uniform(-1.5, 1.5, size=(40, 3)).astype(np.float32):
                state = int(rng.integers(0, 2**32))
                d, drawn = g.sample_vmm(vmms[vi:vi + 1], x, par, state)
                if len(drawn) != 3:
                    continue  # a kappa = 0 lobe (uniform sphere by rejection): another method here
                p = base(abi.PG_PROBE_VMM_SAMPLE, vmm=vi, flags=abi.PROBE_PARALLAX * par)
                p["x"] = x
                p["u"][4], p["u"][2], p["u"][3] = drawn
                add(p, list(d) + [0] * 5, "vmm_sample")

    # getNewDirection (raytrace.rgen:923-960) + evalBsdf / pdf (:1176) for every
    # material, guided or not, with or without a region, guide-all rule (the
    # reference's: every non-discrete material is guided)
    for mi in range(len(mats)):
        for guided in (0, 1):
            for region in (1, 0) if guided else (1,):
                ns = unit(rng, 60)
                wis = hemi(rng, ns, 0.05)
                for n, wi in zip(ns, wis):
                    vi = int(rng.integers(0, len(vmms)))
                    par = int(rng.integers(0, 2))
                    x = rng.uniform(-1.5, 1.5, 3).astype(np.float32)
                    front = int(rng.integers(0, 2)) if mats[mi]["type"] == 2 else 1
                    state = int(rng.integers(0, 2**32))
                    d, pdf, tc, drawn = g.new_direction(refm[mi], x, n, wi, front, vmms[vi:vi + 1],
                                                        0 if region else -1, guided, 0.5, par, state)
                    flags = (abi.PROBE_FRONT * front) | (abi.PROBE_PARALLAX * par) | abi.PROBE_GUIDE_ALL
                    flags |= (abi.PROBE_GUIDED * guided) | (abi.PROBE_REGION * region)
                    p = base(abi.PG_PROBE_CONTINUE, mi, vi, flags)
                    p["n"], p["wi"], p["x"], p["c"] = n, wi, x, 0.5
                    t = int(mats[mi]["type"])
                    guided_here = guided and t not in (1, 2, 5)
                    u = list(drawn)
                    if guided_here:
                        if not region:
                            assert not u
                        else:
                            p["u"][0] = u.pop(0)
                            if p["u"][0] < 0.5:  # the guide: lobe, r1, r2
                                if len(u) != 3:
                                    continue
                                p["u"][4], p["u"][2], p["u"][3] = u
                                u = []
                    if u:
                        if t == 2:                    # dielectric: the Fresnel choice
                            p["u"][1] = u[0]
                        elif t == 4:                  # Phong: lobe choice, then the warp
                            if len(u) != 3:
                                continue
                            p["u"][1:4] = u
                        elif t in (0, 7):             # diffuse, Beckmann: the warp
                            if len(u) != 2:
                                continue
                            p["u"][2:4] = u
                    add(p, list(d) + [pdf] + list(tc) + [0], f"continue_{mi}_{guided}{region}")

    # toWorld (transform.glsl:7-38)
    for v, n in zip(unit(rng, 300), unit(rng, 300)):
        p = base(abi.PG_PROBE_TO_WORLD)
        p["wo"], p["n"] = v, n
        add(p, list(g.to_world(v, n)) + [0] * 5, "to_world")

    # sample recording (raytrace.rgen:973-990, 1179-1200): random event
    # sequences of one path, committed weights and flags
    rec_events, rec_want = [], []
    for _ in range(200):
        n_ev = int(rng.integers(1, 24))
        kinds = (rng.random(n_ev) < 0.55).astype(np.int32) ^ 1  # 0 vertex, 1 radiance
        pdfs = rng.uniform(0.05, 5.0, n_ev).astype(np.float32)
        tcs = rng.uniform(0.0, 1.2, (n_ev, 3)).astype(np.float32)
        regions = rng.integers(0, 4096, n_ev).astype(np.uint32)
        lights = rng.exponential(1.0, (n_ev, 3)).astype(np.float32) * (rng.random((n_ev, 1)) < 0.8)
        w, fl = g.record_path(kinds, pdfs, tcs, regions, lights)
        ev = np.zeros(n_ev, dtype=[("kind", "<i4"), ("pdf", "<f4"), ("tc", "<f4", (3,)), ("region", "<u4"),
                                   ("light", "<f4", (3,))])
        ev["kind"], ev["pdf"], ev["tc"], ev["region"], ev["light"] = kinds, pdfs, tcs, regions, lights
        rec_events.append(ev)
        rec_want.append(np.stack([w, fl.view(np.float32)], axis=1) if len(w) else np.zeros((0, 2), np.float32))

    # ADRRS weight window (raytrace.rgen:830-869) and approxDiffuse (:815-828),
    # from a random sequence of their own; window cases whose decisions sit
    # within 1e-4 of a boundary are skipped (FP32 rounding could flip them)
    rng2 = np.random.default_rng(20261204)
    made = 0
    while made < 600:
        est = (rng2.uniform(0.0, 2.0, 3) * (rng2.random() < 0.95)).astype(np.float32)
        adj = rng2.uniform(0.01, 2.0, 3).astype(np.float32)
        thr = (rng2.uniform(0.0, 1.0, 3) * np.exp(rng2.uniform(-4, 4))).astype(np.float32)
        s_ = float(rng2.choice([2.0, 5.0, 10.0]))
        state = int(rng2.integers(1, 2 ** 31))
        q, nn, drawn = g.weight_window(est, thr, adj, s_, state)
        e64, a64, t64 = est.astype(np.float64), adj.astype(np.float64), thr.astype(np.float64)
        center = np.linalg.norm(e64 / a64)
        lower, v = 2 * center / (1 + s_), np.linalg.norm(t64)
        upper = s_ * lower
        if lower > 0 and (abs(v - lower) < 1e-4 * lower or abs(v - upper) < 1e-4 * upper):
            continue
        if len(drawn) and abs(float(drawn[0]) - (int(v / upper) + 1 - v / upper)) < 1e-4:
            continue
        p = base(abi.PG_PROBE_WEIGHT_WINDOW)
        p["wi"], p["wo"], p["x"], p["a"] = thr, adj, est, s_
        if len(drawn):
            p["u"][0] = drawn[0]
        add(p, [q, nn] + [0] * 6, "weight_window")
        made += 1
    for mi, m in enumerate(mats):
        if int(m["type"]) not in (abi.PG_MAT_DIFFUSE, abi.PG_MAT_PHONG, abi.PG_MAT_BECKMANN):
            continue
        for n, w in zip(unit(rng2, 60), unit(rng2, 60)):
            w = w if w @ n > 0 else -w
            p = base(abi.PG_PROBE_APPROX_DIFFUSE, mi)
            p["n"], p["wi"] = n, w
            add(p, list(g.approx_diffuse(refm[mi], n, w)) + [0] * 5, "approx_diffuse")

    np.savez_compressed(
        out, mats=mats, vmms=vmms, probes=np.array(probes, dtype=P), want=np.array(want), tags=np.array(tags),
        rec_offsets=np.cumsum([0] + [len(e) for e in rec_events]).astype(np.int64),
        rec_events=np.concatenate(rec_events),
        rec_slot_offsets=np.cumsum([0] + [len(w) for w in rec_want]).astype(np.int64),
        rec_want=np.concatenate(rec_want))
    print(f"{out}: {len(probes)} probes, {len(rec_events)} recorded paths")


if __name__ == "__main__":
    main()
