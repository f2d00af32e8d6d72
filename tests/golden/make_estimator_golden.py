"""Generates tests/golden/estimator_ref.npz: converged images of the
reference's own path estimator - raytrace(), nextEventEstimation(),
sampleLights(), getNewDirection() and the hit / miss shaders of
shaders/raytrace*.r*, compiled as host C++ by oracle/build_glsl_ref.py and run
over library scenes by oracle/glsl_ref_render.inc - for the GPU renderer to
converge to (tests/test_estimator_ref_gpu.py).

Each case renders PARTS independent parts (frame seeds 1..PARTS) of SPP
samples per pixel and keeps, per part, the mean radiance of every 4 x 4 pixel
block: the GPU test compares block means with the spread of the parts as the
noise scale.  Scenes: the procedural Cornell box with its glass icosphere,
the Mitsuba scene of tests/test_scene.py (Phong, Fresnel conductor, Beckmann
rough conductor, mirror, diffuse) with and without an environment map, and
the Cornell box guided by a fixed set of region mixtures (the reference's
rule: every non-discrete material guided).  Run from the repository root:

    python tests/golden/make_estimator_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import __graft_entry__ as entry  # noqa: E402

pkg = entry.load_package()
abi = pkg.abi

from oracle import build_glsl_ref  # noqa: E402
from oracle.glsl_ref import GlslRef  # noqa: E402
from oracle.oracle import Oracle  # noqa: E402
from estimator_scenes import CASES, GUIDE_SPLITS, PARTS, PATH_LENGTH, SPP, blocks, guide_states, make_scene  # noqa: E402

OUT = Path(__file__).resolve().parent / "estimator_ref.npz"


def main(out: Path = OUT, parts: int = PARTS, spp: int = SPP):
    build_glsl_ref.build_glsl_ref()
    g = GlslRef()
    arrays = {}
    for case, (scene_name, nee, mis, guided) in CASES.items():
        sc = make_scene(scene_name)
        exp = sc.export()
        guide = None
        if guided:
            st, root = guide_states(sc, GUIDE_SPLITS)
            vmm = Oracle().pack_vmm_theta(st, use_parallax=True)
            guide = {"vmm": vmm, "root": root, "split_count": GUIDE_SPLITS, "use_parallax": 1}
            arrays[f"{case}__states"] = st
        res = []
        for p in range(parts):
            img = g.render(exp, path_length=PATH_LENGTH, spp=spp, frame_seed=p + 1, use_nee=bool(nee),
                           use_mis=bool(mis), guide=guide, guiding_prob=0.5) / spp
            res.append(blocks(img).astype(np.float32))
        arrays[f"{case}__blocks"] = np.stack(res)
        b = arrays[f"{case}__blocks"]
        print(f"{case}: mean {b.mean():.5f}, part spread {b.mean(axis=(1, 2, 3)).std() / b.mean():.4f}")
        sc.close()
    np.savez_compressed(out, path_length=PATH_LENGTH, parts=parts, spp=spp, guide_splits=GUIDE_SPLITS, **arrays)
    print(out)


if __name__ == "__main__":
    main()
