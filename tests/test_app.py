"""The C++ driver over include/pathguiding.hpp (app/pg_render.cpp): argument
and scene-file errors on CPU; a guided and a plain render on the GPU, checked
against the Python path's render of the same scene."""
from __future__ import annotations

import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
EXE = ROOT / "rtx-pathtracer_gb300" / "pg_render"


@pytest.fixture(scope="module")
def exe(pkg):
    import __graft_entry__ as entry
    entry.build()
    assert EXE.exists()
    return EXE


def read_pfm(path: Path) -> np.ndarray:
    data = path.read_bytes()
    head = data.split(b"\n", 3)
    assert head[0] == b"PF"
    w, h = map(int, head[1].split())
    assert float(head[2]) < 0  # little endian
    img = np.frombuffer(head[3], dtype="<f4").reshape(h, w, 3)
    return img[::-1]


def test_usage_and_scene_errors(exe, tmp_path):
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode != 0 and "WIDTH HEIGHT IC_SIZE GUIDING_SPLITS" in r.stderr
    r = subprocess.run([str(exe), "8", "8", "0", "4", str(tmp_path / "missing.xml")], capture_output=True, text=True)
    assert r.returncode != 0 and "PG_ERR_IO" in r.stderr
    bad = tmp_path / "bad.xml"
    bad.write_text("<scene><shape type='torus'/></scene>")
    r = subprocess.run([str(exe), "8", "8", "0", "4", str(bad)], capture_output=True, text=True)
    assert r.returncode != 0 and "PG_ERR_PARSE" in r.stderr
    r = subprocess.run([str(exe), "8", "8", "0", "4", "cornell", "--bogus"], capture_output=True, text=True)
    assert r.returncode != 0


@pytest.mark.gpu
def test_guided_and_plain_renders(exe, tmp_path, cuda, pkg, abi):
    W, H = 96, 54
    out = {}
    for mode in ("guided", "plain", "split"):
        pfm = tmp_path / f"{mode}.pfm"
        args = [str(exe), str(W), str(H), "0", "8", "cornell", "--spp", "256", "--out", str(pfm)]
        if mode == "plain":
            args.append("--no-guiding")
        if mode == "split":  # region splitting at a threshold the training passes reach
            args += ["--split-regions", "400"]
        r = subprocess.run(args, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        info = json.loads(r.stdout.strip().splitlines()[-1])
        assert info["spp"] == 256 + 63
        img = read_pfm(pfm)
        assert img.shape == (H, W, 3) and np.isfinite(img).all()
        assert abs(img.mean() - info["mean"]) < 1e-6 * max(1.0, info["mean"])
        out[mode] = (img, info)
    assert out["guided"][1]["sorted_records"] > 0 and out["guided"][1]["regions_with_samples"] > 0
    assert out["guided"][1]["regions"] == 256 and out["split"][1]["regions"] > 256
    torch = cuda
    sc = pkg.Scene.cornell(W, H)
    img = torch.zeros(W * H * 3, dtype=torch.float32, device="cuda")
    sc.render(abi.render_params(spp=1024, max_depth=10, seed=99), img)
    ref = img.cpu().numpy().reshape(H, W, 3) / 1024
    for mode in ("guided", "plain", "split"):
        assert abs(out[mode][0].mean() - ref.mean()) / ref.mean() < 0.03, mode
    # the same plain render written as OpenEXR (writeEXR) holds the same pixels
    exr = tmp_path / "plain.exr"
    r = subprocess.run([str(exe), str(W), str(H), "0", "8", "cornell", "--spp", "256", "--no-guiding", "--out",
                        str(exr)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    np.testing.assert_array_equal(pkg.read_exr(exr), out["plain"][0])


def test_cache_modes_need_a_capacity(exe):
    for flag in ("--irradiance-cache", "--adrrs"):
        r = subprocess.run([str(exe), "8", "8", "0", "4", "cornell", flag], capture_output=True, text=True)
        assert r.returncode != 0 and "IC_SIZE" in r.stderr


@pytest.mark.gpu
def test_irradiance_cache_and_adrrs_renders(exe, tmp_path, cuda, pkg, abi):
    """IC_SIZE with --irradiance-cache (prepare frames, then frames that use and
    grow the cache) and with --adrrs (the estimate frame, then roulette and
    splitting): images of the Cornell box near the plain render's mean (the
    cache's irradiance is an approximation: within 10 %; ADRRS is unbiased:
    within 3 %)."""
    W, H = 96, 54
    torch = cuda
    sc = pkg.Scene.cornell(W, H)
    img = torch.zeros(W * H * 3, dtype=torch.float32, device="cuda")
    sc.render(abi.render_params(spp=1024, max_depth=10, seed=99), img)
    ref = float(img.mean()) / 1024
    sc.close()
    for mode, tol in (("--irradiance-cache", 0.10), ("--adrrs", 0.03)):
        pfm = tmp_path / "ic.pfm"
        r = subprocess.run([str(exe), str(W), str(H), "20000", "8", "cornell", "--spp", "256", "--no-guiding",
                            "--prepare-frames", "20", mode, "--out", str(pfm)], capture_output=True, text=True,
                           timeout=300)
        assert r.returncode == 0, r.stderr
        info = json.loads(r.stdout.strip().splitlines()[-1])
        assert info["irradiance_cache_entries"] > 20 and info["adrrs"] == (mode == "--adrrs")
        got = read_pfm(pfm)
        assert np.isfinite(got).all()
        assert abs(got.mean() - ref) / ref < tol, (mode, got.mean(), ref)
