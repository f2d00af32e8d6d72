"""Textures on the GPU tracer: alpha-tested hits (raytrace.rahit:21-46) bit-exact
against the CPU traversal twin for closest and any-hit queries, the hits the
alpha test drops, and textured diffuse reflectance (raytrace.rgen:233-249) in
renders against the FP64 renderer (same seed, and converged)."""
from __future__ import annotations

import numpy as np
import pytest

from pngutil import write_texture_scene
from test_trace_gpu import assert_same_seed_parity, dev, host, make_rays, render_gpu, tracer  # noqa: F401

pytestmark = pytest.mark.gpu


@pytest.fixture()
def scene(tmp_path, pkg):
    write_texture_scene(tmp_path)
    return lambda w, h: pkg.Scene.load(tmp_path / "scene.xml", w, h)


def quad_rays(abi, rng, n):
    """Rays from in front of the textured quad (z = 0, x in [-1, 1], y in [0, 2]) through it."""
    rays = np.zeros(n, dtype=abi.RAY_DTYPE)
    org = np.stack([rng.uniform(-2, 2, n), rng.uniform(0.2, 2.5, n), rng.uniform(1.0, 4.0, n)], 1)
    tgt = np.stack([rng.uniform(-1.1, 1.1, n), rng.uniform(-0.1, 2.1, n), np.zeros(n)], 1)
    d = tgt - org
    rays["org"] = org
    rays["dir"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays["tmin"] = 1e-3
    rays["tmax"] = 1e30
    return rays


def test_alpha_tested_hits_bit_exact(scene, cuda, pkg, abi, tracer):
    torch = cuda
    sc = scene(32, 24)
    exp = sc.export()
    rng = np.random.default_rng(21)
    rays = np.concatenate([quad_rays(abi, rng, 150000), make_rays(abi, rng, exp, 50000)])
    d_rays = dev(torch, rays)
    d_hits = torch.zeros(rays.shape[0] * abi.HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    sc.trace_closest(d_rays, rays.shape[0], d_hits)
    torch.cuda.synchronize()
    got = host(d_hits, abi.HIT_DTYPE)
    want = tracer.closest(exp, rays)
    same = got.view(np.uint32).reshape(-1, 4) == want.view(np.uint32).reshape(-1, 4)
    bad = np.where(~same.all(axis=1))[0]
    assert bad.size == 0, f"{bad.size} hits differ; first {bad[:5]}: gpu {got[bad[:3]]} cpu {want[bad[:3]]}"
    # the checkerboard's transparent half lets about half of the rays aimed at the quad through
    quad_tris = np.where(exp["mats"]["texture"][exp["tri_mat"]] > 0)[0]
    on_quad = np.isin(got["prim"][:150000], quad_tris).mean()
    assert 0.3 < on_quad < 0.7, on_quad
    # any-hit queries up to the quad and beyond it
    rays["tmax"] = rng.uniform(0.5, 8.0, rays.shape[0])
    d_rays = dev(torch, rays)
    d_occ = torch.zeros(rays.shape[0], dtype=torch.int32, device="cuda")
    sc.trace_any(d_rays, rays.shape[0], d_occ)
    torch.cuda.synchronize()
    occ = d_occ.cpu().numpy().view(np.uint32)
    np.testing.assert_array_equal(occ, tracer.any(exp, rays))
    assert 0.05 < occ.mean() < 0.95


def test_opaque_texture_changes_no_hit(scene, cuda, pkg, abi, tmp_path, tracer):
    """With an opaque texture every hit stands: the same hits as without the alpha test."""
    from pngutil import leaf_texture, png_bytes
    torch = cuda
    tex = leaf_texture()
    tex[..., 3] = 255
    (tmp_path / "leaf.png").write_bytes(png_bytes(tex, 6))
    sc = scene(32, 24)
    exp = sc.export()
    rays = quad_rays(abi, np.random.default_rng(3), 50000)
    d_rays = dev(torch, rays)
    d_hits = torch.zeros(rays.shape[0] * abi.HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    sc.trace_closest(d_rays, rays.shape[0], d_hits)
    torch.cuda.synchronize()
    got = host(d_hits, abi.HIT_DTYPE)
    plain = dict(exp)
    plain["tri_verts"] = exp["tri_verts"].copy()
    plain["tri_verts"][:, 7] = 0.0  # no texture ids: no alpha test
    want = tracer.closest(plain, rays)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


def test_textured_render_same_seed(scene, cuda, abi, tmp_path, tracer):
    """Textured reflectance with the same random numbers as the FP64 renderer.
    The texture is made opaque here: the alpha test's hash takes the texture
    coordinate times 1e8, so FP32 and FP64 hit points draw unrelated numbers
    for it; alpha-tested images are compared converged (next test)."""
    from pngutil import leaf_texture, png_bytes
    tex = leaf_texture()
    tex[..., 3] = 255
    (tmp_path / "leaf.png").write_bytes(png_bytes(tex, 6))
    sc = scene(48, 36)
    params = abi.render_params(spp=4, max_depth=6, seed=5)
    got, _ = render_gpu(cuda, sc, params)
    want = tracer.render(sc.export(), params)
    assert want.mean() > 0
    assert_same_seed_parity(got, want, "textured scene")


def test_textured_render_converges(scene, cuda, abi, tracer):
    sc = scene(32, 24)
    spp = 1024
    img, _ = render_gpu(cuda, sc, abi.render_params(spp=spp, max_depth=6, seed=8))
    img /= spp
    ref = tracer.render(sc.export(), abi.render_params(spp=256, max_depth=6, seed=91)) / 256
    m = ref.mean()
    assert abs(img.mean() - m) / m < 0.03, (img.mean(), m)
    blk = lambda x: x.reshape(3, 8, 4, 8, 3).mean(axis=(1, 3))
    rel = np.abs(blk(img) - blk(ref)) / (blk(ref) + 0.05 * m)
    assert rel.max() < 0.12, rel.max()
