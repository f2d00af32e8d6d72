"""The reference's remaining materials on the GPU tracer - Phong, the Fresnel
conductor, the Beckmann rough conductor (raytrace.rgen:145-333, 483-599) -
against the FP64 renderer (oracle/pg_oracle_trace.cpp) on a Mitsuba scene that
holds all of them: same-seed images, and the three estimators (BSDF only,
NEE only, MIS) converging to one another, which checks every sampler against
its pdf."""
from __future__ import annotations

import numpy as np
import pytest

from test_scene import MITSUBA, QUAD_OBJ
from test_trace_gpu import assert_same_seed_parity, render_gpu, tracer  # noqa: F401 (fixture)

pytestmark = pytest.mark.gpu


@pytest.fixture()
def scene(tmp_path, pkg):
    (tmp_path / "quad.obj").write_text(QUAD_OBJ)
    (tmp_path / "scene.xml").write_text(MITSUBA)
    return lambda w, h: pkg.Scene.load(tmp_path / "scene.xml", w, h)


@pytest.mark.parametrize("nee,mis", [(1, 1), (0, 0), (1, 0)])
def test_materials_same_seed(nee, mis, scene, cuda, abi, tracer):
    sc = scene(48, 36)
    types = set(sc.export()["mats"]["type"].tolist())
    assert {abi.PG_MAT_PHONG, abi.PG_MAT_CONDUCTOR, abi.PG_MAT_BECKMANN, abi.PG_MAT_SPECULAR} <= types
    params = abi.render_params(spp=4, max_depth=8, seed=13, use_nee=nee, use_mis=mis)
    got, _ = render_gpu(cuda, sc, params)
    want = tracer.render(sc.export(), params)
    assert want.mean() > 0
    assert_same_seed_parity(got, want, f"materials nee={nee} mis={mis}")


def test_materials_estimators_converge(scene, cuda, abi, tracer):
    sc = scene(32, 24)
    spp = 2048
    imgs = {}
    for name, nee, mis in (("bsdf", 0, 0), ("nee", 1, 0), ("mis", 1, 1)):
        imgs[name], _ = render_gpu(cuda, sc, abi.render_params(spp=spp, max_depth=8, seed=31, use_nee=nee,
                                                               use_mis=mis))
        imgs[name] /= spp
    ref = tracer.render(sc.export(), abi.render_params(spp=512, max_depth=8, seed=77)) / 512
    m = ref.mean()
    blk = lambda x: x.reshape(3, 8, 4, 8, 3).mean(axis=(1, 3))
    for name, img in imgs.items():
        assert abs(img.mean() - m) / m < 0.03, f"{name}: mean {img.mean()} vs f64 {m}"
        rel = np.abs(blk(img) - blk(ref)) / (blk(ref) + 0.05 * m)
        assert rel.max() < 0.12, f"{name}: block rel err {rel.max():.3f}"


def test_materials_guided_same_seed(scene, cuda, pkg, abi, tracer):
    torch = cuda
    sc = scene(48, 36)
    i = sc.info()
    P = i.camera.width * i.camera.height
    ctx = pkg.FitContext(abi.default_fit_config(), max_regions=64)
    ctx.set_regions(6, np.array(i.aabb, dtype=np.float32))
    rec = torch.zeros(P * 16 * 40, dtype=torch.uint8, device="cuda")
    render_gpu(torch, sc, abi.render_params(spp=8, max_depth=8, seed=1, record_samples=1), guide=ctx, records=rec)
    vmm = torch.zeros(64 * 720, dtype=torch.uint8, device="cuda")
    ctx.update(rec, P * 16, vmm)
    torch.cuda.synchronize()
    boxes = ctx.region_aabbs()
    guide = {"vmm": vmm.cpu().numpy(), "root": np.concatenate([boxes[:, :3].min(0), boxes[:, 3:].max(0)]),
             "split_count": 6, "use_parallax": int(abi.default_fit_config().use_parallax)}
    params = abi.render_params(spp=4, max_depth=8, seed=19, use_guiding=1, guiding_prob=0.5)
    got, _ = render_gpu(torch, sc, params, guide=ctx)
    want = tracer.render(sc.export(), params, guide=guide)
    assert_same_seed_parity(got, want, "materials guided")
    ctx.close()


@pytest.mark.parametrize("nee,mis", [(1, 1), (0, 0), (1, 0)])
def test_envmap_same_seed(nee, mis, scene, cuda, abi, tracer):
    """The environment map lights misses and is sampled by NEE (a uniform
    direction in the hemisphere), MIS-weighted like the other lights."""
    from test_exr import sky
    sc = scene(48, 36)
    sc.set_envmap(sky())
    params = abi.render_params(spp=4, max_depth=8, seed=23, use_nee=nee, use_mis=mis)
    got, _ = render_gpu(cuda, sc, params)
    want = tracer.render(sc.export(), params)
    assert_same_seed_parity(got, want, f"envmap nee={nee} mis={mis}")


def test_envmap_estimators_converge(scene, cuda, abi, tracer):
    from test_exr import sky
    sc = scene(32, 24)
    sc.set_envmap(sky())
    spp = 2048
    imgs = {}
    for name, nee, mis in (("bsdf", 0, 0), ("nee", 1, 0), ("mis", 1, 1)):
        imgs[name], _ = render_gpu(cuda, sc, abi.render_params(spp=spp, max_depth=8, seed=41, use_nee=nee,
                                                               use_mis=mis))
        imgs[name] /= spp
    ref = tracer.render(sc.export(), abi.render_params(spp=512, max_depth=8, seed=97)) / 512
    m = ref.mean()
    blk = lambda x: x.reshape(3, 8, 4, 8, 3).mean(axis=(1, 3))
    for name, img in imgs.items():
        assert abs(img.mean() - m) / m < 0.03, f"{name}: mean {img.mean()} vs f64 {m}"
        rel = np.abs(blk(img) - blk(ref)) / (blk(ref) + 0.05 * m)
        assert rel.max() < 0.15, f"{name}: block rel err {rel.max():.3f}"
