"""Host side of the tracer, on CPU: the built-in scenes, the binned-SAH BVH
(src/SceneLoader.cpp builds the reference's acceleration structures through
Vulkan; here the tree is ours and is checked for structure and against brute
force), the Mitsuba/OBJ loader (SceneLoader::loadMitsubaScene,
src/SceneLoader.cpp:450-556) with its errors, and pg_render's argument checks,
which run before any device work.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest


@pytest.fixture(scope="module")
def tracer(oracle):
    from oracle.oracle import TraceOracle
    return TraceOracle()


def check_bvh(exp):
    """Structure of the four-wide BVH: every triangle in exactly one leaf, leaf
    boxes bound their triangles, child boxes nest, every node has one parent."""
    nodes, tv, order = exp["nodes"], exp["tri_verts"], exp["tri_order"]
    T = tv.shape[0]
    assert sorted(order.tolist()) == list(range(T)), "tri_order is a permutation"
    # tri_verts row i holds triangle order[i]; its original id sits in the bits of float [3]
    assert np.array_equal(tv[:, 3].view(np.uint32), order)
    pos, idx = exp["pos"], exp["idx"]
    covered = np.zeros(T, dtype=np.int32)
    seen_nodes = np.zeros(len(nodes), dtype=np.int32)
    stack = [0] if len(nodes) else []
    if len(nodes):
        seen_nodes[0] = 1
    while stack:
        i = stack.pop()
        n = nodes[i]
        for c in range(4):
            lo, hi = n["lo"][:, c], n["hi"][:, c]
            cnt, ch = int(n["count"][c]), int(n["child"][c])
            if cnt > 0:
                assert cnt <= 4, "leaf size"
                assert 0 <= ch and ch + cnt <= T
                covered[ch:ch + cnt] += 1
                v = pos[idx[order[ch:ch + cnt]]].reshape(-1, 3)
                assert (v >= lo - 1e-6).all() and (v <= hi + 1e-6).all(), "leaf box bounds its triangles"
            elif ch >= 0:
                assert 0 < ch < len(nodes)
                assert seen_nodes[ch] == 0, "each node has one parent"
                seen_nodes[ch] = 1
                kid = nodes[ch]
                for c2 in range(4):
                    if kid["count"][c2] > 0 or kid["child"][c2] >= 0:
                        assert (kid["lo"][:, c2] >= lo).all() and (kid["hi"][:, c2] <= hi).all(), "boxes nest"
                stack.append(ch)
            else:
                assert not (lo <= hi).any(), "empty slots have empty boxes"
    assert (covered == 1).all(), "every triangle in exactly one leaf"
    assert seen_nodes.all(), "no orphan nodes"
    # four-wide: most nodes use all four slots
    if len(nodes) > 8:
        assert np.mean((nodes["child"] >= 0).sum(axis=1) == 4) > 0.5


def brute_closest(exp, rays):
    """Closest triangle hit by double-precision Moller-Trumbore over all triangles."""
    pos, idx = exp["pos"].astype(np.float64), exp["idx"]
    a, b, c = pos[idx[:, 0]], pos[idx[:, 1]], pos[idx[:, 2]]
    e1, e2 = b - a, c - a
    out_t = np.full(rays.shape[0], np.inf)
    out_p = np.full(rays.shape[0], 0xFFFFFFFF, dtype=np.uint64)
    for r in range(rays.shape[0]):
        o = rays["org"][r].astype(np.float64)
        d = rays["dir"][r].astype(np.float64)
        p = np.cross(d, e2)
        det = np.einsum("ij,ij->i", e1, p)
        ok = np.abs(det) > 1e-30
        inv = np.where(ok, 1.0 / np.where(ok, det, 1.0), 0.0)
        s = o - a
        u = np.einsum("ij,ij->i", s, p) * inv
        q = np.cross(s, e1)
        v = (q @ d) * inv
        t = np.einsum("ij,ij->i", e2, q) * inv
        hit = ok & (u >= 0) & (v >= 0) & (u + v <= 1) & (t >= rays["tmin"][r]) & (t <= rays["tmax"][r])
        if hit.any():
            k = np.argmin(np.where(hit, t, np.inf))
            out_t[r], out_p[r] = t[k], k
    return out_t, out_p


def random_rays(rng, aabb, n, tmin=1e-3, tmax=1e30):
    lo, hi = np.asarray(aabb[:3]), np.asarray(aabb[3:])
    rays = np.zeros(n, dtype=np.dtype([("org", "<f4", (3,)), ("tmin", "<f4"), ("dir", "<f4", (3,)),
                                       ("tmax", "<f4")]))
    rays["org"] = lo + (hi - lo) * rng.random((n, 3))
    d = rng.normal(size=(n, 3))
    rays["dir"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays["tmin"], rays["tmax"] = tmin, tmax
    return rays


def test_cornell_scene_contents(pkg, abi):
    sc = pkg.Scene.cornell(64, 48, ico_level=3)
    i = sc.info()
    assert i.n_spheres == 0 and i.n_triangles > 12 and i.n_lights == 1
    assert i.camera.width == 64 and i.camera.height == 48
    exp = sc.export()
    types = set(exp["mats"]["type"].tolist())
    assert {abi.PG_MAT_DIFFUSE, abi.PG_MAT_LIGHT, abi.PG_MAT_DIELECTRIC} <= types
    lo, hi = np.array(i.aabb[:3]), np.array(i.aabb[3:])
    assert np.allclose(lo, exp["pos"].min(0)) and np.allclose(hi, exp["pos"].max(0))
    check_bvh(exp)


@pytest.mark.parametrize("grid", [0, 1, 16, 64])
def test_plates_scene_bvh(pkg, grid):
    sc = pkg.Scene.plates(32, 18, occluder_grid=grid, seed=3)
    i = sc.info()
    assert i.n_lights == 4 and i.n_spheres == 4
    check_bvh(sc.export())


def test_bvh_closest_matches_brute_force(pkg, tracer):
    sc = pkg.Scene.plates(32, 18, occluder_grid=12, seed=5)
    exp = sc.export()
    rng = np.random.default_rng(11)
    rays = random_rays(rng, exp["info"].aabb, 600)
    hits = tracer.closest(exp, rays, threads=2)
    bt, bp = brute_closest(exp, rays)
    tri = hits["prim"] & np.uint32(0x80000000) == 0
    tri &= hits["prim"] != 0xFFFFFFFF
    # spheres are not in the brute force: take rays whose BVH hit is a
    # triangle or a miss, and whose brute-force hit is nearer than any sphere
    sph = (hits["prim"] != 0xFFFFFFFF) & ~tri
    sel = ~sph
    agree = np.where(tri[sel], hits["prim"][sel] == bp[sel], bp[sel] == 0xFFFFFFFF)
    assert agree.mean() > 0.995, f"prim agreement {agree.mean():.4f}"
    both = sel & tri & (hits["prim"] == bp)
    assert np.allclose(hits["t"][both], bt[both], rtol=1e-4, atol=1e-5)


def test_any_hit_consistent_with_closest(pkg, tracer):
    sc = pkg.Scene.cornell(32, 24, ico_level=3)
    exp = sc.export()
    rng = np.random.default_rng(3)
    rays = random_rays(rng, exp["info"].aabb, 4000)
    rays["tmax"] = rng.uniform(0.01, 3.0, size=rays.shape[0])
    hits = tracer.closest(exp, rays, threads=2)
    occ = tracer.any(exp, rays, threads=2)
    assert np.array_equal(occ.astype(bool), hits["prim"] != 0xFFFFFFFF)


def test_empty_and_degenerate_rays(pkg, tracer):
    sc = pkg.Scene.cornell(16, 16, ico_level=1)
    exp = sc.export()
    rays = random_rays(np.random.default_rng(0), exp["info"].aabb, 8)
    rays["tmax"][:4] = 0.0005  # tmax < tmin: nothing can be hit
    hits = tracer.closest(exp, rays, threads=1)
    assert (hits["prim"][:4] == 0xFFFFFFFF).all()
    assert tracer.closest(exp, rays[:0]).shape == (0,)


MITSUBA = """<?xml version="1.0" encoding="utf-8"?>
<scene version="0.5.0">
  <sensor type="perspective">
    <float name="fov" value="40"/>
    <transform name="toWorld">
      <lookAt origin="0, 1, 6" target="0, 1, 0" up="0, 1, 0"/>
    </transform>
  </sensor>
  <bsdf type="twosided" id="white">
    <bsdf type="diffuse"><rgb name="reflectance" value="0.7, 0.6, 0.5"/></bsdf>
  </bsdf>
  <bsdf type="roughconductor" id="metal">
    <string name="distribution" value="beckmann"/><float name="alpha" value="0.2"/>
    <spectrum name="eta" value="0.370"/><spectrum name="k" value="2.820"/>
  </bsdf>
  <bsdf type="phong" id="plastic">
    <rgb name="diffuseReflectance" value="0.3, 0.4, 0.5"/><rgb name="specularReflectance" value="0.2, 0.2, 0.2"/>
    <float name="exponent" value="40"/>
  </bsdf>
  <shape type="obj">
    <string name="filename" value="quad.obj"/>
    <ref id="white"/>
  </shape>
  <shape type="cube">
    <transform name="toWorld"><scale value="0.5"/><translate x="0" y="0.5" z="0"/></transform>
    <ref id="metal"/>
  </shape>
  <shape type="sphere">
    <point name="center" x="1" y="2" z="0"/>
    <float name="radius" value="0.25"/>
    <bsdf type="dielectric"><float name="intIOR" value="1.596"/><float name="extIOR" value="1.2"/></bsdf>
  </shape>
  <shape type="sphere">
    <point name="center" x="-1.2" y="0.6" z="0.5"/>
    <float name="radius" value="0.5"/>
    <bsdf type="conductor"><spectrum name="eta" value="0.2"/><spectrum name="k" value="3.9"/></bsdf>
  </shape>
  <shape type="sphere">
    <point name="center" x="1.3" y="0.4" z="0.8"/>
    <float name="radius" value="0.4"/>
    <bsdf type="conductor"><string name="material" value="none"/></bsdf>
  </shape>
  <shape type="rectangle">
    <transform name="toWorld"><rotate x="1" angle="90"/><translate x="0" y="1" z="-2"/></transform>
    <ref id="plastic"/>
  </shape>
  <shape type="rectangle">
    <transform name="toWorld"><translate x="0" y="3" z="0"/></transform>
    <emitter type="area"><rgb name="radiance" value="10, 9, 8"/></emitter>
  </shape>
</scene>
"""

QUAD_OBJ = """# floor
v -2 0 -2
v 2 0 -2
v 2 0 2
v -2 0 2
vn 0 1 0
f 1//1 2//1 3//1 4//1
"""


def test_mitsuba_loader(pkg, abi, tmp_path):
    (tmp_path / "quad.obj").write_text(QUAD_OBJ)
    (tmp_path / "scene.xml").write_text(MITSUBA)
    sc = pkg.Scene.load(tmp_path / "scene.xml", 40, 30)
    i = sc.info()
    assert i.n_triangles == 2 + 12 + 2 + 2 and i.n_spheres == 3 and i.n_lights == 1
    cam = i.camera
    assert (cam.width, cam.height) == (40, 30) and abs(cam.vfov_deg - 40) < 1e-6
    assert list(cam.origin) == [0, 1, 6] and list(cam.target) == [0, 1, 0]
    exp = sc.export()
    mats = exp["mats"]
    by_type = {int(t): m for t, m in zip(mats["type"], mats)}
    assert np.allclose(by_type[abi.PG_MAT_DIFFUSE]["albedo"], [0.7, 0.6, 0.5])
    metal = by_type[abi.PG_MAT_BECKMANN]  # roughconductor: the reference's Beckmann conductor
    assert abs(metal["roughness"] - 0.2) < 1e-7 and abs(metal["eta"] - 0.37) < 1e-7 and abs(metal["k"] - 2.82) < 1e-6
    phong = by_type[abi.PG_MAT_PHONG]
    assert np.allclose(phong["albedo"], [0.3, 0.4, 0.5]) and np.allclose(phong["specular"], 0.2)
    assert phong["exponent"] == 40
    cond = by_type[abi.PG_MAT_CONDUCTOR]
    assert abs(cond["eta"] - 0.2) < 1e-7 and abs(cond["k"] - 3.9) < 1e-6
    assert abi.PG_MAT_SPECULAR in by_type  # conductor with material "none": a mirror
    assert abs(by_type[abi.PG_MAT_DIELECTRIC]["ior"] - 1.596 / 1.2) < 1e-6  # intIOR / extIOR
    assert np.allclose(by_type[abi.PG_MAT_LIGHT]["emission"], [10, 9, 8])
    assert np.allclose(exp["spheres"]["center"][0], [1, 2, 0]) and abs(exp["spheres"]["radius"][0] - 0.25) < 1e-7
    # the unit cube scaled by 0.5 and lifted by 0.5 spans [-0.5, 0.5] x [0, 1] x [-0.5, 0.5]
    cube = exp["pos"][exp["idx"][exp["tri_mat"] == int(np.where(mats["type"] == abi.PG_MAT_BECKMANN)[0][0])]].reshape(-1, 3)
    assert np.allclose(cube.min(0), [-0.5, 0.0, -0.5]) and np.allclose(cube.max(0), [0.5, 1.0, 0.5])
    check_bvh(exp)


@pytest.mark.parametrize("text,status", [
    (None, "PG_ERR_IO"),
    ("<scene><shape type='obj'>", "PG_ERR_PARSE"),
    ("<notascene/>", "PG_ERR_PARSE"),
    ("<scene><shape type='torus'/></scene>", "PG_ERR_PARSE"),
    ("<scene><shape type='sphere'><ref id='nope'/></shape></scene>", "PG_ERR_PARSE"),
    ("<scene><shape type='obj'/></scene>", "PG_ERR_PARSE"),
    ("<scene><shape type='obj'><string name='filename' value='missing.obj'/></shape></scene>", "PG_ERR_IO"),
    ("<scene></scene>", "PG_ERR_PARSE"),
])
def test_mitsuba_loader_errors(pkg, abi, tmp_path, text, status):
    path = tmp_path / "bad.xml"
    if text is not None:
        path.write_text(text)
    with pytest.raises(pkg.PathGuideError) as e:
        pkg.Scene.load(path, 8, 8)
    assert e.value.status == getattr(abi, status), str(e.value)


def test_render_argument_errors(pkg, abi):
    sc = pkg.Scene.cornell(8, 8, ico_level=1)
    fake_image = 0x1000  # never touched: every case fails its checks first
    bad = [abi.render_params(max_depth=0), abi.render_params(max_depth=65),
           abi.render_params(use_guiding=1), abi.render_params(record_samples=1)]
    for p in bad:
        with pytest.raises(pkg.PathGuideError) as e:
            sc.render(p, fake_image)
        assert e.value.status == abi.PG_ERR_ARG
    lib = pkg.library()
    assert lib.pg_render(None, C.byref(abi.render_params()), None, fake_image, None, None, None) == abi.PG_ERR_ARG
    with pytest.raises(pkg.PathGuideError):
        pkg.Scene.cornell(0, 8)
    with pytest.raises(pkg.PathGuideError):
        pkg.Scene.plates(8, 8, occluder_grid=5000)
