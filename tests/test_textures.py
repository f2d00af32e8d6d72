"""Textures on the host: the PNG decoder (every colour type and scanline
filter, against the pixels the test encoded), Mitsuba bitmap textures with a
texture-referencing diffuse BSDF (src/SceneLoader.cpp:515-587), OBJ texture
coordinates with the reference's v flip (:288-291), and the texture id each
BVH triangle carries for the alpha test."""
from __future__ import annotations

import numpy as np
import pytest

from pngutil import expected_rgba, leaf_texture, png_bytes, write_texture_scene


@pytest.mark.parametrize("ctype", [0, 2, 3, 4, 6])
def test_png_colour_types_and_filters(ctype, pkg, tmp_path):
    rng = np.random.default_rng(ctype)
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    h, w = 13, 17
    palette = trns = None
    if ctype == 3:
        palette = rng.integers(0, 256, size=(20, 3))
        trns = rng.integers(0, 256, size=7)
        px = rng.integers(0, 20, size=(h, w, 1)).astype(np.uint8)
    else:
        px = rng.integers(0, 256, size=(h, w, ch)).astype(np.uint8)
    path = tmp_path / f"t{ctype}.png"
    path.write_bytes(png_bytes(px, ctype, palette, trns))
    got = pkg.read_png(path)
    np.testing.assert_array_equal(got, expected_rgba(px, ctype, palette, trns))


def test_png_errors(pkg, abi, tmp_path):
    good = png_bytes(np.zeros((2, 2, 4), np.uint8), 6)
    cases = {
        "sig.png": b"notapng" + good[7:],
        "trunc.png": good[:40],
        "bits16.png": good[:24] + bytes([16]) + good[25:],  # IHDR bit depth (the CRC is not checked)
    }
    for name, data in cases.items():
        (tmp_path / name).write_bytes(data)
        with pytest.raises(pkg.PathGuideError):
            pkg.read_png(tmp_path / name)
    with pytest.raises(pkg.PathGuideError) as e:
        pkg.read_png(tmp_path / "missing.png")
    assert e.value.status == abi.PG_ERR_IO


def test_mitsuba_bitmap_texture(pkg, abi, tmp_path):
    write_texture_scene(tmp_path)
    sc = pkg.Scene.load(tmp_path / "scene.xml", 32, 24)
    exp = sc.export()
    mats = exp["mats"]
    tex_mats = np.where(mats["texture"] > 0)[0]
    assert len(tex_mats) == 1
    m = mats[tex_mats[0]]
    assert m["type"] == abi.PG_MAT_DIFFUSE and np.allclose(m["albedo"], 1.0) and m["texture"] == 1
    assert exp["tex_info"].shape == (1, 4) and list(exp["tex_info"][0][:3]) == [0, 32, 32]
    np.testing.assert_array_equal(exp["tex_data"].reshape(32, 32, 4), leaf_texture())
    # the textured quad's two triangles carry (u, 1 - v) of their corners
    tri = np.where(exp["tri_mat"] == tex_mats[0])[0]
    assert len(tri) == 2
    uv = exp["tri_uv"][tri].reshape(-1, 3, 2)
    assert np.allclose(uv[0], [[0, 1], [1, 1], [1, 0]]) and np.allclose(uv[1], [[0, 1], [1, 0], [0, 0]])
    # the BVH triangles of that material carry the texture id in v1.w, all others 0
    tex_bits = exp["tri_verts"][:, 7].view(np.uint32)
    ids = exp["tri_verts"][:, 3].view(np.uint32)
    assert (tex_bits[np.isin(ids, tri)] == 1).all() and (tex_bits[~np.isin(ids, tri)] == 0).all()


def test_unreadable_textures_are_reported(pkg, abi, tmp_path):
    write_texture_scene(tmp_path)
    (tmp_path / "trunc.jpg").write_bytes(b"\xff\xd8\xff\xe0" + b"\0" * 64)
    (tmp_path / "prog.jpg").write_bytes(b"\xff\xd8\xff\xc2\x00\x11" + b"\x08" + b"\0" * 16)
    (tmp_path / "junk.tga").write_bytes(b"\0" * 64)
    for name, words in (("trunc.jpg", "JPEG"), ("prog.jpg", "progressive"), ("junk.tga", "PNG")):
        text = (tmp_path / "scene.xml").read_text()
        (tmp_path / "s2.xml").write_text(text.replace("leaf.png", name))
        with pytest.raises(pkg.PathGuideError) as e:
            pkg.Scene.load(tmp_path / "s2.xml", 8, 8)
        assert words in str(e.value), str(e.value)


@pytest.mark.parametrize("mode", ["grey", "444", "420", "420_restart"])
def test_jpeg_baseline(mode, pkg, tmp_path):
    """Baseline JPEG decoding against the pixels the test's own encoder implies:
    at most one level off (float IDCT and colour rounding), almost always exact."""
    from jpegutil import write_jpeg
    rng = np.random.default_rng(len(mode))
    H, W = 37, 53  # partial MCUs on both edges
    y, x = np.mgrid[0:H, 0:W]
    Y = np.clip(128 + 80 * np.sin(x / 5.0) * np.cos(y / 7.0) + rng.normal(0, 6, (H, W)), 0, 255).astype(np.uint8)
    Cb = np.clip(128 + 40 * np.cos(x / 9.0), 0, 255).astype(np.uint8)
    Cr = np.clip(128 + 30 * np.sin(y / 6.0), 0, 255).astype(np.uint8)
    u, v = np.meshgrid(np.arange(8), np.arange(8))
    ql, qc = (1 + (u + v)).reshape(-1), (2 + 2 * (u + v)).reshape(-1)
    if mode == "grey":
        data, want = write_jpeg([Y], [(1, 1)], [ql])
    elif mode == "444":
        data, want = write_jpeg([Y, Cb, Cr], [(1, 1)] * 3, [ql, qc, qc])
    else:
        data, want = write_jpeg([Y, Cb, Cr], [(2, 2), (1, 1), (1, 1)], [ql, qc, qc],
                                restart=3 if mode.endswith("restart") else 0)
    (tmp_path / "t.jpg").write_bytes(data)
    # through a scene texture (the decoder is reached by signature)
    write_texture_scene(tmp_path)
    (tmp_path / "scene.xml").write_text((tmp_path / "scene.xml").read_text().replace("leaf.png", "t.jpg"))
    sc = pkg.Scene.load(tmp_path / "scene.xml", 8, 8)
    exp = sc.export()
    assert list(exp["tex_info"][0][1:3]) == [W, H]
    got = exp["tex_data"].reshape(H, W, 4).astype(np.int32)
    diff = np.abs(got - want.astype(np.int32))
    assert diff.max() <= 1 and (diff > 0).mean() < 0.02, (diff.max(), (diff > 0).mean())
