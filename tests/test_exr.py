"""OpenEXR images (pg_exr_read / pg_exr_write, the reference's readEXR /
writeEXR, src/CommonOps.cpp:12-65) and the envmap emitter of Mitsuba files.
The reader's ZIP path (a project-written inflate) is checked against files
compressed here with Python's zlib, and, where the reference tree is present,
against the reference's own scene images decoded with Python's zlib."""
from __future__ import annotations

import glob
import os
import struct
import zlib
from pathlib import Path

import numpy as np
import pytest

REF_SCENES = "/root/reference/scenes"


def exr_header(data: bytes):
    pos, attrs = 8, {}
    while True:
        end = data.index(b"\0", pos)
        name = data[pos:end].decode()
        pos = end + 1
        if not name:
            break
        end = data.index(b"\0", pos)
        typ = data[pos:end].decode()
        pos = end + 1
        size, = struct.unpack("<i", data[pos:pos + 4])
        attrs[name] = (typ, data[pos + 4:pos + 4 + size])
        pos += 4 + size
    ch, chans, p = attrs["channels"][1], [], 0
    while ch[p] != 0:
        e = ch.index(b"\0", p)
        nm = ch[p:e].decode()
        pt, = struct.unpack("<i", ch[p + e - p + 1:e + 5])
        chans.append((nm, pt))
        p = e + 17
    return attrs, chans, pos


def decode_exr_python(path):
    """An independent ZIP / ZIPS / NONE decoder over Python's zlib."""
    data = open(path, "rb").read()
    attrs, chans, pos = exr_header(data)
    comp = attrs["compression"][1][0]
    x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"][1])
    W, H = x1 - x0 + 1, y1 - y0 + 1
    lines = {0: 1, 2: 1, 3: 16}[comp]
    nchunks = (H + lines - 1) // lines
    offsets = struct.unpack(f"<{nchunks}Q", data[pos:pos + 8 * nchunks])
    size_of = {0: 4, 1: 2, 2: 4}
    row = sum(W * size_of[t] for _, t in chans)
    img = np.zeros((H, W, 3), dtype=np.float32)
    for off in offsets:
        y, n = struct.unpack("<ii", data[off:off + 8])
        raw = data[off + 8:off + 8 + n]
        nl = min(lines, H - (y - y0))
        if n != row * nl:
            t = np.frombuffer(zlib.decompress(raw), dtype=np.uint8).astype(np.int32)
            t = (np.cumsum(t - 128) + 128) & 0xFF  # predictor: t[i] = t[i-1] + t[i] - 128 (mod 256)
            t[0] = np.frombuffer(zlib.decompress(raw), dtype=np.uint8)[0]
            t = t.astype(np.uint8)
            half = (t.size + 1) // 2
            out = np.empty_like(t)
            out[0::2] = t[:half]
            out[1::2] = t[half:]
            raw = out.tobytes()
        for l in range(nl):
            line, at = raw[row * l:row * (l + 1)], 0
            for name, typ in chans:
                dt = {0: "<u4", 1: "<f2", 2: "<f4"}[typ]
                v = np.frombuffer(line[at:at + W * size_of[typ]], dtype=dt).astype(np.float32)
                at += W * size_of[typ]
                c = {"R": 0, "G": 1, "B": 2}.get(name)
                if c is not None:
                    img[y - y0 + l, :, c] = v
    return img


def write_zip_exr(path, img, half=True, lines=16):
    """A ZIP (or ZIPS with lines=1) compressed EXR written with Python's zlib."""
    H, W, _ = img.shape
    typ, dt = (1, "<f2") if half else (2, "<f4")
    def attr(name, typ_, payload):
        return name.encode() + b"\0" + typ_.encode() + b"\0" + struct.pack("<i", len(payload)) + payload
    chl = b"".join(n.encode() + b"\0" + struct.pack("<i", typ) + b"\0\0\0\0" + struct.pack("<ii", 1, 1)
                   for n in ("B", "G", "R")) + b"\0"
    win = struct.pack("<iiii", 0, 0, W - 1, H - 1)
    head = struct.pack("<ii", 20000630, 2) + attr("channels", "chlist", chl) + \
        attr("compression", "compression", bytes([3 if lines == 16 else 2])) + attr("dataWindow", "box2i", win) + \
        attr("displayWindow", "box2i", win) + attr("lineOrder", "lineOrder", b"\0") + \
        attr("pixelAspectRatio", "float", struct.pack("<f", 1.0)) + \
        attr("screenWindowCenter", "v2f", struct.pack("<ff", 0, 0)) + \
        attr("screenWindowWidth", "float", struct.pack("<f", 1.0)) + b"\0"
    chunks = []
    for y in range(0, H, lines):
        nl = min(lines, H - y)
        raw = b"".join(img[y + l, :, c].astype(dt).tobytes() for l in range(nl) for c in (2, 1, 0))
        r = np.frombuffer(raw, dtype=np.uint8)
        half_n = (r.size + 1) // 2
        t = np.concatenate([r[0::2], r[1::2]]).astype(np.int32)  # interleave
        p = t.copy()
        p[1:] = (t[1:] - t[:-1] + 128) & 0xFF  # predictor
        assert half_n == r[0::2].size
        comp = zlib.compress(p.astype(np.uint8).tobytes(), 6)
        chunks.append(struct.pack("<ii", y, len(comp)) + comp)
    table, off = b"", len(head) + 8 * len(chunks)
    for c in chunks:
        table += struct.pack("<Q", off)
        off += len(c)
    open(path, "wb").write(head + table + b"".join(chunks))


def test_round_trip_float(pkg, tmp_path):
    rng = np.random.default_rng(1)
    img = (rng.random((37, 53, 3)) * 10).astype(np.float32)
    pkg.write_exr(tmp_path / "a.exr", img)
    back = pkg.read_exr(tmp_path / "a.exr")
    assert back.shape == img.shape and np.array_equal(back, img)
    np.testing.assert_array_equal(decode_exr_python(tmp_path / "a.exr"), img)


@pytest.mark.parametrize("half,lines", [(True, 16), (False, 16), (True, 1)])
def test_zip_compressed(pkg, tmp_path, half, lines):
    rng = np.random.default_rng(2)
    img = np.zeros((45, 61, 3), dtype=np.float32)
    img[..., 0] = np.linspace(0, 4, 61)[None, :]
    img[..., 1] = np.linspace(0, 1, 45)[:, None]
    img[..., 2] = rng.random((45, 61))
    if half:
        img = img.astype(np.float16).astype(np.float32)
    write_zip_exr(tmp_path / "z.exr", img, half=half, lines=lines)
    back = pkg.read_exr(tmp_path / "z.exr")
    np.testing.assert_array_equal(back, img)


def test_errors(pkg, tmp_path):
    with pytest.raises(pkg.PathGuideError) as e:
        pkg.read_exr(tmp_path / "missing.exr")
    assert e.value.status == pkg.abi.PG_ERR_IO
    (tmp_path / "bad.exr").write_bytes(b"not an exr file at all")
    with pytest.raises(pkg.PathGuideError):
        pkg.read_exr(tmp_path / "bad.exr")


@pytest.mark.skipif(not os.path.isdir(REF_SCENES), reason="reference scenes not present")
def test_reference_scene_images(pkg):
    files = sorted(glob.glob(os.path.join(REF_SCENES, "*", "*.exr")))[:6]
    assert files
    for f in files:
        got = pkg.read_exr(f)
        want = decode_exr_python(f)
        assert got.shape == want.shape and np.isfinite(got).all()
        np.testing.assert_array_equal(got, want, err_msg=f)


ENV_SCENE = """<?xml version="1.0" encoding="utf-8"?>
<scene version="0.5.0">
  <sensor type="perspective"><float name="fov" value="45"/>
    <transform name="toWorld"><lookAt origin="0, 1, 4" target="0, 1, 0" up="0, 1, 0"/></transform>
  </sensor>
  <shape type="sphere"><point name="center" x="0" y="1" z="0"/><float name="radius" value="0.8"/>
    <bsdf type="diffuse"><rgb name="reflectance" value="0.5, 0.5, 0.5"/></bsdf></shape>
  <emitter type="envmap"><string name="filename" value="sky.exr"/></emitter>
</scene>
"""


def sky(h=32, w=64):
    v = (np.arange(h) + 0.5) / h
    u = (np.arange(w) + 0.5) / w
    img = np.zeros((h, w, 3), dtype=np.float32)
    img[..., 2] = (1.0 - v)[:, None] * 1.5
    img[..., 1] = 0.6 * (1.0 - v)[:, None] + 0.1
    img[..., 0] = 0.3 + 0.2 * np.cos(2 * np.pi * u)[None, :]
    img[3:6, 10:14] = 40.0  # a sun
    return img


def test_envmap_emitter_loads(pkg, tmp_path):
    pkg.write_exr(tmp_path / "sky.exr", sky())
    (tmp_path / "scene.xml").write_text(ENV_SCENE)
    sc = pkg.Scene.load(tmp_path / "scene.xml", 32, 24)
    np.testing.assert_array_equal(sc.envmap(), sky())
    assert sc.info().n_lights == 1  # the environment
    assert "env" in sc.export()
    sc.set_envmap(None)
    assert sc.envmap() is None and sc.info().n_lights == 0
    (tmp_path / "scene2.xml").write_text(ENV_SCENE.replace("sky.exr", "none.exr"))
    with pytest.raises(pkg.PathGuideError) as e:
        pkg.Scene.load(tmp_path / "scene2.xml", 8, 8)
    assert e.value.status == pkg.abi.PG_ERR_IO


REF_SCENES = Path("/root/reference/scenes")


@pytest.mark.skipif(not (REF_SCENES / "envMap" / "envmap.exr").exists(), reason="reference scenes absent")
def test_piz_reference_envmap(pkg):
    """The reference's PIZ-compressed environment map (half RGB, 512 x 256): the
    decoded panorama was inspected (a gallery interior with windows); its
    checksum pins the decoder.  The scenes that use it load."""
    import hashlib
    a = pkg.read_exr(REF_SCENES / "envMap" / "envmap.exr")
    assert a.shape == (256, 512, 3) and np.isfinite(a).all() and a.min() >= 0.0
    assert hashlib.sha256(np.ascontiguousarray(a, dtype=np.float32).tobytes()).hexdigest() == \
        "b55a24c28fe07a55e325eaccd7b917c055c5cf8af09412421f4486d2d8807ba5"
    for name in ("envMap/envMap.xml", "testSpheres/testSpheres.xml"):
        sc = pkg.Scene.load(REF_SCENES / name, 32, 24)
        assert sc.envmap() is not None
        sc.close()
