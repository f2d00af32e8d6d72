"""PNG writer for the texture tests: explicit scanline filters (0-4) so the
decoder's unfiltering is exercised, zlib from Python's standard library."""
from __future__ import annotations

import struct
import zlib

import numpy as np


def _chunk(tag: bytes, body: bytes) -> bytes:
    return struct.pack(">I", len(body)) + tag + body + struct.pack(">I", zlib.crc32(tag + body) & 0xFFFFFFFF)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
    return np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))


def png_bytes(px: np.ndarray, ctype: int, palette=None, trns=None, filters=(0, 1, 2, 3, 4)) -> bytes:
    """px: (h, w, channels) uint8 for colour types 0 (1), 2 (3), 3 (1: indices),
    4 (2), 6 (4); row y uses filters[y % len(filters)]."""
    h, w, ch = px.shape
    bpp = ch
    raw = bytearray()
    prev = np.zeros(w * ch, dtype=np.int32)
    for y in range(h):
        row = px[y].reshape(-1).astype(np.int32)
        left = np.concatenate([np.zeros(bpp, np.int32), row[:-bpp]])
        upleft = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]])
        f = filters[y % len(filters)]
        if f == 0:
            out = row
        elif f == 1:
            out = row - left
        elif f == 2:
            out = row - prev
        elif f == 3:
            out = row - ((left + prev) >> 1)
        else:
            out = row - _paeth(left, prev, upleft)
        raw.append(f)
        raw.extend((out & 0xFF).astype(np.uint8).tobytes())
        prev = row
    ihdr = struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0)
    data = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", ihdr)
    if palette is not None:
        data += _chunk(b"PLTE", np.asarray(palette, dtype=np.uint8).reshape(-1).tobytes())
    if trns is not None:
        data += _chunk(b"tRNS", np.asarray(trns, dtype=np.uint8).tobytes())
    # two IDAT chunks: the decoder joins them
    z = zlib.compress(bytes(raw), 6)
    data += _chunk(b"IDAT", z[: len(z) // 2]) + _chunk(b"IDAT", z[len(z) // 2:]) + _chunk(b"IEND", b"")
    return data


def expected_rgba(px: np.ndarray, ctype: int, palette=None, trns=None) -> np.ndarray:
    h, w, _ = px.shape
    out = np.full((h, w, 4), 255, dtype=np.uint8)
    if ctype == 0:
        out[..., :3] = px[..., :1]
    elif ctype == 2:
        out[..., :3] = px
    elif ctype == 3:
        pal = np.asarray(palette, dtype=np.uint8).reshape(-1, 3)
        out[..., :3] = pal[px[..., 0]]
        if trns is not None:
            a = np.full(pal.shape[0], 255, dtype=np.uint8)
            a[: len(trns)] = trns
            out[..., 3] = a[px[..., 0]]
    elif ctype == 4:
        out[..., :3] = px[..., :1]
        out[..., 3] = px[..., 1]
    else:
        out[:] = px
    return out


# A floor quad with texture coordinates and an alpha-textured quad standing on
# it; the texture's alpha is a 4 x 4 checkerboard of 0 and 255 with a soft band.
TEXTURE_OBJ = """# textured quad in the plane z = 0, x in [-1, 1], y in [0, 2]
v -1 0 0
v 1 0 0
v 1 2 0
v -1 2 0
vt 0 0
vt 1 0
vt 1 1
vt 0 1
f 1/1 2/2 3/3 4/4
"""

FLOOR_OBJ = """# floor
v -3 0 -3
v 3 0 -3
v 3 0 3
v -3 0 3
f 1 2 3 4
"""

TEXTURE_SCENE = """<?xml version="1.0" encoding="utf-8"?>
<scene version="0.5.0">
  <sensor type="perspective">
    <float name="fov" value="45"/>
    <transform name="toWorld"><lookAt origin="0.3, 1.2, 4" target="0, 1, 0" up="0, 1, 0"/></transform>
  </sensor>
  <texture type="bitmap" id="leaf">
    <string name="filename" value="leaf.png"/>
  </texture>
  <bsdf type="diffuse" id="cutout"><ref name="reflectance" id="leaf"/></bsdf>
  <bsdf type="diffuse" id="grey"><rgb name="reflectance" value="0.6, 0.6, 0.6"/></bsdf>
  <shape type="obj"><string name="filename" value="quad.obj"/><ref id="cutout"/></shape>
  <shape type="obj"><string name="filename" value="floor.obj"/><ref id="grey"/></shape>
  <shape type="rectangle">
    <transform name="toWorld"><scale value="0.5"/><rotate x="1" angle="90"/><translate x="0" y="3" z="1"/></transform>
    <emitter type="area"><rgb name="radiance" value="20, 20, 20"/></emitter>
  </shape>
</scene>
"""


def leaf_texture(n: int = 32) -> np.ndarray:
    """RGBA: a colour gradient; alpha a 4 x 4 checkerboard (0 / 255) with
    intermediate values on one band of rows."""
    y, x = np.mgrid[0:n, 0:n]
    rgba = np.zeros((n, n, 4), dtype=np.uint8)
    rgba[..., 0] = (40 + 200 * x / (n - 1)).astype(np.uint8)
    rgba[..., 1] = (220 - 150 * y / (n - 1)).astype(np.uint8)
    rgba[..., 2] = 60
    rgba[..., 3] = np.where(((x * 4 // n) + (y * 4 // n)) % 2 == 0, 255, 0)
    rgba[n // 2: n // 2 + 3, :, 3] = np.linspace(0, 255, n).astype(np.uint8)
    return rgba


def write_texture_scene(dirpath) -> None:
    (dirpath / "quad.obj").write_text(TEXTURE_OBJ)
    (dirpath / "floor.obj").write_text(FLOOR_OBJ)
    (dirpath / "leaf.png").write_bytes(png_bytes(leaf_texture(), 6))
    (dirpath / "scene.xml").write_text(TEXTURE_SCENE)
