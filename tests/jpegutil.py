"""Baseline JPEG writer for the texture tests (sequential DCT, Huffman coding
with the test's own flat code tables, optional restart intervals and 2 x 2
luma sampling), and the pixels a conforming decoder must produce from the
quantised coefficients it wrote (float64 inverse DCT, chroma replicated,
JFIF YCbCr -> RGB)."""
from __future__ import annotations

import struct

import numpy as np

ZIGZAG = np.array([0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13,
                   6, 7, 14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59, 52, 45,
                   38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63])
_C = np.array([[(np.sqrt(0.5) if u == 0 else 1.0) * 0.5 * np.cos((2 * x + 1) * u * np.pi / 16) for u in range(8)]
               for x in range(8)])  # C[x, u]

# code tables: DC categories 0..11 all of length 4; AC: EOB, ZRL and every run/size, all of length 8
DC_SYMS = list(range(12))
AC_SYMS = [0x00, 0xF0] + [(r << 4) | s for r in range(16) for s in range(1, 11)]


def _table(symbols, length):
    counts = [0] * 16
    counts[length - 1] = len(symbols)
    codes = {s: (i, length) for i, s in enumerate(symbols)}
    return bytes(counts) + bytes(symbols), codes


DC_TABLE, DC_CODES = _table(DC_SYMS, 4)
AC_TABLE, AC_CODES = _table(AC_SYMS, 8)


class _Writer:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, v, n):
        for i in range(n - 1, -1, -1):
            self.acc = (self.acc << 1) | ((v >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc = self.n = 0

    def flush(self):
        while self.n:
            self.put(1, 1)


def _cat(v):
    return 0 if v == 0 else int(abs(v)).bit_length()


def _bits(v, s):
    return v if v >= 0 else v + (1 << s) - 1


def _fdct(block):
    return _C.T @ block @ _C  # F[v, u] for samples f[y, x]


def _seg(marker, body):
    return bytes([0xFF, marker]) + struct.pack(">H", len(body) + 2) + body


def write_jpeg(planes, sampling, quant, restart=0):
    """planes: list of 2-D uint8 arrays (Y or Y, Cb, Cr) at full size; sampling:
    (h, v) per component; quant: 64-entry tables (natural order) per component.
    Returns (jpeg bytes, decoded planes the decoder must reproduce)."""
    H, W = planes[0].shape
    hmax, vmax = max(s[0] for s in sampling), max(s[1] for s in sampling)
    mx, my = -(-W // (8 * hmax)), -(-H // (8 * vmax))
    comps = []
    for p, (h, v) in zip(planes, sampling):
        # the component's samples: full-resolution plane averaged over its subsampling box
        fy, fx = vmax // v, hmax // h
        Hc, Wc = my * v * 8, mx * h * 8
        full = np.pad(p.astype(np.float64), ((0, Hc * fy - H), (0, Wc * fx - W)), mode="edge")
        comps.append(full.reshape(Hc, fy, Wc, fx).mean(axis=(1, 3)))
    coefs = []  # per component: blocks (by, bx) of quantised natural-order coefficients
    recon = []
    for c, q in zip(comps, quant):
        bh, bw = c.shape[0] // 8, c.shape[1] // 8
        qc = np.zeros((bh, bw, 8, 8), dtype=np.int64)
        rc = np.zeros_like(c)
        for by in range(bh):
            for bx in range(bw):
                F = _fdct(c[by * 8:by * 8 + 8, bx * 8:bx * 8 + 8] - 128.0)
                qq = np.round(F / q.reshape(8, 8)).astype(np.int64)
                qc[by, bx] = qq
                rc[by * 8:by * 8 + 8, bx * 8:bx * 8 + 8] = np.clip(np.round(_C @ (qq * q.reshape(8, 8)) @ _C.T + 128.0), 0, 255)
        coefs.append(qc)
        recon.append(rc.astype(np.uint8))
    w = _Writer()
    preds = [0] * len(planes)
    count = 0
    rst = 0
    for y in range(my):
        for x in range(mx):
            if restart and count == restart:
                w.flush()
                w.out += bytes([0xFF, 0xD0 + rst])
                rst = (rst + 1) % 8
                preds = [0] * len(planes)
                count = 0
            count += 1
            for ci, (h, v) in enumerate(sampling):
                for vv in range(v):
                    for hh in range(h):
                        blk = coefs[ci][y * v + vv, x * h + hh].reshape(-1)[ZIGZAG]
                        d = int(blk[0]) - preds[ci]
                        preds[ci] = int(blk[0])
                        s = _cat(d)
                        w.put(*DC_CODES[s])
                        if s:
                            w.put(_bits(d, s), s)
                        run = 0
                        last = max([k for k in range(1, 64) if blk[k] != 0], default=0)
                        for k in range(1, last + 1):
                            a = int(blk[k])
                            if a == 0:
                                run += 1
                                continue
                            while run >= 16:
                                w.put(*AC_CODES[0xF0])
                                run -= 16
                            s = _cat(a)
                            w.put(*AC_CODES[(run << 4) | s])
                            w.put(_bits(a, s), s)
                            run = 0
                        if last < 63:
                            w.put(*AC_CODES[0x00])
    w.flush()
    out = bytearray(b"\xff\xd8")
    out += _seg(0xE0, b"JFIF\0\x01\x01\0\0\x01\0\x01\0\0")
    for i, q in enumerate(quant):
        out += _seg(0xDB, bytes([i]) + bytes(np.asarray(q, dtype=np.uint8)[ZIGZAG]))
    sof = struct.pack(">BHHB", 8, H, W, len(planes))
    for i, (h, v) in enumerate(sampling):
        sof += bytes([i + 1, (h << 4) | v, i])
    out += _seg(0xC0, sof)
    out += _seg(0xC4, bytes([0x00]) + DC_TABLE) + _seg(0xC4, bytes([0x10]) + AC_TABLE)
    if restart:
        out += _seg(0xDD, struct.pack(">H", restart))
    sos = bytes([len(planes)]) + b"".join(bytes([i + 1, 0x00]) for i in range(len(planes))) + bytes([0, 63, 0])
    out += _seg(0xDA, sos) + bytes(w.out) + b"\xff\xd9"
    # decoded pixels: components replicated to full resolution, then YCbCr -> RGB
    rgba = np.full((H, W, 4), 255, dtype=np.uint8)
    full = []
    for rc, (h, v) in zip(recon, sampling):
        fy, fx = vmax // v, hmax // h
        full.append(np.repeat(np.repeat(rc, fy, axis=0), fx, axis=1)[:H, :W].astype(np.float64))
    if len(full) == 1:
        rgba[..., :3] = full[0][..., None]
    else:
        Y, cb, cr = full[0], full[1] - 128.0, full[2] - 128.0
        rgb = np.stack([Y + 1.402 * cr, Y - 0.344136 * cb - 0.714136 * cr, Y + 1.772 * cb], -1)
        rgba[..., :3] = np.clip(np.round(rgb), 0, 255)
    return bytes(out), rgba
