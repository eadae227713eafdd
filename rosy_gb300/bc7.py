"""BC7 blocks on the host: field packing, seeded blocks of every mode, and a
simple encoder for synthetic assets.

The engine's assets arrive BC7-compressed from its offline packager (NVTT, out
of scope here); the renderer decodes them on the device (rz_bc7_decode, and
rz_set_asset for RZ_TEXELS_BC7 textures). This module makes BC7 data to feed
that path: `blocks_of_mode` builds valid blocks of one mode with the partition,
rotation and index-selection fields stepped through their values and every
other bit random, and `encode` compresses RGBA8 images with the single-subset
mode 6 (endpoints along each block's principal axis, 4-bit indices) — enough
for test and benchmark textures, not an optimising encoder.
"""
from __future__ import annotations

import numpy as np

from . import _abi
from . import scene as sc

# Per mode: subsets, partition bits, rotation bits, index-selection bits, colour
# bits, alpha bits, P-bits kind (0 none, 1 per endpoint, 2 per subset), index
# bits, secondary index bits.
MODES = [
    (3, 4, 0, 0, 4, 0, 1, 3, 0), (2, 6, 0, 0, 6, 0, 2, 3, 0), (3, 6, 0, 0, 5, 0, 0, 2, 0), (2, 6, 0, 0, 7, 0, 1, 2, 0),
    (1, 0, 2, 1, 5, 6, 0, 2, 3), (1, 0, 2, 0, 7, 8, 0, 2, 2), (1, 0, 0, 0, 7, 7, 1, 4, 0), (2, 6, 0, 0, 5, 5, 1, 2, 0),
]
WEIGHTS4 = np.array([0, 4, 9, 13, 17, 21, 26, 30, 34, 38, 43, 47, 51, 55, 60, 64], np.int32)


def chain_blocks(width: int, height: int, levels: int) -> list[tuple[int, int]]:
    """(blocks per row, block rows) of every level of a mip chain."""
    out = []
    for l in range(levels):
        w, h = max(1, width >> l), max(1, height >> l)
        out.append((max(1, (w + 3) // 4), max(1, (h + 3) // 4)))
    return out


def chain_bytes(width: int, height: int, levels: int) -> int:
    return sum(bw * bh * 16 for bw, bh in chain_blocks(width, height, levels))


def _to_bytes(values: list[int]) -> np.ndarray:
    return np.frombuffer(b"".join(v.to_bytes(16, "little") for v in values), np.uint8).reshape(-1, 16).copy()


def blocks_of_mode(rng: np.random.Generator, mode: int, n: int) -> np.ndarray:
    """(n, 16) uint8 blocks of `mode` (0-7; 8 = the reserved mode, first byte 0):
    block i has partition i mod 2^pb, rotation i mod 2^rb and index selection
    (i >> 2) mod 2^isb; every other bit is random."""
    raw = rng.integers(0, 256, (n, 16), dtype=np.uint8)
    if mode == 8:
        raw[:, 0] = 0
        return raw
    ns, pb, rb, isb = MODES[mode][:4]
    vals = []
    for i in range(n):
        v = int.from_bytes(raw[i].tobytes(), "little")
        pos = mode + 1
        v = (v >> pos << pos) | (1 << mode)  # mode prefix: `mode` zero bits, then a one
        fields = [(pb, i % (1 << pb) if pb else 0), (rb, i % (1 << rb) if rb else 0),
                  (isb, (i >> 2) % (1 << isb) if isb else 0)]
        for bits, val in fields:
            if bits:
                v = (v & ~(((1 << bits) - 1) << pos)) | (val << pos)
                pos += bits
        vals.append(v)
    return _to_bytes(vals)


def mixed_blocks(rng: np.random.Generator, n: int) -> np.ndarray:
    """(n, 16) blocks cycling through modes 0-7 (partitions and fields stepped as in blocks_of_mode)."""
    per = [blocks_of_mode(rng, m, (n + 7) // 8) for m in range(8)]
    out = np.empty((n, 16), np.uint8)
    for i in range(n):
        out[i] = per[i % 8][i // 8]
    return out


def _quantize_endpoint(p: np.ndarray) -> tuple[np.ndarray, int]:
    """An RGBA point as 7-bit channels and one P-bit: the (value << 1) | p nearest to it."""
    best = None
    for pbit in (0, 1):
        e = np.clip(np.rint((p - pbit) / 2.0), 0, 127).astype(np.int32)
        err = float((((e << 1) | pbit) - p) @ (((e << 1) | pbit) - p))
        if best is None or err < best[0]:
            best = (err, e, pbit)
    return best[1], best[2]


def _encode_block(px: np.ndarray) -> int:
    """Mode 6 block of 16 RGBA8 texels (16, 4): the endpoints are the extremes of
    the texels along their principal axis (7 bits + a P-bit each), the indices
    the nearest of the 16 weights along the quantized endpoint line."""
    f = px.astype(np.float64)
    mean = f.mean(0)
    c = f - mean
    _, vecs = np.linalg.eigh(c.T @ c)
    axis = vecs[:, -1]
    t = c @ axis
    e0, p0 = _quantize_endpoint(np.clip(mean + t.min() * axis, 0, 255))
    e1, p1 = _quantize_endpoint(np.clip(mean + t.max() * axis, 0, 255))
    q0 = (e0 << 1) | p0
    q1 = (e1 << 1) | p1
    d = (q1 - q0).astype(np.float64)
    dd = float((d * d).sum())
    if dd > 0:
        t = ((px.astype(np.float64) - q0) @ d) / dd
    else:
        t = np.zeros(16)
    idx = np.abs(t[:, None] * 64.0 - WEIGHTS4[None, :]).argmin(1)
    if idx[0] >= 8:  # texel 0's index is stored with 3 bits: swap the endpoints
        e0, e1, p0, p1 = e1, e0, p1, p0
        idx = 15 - idx
    v, pos = 1 << 6, 7
    for ch in range(4):
        for e in (e0, e1):
            v |= int(e[ch]) << pos
            pos += 7
    v |= p0 << pos
    v |= p1 << (pos + 1)
    pos += 2
    for i in range(16):
        bits = 3 if i == 0 else 4
        v |= int(idx[i]) << pos
        pos += bits
    assert pos == 128
    return v


def encode(rgba: np.ndarray) -> np.ndarray:
    """(H, W, 4) uint8 image -> (ceil(H/4) * ceil(W/4), 16) BC7 mode-6 blocks in rows
    (edge blocks repeat the last row / column)."""
    h, w = rgba.shape[:2]
    bh, bw = max(1, (h + 3) // 4), max(1, (w + 3) // 4)
    ys = np.minimum(np.arange(bh * 4), h - 1)
    xs = np.minimum(np.arange(bw * 4), w - 1)
    padded = rgba[ys][:, xs]
    vals = []
    for by in range(bh):
        for bx in range(bw):
            vals.append(_encode_block(padded[4 * by:4 * by + 4, 4 * bx:4 * bx + 4].reshape(16, 4)))
    return _to_bytes(vals)


def texture_to_bc7(t: sc.Texture) -> sc.Texture:
    """An RGBA8 scene texture compressed level by level (mode 6)."""
    assert t.format == _abi.TEXELS_RGBA8
    chunks, off = [], 0
    for l in range(t.levels):
        w, h = max(1, t.width >> l), max(1, t.height >> l)
        lvl = t.texels[off:off + w * h * 4].reshape(h, w, 4)
        chunks.append(encode(lvl).reshape(-1))
        off += w * h * 4
    return sc.Texture(t.width, t.height, t.levels, t.image_type, np.concatenate(chunks), _abi.TEXELS_BC7)


def random_texture(rng: np.random.Generator, width: int, height: int, levels: int, image_type: int) -> sc.Texture:
    """A BC7 texture whose blocks cycle through every mode (mixed_blocks)."""
    n = chain_bytes(width, height, levels) // 16
    return sc.Texture(width, height, levels, image_type, mixed_blocks(rng, n).reshape(-1), _abi.TEXELS_BC7)
