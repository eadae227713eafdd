"""CPU checks of the upsampler oracle (oracle/upsampler_ref.py): BF16 rounding,
the pixel-shuffle and bilinear conventions, the parameter layout shared with the
C ABI, and the backward formulas against central finite differences."""
import os
import re

import numpy as np

from oracle import upsampler_ref as U
from rosy_gb300 import upsampler as up

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _gbuffer(rng, H, W, sources=False):
    n = rng.normal(size=(H, W, 3))
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    s = np.abs(n).sum(-1, keepdims=True)
    oct_ = (n[..., :2] / s).astype(np.float16)
    gb = {
        "color": rng.integers(0, 256, (H, W, 4), dtype=np.uint8),
        "albedo": rng.integers(0, 256, (H, W, 4), dtype=np.uint8),
        "normal": oct_,
        "depth": rng.uniform(0.0, 0.3, (H, W)).astype(np.float32),
    }
    if sources:  # every mask value, 0xFFFF and 0 included
        gb["sources"] = rng.integers(0, 65536, (H, W), dtype=np.uint16)
        gb["sources"][0, 0], gb["sources"][0, 1] = 0xFFFF, 0
    return gb


def test_bf16_rounding_known_values():
    vals = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, 1.0 + 2.0 ** -9, -2.5, 0.0, 3.0e38], np.float32)
    want = np.array([1.0, 1.0, 1.0 + 2 * 2.0 ** -7, 1.0, -2.5, 0.0, 3.0e38], np.float32)
    got = U.bf16(vals)
    assert got[:6].tolist() == want[:6].tolist()
    # every output is a BF16 value (low 16 bits zero)
    assert np.all(got.view(np.uint32) & 0xFFFF == 0)


def test_parameter_layout_matches_header():
    hdr = open(os.path.join(ROOT, "include", "rosy_gb300.h")).read()
    n = int(re.search(r"#define RZ_UPSAMPLER_PARAM_COUNT (\d+)u", hdr).group(1))
    assert U.PARAM_COUNT == n == up.PARAM_COUNT
    assert U.OFFSETS == up.OFFSETS
    p = up.init_params(3)
    q = U.init_params(3)
    assert np.array_equal(p, q)
    w0 = p[U.OFFSETS[0][0]:U.OFFSETS[0][1]].reshape(32, 9, 16)
    assert np.all(w0[:, :, 14:] == 0) and np.all(w0[:, :, :14] != 0)
    w3 = p[U.OFFSETS[3][0]:U.OFFSETS[3][1]].reshape(16, 9, 32)
    assert np.all(w3[12:] == 0)


def test_x2_base_with_sub_pixel_sources():
    """Masks that keep every source (or none) give the bilinear base bit for bit;
    one kept source gives its colour; two give their renormalised mean."""
    rng = np.random.default_rng(4)
    c = rng.integers(0, 256, (5, 7, 4), dtype=np.uint8)
    bil = U.bilinear_base(c)
    assert np.array_equal(U.x2_base(c, np.full((5, 7), 0xFFFF, np.uint16)), bil)
    assert np.array_equal(U.x2_base(c, np.zeros((5, 7), np.uint16)), bil)
    assert np.array_equal(U.x2_base(c, None), bil)
    cf = c[..., :3].astype(np.float32) / np.float32(255.0)
    y, x = 2, 3
    m = np.full((5, 7), 0xFFFF, np.uint16)
    # point k = 1 (upper row, right half): sources own, right, up, up-right
    m[y, x] = (0xFFFF & ~(0xF << 4)) | (0b1000 << 4)  # only the up-right diagonal (weight 1/16, exact reciprocal)
    b = U.x2_base(c, m)
    assert np.array_equal(b[2 * y, 2 * x + 1], cf[y - 1, x + 1])
    m[y, x] = (0xFFFF & ~(0xF << 4)) | (0b0101 << 4)  # own and the one above
    b = U.x2_base(c, m, np.float64)
    want = (0.5625 * cf[y, x].astype(np.float64) + 0.1875 * cf[y - 1, x]) / 0.75
    assert np.allclose(b[2 * y, 2 * x + 1], want)
    # the feature channels carry the kept weight of each point
    gb = _gbuffer(rng, 5, 7, sources=True)
    f = U.features(gb, exact=True)
    assert f[0, 0, 10:14].tolist() == [1.0, 1.0, 1.0, 1.0] and f[0, 1, 10:14].tolist() == [0.0, 0.0, 0.0, 0.0]


def test_shuffle_and_bilinear_conventions():
    rng = np.random.default_rng(1)
    net = rng.normal(size=(3, 5, 12))
    full = U.shuffle(net)
    assert np.array_equal(U.unshuffle(full), net)
    # channel (2i + j) * 3 + k lands on pixel (2y + i, 2x + j)
    assert full[2 * 1 + 1, 2 * 2 + 0, 2] == net[1, 2, (2 * 1 + 0) * 3 + 2]
    flat = np.full((4, 6, 4), 77, np.uint8)
    assert np.all(U.bilinear_base(flat) == np.float32(77) / np.float32(255))
    c = rng.integers(0, 256, (4, 6, 4), dtype=np.uint8)
    b = U.bilinear_base(c, np.float64)
    cf = c[..., :3] / 255.0
    # pixel (2y+1, 2x) samples low-res (y + 0.25, x - 0.25): 0.75/0.25 weights with the row below / column left
    y, x = 1, 3
    want = 0.5625 * cf[y, x] + 0.1875 * cf[y, x - 1] + 0.1875 * cf[y + 1, x] + 0.0625 * cf[y + 1, x - 1]
    assert np.allclose(b[2 * y + 1, 2 * x], want)


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(7)
    H, W = 5, 6
    gb = _gbuffer(rng, H, W, sources=True)
    target = rng.integers(0, 256, (2 * H, 2 * W, 4), dtype=np.uint8)
    p = U.init_params(11, last_scale=1.0).astype(np.float64)
    for (wo, bo), (cin, cout) in zip(U.OFFSETS, U.LAYERS):
        p[bo:bo + cout] = rng.normal(0.0, 0.1, cout)
    g, loss = U.gradients(p, gb, target, exact=True)
    real = np.flatnonzero(p != 0.0)
    idx = rng.choice(real, 48, replace=False)
    eps = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += eps
        lp = U.forward(q, gb, target, exact=True)["loss"]
        q[i] -= 2 * eps
        lm = U.forward(q, gb, target, exact=True)["loss"]
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-4 * max(1.0, abs(fd)), (i, fd, g[i])
    # padded channels have zero gradient
    w0 = g[U.OFFSETS[0][0]:U.OFFSETS[0][1]].reshape(32, 9, 16)
    assert np.all(w0[:, :, 14:] == 0)
    w3 = g[U.OFFSETS[3][0]:U.OFFSETS[3][1]].reshape(16, 9, 32)
    assert np.all(w3[12:] == 0)


def test_zero_last_layer_is_bilinear():
    rng = np.random.default_rng(2)
    gb = _gbuffer(rng, 4, 7)
    p = U.init_params(0)
    wo, bo = U.OFFSETS[3]
    p[wo:bo + 16] = 0.0
    f = U.forward(p, gb)
    assert np.array_equal(f["rgba8"], U.to_rgba8(U.bilinear_base(gb["color"])))
