"""CPU oracle of the learned upsampler (test infrastructure only).

A numpy restatement of the network the CUDA kernels in
rosy_gb300/csrc/rz_upsample.cu run: input features from the G-buffer, four 3x3
convolutions with zero padding (16 -> 32 -> 32 -> 32 -> 12 channels, ReLU after
the first three), pixel shuffle x2 added to the x2 base of the input colour,
the loss sum of squared errors against a full-resolution target, and the
gradients of that sum with respect to every parameter.

The x2 base is bilinear; with the G-buffer's sub-pixel sources (a u16 mask per
pixel: bit 4k + s = source s of sample point k shows the point's triangle) it
keeps only the bilinear sources that show the triangle at each full-resolution
pixel and renormalises their weights (plain bilinear where none does).

Values are rounded to BF16 (round to nearest even) at exactly the points where
the kernels store BF16: the features, the weights, the activations after ReLU,
the loss gradient at the network output and the masked input gradients.
Sums are taken in float64, so the only differences from the kernels' FP32
tensor-core accumulation are summation order and its rare effect on a BF16
rounding. The reference renderer has no learned part; nothing here follows a
reference file.

Parameter layout (one float32 array): per layer l the weights [cout][9][cin]
(tap = 3 * ky + kx for offsets (ky - 1, kx - 1)) then the biases [cout], with
(cin, cout) = (16, 32), (32, 32), (32, 32), (32, 16).
"""
from __future__ import annotations

import numpy as np

LAYERS = [(16, 32), (32, 32), (32, 32), (32, 16)]
OUT_CHANNELS = 12
REAL_IN_CHANNELS = 14  # colour 3, albedo 3, normal 2, coverage, depth, matched source weight of 4 points
BILINEAR_WEIGHTS = (0.5625, 0.1875, 0.1875, 0.0625)  # own, horizontal, vertical, diagonal source


def layer_offsets():
    """[(weight offset, bias offset)] per layer, and the total parameter count."""
    out, o = [], 0
    for cin, cout in LAYERS:
        out.append((o, o + 9 * cin * cout))
        o += 9 * cin * cout + cout
    return out, o


OFFSETS, PARAM_COUNT = layer_offsets()


def split(params: np.ndarray):
    """[(W (cout, 9, cin), b (cout,))] views of a flat parameter array."""
    res = []
    for (wo, bo), (cin, cout) in zip(OFFSETS, LAYERS):
        res.append((params[wo:bo].reshape(cout, 9, cin), params[bo:bo + cout]))
    return res


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to the nearest BF16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)
    nan = np.isnan(a)
    if nan.any():
        out = np.where(nan, a, out)
    return out.reshape(np.shape(x))


def features(gb: dict, exact: bool = False) -> np.ndarray:
    """(H, W, 16) input channels: float32 BF16-rounded, or float64 unrounded with exact=True."""
    ft = np.float64 if exact else np.float32
    c = gb["color"].astype(ft)
    a = gb["albedo"].astype(ft)
    H, W = c.shape[:2]
    f = np.zeros((H, W, 16), ft)
    f[..., 0:3] = c[..., 0:3] / ft(255.0)
    f[..., 3:6] = a[..., 0:3] / ft(255.0)
    f[..., 6:8] = gb["normal"].astype(ft)
    f[..., 8] = a[..., 3] / ft(255.0)
    f[..., 9] = np.minimum(gb["depth"].astype(ft) * ft(16.0), ft(4.0))
    src = gb.get("sources")
    if src is not None:
        for k in range(4):
            f[..., 10 + k] = matched_weight(src, k, ft)
    return f if exact else bf16(f)


def matched_weight(sources: np.ndarray, k: int, ft=np.float32) -> np.ndarray:
    """Sum of the bilinear weights of sample point k's sources that show its triangle."""
    m = (sources.astype(np.uint32) >> (4 * k)) & 15
    ws = np.zeros(sources.shape, ft)
    for s, w in enumerate(BILINEAR_WEIGHTS):
        ws = np.where((m >> s) & 1, ws + ft(w), ws)
    return ws


def conv3x3(x: np.ndarray, w: np.ndarray) -> np.ndarray:
    """y[p, co] = sum over taps and ci of x[p + offset(tap), ci] * w[co, tap, ci], zero padding, float64."""
    H, W, _ = x.shape
    xp = np.zeros((H + 2, W + 2, x.shape[2]), np.float64)
    xp[1:-1, 1:-1] = x
    y = np.zeros((H, W, w.shape[0]), np.float64)
    for tap in range(9):
        ky, kx = divmod(tap, 3)
        y += xp[ky:ky + H, kx:kx + W] @ w[:, tap, :].astype(np.float64).T
    return y


def conv3x3_input_grad(dy: np.ndarray, w: np.ndarray) -> np.ndarray:
    """dx[q, ci] = sum over taps and co of dy[q - offset(tap), co] * w[co, tap, ci], float64."""
    H, W, _ = dy.shape
    dyp = np.zeros((H + 2, W + 2, dy.shape[2]), np.float64)
    dyp[1:-1, 1:-1] = dy
    dx = np.zeros((H, W, w.shape[2]), np.float64)
    for tap in range(9):
        ky, kx = divmod(tap, 3)
        # dy at q - (ky - 1, kx - 1) = padded index q + (2 - ky, 2 - kx)
        dx += dyp[2 - ky:2 - ky + H, 2 - kx:2 - kx + W] @ w[:, tap, :].astype(np.float64)
    return dx


def conv3x3_weight_grad(x: np.ndarray, dy: np.ndarray) -> np.ndarray:
    """dw[co, tap, ci] = sum over pixels of x[p + offset(tap), ci] * dy[p, co], float64."""
    H, W, cin = x.shape
    xp = np.zeros((H + 2, W + 2, cin), np.float64)
    xp[1:-1, 1:-1] = x
    d = dy.reshape(-1, dy.shape[2]).astype(np.float64)
    dw = np.zeros((dy.shape[2], 9, cin), np.float64)
    for tap in range(9):
        ky, kx = divmod(tap, 3)
        dw[:, tap, :] = d.T @ xp[ky:ky + H, kx:kx + W].reshape(-1, cin)
    return dw


def x2_base(color: np.ndarray, sources: np.ndarray | None = None, ft=np.float32) -> np.ndarray:
    """(2H, 2W, 3) x2 base of RGBA8 colour / 255: bilinear, or with sub-pixel sources
    the weighted sum of each point's four sources with the weights of its mask: the
    bilinear weight times the reciprocal of the kept weights' sum for each kept
    source, zero for the others (summed in the kernels' order; every source kept, or
    none, is bilinear)."""
    bil = bilinear_base(color, ft)
    if sources is None:
        return bil
    c = color[..., :3].astype(ft) / ft(255.0)
    H, W = c.shape[:2]
    out = np.zeros((2 * H, 2 * W, 3), ft)
    ys = np.arange(H)
    xs = np.arange(W)
    for i in range(2):
        yn = np.clip(ys - 1, 0, H - 1) if i == 0 else np.clip(ys + 1, 0, H - 1)
        for j in range(2):
            xn = np.clip(xs - 1, 0, W - 1) if j == 0 else np.clip(xs + 1, 0, W - 1)
            k = 2 * i + j
            m = ((sources.astype(np.uint32) >> (4 * k)) & 15)
            wt = source_weights(ft)[m]  # (H, W, 4)
            srcs = (c, c[:, xn], c[yn, :], c[yn][:, xn])
            b = wt[..., 0:1] * srcs[0]
            for s in range(1, 4):
                b = b + wt[..., s:s + 1] * srcs[s]
            out[i::2, j::2] = b
    return out


def source_weights(ft=np.float32) -> np.ndarray:
    """(16, 4) weights of the x2 base per source mask: for a kept source its bilinear
    weight times the reciprocal of the kept weights' sum, zero for the others;
    mask 0 is plain bilinear."""
    t = np.zeros((16, 4), ft)
    for m in range(16):
        inv = ft(1.0) / matched_weight(np.array([m], np.uint16), 0, ft)[0] if m else ft(0.0)
        for s, w in enumerate(BILINEAR_WEIGHTS):
            t[m, s] = ft(w) if m == 0 else (ft(w) * inv if (m >> s) & 1 else ft(0.0))
    return t


def bilinear_base(color: np.ndarray, ft=np.float32) -> np.ndarray:
    """(2H, 2W, 3) float32 bilinear x2 upsampling of RGBA8 colour / 255, edges clamped,
    summed in the kernels' order: 0.5625 c00 + 0.1875 c01 + 0.1875 c10 + 0.0625 c11."""
    c = color[..., :3].astype(ft) / ft(255.0)
    H, W = c.shape[:2]
    out = np.zeros((2 * H, 2 * W, 3), ft)
    ys = np.arange(H)
    xs = np.arange(W)
    for i in range(2):
        yn = np.clip(ys - 1, 0, H - 1) if i == 0 else np.clip(ys + 1, 0, H - 1)
        for j in range(2):
            xn = np.clip(xs - 1, 0, W - 1) if j == 0 else np.clip(xs + 1, 0, W - 1)
            c00 = c
            c01 = c[:, xn]
            c10 = c[yn, :]
            c11 = c[yn][:, xn]
            b = ft(0.5625) * c00
            b = b + ft(0.1875) * c01
            b = b + ft(0.1875) * c10
            b = b + ft(0.0625) * c11
            out[i::2, j::2] = b
    return out


def shuffle(net: np.ndarray) -> np.ndarray:
    """(H, W, 12) -> (2H, 2W, 3): channel (2 i + j) * 3 + k goes to pixel (2y + i, 2x + j)."""
    H, W = net.shape[:2]
    out = np.zeros((2 * H, 2 * W, 3), net.dtype)
    for i in range(2):
        for j in range(2):
            s = 2 * i + j
            out[i::2, j::2] = net[..., 3 * s:3 * s + 3]
    return out


def unshuffle(full: np.ndarray) -> np.ndarray:
    """Inverse of shuffle: (2H, 2W, 3) -> (H, W, 12)."""
    H, W = full.shape[0] // 2, full.shape[1] // 2
    out = np.zeros((H, W, 12), full.dtype)
    for i in range(2):
        for j in range(2):
            s = 2 * i + j
            out[..., 3 * s:3 * s + 3] = full[i::2, j::2]
    return out


def to_rgba8(v: np.ndarray) -> np.ndarray:
    q = np.clip(v, 0.0, 1.0).astype(np.float32)
    rgb = np.floor(q * np.float32(255.0) + np.float32(0.5)).astype(np.uint8)
    out = np.full(v.shape[:2] + (4,), 255, np.uint8)
    out[..., :3] = rgb
    return out


def forward(params: np.ndarray, gb: dict, target: np.ndarray | None = None, exact: bool = False) -> dict:
    """Runs the network; with a (2H, 2W, 4) RGBA8 target also the loss sum and the
    BF16 loss gradient at the network output. exact=True drops every BF16 rounding
    and computes in float64 (for finite-difference checks of the formulas)."""
    ft = np.float64 if exact else np.float32
    rnd = (lambda a: a) if exact else bf16
    layers = split(np.asarray(params, ft))
    x = features(gb, exact)
    acts = [x]
    for l in range(3):
        w, b = layers[l]
        y = conv3x3(acts[-1], rnd(w)) + b.astype(np.float64)
        acts.append(rnd(np.maximum(y, 0.0).astype(ft)))
    w3, b3 = layers[3]
    net = (conv3x3(acts[-1], rnd(w3)).astype(ft) + b3.astype(ft))[..., :OUT_CHANNELS]
    v = x2_base(gb["color"], gb.get("sources"), ft) + shuffle(net)
    out = {"acts": acts, "v": v, "rgba8": to_rgba8(v)}
    if target is not None:
        t = target[..., :3].astype(ft) / ft(255.0)
        d = v - t
        out["loss"] = float(np.sum(d.astype(np.float64) ** 2))
        dy = np.zeros(acts[-1].shape[:2] + (16,), ft)
        dy[..., :OUT_CHANNELS] = unshuffle(ft(2.0) * d)
        out["dy3"] = rnd(dy)
    return out


def gradients(params: np.ndarray, gb: dict, target: np.ndarray, exact: bool = False) -> tuple[np.ndarray, float]:
    """Gradient of the loss sum with respect to every parameter (float64), and the loss sum."""
    ft = np.float64 if exact else np.float32
    rnd = (lambda a: a) if exact else bf16
    layers = split(np.asarray(params, ft))
    f = forward(params, gb, target, exact)
    acts = f["acts"]
    grads = np.zeros(PARAM_COUNT, np.float64)
    dy = f["dy3"]
    for l in (3, 2, 1, 0):
        w, _ = layers[l]
        wo, bo = OFFSETS[l]
        cin, cout = LAYERS[l]
        grads[wo:bo] = conv3x3_weight_grad(acts[l], dy).reshape(-1)
        grads[bo:bo + cout] = dy.reshape(-1, cout).astype(np.float64).sum(axis=0)
        if l > 0:
            dx = conv3x3_input_grad(dy, rnd(w))
            dy = rnd(np.where(acts[l] > 0, dx, 0.0).astype(ft))
    return grads, f["loss"]


def init_params(seed: int = 0, last_scale: float = 0.1) -> np.ndarray:
    """He-normal weights (zero for padded channels), zero biases; the last layer scaled
    by `last_scale` so that the untrained network starts close to bilinear."""
    rng = np.random.Generator(np.random.PCG64(seed))
    p = np.zeros(PARAM_COUNT, np.float32)
    for l, ((wo, bo), (cin, cout)) in enumerate(zip(OFFSETS, LAYERS)):
        real_in = REAL_IN_CHANNELS if l == 0 else cin
        real_out = OUT_CHANNELS if l == 3 else cout
        w = np.zeros((cout, 9, cin), np.float32)
        std = np.sqrt(2.0 / (9 * real_in))
        w[:real_out, :, :real_in] = rng.normal(0.0, std, (real_out, 9, real_in)).astype(np.float32)
        if l == 3:
            w *= np.float32(last_scale)
        p[wo:bo] = w.reshape(-1)
    return p
