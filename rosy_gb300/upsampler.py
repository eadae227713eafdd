"""Python mirror of the learned upsampler's C ABI (rz_upsampler_*), plus its
parameter layout, initialisation and the training loop over frames that the
plain renderer generates.

The network reconstructs a 2W x 2H RGBA8 frame from a W x H G-buffer (see
include/rosy_gb300.h). All compute runs in the library's CUDA kernels; torch is
used only to hold device buffers.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _abi, _lib

LAYERS = [(16, 32), (32, 32), (32, 32), (32, 16)]
OUT_CHANNELS = 12
REAL_IN_CHANNELS = 14  # colour 3, albedo 3, normal 2, coverage, depth, matched source weight of 4 points


def _offsets():
    out, o = [], 0
    for cin, cout in LAYERS:
        out.append((o, o + 9 * cin * cout))
        o += 9 * cin * cout + cout
    return out, o


OFFSETS, PARAM_COUNT = _offsets()


def init_params(seed: int = 0, last_scale: float = 0.1) -> np.ndarray:
    """He-normal weights on the real channels (padded input channels 14..15 of
    layer 0 and output channels 12..15 of layer 3 stay zero), zero biases; the
    last layer is scaled by `last_scale` so the untrained network is close to
    plain bilinear upsampling."""
    rng = np.random.Generator(np.random.PCG64(seed))
    p = np.zeros(PARAM_COUNT, np.float32)
    for l, ((wo, bo), (cin, cout)) in enumerate(zip(OFFSETS, LAYERS)):
        real_in = REAL_IN_CHANNELS if l == 0 else cin
        real_out = OUT_CHANNELS if l == 3 else cout
        w = np.zeros((cout, 9, cin), np.float32)
        w[:real_out, :, :real_in] = rng.normal(0.0, math.sqrt(2.0 / (9 * real_in)), (real_out, 9, real_in))
        if l == 3:
            w *= np.float32(last_scale)
        p[wo:bo] = w.reshape(-1)
    return p


def conv_flops(width: int, height: int, real_channels: bool = True, real_in: int = REAL_IN_CHANNELS) -> int:
    """Multiply-add FLOPs (2 per MAC) of one inference at W x H: with real channels
    (real_in in: 14 with sub-pixel sources, 10 without; 12 out) or with the padded
    channels the tensor cores execute."""
    chans = [(real_in, 32), (32, 32), (32, 32), (32, OUT_CHANNELS)] if real_channels else LAYERS
    return sum(2 * 9 * ci * co for ci, co in chans) * width * height


class Upsampler:
    def __init__(self, device: int = 0, max_width: int = 960, max_height: int = 540):
        self._lib = _lib.load()
        self._u = C.c_void_p()
        rc = self._lib.rz_upsampler_create(C.byref(self._u), device, max_width, max_height)
        if rc != 0:
            raise _lib.RzError(rc, "rz_upsampler_create")
        self.max_width, self.max_height = max_width, max_height

    def _check(self, rc: int, what: str) -> None:
        if rc != 0:
            raise _lib.RzError(rc, what)

    def close(self) -> None:
        if self._u:
            self._lib.rz_upsampler_destroy(self._u)
            self._u = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params: np.ndarray, stream: int | None = None) -> None:
        p = np.ascontiguousarray(params, np.float32)
        assert p.size == PARAM_COUNT
        self._check(self._lib.rz_upsampler_set_params(self._u, p.ctypes.data_as(C.POINTER(C.c_float)), p.size,
                                                       stream), "rz_upsampler_set_params")

    def params(self, stream: int | None = None) -> np.ndarray:
        p = np.zeros(PARAM_COUNT, np.float32)
        self._check(self._lib.rz_upsampler_get_params(self._u, p.ctypes.data_as(C.POINTER(C.c_float)), p.size,
                                                       stream), "rz_upsampler_get_params")
        return p

    def infer(self, gb: _abi.RzGbuffer, out_ptr: int, stream: int | None = None) -> None:
        self._check(self._lib.rz_upsampler_infer(self._u, C.byref(gb), out_ptr, stream), "rz_upsampler_infer")

    def accumulate(self, gb: _abi.RzGbuffer, target_ptr: int, out_ptr: int | None = None,
                   stream: int | None = None) -> None:
        self._check(self._lib.rz_upsampler_accumulate(self._u, C.byref(gb), target_ptr, out_ptr, stream),
                    "rz_upsampler_accumulate")

    def grads(self, stream: int | None = None) -> tuple[np.ndarray, float, int]:
        g = np.zeros(PARAM_COUNT, np.float32)
        loss = C.c_double()
        values = C.c_uint64()
        self._check(self._lib.rz_upsampler_get_grads(self._u, g.ctypes.data_as(C.POINTER(C.c_float)), g.size,
                                                      C.byref(loss), C.byref(values), stream),
                    "rz_upsampler_get_grads")
        return g, loss.value, values.value

    def loss(self, stream: int | None = None) -> tuple[float, int]:
        loss = C.c_double()
        values = C.c_uint64()
        self._check(self._lib.rz_upsampler_get_grads(self._u, None, 0, C.byref(loss), C.byref(values), stream),
                    "rz_upsampler_get_grads")
        return loss.value, values.value

    def adam_step(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8,
                  grad_scale: float = 1.0, stream: int | None = None) -> None:
        self._check(self._lib.rz_upsampler_adam_step(self._u, lr, beta1, beta2, eps, grad_scale, stream),
                    "rz_upsampler_adam_step")

    def status(self, stream: int | None = None) -> int:
        f = C.c_uint32()
        self._check(self._lib.rz_upsampler_status(self._u, C.byref(f), stream), "rz_upsampler_status")
        return f.value

    def set_wait_limit(self, cycles: int) -> None:
        """Time limit (SM cycles) of each wait in the kernels of the following calls (0: default)."""
        self._check(self._lib.rz_upsampler_set_wait_limit(self._u, cycles), "rz_upsampler_set_wait_limit")


def selftest_gemm(a_ptr: int, b_ptr: int, d_ptr: int, n: int, k: int, stream: int | None = None) -> int:
    """Runs the tensor-core self-test GEMM (see rz_upsampler_selftest_gemm); returns its status code."""
    return _lib.load().rz_upsampler_selftest_gemm(a_ptr, b_ptr, d_ptr, n, k, stream)


def psnr(a: np.ndarray, b: np.ndarray) -> float:
    """PSNR in dB of the RGB channels of two RGBA8 images (inf when equal)."""
    d = a[..., :3].astype(np.float64) - b[..., :3].astype(np.float64)
    mse = float(np.mean(d * d))
    return float("inf") if mse == 0.0 else 10.0 * math.log10(255.0 * 255.0 / mse)
