"""Generates tests/golden/bc7_hw.npz: BC7 blocks of every mode and the RGBA8
texels the GPU's texture unit decodes them to — the decoder behind the
reference's VK_FORMAT_BC7_*_BLOCK images (src/Engine/Graphics.cpp:3632-3647).
Needs a CUDA GPU; run from the repository root after building the library:

    python tests/golden/make_bc7_golden.py [output.npz]

Blocks (seed 2026, 64 per row of 4x4 texels): 128 of each mode 0-7 with the
partition, rotation and index-selection fields stepped through their values and
every other bit random, 64 of the reserved mode (first byte 0), and 64 of fully
random bytes (the natural mode mix): a 256 x 72 texel image.
"""
import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)


def make_blocks() -> np.ndarray:
    from rosy_gb300 import bc7

    rng = np.random.default_rng(2026)
    parts = [bc7.blocks_of_mode(rng, m, 128) for m in range(8)]
    parts.append(bc7.blocks_of_mode(rng, 8, 64))
    parts.append(rng.integers(0, 256, (64, 16), dtype=np.uint8))
    return np.concatenate(parts)


def main() -> None:
    import torch

    from rosy_gb300 import _lib

    out_path = sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "tests", "golden", "bc7_hw.npz")
    lib = _lib.load()
    blocks = make_blocks()
    bw = 64
    bh = len(blocks) // bw
    w, h = 4 * bw, 4 * bh
    d_blocks = torch.from_numpy(blocks.reshape(-1)).cuda()
    d_out = torch.zeros(h * w, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = lib.rz_bc7_decode_texture_unit(C.c_void_p(d_blocks.data_ptr()), w, h, C.c_void_p(d_out.data_ptr()))
    assert rc == 0, f"rz_bc7_decode_texture_unit: {rc}"
    rgba = d_out.cpu().numpy().view(np.uint8).reshape(h, w, 4)
    np.savez_compressed(out_path, blocks=blocks, width=w, height=h, rgba=rgba,
                        source="GB300 texture unit: BC7 CUDA array, point sampling at texel centres")
    print(f"wrote {out_path}: {len(blocks)} blocks, {w}x{h} texels")


if __name__ == "__main__":
    main()
