"""GPU tests of BC7 decoding (rz_bc7_decode) against the GPU's own texture unit
(the decoder the reference's BC7 images go through), the committed golden
vectors and the scalar oracle; and of BC7 textures through rz_set_asset into a
rendered frame."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import oracle
from rosy_gb300 import _lib, bc7
from rosy_gb300 import scene as sc
from rosy_gb300.graphics import render_scene

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "bc7_hw.npz")


def _decode(blocks: np.ndarray, w: int, h: int, texture_unit: bool = False) -> np.ndarray:
    import torch

    lib = _lib.load()
    d_blocks = torch.from_numpy(np.ascontiguousarray(blocks, np.uint8).reshape(-1)).cuda()
    d_out = torch.full((h * w,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    if texture_unit:
        rc = lib.rz_bc7_decode_texture_unit(C.c_void_p(d_blocks.data_ptr()), w, h, C.c_void_p(d_out.data_ptr()))
    else:
        rc = lib.rz_bc7_decode(C.c_void_p(d_blocks.data_ptr()), w, h, C.c_void_p(d_out.data_ptr()), None)
    assert rc == 0, rc
    torch.cuda.synchronize()
    return d_out.cpu().numpy().view(np.uint8).reshape(h, w, 4)


@pytest.mark.parametrize("mode", list(range(9)))
def test_every_mode_matches_texture_unit(gpu, mode):
    rng = np.random.default_rng(100 + mode)
    blocks = bc7.blocks_of_mode(rng, mode, 64 * 16)  # all 64 partitions, 16 times each
    w, h = 4 * 64, 4 * 16
    hw = _decode(blocks, w, h, texture_unit=True)
    got = _decode(blocks, w, h)
    bad = np.argwhere((got != hw).any(-1))
    assert len(bad) == 0, f"mode {mode}: {len(bad)} texels differ, first {bad[:4].tolist()}"
    assert np.array_equal(oracle.bc7_decode(blocks, w, h), hw)


def test_golden_vectors(gpu):
    g = np.load(GOLDEN)
    w, h = int(g["width"]), int(g["height"])
    assert np.array_equal(_decode(g["blocks"], w, h), g["rgba"])


@pytest.mark.parametrize("w,h", [(1, 1), (2, 2), (3, 5), (13, 7), (130, 66), (4, 1)])
def test_partial_blocks_match_oracle(gpu, w, h):
    rng = np.random.default_rng(w * 1000 + h)
    n = max(1, (w + 3) // 4) * max(1, (h + 3) // 4)
    blocks = bc7.mixed_blocks(rng, n)
    assert np.array_equal(_decode(blocks, w, h), oracle.bc7_decode(blocks, w, h))


def test_large_image_matches_texture_unit(gpu):
    """4096 x 4096 texels (a million blocks, all modes) against the texture unit."""
    rng = np.random.default_rng(7)
    base = bc7.mixed_blocks(rng, 4096)
    blocks = base[rng.integers(0, len(base), 1024 * 1024)]
    hw = _decode(blocks, 4096, 4096, texture_unit=True)
    got = _decode(blocks, 4096, 4096)
    assert np.array_equal(got, hw)


def _bc7_scene(seed: int) -> sc.Scene:
    """The tiny scene with every texture replaced by a BC7 texture of the same
    size and type whose blocks cycle through all modes."""
    s = sc.tiny(seed)
    rng = np.random.default_rng(seed)
    s.textures = [bc7.random_texture(rng, t.width, t.height, t.levels, t.image_type) for t in s.textures]
    return s


def _decoded_copy(s: sc.Scene) -> sc.Scene:
    """The same scene with its BC7 textures decoded to RGBA8 by the oracle."""
    import copy

    out = copy.copy(s)
    texs = []
    for t in s.textures:
        lv, off = [], 0
        for l in range(t.levels):
            w, h = max(1, t.width >> l), max(1, t.height >> l)
            nb = max(1, (w + 3) // 4) * max(1, (h + 3) // 4) * 16
            lv.append(oracle.bc7_decode(t.texels[off:off + nb], w, h).reshape(-1))
            off += nb
        texs.append(sc.Texture(t.width, t.height, t.levels, t.image_type, np.concatenate(lv)))
    out.textures = texs
    return out


@pytest.mark.parametrize("seed", [0, 1])
def test_frame_with_bc7_textures_matches_oracle(gpu, seed):
    s = _bc7_scene(seed)
    assert all(t.format == 1 for t in s.textures)
    out = render_scene(s, device=0)
    ref = oracle.render(s)
    assert np.array_equal(out["ids"], ref["ids"])
    assert np.array_equal(out["depth"].view(np.uint32), ref["depth"].view(np.uint32))
    d = np.abs(out["color"].astype(np.int32) - ref["color"].astype(np.int32)).max()
    assert d <= 1, d
    # uploading BC7 blocks renders exactly what uploading their decoded texels renders
    plain = render_scene(_decoded_copy(s), device=0)
    assert np.array_equal(out["color"], plain["color"])


def test_dds_file_through_to_frame(gpu, tmp_path):
    """Textures written as .dds files (mode-6 encoded), read back with rz_dds_read
    and rendered: the frame equals the oracle's."""
    from rosy_gb300 import dds

    s = sc.tiny(3)
    texs = []
    for i, t in enumerate(s.textures):
        b = bc7.texture_to_bc7(t)
        path = str(tmp_path / f"img{i}.dds")
        dds.write_dds(path, b.width, b.height, b.levels, b.texels)
        texs.append(dds.texture_from_dds(path, t.image_type))
        assert np.array_equal(texs[-1].texels, b.texels)
    s.textures = texs
    out = render_scene(s, device=0)
    ref = oracle.render(s)
    assert np.array_equal(out["ids"], ref["ids"])
    assert np.abs(out["color"].astype(np.int32) - ref["color"].astype(np.int32)).max() <= 1
