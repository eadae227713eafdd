"""CPU tests of BC7 and .dds handling: the oracle's BC7 decoder against the
golden vectors the GPU's texture unit produced (the decoder the reference's BC7
images go through), hand-derived blocks, partial blocks, the host-side encoder,
and the library's .dds reader (rz_dds_parse / rz_dds_read) on good and
malformed files, mirroring dds::readImage (src/libs/dds.hpp:409-574)."""
import os

import numpy as np
import pytest

from oracle import oracle
from rosy_gb300 import _lib, bc7, dds
from rosy_gb300 import scene as sc

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "bc7_hw.npz")


def test_oracle_matches_texture_unit_golden():
    g = np.load(GOLDEN)
    w, h = int(g["width"]), int(g["height"])
    blocks = g["blocks"]
    assert len(blocks) == 1152 and (w, h) == (256, 72)
    # the fixture's blocks are the generator's (so the file and the script agree)
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_bc7_golden", os.path.join(os.path.dirname(GOLDEN),
                                                                                 "make_bc7_golden.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    assert np.array_equal(blocks, gen.make_blocks())
    assert np.array_equal(oracle.bc7_decode(blocks, w, h), g["rgba"])
    # every mode is present, and the reserved mode decodes to zeros
    modes = [(int(b[0]) & -int(b[0])).bit_length() - 1 if b[0] else 8 for b in blocks]
    assert set(modes) == set(range(9))
    assert not g["rgba"][64:68].any()


def _mode6(ends, pbits, idx) -> np.ndarray:
    v, pos = 1 << 6, 7
    for ch in ends:
        for e in ch:
            v |= e << pos
            pos += 7
    for p in pbits:
        v |= p << pos
        pos += 1
    for i in range(16):
        v |= idx[i] << pos
        pos += 3 if i == 0 else 4
    assert pos == 128
    return np.frombuffer(v.to_bytes(16, "little"), np.uint8)


def test_hand_derived_mode6_block():
    # endpoints (R, G, B, A) = (127,0,64,127) / (0,127,64,127) in 7 bits, P-bits 1 / 0:
    # widened e0 = (255, 1, 129, 255), e1 = (0, 254, 128, 254); weight 34 for index 8:
    # ((64-34)*e0 + 34*e1 + 32) >> 6 = (120, 135, 128, 254)
    idx = [0] * 16
    idx[1], idx[15] = 8, 15
    blk = _mode6([(127, 0), (0, 127), (64, 64), (127, 127)], (1, 0), idx)
    px = oracle.bc7_decode(blk, 4, 4).reshape(16, 4)
    assert px[0].tolist() == [255, 1, 129, 255]
    assert px[1].tolist() == [120, 135, 128, 254]
    assert px[15].tolist() == [0, 254, 128, 254]
    assert all(px[i].tolist() == [255, 1, 129, 255] for i in range(2, 15))


def test_reserved_mode_is_zero():
    assert not oracle.bc7_decode(np.zeros(16, np.uint8), 4, 4).any()


@pytest.mark.parametrize("w,h", [(1, 1), (3, 2), (13, 7), (6, 9)])
def test_partial_blocks_are_crops(w, h):
    rng = np.random.default_rng(w * 31 + h)
    bw, bh = (w + 3) // 4, (h + 3) // 4
    blocks = bc7.mixed_blocks(rng, bw * bh)
    full = oracle.bc7_decode(blocks, 4 * bw, 4 * bh)
    assert np.array_equal(oracle.bc7_decode(blocks, w, h), full[:h, :w])


def test_blocks_of_mode_fields():
    rng = np.random.default_rng(0)
    for m in range(8):
        b = bc7.blocks_of_mode(rng, m, 70)
        v = [int.from_bytes(x.tobytes(), "little") for x in b]
        assert all(x & ((1 << (m + 1)) - 1) == 1 << m for x in v)
        pb = bc7.MODES[m][1]
        if pb:
            assert [(x >> (m + 1)) & ((1 << pb) - 1) for x in v] == [i % (1 << pb) for i in range(70)]


def test_encoder_round_trip():
    y, x = np.mgrid[0:37, 0:50]
    # channels that rise and fall together along one direction lie on a line in
    # every block, which mode 6 represents up to endpoint and weight rounding
    t = x + 2 * y
    img = np.stack([t * 2, 255 - t * 2, t + 40, 200 - t], -1).clip(0, 255).astype(np.uint8)
    blocks = bc7.encode(img)
    assert blocks.shape == (13 * 10, 16)
    assert np.abs(oracle.bc7_decode(blocks, 50, 37).astype(int) - img).max() <= 2
    assert all((int(b[0]) & 0x7F) == 0x40 for b in blocks)  # mode 6
    # a two-dimensional gradient is approximated by each block's principal line
    img2 = np.stack([x * 5, y * 6, (x + y) * 2, 255 - 3 * y], -1).clip(0, 255).astype(np.uint8)
    assert np.abs(oracle.bc7_decode(bc7.encode(img2), 50, 37).astype(int) - img2).mean() < 3.0
    t = sc.make_texture(np.random.default_rng(1), 32, sc.IMAGE_COLOR)
    b = bc7.texture_to_bc7(t)
    assert b.format == 1 and len(b.texels) == bc7.chain_bytes(32, 32, t.levels)


def _info(data: bytes):
    return dds.DdsImage(data=data).info


def test_dds_round_trip(tmp_path):
    rng = np.random.default_rng(5)
    blocks = bc7.mixed_blocks(rng, bc7.chain_bytes(20, 12, 4) // 16)
    data = dds.dds_bytes(20, 12, 4, blocks, dxgi=dds.DXGI_BC7_UNORM, alpha=False)
    im = dds.DdsImage(data=data)
    i = im.info
    assert (i.width, i.height, i.levels, i.dxgi_format, i.supports_alpha) == (20, 12, 4, 98, 0)
    assert i.data_bytes == blocks.size and np.array_equal(im.blocks, blocks.reshape(-1))
    path = str(tmp_path / "a.dds")
    dds.write_dds(path, 20, 12, 4, blocks)
    t = dds.texture_from_dds(path, sc.IMAGE_NORMAL_MAP)
    assert (t.width, t.height, t.levels, t.image_type, t.format) == (20, 12, 4, sc.IMAGE_NORMAL_MAP, 1)
    assert np.array_equal(t.texels, blocks.reshape(-1))
    # mipmapCount 0 reads as one level; extra bytes after the levels are ignored
    assert _info(dds.dds_bytes(8, 8, 1, np.zeros((4, 16), np.uint8), mip_count=0) + b"xx").levels == 1


@pytest.mark.parametrize("case,code", [
    ("short", 11), ("magic", 11), ("dx10_short", 11), ("legacy_fourcc", 3), ("not_bc7", 3),
    ("array", 3), ("truncated_mips", 11), ("zero_width", 11), ("array_zero", 11), ("huge_width", 11),
])
def test_dds_rejects_malformed(case, code):
    blocks = np.zeros((bc7.chain_bytes(16, 16, 3) // 16, 16), np.uint8)
    good = dds.dds_bytes(16, 16, 3, blocks)
    data = {
        "short": good[:100],
        "magic": dds.dds_bytes(16, 16, 3, blocks, magic=b"DDS\0"),
        "dx10_short": good[:140],
        "legacy_fourcc": dds.dds_bytes(16, 16, 3, blocks, four_cc=b"DXT1"),
        "not_bc7": dds.dds_bytes(16, 16, 3, blocks, dxgi=71),  # BC1_UNORM
        "array": dds.dds_bytes(16, 16, 3, blocks, array_size=2),
        "truncated_mips": good[:-1],
        "zero_width": dds.dds_bytes(0, 16, 1, blocks[:4]),
        "array_zero": dds.dds_bytes(16, 16, 3, blocks, array_size=0),
        # (width + 3) / 4 must not wrap in 32 bits: 2^32 - 1 texels wide needs far more than the file holds
        "huge_width": good[:16] + (0xFFFFFFFF).to_bytes(4, "little") + good[20:],
    }[case]
    with pytest.raises(_lib.RzError) as e:
        dds.DdsImage(data=data)
    assert e.value.code == code


def test_dds_read_missing_file(tmp_path):
    with pytest.raises(_lib.RzError) as e:
        dds.DdsImage(path=str(tmp_path / "none.dds"))
    assert e.value.code == 8  # RZ_OPEN_FAILED


def test_rsy_scene_loads_dds_images(tmp_path):
    """scene_from_rsy reads the asset's named images as BC7 textures; a missing
    one becomes a 1x1 white texture and is listed."""
    from test_rsy import _asset

    from rosy_gb300 import rsy

    a, _ = _asset()
    a.images = [(sc.IMAGE_COLOR, "col.dds"), (sc.IMAGE_NORMAL_MAP, "missing.dds")]
    blocks = bc7.encode(np.full((8, 8, 4), 200, np.uint8))
    dds.write_dds(str(tmp_path / "col.dds"), 8, 8, 1, blocks)
    path = str(tmp_path / "a.rsy")
    rsy.write_rsy(path, a)
    s = rsy.scene_from_rsy(path)
    assert s.textures[0].format == 1 and (s.textures[0].width, s.textures[0].height) == (8, 8)
    assert s.textures[1].format == 0 and s.textures[1].width == 1
    assert s.missing_images == ["missing.dds"]


def test_dds_parser_survives_random_and_mutated_files():
    """Random bytes and random byte edits of a valid file: the parser returns a
    result code (or parses) and never reads out of bounds or crashes."""
    hypothesis = pytest.importorskip("hypothesis")
    from hypothesis import given, settings
    from hypothesis import strategies as st

    blocks = bc7.mixed_blocks(np.random.default_rng(9), bc7.chain_bytes(12, 8, 3) // 16)
    good = dds.dds_bytes(12, 8, 3, blocks)

    @settings(max_examples=300, deadline=None, derandomize=True)
    @given(st.binary(max_size=400))
    def random_bytes(data):
        try:
            im = dds.DdsImage(data=data)
            assert im.info.data_bytes <= len(data)
        except _lib.RzError as e:
            assert e.code in (3, 11)

    @settings(max_examples=300, deadline=None, derandomize=True)
    @given(st.lists(st.tuples(st.integers(0, len(good) - 1), st.integers(0, 255)), max_size=8),
           st.integers(0, len(good)))
    def mutated(edits, cut):
        data = bytearray(good)
        for pos, val in edits:
            data[pos] = val
        data = bytes(data[:cut])
        try:
            im = dds.DdsImage(data=data)
            assert 148 + im.info.data_bytes <= len(data)
            assert im.info.levels >= 1 and im.info.width > 0 and im.info.height > 0
        except _lib.RzError as e:
            assert e.code in (3, 11)

    random_bytes()
    mutated()
