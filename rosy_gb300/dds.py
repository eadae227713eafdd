""".dds images: a writer for BC7 files (the layout the engine's packager
writes and dds::readFile reads, src/libs/dds.hpp:409-596) and the library's
reader (rz_dds_read / rz_dds_parse) turning a file into a BC7 scene.Texture."""
from __future__ import annotations

import ctypes as C
import struct

import numpy as np

from . import _abi, _lib
from . import scene as sc
from .bc7 import chain_bytes

DXGI_BC7_TYPELESS = 97
DXGI_BC7_UNORM = 98
DXGI_BC7_UNORM_SRGB = 99
DDPF_ALPHAPIXELS = 0x1
DDPF_FOURCC = 0x4


def dds_bytes(width: int, height: int, levels: int, blocks: np.ndarray, dxgi: int = DXGI_BC7_UNORM_SRGB,
              alpha: bool = True, mip_count: int | None = None, four_cc: bytes = b"DX10", array_size: int = 1,
              magic: bytes = b"DDS ") -> bytes:
    """A .dds file: magic, 124-byte header, DX10 header, the blocks. The optional
    arguments exist to build malformed files for tests."""
    flags = 0x1 | 0x2 | 0x4 | 0x1000 | (0x20000 if levels > 1 else 0)
    pf = struct.pack("<II4sIIIII", 32, DDPF_FOURCC | (DDPF_ALPHAPIXELS if alpha else 0), four_cc, 0, 0, 0, 0, 0)
    mips = levels if mip_count is None else mip_count
    header = struct.pack("<7I", 124, flags, height, width, chain_bytes(width, height, 1), 0, mips)
    header += b"\0" * 44 + pf + struct.pack("<5I", 0x1000 | (0x400008 if levels > 1 else 0), 0, 0, 0, 0)
    assert len(header) == 124
    dx10 = struct.pack("<5I", dxgi, 3, 0, array_size, 0)
    return magic + header + dx10 + np.ascontiguousarray(blocks, np.uint8).tobytes()


def write_dds(path: str, width: int, height: int, levels: int, blocks: np.ndarray, **kw) -> None:
    with open(path, "wb") as f:
        f.write(dds_bytes(width, height, levels, blocks, **kw))


class DdsImage:
    """A .dds file read by the library: info (width, height, levels, dxgi_format,
    supports_alpha, data_bytes) and the blocks of all levels."""

    def __init__(self, path: str | None = None, data: bytes | None = None):
        lib = _lib.load()
        self._lib = lib
        self._h = C.c_void_p()
        if path is not None:
            rc = lib.rz_dds_read(path.encode(), C.byref(self._h))
            what = f"rz_dds_read({path})"
        else:
            buf = C.create_string_buffer(data, len(data)) if data else None
            rc = lib.rz_dds_parse(buf, len(data or b""), C.byref(self._h))
            what = "rz_dds_parse"
        if rc != 0:
            raise _lib.RzError(rc, what)
        self.info = _abi.RzDdsInfo()
        rc = lib.rz_dds_get_info(self._h, C.byref(self.info))
        if rc != 0:
            raise _lib.RzError(rc, "rz_dds_get_info")
        self.blocks = np.ctypeslib.as_array(C.cast(self.info.data, C.POINTER(C.c_uint8)),
                                            (self.info.data_bytes,)).copy()
        lib.rz_dds_free(self._h)
        self._h = C.c_void_p()

    def texture(self, image_type: int) -> sc.Texture:
        """The image as a BC7 texture of the given type (the engine picks sRGB or
        UNORM sampling from the type, src/Engine/Graphics.cpp:3632-3647)."""
        i = self.info
        return sc.Texture(i.width, i.height, i.levels, image_type, self.blocks, _abi.TEXELS_BC7)


def texture_from_dds(path: str, image_type: int) -> sc.Texture:
    return DdsImage(path).texture(image_type)
