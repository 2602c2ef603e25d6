"""Image writers for sRGB8 RGBA pixels (the output of ``GpuRasterizer.encode_rgba8``,
``encode_mask_rgba8`` and ``render_scene_rgba8``), mirroring ``Image::write``
(src/image.rs:121-229): BMP, raw RGBA and PPM go through the library's
``rz_write_image`` (host code, no GPU needed); PNG is written with zlib here.
"""
from __future__ import annotations

import ctypes
import struct
import zlib

import numpy as np

from . import _ffi

BMP, RGBA, PPM = 0, 1, 2
_FORMATS = {"bmp": BMP, "rgba": RGBA, "ppm": PPM}


def encode(rgba8: np.ndarray, fmt: str = "bmp") -> bytes:
    """File bytes of a (height, width, 4) uint8 image in ``fmt`` ("bmp", "rgba", "ppm", "png")."""
    img = np.ascontiguousarray(rgba8, dtype=np.uint8)
    if img.ndim != 3 or img.shape[2] != 4:
        raise ValueError("expected (height, width, 4) uint8")
    h, w = img.shape[:2]
    if fmt == "png":
        return _png(img)
    code = _FORMATS[fmt]
    lib = _ffi.load()
    n = ctypes.c_uint64(0)
    st = lib.rz_write_image(img.ctypes.data, w, h, code, None, 0, ctypes.byref(n))
    if st != 0:
        raise _ffi.RasterizeError(st, "rz_write_image: cannot encode %dx%d as %s" % (w, h, fmt))
    out = np.zeros(n.value, dtype=np.uint8)
    st = lib.rz_write_image(img.ctypes.data, w, h, code, out.ctypes.data, out.size, ctypes.byref(n))
    if st != 0:
        raise _ffi.RasterizeError(st, "rz_write_image failed")
    return out.tobytes()


def _png(img: np.ndarray) -> bytes:
    # Image::write_png (src/image.rs:214-229): 8-bit RGBA, one IDAT stream
    # (filter type 0 on every row; the compressed bytes depend on the deflate
    # implementation, the decoded pixels do not)
    h, w = img.shape[:2]

    def chunk(tag: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    raw = np.concatenate([np.zeros((h, 1), dtype=np.uint8), img.reshape(h, w * 4)], axis=1).tobytes()
    ihdr = struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)
    return b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", ihdr) + chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b"")


def write(rgba8: np.ndarray, path: str, fmt: str | None = None) -> None:
    """Writes the image to ``path``; the format defaults to the file extension."""
    if fmt is None:
        fmt = path.rsplit(".", 1)[-1].lower()
    with open(path, "wb") as f:
        f.write(encode(rgba8, fmt))
