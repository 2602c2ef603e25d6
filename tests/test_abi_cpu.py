"""CPU-side checks: the C-ABI library builds, loads and exports every symbol
of include/rasterize_gb300.h; host-side logic (path model, SVG parser, batch
packing) behaves like the reference.  No compute call needs a GPU here."""
import ctypes
import math

import numpy as np
import pytest

from rasterize_gb300 import FillRule, MaskBatch, Path, PathBuilder, Transform, _ffi, parse_svg_path
from rasterize_gb300 import workloads as W


def test_library_exports_every_header_symbol():
    lib = _ffi.load()
    names = _ffi.header_symbols()
    assert len(names) >= 10
    for name in names:
        assert hasattr(lib, name), name
    assert lib.rz_version().startswith(b"rasterize_gb300")


def test_create_without_gpu_reports_no_device():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = _ffi.load()
    st = ctypes.c_int32(-1)
    assert not lib.rz_create(0, ctypes.byref(st))
    assert st.value == 4  # RZ_ERR_NO_DEVICE


def test_null_context_is_invalid():
    lib = _ffi.load()
    assert lib.rz_synchronize(None) == 2
    assert lib.rz_last_error(None) == b"no context"


def test_builder_matches_reference_semantics():
    b = PathBuilder().move_to((1, 1)).line_to((1, 1)).line_to((2, 1)).line_to((2, 2)).close()
    b.line_to((5, 5))  # after close the position is the subpath start (src/path.rs:857-866)
    p = b.build()
    assert p.n_subpaths == 2
    assert list(p.subpath_off) == [0, 2, 3]
    assert list(p.closed) == [1, 0]
    assert tuple(p.pts[2, :2]) == (1.0, 1.0)


def test_svg_parser_relative_and_smooth():
    cmds = list(parse_svg_path("m1,1 l2,0 s1,1 2,2 t3,3 z M0 0 1.5.5"))
    ops = [c[0] for c in cmds]
    assert ops == ["M", "L", "C", "Q", "Z", "M", "L"]
    assert cmds[1][1] == (3.0, 1.0)
    assert cmds[2][1] == (3.0, 1.0)  # smooth cubic after a line reflects nothing
    assert cmds[-1][1] == (1.5, 0.5)
    p = Path.parse("M1,1 v2 h1 v-2 Z")
    assert p.n_segments == 3 and p.n_subpaths == 1


def test_squirrel_parses():
    import json
    import os
    fx = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_fixtures.json")))
    p = Path.parse(fx["squirrel"])
    assert p.n_subpaths == 2 and p.n_segments == 26


def test_batch_packing():
    paths, sizes, rules = W.glyph_batch(seed=1, n=50)
    b = MaskBatch(paths, sizes, fill_rules=rules)
    assert b.n_paths == 50
    assert b.sub_off[-1] == b.n_segments
    assert list(b.path_sub) == list(range(51))
    for i in range(50):
        d = b.descs[i]
        assert d.row_stride % 4 == 0 and d.offset % 4 == 0 and d.row_stride >= d.width
    last = b.descs[49]
    assert last.offset + last.row_stride * last.height <= b.out_len


def test_workload_shapes():
    paths, sizes, _ = W.glyph_batch(seed=2, n=2000)
    segs = np.array([p.n_segments for p in paths])
    sides = np.array([w for w, _ in sizes])
    assert segs.min() >= 10 and segs.max() <= 400
    assert sides.min() >= 16 and sides.max() <= 256
    path, rule, (w, h) = W.large_path(seed=1, n_segments=2000)
    kinds = np.bincount(path.kind, minlength=4) / path.n_segments
    assert abs(kinds[0] - 0.4) < 0.05 and abs(kinds[3] - 0.1) < 0.03
    assert rule == FillRule.EvenOdd and (w, h) == (4096, 4096)


@pytest.mark.parametrize("fmt", ["bmp", "rgba", "ppm"])
def test_image_writers_match_reference_layout(fmt):
    """rz_write_image against the oracle's byte-for-byte restatement of
    Image::write_bmp / write_rgba / write_ppm (src/image.rs:136-212)."""
    from oracle import oracle as O
    from rasterize_gb300 import image
    rng = np.random.default_rng(3)
    for h, w in [(1, 1), (3, 5), (17, 9), (0, 4)]:
        img = rng.integers(0, 256, size=(h, w, 4), dtype=np.uint8)
        got = image.encode(img, fmt)
        want = {"bmp": O.write_bmp, "rgba": O.write_rgba, "ppm": O.write_ppm}[fmt](img)
        assert got == want, (fmt, h, w)


def test_png_writer_decodes_back():
    import struct
    import zlib
    from rasterize_gb300 import image
    rng = np.random.default_rng(4)
    img = rng.integers(0, 256, size=(7, 11, 4), dtype=np.uint8)
    data = image.encode(img, "png")
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, ihdr = 8, b"", None
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        tag, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        assert struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0] == zlib.crc32(tag + body) & 0xFFFFFFFF
        if tag == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    assert ihdr == (11, 7, 8, 6, 0, 0, 0)
    raw = np.frombuffer(zlib.decompress(idat), dtype=np.uint8).reshape(7, 1 + 11 * 4)
    assert (raw[:, 0] == 0).all()
    assert (raw[:, 1:].reshape(7, 11, 4) == img).all()


def test_image_writer_rejects_bad_format():
    lib = _ffi.load()
    n = ctypes.c_uint64(0)
    img = np.zeros(4, dtype=np.uint8)
    assert lib.rz_write_image(img.ctypes.data, 1, 1, 9, None, 0, ctypes.byref(n)) == 2
    assert lib.rz_write_image(img.ctypes.data, 1, 1, 0, None, 0, ctypes.byref(n)) == 0 and n.value == 126
    small = np.zeros(10, dtype=np.uint8)
    assert lib.rz_write_image(img.ctypes.data, 1, 1, 0, small.ctypes.data, 10, ctypes.byref(n)) == 7


@pytest.mark.parametrize("join,cap", [(0, 0), (1, 1), (2, 2), (0, 2), (2, 1)])
def test_stroke_path_matches_oracle_bit_for_bit(join, cap):
    """rz_stroke_path (host C++) against the oracle's restatement of
    Path::stroke on random open and closed paths with lines, quads, cubics
    and arcs, every join and cap."""
    from oracle import oracle as O
    from rasterize_gb300 import LineCap, LineJoin, StrokeStyle
    rng = np.random.default_rng(10 + 3 * join + cap)
    for trial in range(6):
        b = PathBuilder().move_to(tuple(rng.uniform(0, 50, 2)))
        for _ in range(int(rng.integers(1, 9))):
            k = rng.integers(4)
            p = [tuple(rng.uniform(0, 50, 2)) for _ in range(3)]
            if k == 0:
                b.line_to(p[0])
            elif k == 1:
                b.quad_to(p[0], p[1])
            elif k == 2:
                b.cubic_to(p[0], p[1], p[2])
            else:
                b.arc_to(tuple(rng.uniform(5, 20, 2)), float(rng.uniform(0, 90)), bool(rng.integers(2)),
                         bool(rng.integers(2)), p[0])
        if trial % 2:
            b.close()
        path = b.build()
        width = float(rng.uniform(0.5, 6.0))
        got = path.stroke(StrokeStyle(width, LineJoin(join), 4.0, LineCap(cap)))
        want = O.stroke(path, width, join, 4.0, cap)
        assert list(got.kind) == list(want.kind)
        assert list(got.subpath_off) == list(want.sub_off)
        assert np.array_equal(got.pts, want.pts)
