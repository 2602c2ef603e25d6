"""Path model mirroring the reference crate's ``Path`` / ``PathBuilder`` / ``FillRule``.

The storage is the structure-of-arrays the C ABI consumes (``rz_path`` in
``include/rasterize_gb300.h``):

* ``kind``    uint8[n]      segment kind (LINE, QUAD, CUBIC, ARC)
* ``pts``     float64[n, 8] up to four control points ``x0 y0 x1 y1 x2 y2 x3 y3``;
  an ARC stores ``sx sy dx dy rx ry x_axis_rot_deg flags`` (flags bit0 = large,
  bit1 = sweep) and is expanded to cubics on the device exactly like
  ``PathBuilder::arc_to`` (src/path.rs:945-972) expands it on the host;
* ``subpath_off`` uint32[m+1] segment offsets of the subpaths
  (``Path::subpaths``, src/path.rs:228-233);
* ``closed``  uint8[m]      whether each subpath was closed.

Rasterizers flatten with ``close=true`` (src/rasterize.rs:307), so every
subpath gets its closing line whatever ``closed`` says.
"""
from __future__ import annotations

import enum
import re

import numpy as np

from .geometry import EPSILON, Transform

SEG_LINE, SEG_QUAD, SEG_CUBIC, SEG_ARC = 0, 1, 2, 3
DEFAULT_FLATNESS = 0.05  # src/path.rs:16


class FillRule(enum.IntEnum):
    """src/path.rs:21-47"""

    NonZero = 0
    EvenOdd = 1

    def alpha_from_winding(self, winding: float) -> float:
        if self == FillRule.EvenOdd:
            return abs(((winding + 1.0) % 2.0) - 1.0)
        v = abs(winding)
        if v >= 1.0:
            return 1.0
        if v < 1e-6:
            return 0.0
        return v


def _close_to(p, q) -> bool:
    """Point::is_close_to (src/geometry.rs:206-211)."""
    return abs(p[0] - q[0]) < EPSILON and abs(p[1] - q[1]) < EPSILON


class LineJoin(enum.IntEnum):
    """LineJoin (src/path.rs:78-95); Miter carries StrokeStyle.miter_limit."""
    Miter = 0
    Bevel = 1
    Round = 2


class LineCap(enum.IntEnum):
    """LineCap (src/path.rs:103-117)."""
    Butt = 0
    Square = 1
    Round = 2


class StrokeStyle:
    """StrokeStyle (src/path.rs:121-137): width, join (Miter(4.0) by default), cap (Butt)."""

    __slots__ = ("width", "line_join", "miter_limit", "line_cap")

    def __init__(self, width: float = 0.0, line_join: LineJoin = LineJoin.Miter, miter_limit: float = 4.0,
                 line_cap: LineCap = LineCap.Butt):
        self.width = float(width)
        self.line_join = LineJoin(line_join)
        self.miter_limit = float(miter_limit)
        self.line_cap = LineCap(line_cap)


class Path:
    """Immutable path in SoA form (src/path.rs:228-233)."""

    __slots__ = ("kind", "pts", "subpath_off", "closed")

    def __init__(self, kind, pts, subpath_off, closed):
        self.kind = np.ascontiguousarray(kind, dtype=np.uint8)
        self.pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 8)
        self.subpath_off = np.ascontiguousarray(subpath_off, dtype=np.uint32)
        self.closed = np.ascontiguousarray(closed, dtype=np.uint8)
        if len(self.subpath_off) == 0:
            self.subpath_off = np.zeros(1, dtype=np.uint32)

    @staticmethod
    def empty() -> "Path":
        return Path(np.zeros(0, np.uint8), np.zeros((0, 8)), np.zeros(1, np.uint32), np.zeros(0, np.uint8))

    @staticmethod
    def builder() -> "PathBuilder":
        return PathBuilder()

    @staticmethod
    def parse(svg: str) -> "Path":
        b = PathBuilder()
        b.append_svg_path(svg)
        return b.build()

    def __len__(self) -> int:
        return max(len(self.subpath_off) - 1, 0)

    @property
    def n_segments(self) -> int:
        return int(self.kind.shape[0])

    @property
    def n_subpaths(self) -> int:
        return len(self)

    def is_empty(self) -> bool:
        return self.n_subpaths == 0

    def stroke(self, style: StrokeStyle) -> "Path":
        """Path::stroke (src/path.rs:374-415) on the host, through the library's
        rz_stroke_path: the outline, every subpath closed."""
        import ctypes
        from . import _ffi
        lib = _ffi.load()
        ps = _ffi.RzPath(self.kind.ctypes.data, self.pts.ctypes.data, self.subpath_off.ctypes.data,
                         self.closed.ctypes.data if self.closed.size else None, self.n_segments, self.n_subpaths)
        st = _ffi.RzStrokeStyle(style.width, style.miter_limit, int(style.line_join), int(style.line_cap))
        ns, nsub = ctypes.c_uint32(0), ctypes.c_uint32(0)
        cap_s, cap_p = 16 * self.n_segments + 64, 2 * self.n_subpaths + 2  # usually enough: one call
        while True:
            kind = np.zeros(cap_s, dtype=np.uint8)
            pts = np.zeros((cap_s, 8), dtype=np.float64)
            sub = np.zeros(cap_p, dtype=np.uint32)
            rc = lib.rz_stroke_path(ctypes.byref(ps), ctypes.byref(st), kind.ctypes.data, pts.ctypes.data, cap_s,
                                    sub.ctypes.data, cap_p, ctypes.byref(ns), ctypes.byref(nsub))
            if rc != 7:  # RZ_ERR_CAPACITY: grow to the sizes it reported
                break
            cap_s, cap_p = ns.value, nsub.value + 1
        if rc != 0:
            raise _ffi.RasterizeError(rc, "rz_stroke_path failed")
        n = ns.value
        return Path(kind[:n], pts[:n], sub[:nsub.value + 1], np.ones(nsub.value, dtype=np.uint8))

    def has_arcs(self) -> bool:
        return bool(np.any(self.kind == SEG_ARC))

    def segments(self):
        """Yields (kind, points) per segment, points as a list of (x, y)."""
        npts = {SEG_LINE: 2, SEG_QUAD: 3, SEG_CUBIC: 4}
        for k, p in zip(self.kind, self.pts):
            k = int(k)
            if k == SEG_ARC:
                yield k, [tuple(p[0:2]), tuple(p[2:4])]
            else:
                yield k, [(p[2 * i], p[2 * i + 1]) for i in range(npts[k])]

    @staticmethod
    def concat(paths) -> "Path":
        """Concatenates paths into one (subpaths kept in order)."""
        kinds, ptss, offs, closed = [], [], [0], []
        base = 0
        for p in paths:
            kinds.append(p.kind)
            ptss.append(p.pts)
            offs.extend((p.subpath_off[1:].astype(np.int64) + base).tolist())
            closed.append(p.closed)
            base += p.n_segments
        return Path(
            np.concatenate(kinds) if kinds else np.zeros(0, np.uint8),
            np.concatenate(ptss) if ptss else np.zeros((0, 8)),
            np.asarray(offs, dtype=np.uint32),
            np.concatenate(closed) if closed else np.zeros(0, np.uint8),
        )


class PathBuilder:
    """Canvas-like builder mirroring src/path.rs:800-1056."""

    def __init__(self):
        self.position = (0.0, 0.0)
        self._kind: list[int] = []
        self._pts: list[list[float]] = []
        self._sub: list[int] = []
        self._closed: list[int] = []

    # -- subpath bookkeeping (src/path.rs:850-870)
    def _segment_start(self, i):
        k = self._kind[i]
        p = self._pts[i]
        return (p[0], p[1])

    def _subpath_finish(self, close: bool):
        n = len(self._kind)
        if n == 0 or (self._sub and self._sub[-1] == n):
            return
        if not self._sub:
            self._sub.append(0)
        if close:
            first = self._sub[-1]
            if first < n:
                self.position = self._segment_start(first)
        self._sub.append(n)
        self._closed.append(1 if close else 0)

    def build(self) -> Path:
        self._subpath_finish(False)
        path = Path(
            np.asarray(self._kind, dtype=np.uint8),
            np.asarray(self._pts, dtype=np.float64).reshape(-1, 8),
            np.asarray(self._sub if self._sub else [0], dtype=np.uint32),
            np.asarray(self._closed, dtype=np.uint8),
        )
        self.__init__()
        return path

    def move_to(self, p):
        self._subpath_finish(False)
        self.position = (float(p[0]), float(p[1]))
        return self

    def close(self):
        self._subpath_finish(True)
        return self

    def line_to(self, p):
        p = (float(p[0]), float(p[1]))
        if not _close_to(self.position, p):
            self._kind.append(SEG_LINE)
            self._pts.append([self.position[0], self.position[1], p[0], p[1], 0.0, 0.0, 0.0, 0.0])
            self.position = p
        return self

    def quad_to(self, p1, p2):
        p0 = self.position
        self._kind.append(SEG_QUAD)
        self._pts.append([p0[0], p0[1], float(p1[0]), float(p1[1]), float(p2[0]), float(p2[1]), 0.0, 0.0])
        self.position = (float(p2[0]), float(p2[1]))
        return self

    def cubic_to(self, p1, p2, p3):
        p0 = self.position
        self._kind.append(SEG_CUBIC)
        self._pts.append([p0[0], p0[1], float(p1[0]), float(p1[1]), float(p2[0]), float(p2[1]),
                          float(p3[0]), float(p3[1])])
        self.position = (float(p3[0]), float(p3[1]))
        return self

    def arc_to(self, radii, x_axis_rot, large, sweep, p):
        """Elliptic arc (src/path.rs:945-972).

        The arc is kept as one ARC segment; the device converts it to at most
        four cubics with the reference's endpoint-to-centre parametrisation
        (src/ellipse.rs:40-96, 159-214) before flattening.
        """
        p = (float(p[0]), float(p[1]))
        src = self.position
        flags = (1 if large else 0) | (2 if sweep else 0)
        self._kind.append(SEG_ARC)
        self._pts.append([src[0], src[1], p[0], p[1], float(radii[0]), float(radii[1]), float(x_axis_rot),
                          float(flags)])
        self.position = p
        return self

    def circle(self, radius: float):
        """src/path.rs:977-996"""
        offset = 0.5522847498307935 * radius
        cx, cy = self.position
        p0 = (cx - radius, cy)
        p1 = (cx, cy - radius)
        p2 = (cx + radius, cy)
        p3 = (cx, cy + radius)
        self.move_to(p0)
        self.cubic_to((p0[0], p0[1] - offset), (p1[0] - offset, p1[1]), p1)
        self.cubic_to((p1[0] + offset, p1[1]), (p2[0], p2[1] - offset), p2)
        self.cubic_to((p2[0], p2[1] + offset), (p3[0] + offset, p3[1]), p3)
        self.cubic_to((p3[0] - offset, p3[1]), (p0[0], p0[1] + offset), p0)
        self.close()
        self.move_to((cx, cy))
        return self

    def append_svg_path(self, text: str):
        for cmd in parse_svg_path(text):
            op = cmd[0]
            if op == "M":
                self.move_to(cmd[1])
            elif op == "L":
                self.line_to(cmd[1])
            elif op == "Q":
                self.quad_to(cmd[1], cmd[2])
            elif op == "C":
                self.cubic_to(cmd[1], cmd[2], cmd[3])
            elif op == "A":
                self.arc_to(cmd[1], cmd[2], cmd[3], cmd[4], cmd[5])
            elif op == "Z":
                self.close()
        return self


class SvgParserError(ValueError):
    pass


_NUM = re.compile(r"[+-]?(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?")
_SEP = re.compile(r"[\s,]*")


def parse_svg_path(text: str):
    """SVG path-data parser with the reference's command semantics
    (src/svg.rs:241-430): implicit repetition, ``m`` continuing as ``l``,
    smooth curves reflecting the previous control point, relative points offset
    by the position before the command.  Yields absolute commands
    ``("M", p) ("L", p) ("Q", p1, p2) ("C", p1, p2, p3) ("A", radii, rot, large, sweep, p) ("Z", p)``.
    """
    i, n = 0, len(text)
    prev_op = None
    prev_cmd = None
    position = (0.0, 0.0)
    subpath_start = (0.0, 0.0)

    def skip(i):
        return _SEP.match(text, i).end()

    def scalar(i):
        i = skip(i)
        m = _NUM.match(text, i)
        if not m:
            raise SvgParserError("expected number at offset %d" % i)
        return float(m.group(0)), m.end()

    def flag(i):
        i = skip(i)
        if i < n and text[i] in "01":
            return text[i] == "1", i + 1
        raise SvgParserError("invalid flag at offset %d" % i)

    while True:
        i = skip(i)
        if i >= n:
            return
        c = text[i]
        if c in "MmLlVvHhCcSsQqTtAaZz":
            op = c
            i += 1
            prev_op = {"m": "l", "M": "L"}.get(op, None if op in "Zz" else op)
        else:
            if prev_op is None:
                raise SvgParserError("invalid command at offset %d" % i)
            op = prev_op
        rel = prev_op is not None and prev_op.islower()

        def point(i):
            x, i = scalar(i)
            y, i = scalar(i)
            if rel:
                return (x + position[0], y + position[1]), i
            return (x, y), i

        if op in "Mm":
            dst, i = point(i)
            subpath_start = dst
            cmd = ("M", dst)
        elif op in "Ll":
            dst, i = point(i)
            cmd = ("L", dst)
        elif op in "Vv":
            y, i = scalar(i)
            cmd = ("L", (position[0], position[1] + y) if op == "v" else (position[0], y))
        elif op in "Hh":
            x, i = scalar(i)
            cmd = ("L", (position[0] + x, position[1]) if op == "h" else (x, position[1]))
        elif op in "Qq":
            p1, i = point(i)
            p2, i = point(i)
            cmd = ("Q", p1, p2)
        elif op in "Tt":
            if prev_cmd is not None and prev_cmd[0] == "Q":
                q1, q2 = prev_cmd[1], prev_cmd[2]
                p1 = (2.0 * q2[0] - q1[0], 2.0 * q2[1] - q1[1])
            else:
                p1 = position
            p2, i = point(i)
            cmd = ("Q", p1, p2)
        elif op in "Cc":
            p1, i = point(i)
            p2, i = point(i)
            p3, i = point(i)
            cmd = ("C", p1, p2, p3)
        elif op in "Ss":
            if prev_cmd is not None and prev_cmd[0] == "C":
                c2, c3 = prev_cmd[2], prev_cmd[3]
                p1 = (2.0 * c3[0] - c2[0], 2.0 * c3[1] - c2[1])
            else:
                p1 = position
            p2, i = point(i)
            p3, i = point(i)
            cmd = ("C", p1, p2, p3)
        elif op in "Aa":
            rx, i = scalar(i)
            ry, i = scalar(i)
            rot, i = scalar(i)
            large, i = flag(i)
            sweep, i = flag(i)
            dst, i = point(i)
            cmd = ("A", (rx, ry), rot, large, sweep, dst)
        else:  # Zz
            cmd = ("Z", subpath_start)
        position = cmd[-1]
        prev_cmd = cmd
        yield cmd
