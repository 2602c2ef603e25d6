"""Paints mirroring the reference's ``Paint`` implementations.

``LinColor`` (src/color.rs:268-374), ``GradLinear`` (src/grad.rs:150-226),
``GradRadial`` (src/grad.rs:300-426), ``GradStop`` / spread / units.  They
are passed to the C ABI as ``rz_paint`` records; stop sorting, the sRGB
conversion of ``linear_colors = false`` and the pixel transform are done by
the library exactly like the reference's constructors and
``Rasterizer::fill``.
"""
from __future__ import annotations

import ctypes
import enum
from dataclasses import dataclass, field

from .geometry import Transform

MAX_STOPS = 16


class Units(enum.IntEnum):
    UserSpaceOnUse = 0
    BoundingBox = 1


class GradSpread(enum.IntEnum):
    Pad = 0
    Repeat = 1
    Reflect = 2


class RzStop(ctypes.Structure):
    _fields_ = [("position", ctypes.c_double), ("color", ctypes.c_float * 4)]


class RzPaint(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("units", ctypes.c_int32), ("spread", ctypes.c_int32),
                ("linear_colors", ctypes.c_int32), ("tr", ctypes.c_double * 6), ("start", ctypes.c_double * 2),
                ("end", ctypes.c_double * 2), ("radius", ctypes.c_double), ("fradius", ctypes.c_double),
                ("color", ctypes.c_float * 4), ("stops", ctypes.POINTER(RzStop)), ("n_stops", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


@dataclass(frozen=True)
class LinColor:
    """Alpha-premultiplied linear RGBA (src/color.rs:268-272)."""

    r: float
    g: float
    b: float
    a: float

    def rgba(self):
        return (self.r, self.g, self.b, self.a)


@dataclass(frozen=True)
class GradStop:
    position: float
    color: LinColor


@dataclass
class GradLinear:
    stops: list
    start: tuple
    end: tuple
    units: Units = Units.UserSpaceOnUse
    linear_colors: bool = True
    spread: GradSpread = GradSpread.Pad
    tr: Transform = field(default_factory=Transform.identity)


@dataclass
class GradRadial:
    stops: list
    center: tuple
    radius: float
    fcenter: tuple
    fradius: float
    units: Units = Units.UserSpaceOnUse
    linear_colors: bool = True
    spread: GradSpread = GradSpread.Pad
    tr: Transform = field(default_factory=Transform.identity)


def to_struct(paint):
    """Returns (RzPaint, keepalive) for a LinColor, GradLinear or GradRadial."""
    p = RzPaint()
    keep = None
    if isinstance(paint, LinColor):
        p.kind = 0
        for i, v in enumerate(paint.rgba()):
            p.color[i] = v
        for i, v in enumerate((1.0, 0.0, 0.0, 0.0, 1.0, 0.0)):
            p.tr[i] = v
        return p, keep
    if len(paint.stops) > MAX_STOPS:
        raise ValueError("at most %d gradient stops" % MAX_STOPS)
    stops = (RzStop * max(len(paint.stops), 1))()
    for i, s in enumerate(paint.stops):
        stops[i].position = s.position
        for c, v in enumerate(s.color.rgba()):
            stops[i].color[c] = v
    keep = stops
    p.stops = ctypes.cast(stops, ctypes.POINTER(RzStop))
    p.n_stops = len(paint.stops)
    p.units = int(paint.units)
    p.spread = int(paint.spread)
    p.linear_colors = 1 if paint.linear_colors else 0
    for i, v in enumerate(paint.tr.m):
        p.tr[i] = v
    if isinstance(paint, GradLinear):
        p.kind = 1
        p.start[0], p.start[1] = paint.start
        p.end[0], p.end[1] = paint.end
    elif isinstance(paint, GradRadial):
        p.kind = 2
        p.start[0], p.start[1] = paint.center
        p.end[0], p.end[1] = paint.fcenter
        p.radius = paint.radius
        p.fradius = paint.fradius
    else:
        raise TypeError("unsupported paint %r" % (paint,))
    return p, keep
