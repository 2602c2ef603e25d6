"""Affine transforms and sizes, mirroring the reference's geometry types.

`Transform` stores ``[m00, m01, m02, m10, m11, m12]`` exactly like
``src/geometry.rs:317`` (``Transform([Scalar; 6])``), so it can be passed to
the C ABI as ``double[6]`` unchanged.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

EPSILON = 2.220446049250313e-16  # src/geometry.rs:14
EPSILON_SQRT = 1.4901161193847656e-08  # src/geometry.rs:16


@dataclass(frozen=True)
class Size:
    """Integer image size (src/rasterize.rs:36-41)."""

    width: int
    height: int


class Transform:
    """2D affine transformation (src/geometry.rs:317-539)."""

    __slots__ = ("m",)

    def __init__(self, m00=1.0, m01=0.0, m02=0.0, m10=0.0, m11=1.0, m12=0.0):
        self.m = (float(m00), float(m01), float(m02), float(m10), float(m11), float(m12))

    @staticmethod
    def identity() -> "Transform":
        return Transform()

    @staticmethod
    def new_translate(tx: float, ty: float) -> "Transform":
        return Transform(1.0, 0.0, tx, 0.0, 1.0, ty)

    @staticmethod
    def new_scale(sx: float, sy: float) -> "Transform":
        return Transform(sx, 0.0, 0.0, 0.0, sy, 0.0)

    @staticmethod
    def new_rotate(a: float) -> "Transform":
        s, c = math.sin(a), math.cos(a)
        return Transform(c, -s, 0.0, s, c, 0.0)

    def apply(self, p):
        m00, m01, m02, m10, m11, m12 = self.m
        x, y = p
        return (x * m00 + y * m01 + m02, x * m10 + y * m11 + m12)

    def __mul__(self, o: "Transform") -> "Transform":
        s00, s01, s02, s10, s11, s12 = self.m
        o00, o01, o02, o10, o11, o12 = o.m
        return Transform(
            s00 * o00 + s01 * o10,
            s00 * o01 + s01 * o11,
            s00 * o02 + s01 * o12 + s02,
            s10 * o00 + s11 * o10,
            s10 * o01 + s11 * o11,
            s10 * o02 + s11 * o12 + s12,
        )

    def pre_concat(self, other: "Transform") -> "Transform":
        return self * other

    def pre_translate(self, tx: float, ty: float) -> "Transform":
        return self * Transform.new_translate(tx, ty)

    def pre_scale(self, sx: float, sy: float) -> "Transform":
        return self * Transform.new_scale(sx, sy)

    def pre_rotate(self, a: float) -> "Transform":
        return self * Transform.new_rotate(a)

    def invert(self):
        """Inverse transform or None (src/geometry.rs:370-384)."""
        m00, m01, m02, m10, m11, m12 = self.m
        det = m00 * m11 - m10 * m01
        if abs(det) <= EPSILON:
            return None
        o00 = m11 / det
        o01 = -m01 / det
        o10 = -m10 / det
        o11 = m00 / det
        o02 = -o00 * m02 - o01 * m12
        o12 = -o10 * m02 - o11 * m12
        return Transform(o00, o01, o02, o10, o11, o12)

    def is_identity(self) -> bool:
        return self.m == (1.0, 0.0, 0.0, 0.0, 1.0, 0.0)

    def __eq__(self, other) -> bool:
        return isinstance(other, Transform) and self.m == other.m

    def __hash__(self) -> int:
        return hash(self.m)

    def __repr__(self) -> str:
        return "Transform(%s)" % ", ".join(repr(v) for v in self.m)
