"""GB300-native (sm_103a) rasterizer with the API of aslpavel/rasterize's hot path.

Public surface mirrors the reference crate: ``Path``, ``PathBuilder``,
``FillRule``, ``Transform``, ``Size``, the ``Rasterizer`` trait and
``GpuRasterizer`` (a drop-in beside ``SignedDifferenceRasterizer``).  Compute
runs in hand-written CUDA kernels behind the C ABI in
``include/rasterize_gb300.h``.
"""
from .geometry import EPSILON, EPSILON_SQRT, Size, Transform
from .path import (DEFAULT_FLATNESS, SEG_ARC, SEG_CUBIC, SEG_LINE, SEG_QUAD, FillRule, LineCap, LineJoin, Path,
                   PathBuilder, StrokeStyle, SvgParserError, parse_svg_path)
from ._ffi import NanError, RasterizeError
from .paint import GradLinear, GradRadial, GradSpread, GradStop, LinColor, Units
from .rasterizer import (BatchPlan, Context, DiffBatch, GpuRasterizer, MaskBatch, Pixel, Rasterizer, Scene,
                         default_context)

__all__ = [
    "EPSILON", "EPSILON_SQRT", "Size", "Transform", "DEFAULT_FLATNESS", "SEG_ARC", "SEG_CUBIC", "SEG_LINE",
    "SEG_QUAD", "FillRule", "LineCap", "LineJoin", "StrokeStyle", "Path", "PathBuilder", "SvgParserError", "parse_svg_path", "NanError",
    "RasterizeError", "BatchPlan", "Context", "DiffBatch", "Scene", "GradLinear", "GradRadial", "GradSpread", "GradStop",
    "LinColor", "Units", "GpuRasterizer", "MaskBatch", "Pixel", "Rasterizer", "default_context",
]
