"""Pins the CPU oracle against the reference's own known-answer tests.

Each test restates a test of aslpavel/rasterize v0.6.7 with the reference's
expected numbers and tolerances (``assert_approx_eq!`` defaults to f64
EPSILON, src/utils.rs:431-441).  Fixture path strings come from
tests/golden/reference_fixtures.json (extracted by tests/golden/make_golden.py).
"""
import json
import math
import os

import numpy as np
import pytest

from oracle import oracle as O
from rasterize_gb300.geometry import EPSILON, Transform
from rasterize_gb300.path import FillRule, Path, PathBuilder

FIX = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_fixtures.json")))


def approx(a, b, eps=EPSILON):
    assert abs(a - b) < eps, "%r != %r" % (a, b)


def test_signed_difference_line():
    """src/rasterize.rs:945-1003"""
    img = np.zeros((2, 5))
    O.signed_difference_line(img, (0.5, 1.0, 3.5, 0.0))
    a0 = (0.5 * (1.0 / 6.0)) / 2.0
    a1 = ((1.0 / 6.0) + (3.0 / 6.0)) / 2.0
    a2 = ((3.0 / 6.0) + (5.0 / 6.0)) / 2.0
    approx(img[0, 0], -a0)
    approx(img[0, 1], a0 - a1)
    approx(img[0, 2], a1 - a2)
    approx(img[0, 3], a0 - a1)
    approx(img[0, 4], -a0)
    approx(img.sum(), -1.0)
    img[:] = 0
    O.signed_difference_line(img, (-1.0, 0.0, 1.0, 1.0))
    approx(img[0, 0], 3.0 / 4.0)
    approx(img[0, 1], 1.0 / 4.0)
    img[:] = 0
    O.signed_difference_line(img, (0.0, -0.5, 2.0, 1.5))
    approx(img[0, 0], 1.0 / 8.0)
    approx(img[0, 1], 1.0 - 2.0 / 8.0)
    approx(img[0, 2], 1.0 / 8.0)
    approx(img[1, 1], 1.0 / 8.0)
    approx(img[1, 2], 0.5 - 1.0 / 8.0)
    img[:] = 0
    O.signed_difference_line(img, (0.1, 0.1, 1.9, 0.9))
    approx(img[0, 0], 0.18)
    approx(img[0, 1], 0.44)
    approx(img[0, 2], 0.18)
    img[:] = 0
    O.signed_difference_line(img, (0.1, 0.1, 0.9, 0.9))
    approx(img[0, 0], 0.4)
    approx(img[0, 1], 0.8 - 0.4)
    img[:] = 0
    O.signed_difference_line(img, (0.5, 0.5, 0.5, 1.75))
    approx(img[0, 0], 1.0 / 4.0)
    approx(img[0, 1], 1.0 / 4.0)
    approx(img[1, 0], 3.0 / 8.0)
    approx(img[1, 1], 3.0 / 8.0)


RASTERIZER_EXPECTED = np.array([
    0.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 0.0,
    0.0, 0.5, 1.0, 1.0, 1.0, 1.0, 1.0, 0.5, 0.0,
    0.0, 0.0, 0.25, 0.75, 1.0, 0.75, 0.25, 0.0, 0.0,
    0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,
]).reshape(4, 9)


def polygon_9x4():
    return (PathBuilder().move_to((1.0, 0.0)).line_to((1.0, 1.0)).line_to((2.0, 2.0)).line_to((4.0, 3.0))
            .line_to((5.0, 3.0)).line_to((7.0, 2.0)).line_to((8.0, 1.0)).line_to((8.0, 0.0)).close().build())


@pytest.mark.parametrize("which", ["sd", "ae"])
def test_rasterizer(which):
    """src/rasterize.rs:1065-1120 (both rasterizers)"""
    path = polygon_9x4()
    if which == "sd":
        img = O.mask(path, Transform.identity(), FillRule.EvenOdd, 9, 4)
    else:
        img = O.mask_ae(path, Transform.identity(), FillRule.EvenOdd, 9, 4)
    for e, p in zip(RASTERIZER_EXPECTED.reshape(-1), img.reshape(-1)):
        approx(e, p)
    # square exactly on pixel edges (the reference only renders it)
    sq = Path.parse(FIX["square_on_pixel_edges"])
    img = O.mask(sq, Transform.identity(), FillRule.EvenOdd, 3, 3)
    assert img.shape == (3, 3)


def path_size(path, tr):
    """Path::size (src/path.rs:439-451)."""
    bb = O.path_bbox(path, tr)
    min_x, min_y, max_x, max_y = bb
    mn = (math.floor(min_x) - 1.0, math.floor(min_y) - 1.0)
    mx = (math.ceil(max_x) + 1.0, math.ceil(max_y) + 1.0)
    w = int(round(mx[0] - mn[0]))
    h = int(round(mx[1] - mn[1]))
    shift = Transform.new_translate(1.0 - min_x, 1.0 - min_y)
    return w, h, shift * tr


@pytest.mark.parametrize("which", ["sd", "ae"])
def test_fill_rule(which):
    """src/rasterize.rs:1122-1161"""
    path = Path.parse(FIX["fill_rule_star_boxes"])
    w, h, tr = path_size(path, Transform.identity())
    fn = O.mask if which == "sd" else O.mask_ae
    y, x0, x1, x2 = 50, 50, 150, 250
    img = fn(path, tr, FillRule.EvenOdd, w, h)
    approx(img[y, x0], 0.0, 1e-6)
    approx(img[y, x1], 0.0, 1e-6)
    approx(img[y, x2], 0.0, 1e-6)
    approx(img.sum(), 13130.0, 1.0)
    img = fn(path, tr, FillRule.NonZero, w, h)
    approx(img[y, x0], 1.0, 1e-6)
    approx(img[y, x1], 1.0, 1e-6)
    approx(img[y, x2], 0.0, 1e-6)
    approx(img.sum(), 16492.5, 1.0)


def test_flatten_structure():
    """src/path.rs:1191-1211: lines of each subpath are connected and the
    closed flatten equals the concatenation of per-subpath flattens."""
    path = Path.parse(FIX["squirrel"])
    tr = Transform.new_rotate(math.pi / 3.0).pre_translate(-10.0, -20.0)
    lines, counts = O.flatten(path, tr, 0.05)
    assert len(lines) == counts.sum()
    off = path.subpath_off
    pos = 0
    for s in range(path.n_subpaths):
        n = int(counts[off[s]:off[s + 1]].sum()) + 1
        sub = lines[pos:pos + n]
        for a, b in zip(sub[:-1], sub[1:]):
            assert abs(a[2] - b[0]) < EPSILON and abs(a[3] - b[1]) < EPSILON
        # the closing line returns to the start
        assert abs(sub[-1][2] - sub[0][0]) < 1e-9 and abs(sub[-1][3] - sub[0][1]) < 1e-9
        pos += n
    assert pos == len(lines)


def test_squirrel_bbox():
    """src/path.rs:1096-1105"""
    path = Path.parse(FIX["squirrel"])
    bb = O.path_bbox(path, Transform.identity())
    approx(bb[0], 0.25)
    approx(bb[1], 1.0)
    approx(bb[2] - bb[0], 15.75)
    approx(bb[3] - bb[1], 14.0)


def test_spread():
    """src/grad.rs:514-525 (Pad=0, Repeat=1, Reflect=2)"""
    approx(O.lib().rzo_spread_at(2, 0.3), 0.3, 1e-6)
    approx(O.lib().rzo_spread_at(2, -0.3), 0.3, 1e-6)
    approx(O.lib().rzo_spread_at(2, 1.3), 0.7, 1e-6)
    approx(O.lib().rzo_spread_at(2, -1.3), 0.7, 1e-6)
    approx(O.lib().rzo_spread_at(1, 0.3), 0.3)
    approx(O.lib().rzo_spread_at(1, -0.3), 0.7)


def test_grad_stops():
    """src/grad.rs:527-540 (stops evaluated through a linear gradient along x)"""
    stops = [(0.0, (1, 0, 0, 1)), (0.5, (0, 1, 0, 1)), (1.0, (0, 0, 1, 1))]
    p = O.make_paint(kind=1, p0=(0.0, 0.0), p1=(1.0, 0.0), stops=stops)
    assert list(O.paint_at(p, -1.0, 0.0)) == [1, 0, 0, 1]
    assert list(O.paint_at(p, 0.25, 0.0)) == [0.5, 0.5, 0.0, 1.0]
    assert list(O.paint_at(p, 0.75, 0.0)) == [0.0, 0.5, 0.5, 1.0]
    assert list(O.paint_at(p, 2.0, 0.0)) == [0, 0, 1, 1]


def test_radial_grad():
    """src/grad.rs:542-568"""
    p = O.make_paint(kind=2, units=1, p0=(0.5, 0.0), r0=0.5, p1=(0.25, 0.0), r1=0.1)
    assert O.radial_offset(p, 0.25, 0.0) < 0.0
    approx(O.radial_offset(p, 0.675, 0.0), 0.5)
    approx(O.radial_offset(p, 1.0, 0.0), 1.0)


def test_linear_grad():
    """src/grad.rs:570-601: stop colours come back exactly at and beyond the stops"""
    c0, c1, c2 = (0.1, 0.2, 0.3, 0.5), (0.4, 0.1, 0.05, 0.5), (0.0, 0.0, 0.0, 0.0)
    p = O.make_paint(kind=1, p0=(0.0, 0.0), p1=(1.0, 1.0), stops=[(0.0, c0), (0.5, c1), (1.0, c2)])
    f32 = lambda c: list(np.asarray(c, dtype=np.float32))
    assert list(O.paint_at(p, -0.5, -0.5)) == f32(c0)
    assert list(O.paint_at(p, 0.0, 0.0)) == f32(c0)
    assert list(O.paint_at(p, 1.0, 0.0)) == f32(c1)
    assert list(O.paint_at(p, 0.0, 1.0)) == f32(c1)
    assert list(O.paint_at(p, 1.0, 1.0)) == f32(c2)
    assert list(O.paint_at(p, 1.5, 1.5)) == f32(c2)


def test_lin_and_srgb():
    """src/color.rs:547-554"""
    L = O.lib()
    for i in range(255):
        v = float(np.float32(i) / np.float32(255.0))
        assert abs(v - L.rzo_linear_to_srgb(L.rzo_srgb_to_linear(v))) < 1e-4
        assert abs(v - L.rzo_srgb_to_linear(L.rzo_linear_to_srgb(v))) < 1e-4


def test_sd_matches_active_edge_random():
    """No reference test cross-checks the two rasterizers on random paths; the
    two independent f64 restatements must agree to rounding.  Control points
    stay inside (0, W-1): where a line crosses x = 0 the reference's
    active-edge iterator starts its pixel walk at ``next_ceil`` of a split
    point that can round to a tiny negative x (src/rasterize.rs:836-893),
    which moves that row's cover to column 1, and the signed-difference
    rasterizer drops geometry beyond x = W-1 (src/rasterize.rs:372-387)."""
    rng = np.random.default_rng(7)
    for trial in range(40):
        b = PathBuilder().move_to(rng.uniform(0.5, 62, 2))
        for _ in range(12):
            k = rng.integers(3)
            if k == 0:
                b.line_to(rng.uniform(0.5, 62, 2))
            elif k == 1:
                b.quad_to(rng.uniform(0.5, 62, 2), rng.uniform(0.5, 62, 2))
            else:
                b.cubic_to(rng.uniform(0.5, 62, 2), rng.uniform(0.5, 62, 2), rng.uniform(-4, 62, 2) * [0, 1] + [30, 0])
        path = b.close().build()
        rule = FillRule(trial % 2)
        sd = O.mask(path, Transform.identity(), rule, 64, 64)
        ae = O.mask_ae(path, Transform.identity(), rule, 64, 64)
        assert np.abs(sd - ae).max() < 1e-9


def test_mask_iter_equals_mask_away_from_right_edge():
    """mask_iter (W+1 columns) and mask (W columns) differ only at the last column."""
    rng = np.random.default_rng(3)
    b = PathBuilder().move_to((5, 5))
    for _ in range(10):
        b.cubic_to(rng.uniform(0, 40, 2), rng.uniform(0, 40, 2), rng.uniform(0, 40, 2))
    path = b.close().build()
    m = O.mask(path, Transform.identity(), FillRule.NonZero, 48, 48)
    it, n = O.mask_iter(path, Transform.identity(), FillRule.NonZero, 48, 48)
    assert n > 0
    assert np.abs(m[:, :40] - it[:, :40]).max() < 1e-12


def test_arc_expansion_and_nan():
    b = PathBuilder().move_to((10, 10)).arc_to((20, 10), 30.0, False, True, (40, 30)).close()
    path = b.build()
    op = O.expand_path(path)
    assert len(op.kind) >= 2 and all(k == 2 for k in op.kind)
    # arc endpoints land (to rounding) on the SVG endpoints
    assert abs(op.pts[0, 0] - 10) < 1e-9 and abs(op.pts[0, 1] - 10) < 1e-9
    last_cubic = op.pts[-1]
    assert abs(last_cubic[6] - 40) < 1e-9 and abs(last_cubic[7] - 30) < 1e-9
    # NaN control point: the reference panics in flatten (src/path.rs:765-767)
    bad = PathBuilder().move_to((0, 0)).line_to((float("nan"), 1)).line_to((3, 3)).close().build()
    with pytest.raises(O.OracleError):
        O.mask(bad, Transform.identity(), FillRule.NonZero, 8, 8)


def test_color_conversion_roundtrip():
    """src/color.rs:538-545: "#ff804010" -> LinColor -> RGBA is the identity."""
    c = np.array([0xFF, 0x80, 0x40, 0x10], dtype=np.uint8)
    lin = O.lin_from_rgba8(c)
    assert list(O.encode_rgba8(lin.reshape(1, 4))[0]) == list(c)


def test_encode_roundtrip_every_byte():
    """Every opaque sRGB byte survives RGBA -> LinColor -> RGBA (the same path
    as the KAT above, over all 256 values of each channel)."""
    lin = np.stack([O.lin_from_rgba8(np.array([v, 255 - v, v // 2, 255], dtype=np.uint8)) for v in range(256)])
    out = O.encode_rgba8(lin)
    assert (out[:, 0] == np.arange(256)).all()
    assert (out[:, 1] == 255 - np.arange(256)).all()
    assert (out[:, 2] == np.arange(256) // 2).all()
    assert (out[:, 3] == 255).all()


def test_encode_edges():
    """unmultiply's alpha <= 1e-6 cut (src/color.rs:308-316), Rust's saturating
    `as u8` (negative and NaN -> 0, >= 255 -> 255) and the mask grey."""
    f = np.float32
    canvas = np.array([[0, 0, 0, 0], [0.5, 0.5, 0.5, f(1e-6)], [1, 1, 1, 1], [2, -1, np.nan, 1],
                       [0.25, 0.5, 1.0, 0.5], [0.001, 0.002, 0.003, 1.0]], dtype=np.float32)
    out = O.encode_rgba8(canvas)
    assert list(out[0]) == [0, 0, 0, 0]
    assert list(out[1]) == [0, 0, 0, 0]
    assert list(out[2]) == [255, 255, 255, 255]
    assert list(out[3]) == [255, 0, 0, 255]
    assert list(out[4][[2, 3]]) == [255, 128]
    m = O.encode_mask_rgba8(np.array([0.0, 1.0, 0.5, -1.0, 2.0]))
    assert list(m[0]) == [255, 255, 255, 255]
    assert list(m[1]) == [0, 0, 0, 255]
    assert m[2][0] == int(np.float32(O.lib().rzo_linear_to_srgb(0.5)) * np.float32(255) + np.float32(0.5))
    assert list(m[3][:3]) == [255] * 3 and list(m[4][:3]) == [0] * 3


STROKE_STYLES = [(1.0, 0, 4.0, 0), (1.0, 2, 4.0, 2), (1.0, 2, 4.0, 2)]  # (width, join, miter, cap) per case


def test_stroke():
    """src/path.rs:1224-1273: the three outlines of test_stroke, compared as
    the reference does (its Display prints 5 decimals)."""
    inputs = [FIX["stroke_inputs"][0], FIX["stroke_inputs"][0], FIX["stroke_inputs"][1]]
    for src, want_svg, (w, j, m, c) in zip(inputs, FIX["stroke_expected"], STROKE_STYLES):
        got = O.stroke(Path.parse(src), w, j, m, c)
        want = Path.parse(want_svg)
        assert list(got.kind) == list(want.kind), (src, list(got.kind), list(want.kind))
        assert list(got.sub_off) == list(want.subpath_off)
        assert np.abs(got.pts - want.pts).max() < 1e-5
