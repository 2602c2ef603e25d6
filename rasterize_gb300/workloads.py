"""Seeded synthetic workloads with the shapes of the reference's headline configs.

No public dataset is involved: every workload is generated from a seed.

* ``small_path``   -- one closed path of 200 cubics, control points U[0,512]^2,
  NonZero, 512x512 mask.
* ``large_path``   -- one closed path of 20,000 segments: 40 % lines, 20 % quads,
  30 % cubics (1 % of them degenerate: coincident control points or a cusp),
  10 % elliptic arcs (radii U[5,400], rotation U[0,360) degrees, random
  large/sweep flags); points U[0,4096]^2, EvenOdd, 4096x4096.
* ``glyph_batch``  -- 10,000 independent closed glyph outlines with a
  log-uniform segment count in [10,400] (70 % cubic / 30 % quad) and a
  log-uniform square bounding box side in [16,256] px, each into its own mask
  (NonZero).  An outline is a star-shaped loop around the box centre
  (vertices at sorted random angles, radius U[0.55,1] of the half side) whose
  curve controls are jittered around the chord, like a font glyph contour.
"""
from __future__ import annotations

import math

import numpy as np

from .geometry import Transform
from .path import SEG_ARC, SEG_CUBIC, SEG_LINE, SEG_QUAD, FillRule, Path


def _path_from_arrays(kind, pts, closed=True):
    kind = np.asarray(kind, dtype=np.uint8)
    return Path(kind, np.asarray(pts, dtype=np.float64).reshape(-1, 8), np.asarray([0, len(kind)], np.uint32),
                np.asarray([1 if closed else 0], np.uint8))


def small_path(seed: int = 0, n_cubics: int = 200, size: int = 512):
    """One closed path of cubics with control points uniform in [0,size]^2."""
    rng = np.random.default_rng(seed)
    p = rng.uniform(0.0, float(size), size=(n_cubics * 3 + 1, 2))
    pts = np.zeros((n_cubics, 8))
    for i in range(n_cubics):
        pts[i] = np.concatenate([p[3 * i], p[3 * i + 1], p[3 * i + 2], p[3 * i + 3]])
    return _path_from_arrays(np.full(n_cubics, SEG_CUBIC), pts), FillRule.NonZero, (size, size)


def large_path(seed: int = 1, n_segments: int = 20000, size: int = 4096):
    """One closed path mixing lines, quads, cubics (1 % degenerate) and arcs."""
    rng = np.random.default_rng(seed)
    kinds = rng.choice([SEG_LINE, SEG_QUAD, SEG_CUBIC, SEG_ARC], size=n_segments, p=[0.4, 0.2, 0.3, 0.1])
    pts = np.zeros((n_segments, 8))
    cur = rng.uniform(0, size, 2)
    for i, k in enumerate(kinds):
        if k == SEG_LINE:
            q = rng.uniform(0, size, 2)
            pts[i, :4] = [cur[0], cur[1], q[0], q[1]]
        elif k == SEG_QUAD:
            c, q = rng.uniform(0, size, 2), rng.uniform(0, size, 2)
            pts[i, :6] = [cur[0], cur[1], c[0], c[1], q[0], q[1]]
        elif k == SEG_CUBIC:
            c1, c2, q = rng.uniform(0, size, 2), rng.uniform(0, size, 2), rng.uniform(0, size, 2)
            if rng.uniform() < 0.01:  # degenerate: coincident controls or a cusp
                if rng.uniform() < 0.5:
                    c1, c2 = cur.copy(), q.copy()
                else:
                    # controls crossed over the chord produce a cusp
                    c1, c2 = q + (q - cur), cur + (cur - q)
            pts[i] = [cur[0], cur[1], c1[0], c1[1], c2[0], c2[1], q[0], q[1]]
        else:
            q = rng.uniform(0, size, 2)
            while abs(q[0] - cur[0]) < 1e-3 and abs(q[1] - cur[1]) < 1e-3:
                q = rng.uniform(0, size, 2)
            rx, ry = rng.uniform(5, 400, 2)
            rot = rng.uniform(0, 360)
            flags = int(rng.integers(0, 2)) | (int(rng.integers(0, 2)) << 1)
            pts[i] = [cur[0], cur[1], q[0], q[1], rx, ry, rot, float(flags)]
        cur = q
    return _path_from_arrays(kinds, pts), FillRule.EvenOdd, (size, size)


def glyph(rng, n_seg: int, side: float, p_cubic: float = 0.7):
    """A star-shaped closed outline inside a side x side box."""
    c = side / 2.0
    R = side / 2.0 - 1.0
    ang = np.sort(rng.uniform(0.0, 2.0 * math.pi, n_seg))
    rad = R * rng.uniform(0.55, 1.0, n_seg)
    v = np.stack([c + rad * np.cos(ang), c + rad * np.sin(ang)], axis=1)
    a = v
    b = np.roll(v, -1, axis=0)
    chord = np.linalg.norm(b - a, axis=1, keepdims=True) + 1e-9
    kinds = np.where(rng.uniform(size=n_seg) < p_cubic, SEG_CUBIC, SEG_QUAD).astype(np.uint8)
    lo, hi = 0.5, side - 0.5
    j1 = rng.normal(0.0, 1.0, (n_seg, 2)) * 0.3 * chord
    j2 = rng.normal(0.0, 1.0, (n_seg, 2)) * 0.3 * chord
    c1 = np.clip(a + (b - a) / 3.0 + j1, lo, hi)
    c2 = np.clip(a + 2.0 * (b - a) / 3.0 + j2, lo, hi)
    cq = np.clip((a + b) / 2.0 + j1, lo, hi)
    pts = np.zeros((n_seg, 8))
    cub = kinds == SEG_CUBIC
    pts[:, 0:2] = a
    pts[cub, 2:4] = c1[cub]
    pts[cub, 4:6] = c2[cub]
    pts[cub, 6:8] = b[cub]
    pts[~cub, 2:4] = cq[~cub]
    pts[~cub, 4:6] = b[~cub]
    return _path_from_arrays(kinds, pts)


def glyph_batch(seed: int = 2, n: int = 10000, seg_range=(10, 400), side_range=(16, 256)):
    """10k uneven glyphs; returns (paths, sizes, rules)."""
    rng = np.random.default_rng(seed)
    lseg = rng.uniform(math.log(seg_range[0]), math.log(seg_range[1]), n)
    lside = rng.uniform(math.log(side_range[0]), math.log(side_range[1]), n)
    paths, sizes = [], []
    for i in range(n):
        nseg = int(round(math.exp(lseg[i])))
        side = int(round(math.exp(lside[i])))
        paths.append(glyph(rng, nseg, float(side)))
        sizes.append((side, side))
    return paths, sizes, [FillRule.NonZero] * n


def identity():
    return Transform.identity()


def _random_stops(rng, n):
    from .paint import GradStop, LinColor
    stops = []
    for _ in range(n):
        a = float(rng.uniform(0.3, 1.0))
        r, g, b = rng.uniform(0, 1, 3) * a
        stops.append(GradStop(float(rng.uniform(0, 1)), LinColor(float(r), float(g), float(b), a)))
    return stops


def random_paint(rng, cx, cy, size, linear_colors=True):
    """50 % solid, 25 % linear, 25 % radial gradient (2-8 stops uniform in [0,1])."""
    from .paint import GradLinear, GradRadial, GradSpread, LinColor, Units
    u = rng.uniform()
    if u < 0.5:
        a = float(rng.uniform(0.3, 1.0))
        r, g, b = rng.uniform(0, 1, 3) * a
        return LinColor(float(r), float(g), float(b), a)
    stops = _random_stops(rng, int(rng.integers(2, 9)))
    spread = GradSpread(int(rng.integers(0, 3)))
    if u < 0.75:
        ang = rng.uniform(0, 2 * math.pi)
        d = size * rng.uniform(0.3, 1.0)
        start = (cx - 0.5 * d * math.cos(ang), cy - 0.5 * d * math.sin(ang))
        end = (cx + 0.5 * d * math.cos(ang), cy + 0.5 * d * math.sin(ang))
        return GradLinear(stops, start, end, Units.UserSpaceOnUse, linear_colors, spread)
    R = size * rng.uniform(0.3, 0.8)
    off = R * 0.4 * rng.uniform(0, 1)
    ang = rng.uniform(0, 2 * math.pi)
    fc = (cx + off * math.cos(ang), cy + off * math.sin(ang))
    fr = float(rng.uniform(0.0, 0.5)) * (R - off)
    return GradRadial(stops, (cx, cy), float(R), fc, fr, Units.UserSpaceOnUse, linear_colors, spread)


def contour(rng, n_seg, radius, p_cubic=0.5, center=(0.0, 0.0)):
    """Star-shaped closed outline around ``center`` (the origin by default): cubic or line segments."""
    ang = np.sort(rng.uniform(0.0, 2.0 * math.pi, n_seg))
    rad = radius * rng.uniform(0.55, 1.0, n_seg)
    v = np.stack([rad * np.cos(ang), rad * np.sin(ang)], axis=1)
    a, b = v, np.roll(v, -1, axis=0)
    chord = np.linalg.norm(b - a, axis=1, keepdims=True) + 1e-9
    kinds = np.where(rng.uniform(size=n_seg) < p_cubic, SEG_CUBIC, SEG_LINE).astype(np.uint8)
    c1 = a + (b - a) / 3.0 + rng.normal(0.0, 1.0, (n_seg, 2)) * 0.3 * chord
    c2 = a + 2.0 * (b - a) / 3.0 + rng.normal(0.0, 1.0, (n_seg, 2)) * 0.3 * chord
    pts = np.zeros((n_seg, 8))
    pts[:, 0:2] = a
    cub = kinds == SEG_CUBIC
    pts[cub, 2:4] = c1[cub]
    pts[cub, 4:6] = c2[cub]
    pts[cub, 6:8] = b[cub]
    pts[~cub, 2:4] = b[~cub]
    if center[0] or center[1]:
        pts[:, 0:2] += center
        pts[cub, 2:8] += np.tile(np.asarray(center, dtype=np.float64), 3)
        pts[~cub, 2:4] += center
    return _path_from_arrays(kinds, pts)


def scene(seed: int = 3, n: int = 2000, size: int = 2048, seg_range=(20, 2000), radius_range=(8, 128),
          linear_colors=True):
    """``n`` filled star-shaped paths (log-uniform 20-2000 cubic/line segments,
    radius log-uniform 8-128 px) under random affine transforms (scale
    0.5-2, any rotation, centre uniform in the canvas), 50 % solid / 25 %
    linear / 25 % radial paints, NonZero, drawn in order on a size x size
    canvas.  Returns a Scene and the per-fill (path, tr, rule, paint)."""
    from .rasterizer import Scene
    rng = np.random.default_rng(seed)
    sc = Scene()
    for _ in range(n):
        nseg = int(round(math.exp(rng.uniform(math.log(seg_range[0]), math.log(seg_range[1])))))
        r = math.exp(rng.uniform(math.log(radius_range[0]), math.log(radius_range[1])))
        path = contour(rng, nseg, r)
        s = rng.uniform(0.5, 2.0)
        ang = rng.uniform(0, 2 * math.pi)
        cx, cy = rng.uniform(0, size, 2)
        tr = Transform.new_translate(cx, cy) * Transform.new_rotate(ang) * Transform.new_scale(s, s)
        # gradients live in the path's own coordinates (UserSpaceOnUse, before tr)
        paint = random_paint(rng, 0.0, 0.0, 2 * r, linear_colors)
        sc.fill(path, paint, tr, FillRule.NonZero)
    return sc


def scene_tree(seed: int = 6, n_groups: int = 40, fills_per_group: int = 10, size: int = 512, seg_range=(20, 200),
               radius_range=(8, 64), linear_colors=True, stroke_fraction=0.2):
    """A layered scene: ``n_groups`` groups of ``fills_per_group`` fills (as
    ``scene``), each group either plain, under Opacity U[0.2, 0.95], clipped by
    a star path (UserSpaceOnUse or BoundingBox units, NonZero or EvenOdd), or a
    clip inside an opacity; every third group under an extra Transform node
    (a small rotation about the canvas centre).  ``stroke_fraction`` of the
    paths are stroked instead of filled (width 1-6, any join and cap)."""
    from .paint import Units
    from .path import LineCap, LineJoin, Path, StrokeStyle
    from .rasterizer import Scene
    rng = np.random.default_rng(seed)
    root = Scene()
    for g in range(n_groups):
        grp = Scene()
        gx, gy = rng.uniform(0.1 * size, 0.9 * size, 2)
        for _ in range(fills_per_group):
            nseg = int(round(math.exp(rng.uniform(math.log(seg_range[0]), math.log(seg_range[1])))))
            r = math.exp(rng.uniform(math.log(radius_range[0]), math.log(radius_range[1])))
            path = contour(rng, nseg, r)
            s = rng.uniform(0.5, 2.0)
            ang = rng.uniform(0, 2 * math.pi)
            cx, cy = np.array([gx, gy]) + rng.normal(0, 0.08 * size, 2)
            tr = Transform.new_translate(cx, cy) * Transform.new_rotate(ang) * Transform.new_scale(s, s)
            if rng.uniform() < stroke_fraction:
                # an open outline stroked (closed every other time), any join and cap
                style = StrokeStyle(rng.uniform(1.0, 6.0), LineJoin(int(rng.integers(3))), 4.0,
                                    LineCap(int(rng.integers(3))))
                if rng.uniform() < 0.5:
                    path = Path(path.kind, path.pts, path.subpath_off, np.zeros_like(path.closed))
                grp.stroke(path, random_paint(rng, 0.0, 0.0, 2 * r, linear_colors), style, tr)
            else:
                grp.fill(path, random_paint(rng, 0.0, 0.0, 2 * r, linear_colors), tr, FillRule.NonZero)
        mode = g % 4
        node = grp
        if mode in (2, 3):
            units = Units(int(rng.integers(2)))
            if units == Units.BoundingBox:
                clip = contour(rng, 24, 0.5, center=(0.5, 0.5))  # in the unit square of the group's bbox
            else:
                clip = contour(rng, 24, rng.uniform(0.1, 0.25) * size, center=(gx, gy))
            node = node.clip(clip, units, FillRule(int(rng.integers(2))))
        if mode in (1, 3):
            node = node.opacity(rng.uniform(0.2, 0.95))
        if g % 3 == 2:
            c = size / 2.0
            node = node.transform(Transform.new_translate(c, c) * Transform.new_rotate(rng.uniform(-0.2, 0.2))
                                  * Transform.new_translate(-c, -c))
        root.add(node)
    return root


def diff_batch(seed: int = 4, n_images: int = 64, paths: int = 256, segs: int = 32, size: int = 1024,
               jitter: float = 2.0, margin: float = 0.0):
    """Differentiable batch: control points (n_images, paths, 3*segs, 2)
    uniform in [-margin, size + margin]^2 (float32) and the jittered copy
    (N(0, jitter px)) the target images are rendered from."""
    rng = np.random.default_rng(seed)
    ctrl = rng.uniform(-margin, size + margin, size=(n_images, paths, 3 * segs, 2)).astype(np.float32)
    target = (ctrl + rng.normal(0.0, jitter, size=ctrl.shape)).astype(np.float32)
    return ctrl, target
