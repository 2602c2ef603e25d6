"""ctypes wrapper around the CPU f64 oracle (oracle/rz_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``; the product package never imports
this module.  Arcs are expanded here exactly like ``PathBuilder::arc_to``
(src/path.rs:945-972) does at path-build time in the reference, so the oracle
sees the same Line/Quad/Cubic segments as the reference's rasterizers.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "librz_oracle.so")
SRC = os.path.join(HERE, "rz_oracle.c")

SEG_LINE, SEG_QUAD, SEG_CUBIC, SEG_ARC = 0, 1, 2, 3
MAX_STOPS = 32

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compiles the oracle with the flags that keep binary64 op order (no FMA contraction)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(SRC):
        tmp = LIB_PATH + ".tmp.%d" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
                               "-o", tmp, SRC, "-lm", "-lpthread"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


class Paint(ctypes.Structure):
    """Mirror of ``rzo_paint`` in rz_oracle.c."""

    _fields_ = [
        ("kind", ctypes.c_int32), ("units", ctypes.c_int32), ("spread", ctypes.c_int32),
        ("linear_colors", ctypes.c_int32),
        ("tr", ctypes.c_double * 6),
        ("p0", ctypes.c_double * 2), ("p1", ctypes.c_double * 2),
        ("r0", ctypes.c_double), ("r1", ctypes.c_double),
        ("nstops", ctypes.c_int32), ("pad", ctypes.c_int32),
        ("stop_pos", ctypes.c_double * MAX_STOPS),
        ("stop_col", (ctypes.c_float * 4) * MAX_STOPS),
        ("solid", ctypes.c_float * 4),
    ]


def lib():
    global _lib
    with _lock:
        if _lib is None:
            L = ctypes.CDLL(build())
            P = ctypes.c_void_p
            L.rzo_flatten.restype = ctypes.c_long
            L.rzo_flatten.argtypes = [P, P, P, ctypes.c_long, P, ctypes.c_double, P, ctypes.c_long, P]
            L.rzo_mask.restype = ctypes.c_int
            L.rzo_mask.argtypes = [P, P, P, ctypes.c_long, P, ctypes.c_int, ctypes.c_double, P] + [ctypes.c_long] * 6
            L.rzo_mask_iter.restype = ctypes.c_long
            L.rzo_mask_iter.argtypes = [P, P, P, ctypes.c_long, P, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_long, ctypes.c_long, P]
            L.rzo_mask_ae.restype = ctypes.c_int
            L.rzo_mask_ae.argtypes = [P, P, P, ctypes.c_long, P, ctypes.c_int, ctypes.c_double, P,
                                      ctypes.c_long, ctypes.c_long]
            L.rzo_signed_difference_line.restype = None
            L.rzo_signed_difference_line.argtypes = [P] + [ctypes.c_long] * 6 + [ctypes.c_double] * 4
            L.rzo_arc_to_cubics.restype = ctypes.c_int
            L.rzo_arc_to_cubics.argtypes = [ctypes.c_double] * 7 + [ctypes.c_int, ctypes.c_int, P, ctypes.c_int]
            L.rzo_alpha_from_winding.restype = ctypes.c_double
            L.rzo_alpha_from_winding.argtypes = [ctypes.c_int, ctypes.c_double]
            L.rzo_paint_at.restype = None
            L.rzo_paint_at.argtypes = [ctypes.POINTER(Paint), ctypes.c_double, ctypes.c_double, P]
            L.rzo_radial_offset.restype = ctypes.c_int
            L.rzo_radial_offset.argtypes = [ctypes.POINTER(Paint), ctypes.c_double, ctypes.c_double, P]
            L.rzo_spread_at.restype = ctypes.c_double
            L.rzo_spread_at.argtypes = [ctypes.c_int, ctypes.c_double]
            for name in ("rzo_l2s", "rzo_s2l", "rzo_into_srgb", "rzo_into_linear"):
                getattr(L, name).restype = None
                getattr(L, name).argtypes = [P, P]
            for name in ("rzo_linear_to_srgb", "rzo_srgb_to_linear"):
                getattr(L, name).restype = ctypes.c_float
                getattr(L, name).argtypes = [ctypes.c_float]
            L.rzo_encode_rgba8.restype = None
            L.rzo_encode_rgba8.argtypes = [P, ctypes.c_long, P]
            L.rzo_encode_mask_rgba8.restype = None
            L.rzo_encode_mask_rgba8.argtypes = [P, ctypes.c_long, P]
            L.rzo_l2s_byte_thresholds.restype = ctypes.c_int
            L.rzo_l2s_byte_thresholds.argtypes = [P]
            L.rzo_lin_from_rgba8.restype = None
            L.rzo_lin_from_rgba8.argtypes = [P, P]
            L.rzo_path_bbox.restype = ctypes.c_int
            L.rzo_path_bbox.argtypes = [P, P, P, ctypes.c_long, P, P]
            L.rzo_fill.restype = ctypes.c_int
            L.rzo_fill.argtypes = [P, P, P, ctypes.c_long, P, ctypes.c_int, ctypes.c_double,
                                   ctypes.POINTER(Paint), P] + [ctypes.c_long] * 5
            L.rzo_scene_render.restype = ctypes.c_int
            L.rzo_scene_render.argtypes = [P, P, P, P, P, ctypes.c_long, P, P, ctypes.POINTER(Paint),
                                           ctypes.c_double, ctypes.c_long, ctypes.c_long, P, P]
            _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _tr(tr):
    m = tr.m if hasattr(tr, "m") else tr
    return np.ascontiguousarray(m, dtype=np.float64)


class OraclePath:
    """Arc-free SoA path as the reference holds it after PathBuilder::build."""

    def __init__(self, kind, pts, sub_off):
        self.kind = np.ascontiguousarray(kind, dtype=np.uint8)
        self.pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 8)
        self.sub_off = np.ascontiguousarray(sub_off, dtype=np.uint32)

    @property
    def nsub(self):
        return len(self.sub_off) - 1


class OracleError(RuntimeError):
    pass


def arc_to_cubics(src, dst, radii, rot, large, sweep):
    """EllipArc::new_param + to_cubics; returns an (n, 8) array, or None when
    new_param yields None (PathBuilder then falls back to line_to)."""
    out = np.zeros((8, 8), dtype=np.float64)
    n = lib().rzo_arc_to_cubics(src[0], src[1], dst[0], dst[1], radii[0], radii[1], rot,
                                int(bool(large)), int(bool(sweep)), _ptr(out), 8)
    if n == -1:
        return None
    if n < 0:
        raise OracleError("arc has no finite cubic count (the reference iterator never terminates)")
    return out[:n]


def expand_path(path, with_map: bool = False):
    """Expands ARC segments into cubics like PathBuilder::arc_to; drops
    subpaths that end up empty (PathBuilder::subpath_finish records none).
    With ``with_map`` also returns, per expanded segment, the input segment
    index it came from, and per expanded subpath the input subpath index."""
    kind = np.asarray(path.kind)
    pts = np.asarray(path.pts).reshape(-1, 8)
    sub = np.asarray(path.subpath_off)
    if not np.any(kind == SEG_ARC):
        op = OraclePath(kind, pts, sub)
        if with_map:
            return op, np.arange(len(kind)), np.arange(len(sub) - 1)
        return op
    ok, op, off, seg_map, sub_map = [], [], [0], [], []
    for s in range(len(sub) - 1):
        for i in range(int(sub[s]), int(sub[s + 1])):
            k = int(kind[i])
            if k != SEG_ARC:
                ok.append(k)
                op.append(pts[i])
                seg_map.append(i)
                continue
            p = pts[i]
            flags = int(p[7])
            cub = arc_to_cubics((p[0], p[1]), (p[2], p[3]), (p[4], p[5]), p[6], flags & 1, flags & 2)
            if cub is None:
                if not (abs(p[0] - p[2]) < 2.220446049250313e-16 and abs(p[1] - p[3]) < 2.220446049250313e-16):
                    ok.append(SEG_LINE)
                    op.append(np.array([p[0], p[1], p[2], p[3], 0, 0, 0, 0], dtype=np.float64))
                    seg_map.append(i)
            else:
                for c in cub:
                    ok.append(SEG_CUBIC)
                    op.append(c)
                    seg_map.append(i)
        if len(ok) > off[-1]:
            off.append(len(ok))
            sub_map.append(s)
    res = OraclePath(np.asarray(ok, np.uint8), np.asarray(op, np.float64).reshape(-1, 8),
                     np.asarray(off, np.uint32))
    if with_map:
        return res, np.asarray(seg_map, dtype=np.int64), np.asarray(sub_map, dtype=np.int64)
    return res


def flatten(path, tr, flatness=0.05):
    """Path::flatten(tr, flatness, close=true).  Returns (lines (n,4), counts)
    where counts holds per-segment line counts then one per subpath closing line."""
    op = path if isinstance(path, OraclePath) else expand_path(path)
    L = lib()
    counts = np.zeros(len(op.kind) + op.nsub, dtype=np.int64)
    n = L.rzo_flatten(_ptr(op.kind), _ptr(op.pts), _ptr(op.sub_off), op.nsub, _ptr(_tr(tr)), flatness,
                      None, 0, _ptr(counts))
    if n < 0:
        raise OracleError("cannot flatten segment with NaN")
    out = np.zeros((max(n, 1), 4), dtype=np.float64)
    L.rzo_flatten(_ptr(op.kind), _ptr(op.pts), _ptr(op.sub_off), op.nsub, _ptr(_tr(tr)), flatness,
                  _ptr(out), n, _ptr(counts))
    return out[:n], counts


def flatten_counts_per_input(path, tr, flatness=0.05):
    """Line counts per input segment (arcs summed over their cubics), then one
    entry per input subpath for its closing line (0 if the subpath vanished)."""
    op, seg_map, sub_map = expand_path(path, with_map=True)
    _, counts = flatten(op, tr, flatness)
    n_in = len(np.asarray(path.kind))
    nsub_in = len(np.asarray(path.subpath_off)) - 1
    out = np.zeros(n_in + nsub_in, dtype=np.int64)
    np.add.at(out, seg_map, counts[:len(seg_map)])
    out[n_in + sub_map] = counts[len(seg_map):]
    return out


def mask(path, tr, fill_rule, width, height, flatness=0.05, img=None, shape=None):
    """SignedDifferenceRasterizer::mask into a zeroed (height, width) f64 image,
    or into ``img`` viewed with ``shape = (start, width, height, row_stride, col_stride)``."""
    op = path if isinstance(path, OraclePath) else expand_path(path)
    if img is None:
        img = np.zeros((height, width), dtype=np.float64)
        shape = (0, width, height, width, 1)
    flat = img.reshape(-1)
    rc = lib().rzo_mask(_ptr(op.kind), _ptr(op.pts), _ptr(op.sub_off), op.nsub, _ptr(_tr(tr)), int(fill_rule),
                        flatness, _ptr(flat), flat.size, *shape)
    if rc < 0:
        raise OracleError("cannot flatten segment with NaN")
    return img


def mask_iter(path, tr, fill_rule, width, height, flatness=0.05):
    """SignedDifferenceRasterizer::mask_iter materialised as a dense image
    (pixels the iterator skips stay 0).  Returns (image, yielded pixel count)."""
    op = path if isinstance(path, OraclePath) else expand_path(path)
    out = np.zeros((height, width), dtype=np.float64)
    n = lib().rzo_mask_iter(_ptr(op.kind), _ptr(op.pts), _ptr(op.sub_off), op.nsub, _ptr(_tr(tr)),
                            int(fill_rule), flatness, width, height, _ptr(out))
    if n < 0:
        raise OracleError("cannot flatten segment with NaN")
    return out, n


def mask_ae(path, tr, fill_rule, width, height, flatness=0.05):
    """ActiveEdgeRasterizer::mask into a zeroed image (independent cross-check)."""
    op = path if isinstance(path, OraclePath) else expand_path(path)
    out = np.zeros((height, width), dtype=np.float64)
    rc = lib().rzo_mask_ae(_ptr(op.kind), _ptr(op.pts), _ptr(op.sub_off), op.nsub, _ptr(_tr(tr)), int(fill_rule),
                           flatness, _ptr(out), width, height)
    if rc < 0:
        raise OracleError("cannot flatten segment with NaN")
    return out


def signed_difference_line(img, line, shape=None):
    flat = img.reshape(-1)
    h, w = img.shape
    if shape is None:
        shape = (0, w, h, w, 1)
    lib().rzo_signed_difference_line(_ptr(flat), flat.size, *shape, *[float(v) for v in line])
    return img


def path_bbox(path, tr):
    op = path if isinstance(path, OraclePath) else expand_path(path)
    out = np.zeros(4)
    if not lib().rzo_path_bbox(_ptr(op.kind), _ptr(op.pts), _ptr(op.sub_off), op.nsub, _ptr(_tr(tr)), _ptr(out)):
        return None
    return out


def make_paint(kind=0, units=0, spread=0, linear_colors=True, tr=None, p0=(0, 0), p1=(0, 0), r0=0.0, r1=0.0,
               stops=(), solid=(0, 0, 0, 0)) -> Paint:
    p = Paint()
    p.kind, p.units, p.spread, p.linear_colors = int(kind), int(units), int(spread), int(bool(linear_colors))
    m = (1, 0, 0, 0, 1, 0) if tr is None else (tr.m if hasattr(tr, "m") else tr)
    for i in range(6):
        p.tr[i] = m[i]
    p.p0[0], p.p0[1] = p0
    p.p1[0], p.p1[1] = p1
    p.r0, p.r1 = r0, r1
    if len(stops) > MAX_STOPS:
        raise ValueError("too many stops")
    p.nstops = len(stops)
    for i, (pos, col) in enumerate(stops):
        p.stop_pos[i] = pos
        for c in range(4):
            p.stop_col[i][c] = col[c]
    for c in range(4):
        p.solid[c] = solid[c]
    return p


def paint_at(paint: Paint, x, y):
    out = np.zeros(4, dtype=np.float32)
    lib().rzo_paint_at(ctypes.byref(paint), x, y, _ptr(out))
    return out


def radial_offset(paint: Paint, x, y):
    out = np.zeros(1)
    if not lib().rzo_radial_offset(ctypes.byref(paint), x, y, _ptr(out)):
        return None
    return float(out[0])


def color_fn(name, rgba):
    a = np.ascontiguousarray(rgba, dtype=np.float32)
    out = np.zeros(4, dtype=np.float32)
    getattr(lib(), name)(_ptr(a), _ptr(out))
    return out


def fill(path, tr, fill_rule, paint: Paint, img, shape=None, flatness=0.05):
    """Rasterizer::fill (default method) into an RGBA f32 image (H, W, 4)."""
    op = path if isinstance(path, OraclePath) else expand_path(path)
    h, w = img.shape[:2]
    if shape is None:
        shape = (0, w, h, w, 1)
    rc = lib().rzo_fill(_ptr(op.kind), _ptr(op.pts), _ptr(op.sub_off), op.nsub, _ptr(_tr(tr)), int(fill_rule),
                        flatness, ctypes.byref(paint), _ptr(img.reshape(-1)), *shape)
    if rc < 0:
        raise OracleError("cannot flatten segment with NaN")
    return img


def scene_render(paths, trs, rules, paints, width, height, bg=(0, 0, 0, 0), flatness=0.05):
    """Scene::render of a Group of Fill nodes in path order over a (height, width)
    RGBA f32 canvas initialised to ``bg`` (view = the canvas, tr = identity)."""
    ops = [p if isinstance(p, OraclePath) else expand_path(p) for p in paths]
    kind = np.ascontiguousarray(np.concatenate([o.kind for o in ops]).astype(np.uint8))
    pts = np.ascontiguousarray(np.concatenate([o.pts for o in ops]).astype(np.float64))
    tab, starts, nsubs = [], [], []
    base = 0
    for o in ops:
        starts.append(len(tab))
        nsubs.append(o.nsub)
        tab.extend((o.sub_off.astype(np.int64) + base).tolist())
        base += len(o.kind)
    tab = np.ascontiguousarray(np.asarray(tab, dtype=np.uint32))
    starts = np.ascontiguousarray(np.asarray(starts, dtype=np.int64))
    nsubs = np.ascontiguousarray(np.asarray(nsubs, dtype=np.int64))
    trs_a = np.ascontiguousarray(np.array([t.m if hasattr(t, "m") else t for t in trs], dtype=np.float64))
    rules_a = np.ascontiguousarray(np.array([int(r) for r in rules], dtype=np.int32))
    paints_a = (Paint * len(paints))(*paints)
    canvas = np.zeros((height, width, 4), dtype=np.float32)
    bg_a = np.ascontiguousarray(bg, dtype=np.float32)
    rc = lib().rzo_scene_render(_ptr(kind), _ptr(pts), _ptr(tab), _ptr(starts), _ptr(nsubs), len(ops), _ptr(trs_a),
                                _ptr(rules_a), paints_a, flatness, width, height, _ptr(bg_a), _ptr(canvas))
    if rc < 0:
        raise OracleError("cannot flatten segment with NaN")
    return canvas


# --------------------------------------------------------------------------- differentiable batch
def diff_forward(ctrl, n_paths, segs, width, height, alpha=0.5, rule=0, flatness=0.05, frozen=None):
    """Alpha channel of ``n_paths`` closed cubic paths (``segs`` segments each,
    control points ``ctrl`` of shape (n_paths, 3*segs, 2)) filled in order with
    a solid paint of alpha ``alpha`` (source-over).  ``frozen``: control points
    whose bisection tree is reused (finite differences, tree held fixed)."""
    c = np.ascontiguousarray(ctrl, dtype=np.float64).reshape(-1)
    fz = None if frozen is None else np.ascontiguousarray(frozen, dtype=np.float64).reshape(-1)
    img = np.zeros((height, width))
    L = lib()
    L.rzo_diff_forward.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_long, ctypes.c_long, ctypes.c_long,
                                   ctypes.c_long, ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_void_p]
    rc = L.rzo_diff_forward(_ptr(c), _ptr(fz) if fz is not None else None, n_paths, segs, width, height, alpha,
                            int(rule), flatness, _ptr(img))
    if rc < 0:
        raise OracleError("cannot flatten segment with NaN")
    return img


def diff_backward(ctrl, n_paths, segs, width, height, image, dl_dimage, alpha=0.5, rule=0, flatness=0.05):
    """d loss / d control points (shape of ``ctrl``) from d loss / d image, the
    tree held fixed (binary64)."""
    c = np.ascontiguousarray(ctrl, dtype=np.float64).reshape(-1)
    img = np.ascontiguousarray(image, dtype=np.float64)
    dl = np.ascontiguousarray(dl_dimage, dtype=np.float64)
    out = np.zeros_like(c)
    L = lib()
    L.rzo_diff_backward.argtypes = [ctypes.c_void_p, ctypes.c_long, ctypes.c_long, ctypes.c_long, ctypes.c_long,
                                    ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p]
    rc = L.rzo_diff_backward(_ptr(c), n_paths, segs, width, height, alpha, int(rule), flatness, _ptr(img), _ptr(dl),
                             _ptr(out))
    if rc < 0:
        raise OracleError("cannot flatten segment with NaN")
    return out.reshape(np.shape(ctrl))


def encode_rgba8(canvas):
    """From<LinColor> for RGBA of every pixel: (..., 4) f32 -> (..., 4) uint8."""
    c = np.ascontiguousarray(canvas, dtype=np.float32)
    out = np.zeros(c.shape, dtype=np.uint8)
    lib().rzo_encode_rgba8(_ptr(c), c.size // 4, _ptr(out))
    return out


def encode_mask_rgba8(mask):
    """Scalar::to_rgba of every mask value (f64): (...) -> (..., 4) uint8."""
    m = np.ascontiguousarray(mask, dtype=np.float64)
    out = np.zeros(m.shape + (4,), dtype=np.uint8)
    lib().rzo_encode_mask_rgba8(_ptr(m), m.size, _ptr(out))
    return out


def lin_from_rgba8(rgba):
    """From<RGBA> for LinColor."""
    a = np.ascontiguousarray(rgba, dtype=np.uint8)
    out = np.zeros(4, dtype=np.float32)
    lib().rzo_lin_from_rgba8(_ptr(a), _ptr(out))
    return out


def write_bmp(rgba8):
    """Image::write_bmp (src/image.rs:165-212) restated byte by byte."""
    img = np.ascontiguousarray(rgba8, dtype=np.uint8)
    h, w = img.shape[:2]
    size = w * h * 4
    head = b"BM" + (size + 122).to_bytes(4, "little") + bytes(4) + (122).to_bytes(4, "little")
    dib = ((108).to_bytes(4, "little") + w.to_bytes(4, "little") + h.to_bytes(4, "little") + bytes([1, 0, 0x20, 0])
           + bytes([3, 0, 0, 0]) + size.to_bytes(4, "little") + bytes([0x13, 0x0B, 0, 0]) * 2 + bytes(8)
           + bytes([0xFF, 0, 0, 0]) + bytes([0, 0xFF, 0, 0]) + bytes([0, 0, 0xFF, 0]) + bytes([0, 0, 0, 0xFF])
           + bytes([0x42, 0x47, 0x52, 0x73]) + bytes(48))
    return head + dib + img[::-1].tobytes()


def write_rgba(rgba8):
    """Image::write_rgba (src/image.rs:136-149)."""
    img = np.ascontiguousarray(rgba8, dtype=np.uint8)
    h, w = img.shape[:2]
    return h.to_bytes(4, "little") + w.to_bytes(4, "little") + img.tobytes()


def write_ppm(rgba8):
    """Image::write_ppm (src/image.rs:151-163)."""
    img = np.ascontiguousarray(rgba8, dtype=np.uint8)
    h, w = img.shape[:2]
    return ("P6 %d %d 255 " % (w, h)).encode() + img[..., :3].tobytes()


def l2s_byte_thresholds():
    """(T[0..255], monotone): the smallest f32 in [0, 1] reaching each sRGB byte."""
    T = np.zeros(256, dtype=np.float32)
    mono = lib().rzo_l2s_byte_thresholds(_ptr(T))
    return T, bool(mono)


# ---------------------------------------------------------------------------
# Scene trees: Pipeline::build_rec / render_rec and Layer (src/scene.rs:153-565)
# restated over the C primitives above.  A tree is nested tuples:
#   ("fill", path, tr, rule, paint)      tr: the fill's own transform (applied first)
#   ("group", [children])
#   ("transform", child, tr)
#   ("opacity", child, opacity)          already clamped (Scene::opacity)
#   ("clip", child, path, units, rule)   units 0 UserSpaceOnUse, 1 BoundingBox
#   ("stroke", path, tr, (width, join, miter_limit, cap), paint)
# Bounding boxes are (x0, y0, x1, y1) tuples of Python floats (binary64).
# ---------------------------------------------------------------------------
_ID = (1.0, 0.0, 0.0, 0.0, 1.0, 0.0)


def _m(tr):
    return tuple(tr.m) if hasattr(tr, "m") else tuple(tr)


def _xf_mul(s, o):
    """Transform * Transform (src/geometry.rs:519-539)."""
    return (s[0] * o[0] + s[1] * o[3], s[0] * o[1] + s[1] * o[4], s[0] * o[2] + s[1] * o[5] + s[2],
            s[3] * o[0] + s[4] * o[3], s[3] * o[1] + s[4] * o[4], s[3] * o[2] + s[4] * o[5] + s[5])


def _bbox_new(x0, y0, x1, y1):
    """BBox::new (src/geometry.rs:552-561)."""
    if not x0 <= x1:
        x0, x1 = x1, x0
    if not y0 <= y1:
        y0, y1 = y1, y0
    return (x0, y0, x1, y1)


def _bbox_extend(b, x, y):
    """BBox::extend (src/geometry.rs:611-633)."""
    x0, y0, x1, y1 = b
    if x < x0:
        x0 = x
    elif x > x1:
        x1 = x
    if y < y0:
        y0 = y
    elif y > y1:
        y1 = y
    return (x0, y0, x1, y1)


def _bbox_union(a, b):
    return _bbox_extend(_bbox_extend(a, b[0], b[1]), b[2], b[3])


def _bbox_intersect(a, b):
    """BBox::intersect with range_intersect (src/geometry.rs:648-657, 677-688)."""
    if a[0] > b[2] or b[0] > a[2] or a[1] > b[3] or b[1] > a[3]:
        return None
    return _bbox_new(max(a[0], b[0]), max(a[1], b[1]), min(a[2], b[2]), min(a[3], b[3]))


def _unit_transform(b):
    """BBox::unit_transform (src/geometry.rs:662-664)."""
    return _xf_mul((1.0, 0.0, b[0], 0.0, 1.0, b[1]), (b[2] - b[0], 0.0, 0.0, 0.0, b[3] - b[1], 0.0))


def _path_bbox(path, tr):
    b = path_bbox(path, tr)
    return None if b is None else tuple(float(v) for v in b)


def _scene_bbox(node, tr):
    """Scene::bbox (src/scene.rs:153-182)."""
    k = node[0]
    if k in ("fill", "stroke"):  # a stroke's bbox does not include the stroke width
        return _path_bbox(node[1], _xf_mul(tr, _m(node[2])))
    if k == "group":
        acc = None
        for c in node[1]:
            cb = _scene_bbox(c, tr)
            acc = cb if acc is None else (acc if cb is None else _bbox_union(acc, cb))
        return acc
    if k == "transform":
        return _scene_bbox(node[1], _xf_mul(tr, _m(node[2])))
    if k == "opacity":
        return _scene_bbox(node[1], tr)
    clip_tr = tr
    if node[3] == 1:
        cb = _scene_bbox(node[1], _ID)
        if cb is None:
            return None
        clip_tr = _xf_mul(tr, _unit_transform(cb))
    child = _scene_bbox(node[1], tr)
    if child is None:
        return None
    clip = _path_bbox(node[2], clip_tr)
    if clip is None:
        return None
    return _bbox_intersect(child, clip)


def _view_apply(view, bbox):
    if view is None:
        return bbox
    if bbox is None:
        return None
    return _bbox_intersect(view, bbox)


def _build_rec(node, view, tr, out):
    """Pipeline::build_rec (src/scene.rs:268-357): appends pipeline nodes
    (children first) and returns the index of this one, or None."""
    k = node[0]
    if k == "stroke":  # the Fill of the outline, NonZero (src/scene.rs:297-306)
        w, j, m, c = node[3]
        node = ("fill", stroke(node[1], w, j, m, c), node[2], 0, node[4])
        k = "fill"
    if k == "fill":
        b = _view_apply(view, _path_bbox(node[1], _xf_mul(tr, _m(node[2]))))
        if b is None:
            return None
        out.append({"kind": "fill", "bbox": b, "tr": tr, "node": node})
    elif k == "group":
        ids = [i for i in (_build_rec(c, view, tr, out) for c in node[1]) if i is not None]
        if not ids:
            return None
        acc = None
        for i in ids:
            acc = out[i]["bbox"] if acc is None else _bbox_union(out[i]["bbox"], acc)
        out.append({"kind": "group", "bbox": acc, "tr": tr, "children": ids})
    elif k == "clip":
        clip_tr = tr
        if node[3] == 1:
            cb = _scene_bbox(node[1], _ID)
            if cb is None:
                return None
            clip_tr = _xf_mul(tr, _unit_transform(cb))
        clip_bbox = _view_apply(view, _path_bbox(node[2], clip_tr))
        if clip_bbox is None:
            return None
        cid = _build_rec(node[1], clip_bbox, tr, out)
        if cid is None:
            return None
        b = _bbox_intersect(clip_bbox, out[cid]["bbox"])
        if b is None:
            return None
        out.append({"kind": "clip", "bbox": b, "tr": tr, "child": cid, "clip": node[2], "clip_tr": clip_tr,
                    "rule": node[4]})
    elif k == "opacity":
        cid = _build_rec(node[1], view, tr, out)
        if cid is None:
            return None
        out.append({"kind": "opacity", "bbox": out[cid]["bbox"], "tr": tr, "child": cid, "opacity": node[2]})
    else:
        return _build_rec(node[1], view, _xf_mul(tr, _m(node[2])), out)
    return len(out) - 1


def _layer_new(b, color=None):
    """Layer::new (src/scene.rs:483-501)."""
    x0, x1 = math.floor(b[0]), math.ceil(b[2])
    y0, y1 = math.floor(b[1]), math.ceil(b[3])
    img = np.zeros((y1 - y0, x1 - x0, 4), dtype=np.float32)
    if color is not None:
        img[:] = np.asarray(color, dtype=np.float32)
    return {"x": x0, "y": y0, "img": img}


def _layer_compose(dst, src, fn):
    """Layer::compose (src/scene.rs:532-565) over the intersection."""
    dh, dw = dst["img"].shape[:2]
    sh, sw = src["img"].shape[:2]
    x0, x1 = max(dst["x"], src["x"]), min(dst["x"] + dw, src["x"] + sw)
    y0, y1 = max(dst["y"], src["y"]), min(dst["y"] + dh, src["y"] + sh)
    if x1 <= x0 or y1 <= y0:
        return
    d = dst["img"][y0 - dst["y"]:y1 - dst["y"], x0 - dst["x"]:x1 - dst["x"]]
    s = src["img"][y0 - src["y"]:y1 - src["y"], x0 - src["x"]:x1 - src["x"]]
    d[...] = fn(d, s)


def _blend_over(dst, src):
    """LinColor::blend_over (src/color.rs:342-344): src + dst * (1 - src.alpha), in f32."""
    return src + dst * (np.float32(1.0) - src[..., 3:4])


def _render(nodes, pid, view, bg, flatness):
    """Pipeline::render (src/scene.rs:384-395)."""
    layer = _layer_new(view if view is not None else nodes[pid]["bbox"], bg)
    _render_rec(nodes, pid, layer, flatness)
    return layer


def _render_rec(nodes, pid, layer, flatness):
    """Pipeline::render_rec (src/scene.rs:397-458)."""
    nd = nodes[pid]
    k = nd["kind"]
    if k == "fill":
        b = nd["bbox"]
        h, w = layer["img"].shape[:2]
        col_min = math.floor(b[0]) - layer["x"]
        col_max = math.ceil(b[2]) - layer["x"] + 1
        row_min = math.floor(b[1]) - layer["y"]
        row_max = math.ceil(b[3]) - layer["y"] + 1
        # `i32 as usize` wraps negatives to huge values; view_shape clamps (src/image.rs:588-605)
        wrap = lambda v, lim: lim if v < 0 else v  # noqa: E731
        row_min = min(wrap(row_min, h), h)
        row_max = max(min(wrap(row_max, h), h), row_min)
        col_min = min(wrap(col_min, w), w)
        col_max = max(min(wrap(col_max, w), w), col_min)
        vw, vh = col_max - col_min, row_max - row_min
        if vw <= 0 or vh <= 0:
            return
        align = (1.0, 0.0, -math.floor(b[0]), 0.0, 1.0, -math.floor(b[1]))
        node = nd["node"]
        tr = _xf_mul(_xf_mul(align, nd["tr"]), _m(node[2]))
        fill(node[1], tr, node[3], node[4], layer["img"], shape=(row_min * w + col_min, vw, vh, w, 1),
             flatness=flatness)
    elif k == "group":
        for c in nd["children"]:
            _render_rec(nodes, c, layer, flatness)
    elif k == "opacity":
        child = _render(nodes, nd["child"], None, None, flatness)
        op = np.float32(nd["opacity"])
        _layer_compose(layer, child, lambda d, s: _blend_over(d, s * op))
    else:
        mlay = _layer_new(nd["bbox"])
        mh, mw = mlay["img"].shape[:2]
        align = (1.0, 0.0, -float(mlay["x"]), 0.0, 1.0, -float(mlay["y"]))
        child = _render(nodes, nd["child"], None, None, flatness)
        m = mask(nd["clip"], _xf_mul(align, nd["clip_tr"]), nd["rule"], mw, mh, flatness=flatness)
        mlayer = {"x": mlay["x"], "y": mlay["y"], "img": m.astype(np.float32)[..., None]}
        _layer_compose(child, mlayer, lambda d, s: d * s)
        _layer_compose(layer, child, _blend_over)


def scene_tree_render(tree, width, height, bg=(0, 0, 0, 0), flatness=0.05):
    """Scene::render (src/scene.rs:186-199) of ``tree`` with view = the canvas
    (0, 0, width, height) and tr = identity: the (height, width, 4) f32 canvas.
    With nothing in view the reference returns an empty layer; the canvas is
    then the background."""
    nodes = []
    root = _build_rec(tree, (0.0, 0.0, float(width), float(height)), _ID, nodes)
    if root is None:
        img = np.zeros((height, width, 4), dtype=np.float32)
        img[:] = np.asarray(bg, dtype=np.float32)
        return img
    return _render(nodes, root, (0.0, 0.0, float(width), float(height)), bg, flatness)["img"]


def stroke(path, width, line_join=0, miter_limit=4.0, line_cap=0):
    """Path::stroke (src/path.rs:374-415): the outline as an OraclePath (every
    subpath closed).  ``path`` carries ``closed`` flags per subpath (arcs
    are expanded first, keeping the flag of the subpath they came from)."""
    op, _, sub_map = expand_path(path, with_map=True)
    closed_in = np.asarray(getattr(path, "closed", np.zeros(0)), dtype=np.uint8)
    closed = np.ascontiguousarray(np.array([closed_in[s] if s < len(closed_in) else 0 for s in sub_map],
                                           dtype=np.uint8))
    L = lib()
    if not hasattr(L, "_stroke_ready"):
        L.rzo_stroke.restype = ctypes.c_long
        L.rzo_stroke.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_long, ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                                          ctypes.c_double, ctypes.c_int, ctypes.c_void_p,
                                                          ctypes.c_void_p, ctypes.c_long, ctypes.c_void_p,
                                                          ctypes.c_long, ctypes.POINTER(ctypes.c_long)]
        L._stroke_ready = True
    cap = max(64, 64 * len(op.kind))
    while True:
        okind = np.zeros(cap, dtype=np.uint8)
        opts = np.zeros((cap, 8), dtype=np.float64)
        osub = np.zeros(cap + 1, dtype=np.uint32)
        nsub = ctypes.c_long(0)
        n = L.rzo_stroke(_ptr(op.kind), _ptr(op.pts), _ptr(op.sub_off), op.nsub, _ptr(closed), float(width),
                         int(line_join), float(miter_limit), int(line_cap), _ptr(okind), _ptr(opts), cap, _ptr(osub),
                         cap + 1, ctypes.byref(nsub))
        if n >= 0:
            break
        cap *= 4
    return OraclePath(okind[:n].copy(), opts[:n].copy(), osub[:nsub.value + 1].copy())
