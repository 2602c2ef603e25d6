"""`Rasterizer` trait mirror and the GPU implementation.

``GpuRasterizer`` implements the reference's ``Rasterizer`` trait
(src/rasterize.rs:44-101) on top of the C ABI: ``name``, ``mask`` (f64 image
with arbitrary strides, SD semantics), ``mask_iter`` (sparse pixels) and
``fill`` (paint + source-over composite), plus the batched entry points the
reference does not have (``mask_batch``).  There is no CPU fallback: without
the CUDA library or a GPU every call raises ``RasterizeError``.
"""
from __future__ import annotations

import abc
import atexit
import ctypes
import os
import weakref
from dataclasses import dataclass

import numpy as np

from . import _ffi
from . import paint as _paint
from .geometry import Size, Transform
from .path import DEFAULT_FLATNESS, FillRule, Path


@dataclass(frozen=True)
class Pixel:
    """src/rasterize.rs:664-672"""

    x: int
    y: int
    alpha: float


class Rasterizer(abc.ABC):
    """Basic rasterizer interface (src/rasterize.rs:44-101)."""

    @abc.abstractmethod
    def name(self) -> str: ...

    @abc.abstractmethod
    def mask(self, path: Path, tr: Transform, img: np.ndarray, fill_rule: FillRule) -> None: ...

    @abc.abstractmethod
    def mask_iter(self, path: Path, tr: Transform, size: Size, fill_rule: FillRule): ...


# Plans and contexts are released before interpreter shutdown tears down the
# CUDA runtime: plans first (they use their context's stream), then contexts.
_live_plans = weakref.WeakSet()
_live_contexts = weakref.WeakSet()
_finalized = [False]


def _release_all():
    for p in list(_live_plans):
        p.close()
    for c in list(_live_contexts):
        c.close()
    _finalized[0] = True


atexit.register(_release_all)


def _path_struct(path: Path):
    keep = (path.kind, path.pts, path.subpath_off, path.closed)
    s = _ffi.RzPath(path.kind.ctypes.data, path.pts.ctypes.data, path.subpath_off.ctypes.data,
                    path.closed.ctypes.data if path.closed.size else None, path.n_segments, path.n_subpaths)
    return s, keep


def _tr_array(tr) -> np.ndarray:
    m = tr.m if hasattr(tr, "m") else tr
    return np.ascontiguousarray(m, dtype=np.float64)


class Context:
    """Owns one ``rz_ctx`` (a CUDA stream and device buffers) on a device."""

    def __init__(self, device: int = 0):
        self.lib = _ffi.load()
        st = ctypes.c_int32(0)
        self.ptr = self.lib.rz_create(device, ctypes.byref(st))
        if not self.ptr:
            raise _ffi.RasterizeError(st.value or 4, "cannot create a context on CUDA device %d" % device)
        self.device = device
        _live_contexts.add(self)

    def check(self, status):
        _ffi.check(self.lib, self.ptr, status)

    @property
    def stream(self) -> int:
        return self.lib.rz_get_stream(self.ptr) or 0

    def set_stream(self, stream_ptr: int):
        """Runs on the given cudaStream_t (0 = the legacy default stream)."""
        self.check(self.lib.rz_set_stream(self.ptr, stream_ptr or None))

    def synchronize(self):
        self.check(self.lib.rz_synchronize(self.ptr))

    def close(self):
        if getattr(self, "ptr", None) and not _finalized[0]:
            for p in list(_live_plans):
                if p.ctx is self:
                    p.close()
            self.lib.rz_destroy(self.ptr)
        self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = {}


def default_context(device: int = 0) -> Context:
    ctx = _default_ctx.get(device)
    if ctx is None:
        ctx = _default_ctx[device] = Context(device)
    return ctx


class MaskBatch:
    """Many independent paths, each rendered into its own f32 mask.

    Masks are packed row-major into one buffer; ``descs`` holds each mask's
    (offset, width, height, row_stride).  Row strides are rounded up to a
    multiple of 4 so rows start 16-byte aligned for vector stores.
    """

    def __init__(self, paths, sizes, transforms=None, fill_rules=None, align: int = 4):
        self.paths = list(paths)
        n = len(self.paths)
        self.kind = np.ascontiguousarray(np.concatenate([p.kind for p in self.paths]) if n else np.zeros(0, np.uint8))
        self.pts = np.ascontiguousarray(np.concatenate([p.pts for p in self.paths]) if n else np.zeros((0, 8)))
        sub = [0]
        psub = [0]
        base = 0
        for p in self.paths:
            sub.extend((p.subpath_off[1:].astype(np.int64) + base).tolist())
            base += p.n_segments
            psub.append(len(sub) - 1)
        self.sub_off = np.ascontiguousarray(np.asarray(sub, dtype=np.uint32))
        self.path_sub = np.ascontiguousarray(np.asarray(psub, dtype=np.uint32))
        self.transforms = None
        if transforms is not None:
            self.transforms = np.ascontiguousarray(np.array([_tr_array(t) for t in transforms]).reshape(n, 6))
        self.fill_rules = None
        if fill_rules is not None:
            self.fill_rules = np.ascontiguousarray(np.asarray([int(r) for r in fill_rules], dtype=np.uint8))
        self.descs = (_ffi.RzMaskDesc * max(n, 1))()
        off = 0
        for i, (w, h) in enumerate(sizes):
            rs = (int(w) + align - 1) // align * align
            self.descs[i] = _ffi.RzMaskDesc(off, int(w), int(h), rs, 0)
            off += rs * int(h)
            off = (off + 3) // 4 * 4
        self.out_len = off
        self.sizes = [(int(w), int(h)) for w, h in sizes]

    @property
    def n_paths(self) -> int:
        return len(self.paths)

    @property
    def n_segments(self) -> int:
        return int(self.kind.shape[0])

    @property
    def pixels(self) -> int:
        return int(sum(w * h for w, h in self.sizes))

    def struct(self, memory=_ffi.RZ_MEM_HOST, device_ptrs=None):
        """rz_path_batch over host arrays, or over ``device_ptrs`` (dict of
        device addresses for kind/pts/sub_off/path_sub/transforms/fill_rules)."""
        if memory == _ffi.RZ_MEM_HOST:
            d = dict(kind=self.kind.ctypes.data, pts=self.pts.ctypes.data, sub_off=self.sub_off.ctypes.data,
                     path_sub=self.path_sub.ctypes.data,
                     transforms=self.transforms.ctypes.data if self.transforms is not None else None,
                     fill_rules=self.fill_rules.ctypes.data if self.fill_rules is not None else None)
        else:
            d = device_ptrs
        return _ffi.RzPathBatch(self.n_paths, self.n_segments, len(self.sub_off) - 1, memory, d["kind"], d["pts"],
                                d["sub_off"], d["path_sub"], d.get("transforms"), d.get("fill_rules"),
                                ctypes.addressof(self.descs))

    def mask(self, out: np.ndarray, i: int) -> np.ndarray:
        d = self.descs[i]
        flat = out.reshape(-1)
        return flat[d.offset:d.offset + d.row_stride * d.height].reshape(d.height, d.row_stride)[:, :d.width]


class Scene:
    """A scene tree (SceneInner, src/scene.rs:19-62).  A Scene made with
    ``Scene()`` is a Group: ``fill`` appends a Fill (with the fill's own
    transform) and ``add`` a child scene; ``opacity``, ``clip`` and
    ``transform`` wrap a scene like the reference's builders (src/scene.rs:85-150,
    nested opacities and transforms merged, a group of one child is the child).
    ``GpuRasterizer.render_scene`` renders it like ``Scene::render`` with
    view = canvas: a Group of Fills goes through ``rz_render_scene``, anything
    else through ``rz_render_scene_tree``."""

    _version = 0  # bumped by every mutation of any Scene: packed trees are reused only while it is unchanged

    def __init__(self, kind: str = "group", children=None, **params):
        self.kind = kind
        self.children = list(children or [])  # fills as (path, tr, rule, paint) tuples, or Scenes
        self.params = params
        self._packed = None
        self._tree = None

    def _touch(self):
        Scene._version += 1
        self._packed = None

    # ---- builders
    def fill(self, path: Path, paint, tr: Transform | None = None, fill_rule: FillRule = FillRule.NonZero):
        """Appends a Fill to this Group (``tr``: the fill's own transform)."""
        if self.kind != "group":
            raise TypeError("fill() appends to a group")
        self.children.append((path, tr or Transform.identity(), FillRule(fill_rule), paint))
        self._touch()
        return self

    def stroke(self, path: Path, paint, style, tr: Transform | None = None):
        """Appends a Stroke (src/scene.rs:29-35) to this Group: ``path``
        stroked with ``style`` (a StrokeStyle), filled NonZero with ``paint``."""
        if self.kind != "group":
            raise TypeError("stroke() appends to a group")
        self.children.append(Scene("stroke", path=path, paint=paint, style=style, tr=tr or Transform.identity()))
        self._touch()
        return self

    def add(self, child: "Scene"):
        """Appends a child scene to this Group."""
        if self.kind != "group":
            raise TypeError("add() appends to a group")
        self.children.append(child)
        self._touch()
        return self

    @staticmethod
    def group(children) -> "Scene":
        """Scene::group (src/scene.rs:101-107): one child is the child itself."""
        children = list(children)
        if len(children) == 1 and isinstance(children[0], Scene):
            return children[0]
        return Scene("group", children)

    def opacity(self, opacity: float) -> "Scene":
        """Scene::opacity (src/scene.rs:110-125): clamped to [0, 1], nested opacities multiply."""
        opacity = min(max(float(opacity), 0.0), 1.0)
        if self.kind == "opacity":
            return self.children[0].opacity(opacity * self.params["opacity"])
        return Scene("opacity", [self], opacity=opacity)

    def clip(self, path: Path, units=_paint.Units.UserSpaceOnUse, fill_rule: FillRule = FillRule.NonZero) -> "Scene":
        """Scene::clip (src/scene.rs:128-136)."""
        return Scene("clip", [self], path=path, units=int(units), rule=FillRule(fill_rule))

    def transform(self, tr: Transform) -> "Scene":
        """Scene::transform (src/scene.rs:139-150): nested transforms compose."""
        if self.kind == "transform":
            return self.children[0].transform(tr * self.params["tr"])
        return Scene("transform", [self], tr=tr)

    # ---- views
    @property
    def fills(self):
        """Every Fill in drawing order as (path, tr, rule, paint)."""
        if self.kind == "group" and all(isinstance(c, tuple) for c in self.children):
            return self.children
        out = []
        for c in self.children:
            out.extend([c] if isinstance(c, tuple) else c.fills)
        return out

    def is_flat(self) -> bool:
        return self.kind == "group" and all(isinstance(c, tuple) for c in self.children)

    def entries_and_nodes(self):
        """The fill entries (fills in drawing order, then clip paths with a
        transparent paint) and the pre-order node list of rz_render_scene_tree."""
        entries, nodes = [], []

        def walk(sc):
            if isinstance(sc, tuple):
                nodes.append(("fill", len(entries)))
                entries.append(sc)
                return
            if sc.kind == "group":
                nodes.append(("group", len(sc.children)))
                for c in sc.children:
                    walk(c)
            elif sc.kind == "opacity":
                nodes.append(("opacity", sc.params["opacity"]))
                walk(sc.children[0])
            elif sc.kind == "transform":
                nodes.append(("transform", sc.params["tr"]))
                walk(sc.children[0])
            elif sc.kind == "stroke":
                nodes.append(("stroke", len(entries), sc.params["style"]))
                entries.append((sc.params["path"], sc.params["tr"], FillRule.NonZero, sc.params["paint"]))
            else:
                i = len(nodes)
                nodes.append(None)
                clip_entry = (sc.params["path"], Transform.identity(), sc.params["rule"], _paint.LinColor(0, 0, 0, 0))
                walk(sc.children[0])
                nodes[i] = ("clip", clip_entry, sc.params["units"])

        walk(self)
        # clip paths become entries after the fills
        out = (_ffi.RzSceneNode * max(len(nodes), 1))()
        for i, nd in enumerate(nodes):
            k = nd[0]
            if k == "fill":
                out[i].kind, out[i].arg = _ffi.NODE_FILL, nd[1]
            elif k == "group":
                out[i].kind, out[i].arg = _ffi.NODE_GROUP, nd[1]
            elif k == "opacity":
                out[i].kind, out[i].opacity = _ffi.NODE_OPACITY, nd[1]
            elif k == "transform":
                out[i].kind = _ffi.NODE_TRANSFORM
                for j in range(6):
                    out[i].tr[j] = nd[1].m[j]
            elif k == "stroke":
                st = nd[2]
                out[i].kind, out[i].arg = _ffi.NODE_STROKE, nd[1]
                out[i].width, out[i].miter_limit = st.width, st.miter_limit
                out[i].line_join, out[i].line_cap = int(st.line_join), int(st.line_cap)
            else:
                out[i].kind, out[i].arg, out[i].units = _ffi.NODE_CLIP, len(entries), nd[2]
                entries.append(nd[1])
        return entries, out, len(nodes)

    def pack(self):
        """(rz_scene struct, keepalive) over host arrays; for a tree also the
        node array: (struct, keepalive, nodes, n_nodes)."""
        key = (len(self.children), self.is_flat())
        if self._packed is not None and self._packed[2] == key:
            return self._packed[0], self._packed[1]
        if self.is_flat():
            entries, nodes, n_nodes = self.children, None, 0
        else:
            entries, nodes, n_nodes = self.entries_and_nodes()
        s, keep = _pack_entries(entries)
        keep = (keep, nodes, n_nodes)
        self._packed = (s, keep, key)
        return s, keep


def _pack_entries(entries):
    """rz_scene over fill entries (path, tr, rule, paint)."""
    paths = [f[0] for f in entries]
    n = len(paths)
    kind = np.ascontiguousarray(np.concatenate([p.kind for p in paths]) if n else np.zeros(0, np.uint8))
    pts = np.ascontiguousarray(np.concatenate([p.pts for p in paths]) if n else np.zeros((0, 8)))
    nseg = np.array([p.n_segments for p in paths], dtype=np.int64)
    seg_base = np.concatenate([[0], np.cumsum(nseg)[:-1]]) if n else np.zeros(0, np.int64)
    parts = [np.zeros(1, np.int64)] + [p.subpath_off[1:].astype(np.int64) + b for p, b in zip(paths, seg_base)]
    sub = np.ascontiguousarray(np.concatenate(parts).astype(np.uint32))
    nsub = np.array([len(p.subpath_off) - 1 for p in paths], dtype=np.int64)
    fsub = np.ascontiguousarray(np.concatenate([[0], np.cumsum(nsub)]).astype(np.uint32))
    trs = np.ascontiguousarray(np.array([f[1].m for f in entries], dtype=np.float64).reshape(-1))
    rules = np.ascontiguousarray(np.array([int(f[2]) for f in entries], dtype=np.uint8))
    structs, keep = [], []
    for f in entries:
        st, k = _paint.to_struct(f[3])
        structs.append(st)
        keep.append(k)
    paints = (_paint.RzPaint * max(n, 1))(*structs)
    fpaint = np.ascontiguousarray(np.arange(n, dtype=np.uint32))
    closed = np.ascontiguousarray(np.concatenate(
        [np.resize(np.asarray(p.closed, np.uint8), len(p.subpath_off) - 1) if len(p.closed) else
         np.zeros(len(p.subpath_off) - 1, np.uint8) for p in paths]) if n else np.zeros(0, np.uint8))
    s = _ffi.RzScene(n, int(kind.shape[0]), len(sub) - 1, n, kind.ctypes.data, pts.ctypes.data, sub.ctypes.data,
                     fsub.ctypes.data, trs.ctypes.data if n else None, rules.ctypes.data if n else None,
                     fpaint.ctypes.data if n else None, ctypes.addressof(paints),
                     closed.ctypes.data if closed.size else None)
    return s, (kind, pts, sub, fsub, trs, rules, fpaint, paints, keep, closed)


def _tune_key(device: str, batch: "MaskBatch", flatness: float) -> str:
    """GPU + batch kernel + batch shape (paths, segments and pixels to two significant digits, flatness)."""
    def sig2(v):
        return "%.1e" % float(v) if v else "0"
    kernel = os.environ.get("RZ_BATCH_KERNEL") or "glyph"
    return "%s|%s|paths=%s|segs=%s|px=%s|f=%g" % (device, kernel, sig2(len(batch.paths)), sig2(batch.n_segments),
                                                  sig2(batch.pixels), flatness)


class DiffBatch:
    """The differentiable batch: ``n_images`` images of (height, width), each
    the alpha channel of ``paths`` closed cubic paths of ``segs`` segments
    filled in order with one solid paint of alpha ``alpha`` (Rasterizer::fill
    + source-over).  ``ctrl_ptr``: device FP32 control points, shape
    (n_images, paths, 3 * segs, 2); segment s is (V_s, C1_s, C2_s, V_{s+1})
    with V_s = point 3s."""

    def __init__(self, n_images, paths, segs, width, height, ctrl_ptr, alpha=0.5, fill_rule=FillRule.NonZero):
        self.n_images, self.paths, self.segs = int(n_images), int(paths), int(segs)
        self.width, self.height = int(width), int(height)
        self.ctrl_ptr, self.alpha, self.fill_rule = int(ctrl_ptr), float(alpha), FillRule(fill_rule)

    @property
    def n_pixels(self):
        return self.n_images * self.width * self.height

    @property
    def n_ctrl(self):
        return self.n_images * self.paths * self.segs * 3 * 2

    def struct(self):
        return _ffi.RzDiffBatch(self.n_images, self.paths, self.segs, self.width, self.height, int(self.fill_rule),
                                self.alpha, self.ctrl_ptr)


class BatchPlan:
    """A device-resident batch bound to its output: work list uploaded once,
    each ``launch()`` replays a captured CUDA graph (no host synchronisation)."""

    def __init__(self, ctx: Context, batch: MaskBatch, device_ptrs: dict, out_ptr: int, flatness: float):
        self.ctx = ctx
        self.batch = batch
        self._struct = batch.struct(_ffi.RZ_MEM_DEVICE, device_ptrs)
        st = ctypes.c_int32(0)
        self.ptr = ctx.lib.rz_batch_plan_create(ctx.ptr, ctypes.byref(self._struct), flatness, out_ptr,
                                                batch.out_len, ctypes.byref(st))
        if not self.ptr:
            ctx.check(st.value or 2)
        _live_plans.add(self)

    def launch(self):
        self.ctx.check(self.ctx.lib.rz_batch_plan_launch(self.ptr))

    def status(self):
        self.ctx.check(self.ctx.lib.rz_batch_plan_status(self.ptr))

    def info(self):
        n, f = ctypes.c_uint64(0), ctypes.c_uint64(0)
        self.ctx.check(self.ctx.lib.rz_batch_plan_info(self.ptr, ctypes.byref(n), ctypes.byref(f)))
        return int(n.value), int(f.value)

    def close(self):
        if getattr(self, "ptr", None) and not _finalized[0]:
            self.ctx.lib.rz_batch_plan_destroy(self.ptr)
        self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuRasterizer(Rasterizer):
    """Signed-difference rasterizer on the GPU (drop-in for
    ``SignedDifferenceRasterizer``, src/rasterize.rs:279-360)."""

    def __init__(self, flatness: float = DEFAULT_FLATNESS, device: int = 0, context: Context | None = None):
        self.flatness = float(flatness)
        self.ctx = context or default_context(device)

    def name(self) -> str:
        return "gpu-signed-difference"

    def mask(self, path: Path, tr: Transform, img: np.ndarray, fill_rule: FillRule) -> None:
        """Rasterizer::mask into a 2-D float64 array (any positive strides)."""
        if img.dtype != np.float64 or img.ndim != 2:
            raise TypeError("mask image must be a 2-D float64 array")
        if any(s < 0 or s % 8 for s in img.strides):
            raise ValueError("mask image strides must be positive multiples of 8 bytes")
        h, w = img.shape
        shape = _ffi.RzShape(0, w, h, img.strides[0] // 8, img.strides[1] // 8)
        ps, keep = _path_struct(path)
        tr_a = _tr_array(tr)
        lib = self.ctx.lib
        self.ctx.check(lib.rz_mask(self.ctx.ptr, ctypes.byref(ps), tr_a.ctypes.data, int(fill_rule), self.flatness,
                                   img.ctypes.data, shape))

    def mask_iter(self, path: Path, tr: Transform, size: Size, fill_rule: FillRule):
        """Rasterizer::mask_iter: yields Pixel(x, y, alpha) in row-major order."""
        ps, keep = _path_struct(path)
        tr_a = _tr_array(tr)
        lib = self.ctx.lib
        n = ctypes.c_uint64(0)
        cap = int(size.width) * int(size.height)
        buf = (_ffi.RzPixel * max(cap, 1))()
        self.ctx.check(lib.rz_mask_iter(self.ctx.ptr, ctypes.byref(ps), tr_a.ctypes.data, int(fill_rule),
                                        self.flatness, int(size.width), int(size.height), buf, cap,
                                        ctypes.byref(n)))
        for i in range(n.value):
            p = buf[i]
            yield Pixel(int(p.x), int(p.y), float(p.alpha))

    def mask_iter_dense(self, path: Path, tr: Transform, size: Size, fill_rule: FillRule) -> np.ndarray:
        out = np.zeros((size.height, size.width), dtype=np.float64)
        for p in self.mask_iter(path, tr, size, fill_rule):
            out[p.y, p.x] = p.alpha
        return out

    def fill(self, path: Path, tr: Transform, fill_rule: FillRule, paint, img: np.ndarray) -> None:
        """Rasterizer::fill: paints ``path`` source-over into a (H, W, 4) float32
        image of premultiplied linear RGBA (any positive pixel strides)."""
        if img.dtype != np.float32 or img.ndim != 3 or img.shape[2] != 4 or img.strides[2] != 4:
            raise TypeError("fill image must be a (H, W, 4) float32 array with contiguous channels")
        if any(st < 0 or st % 16 for st in img.strides[:2]):
            raise ValueError("fill image pixel strides must be positive multiples of 16 bytes")
        h, w = img.shape[:2]
        shape = _ffi.RzShape(0, w, h, img.strides[0] // 16, img.strides[1] // 16)
        ps, keep = _path_struct(path)
        pst, pkeep = _paint.to_struct(paint)
        tr_a = _tr_array(tr)
        lib = self.ctx.lib
        self.ctx.check(lib.rz_fill(self.ctx.ptr, ctypes.byref(ps), tr_a.ctypes.data, int(fill_rule), self.flatness,
                                   ctypes.addressof(pst), img.ctypes.data, shape))

    def render_scene(self, scene: Scene, width: int, height: int, bg=None, tree: bool | None = None) -> np.ndarray:
        """Scene::render over a (height, width, 4) float32 canvas initialised to bg
        (``tree=True`` sends a flat group through the scene-tree path too)."""
        canvas = np.zeros((height, width, 4), dtype=np.float32)
        self._render(scene, width, height, bg, canvas, None, tree)
        return canvas

    def render_scene_rgba8(self, scene: Scene, width: int, height: int, bg=None, tree: bool | None = None) -> np.ndarray:
        """Scene::render, then `to_rgba` of every pixel: (height, width, 4) uint8
        sRGB, encoded on the GPU (in the composite's epilogue for a flat group)."""
        out = np.zeros((height, width, 4), dtype=np.uint8)
        self._render(scene, width, height, bg, None, out, tree)
        return out

    def _render(self, scene, width, height, bg, canvas, rgba8, tree):
        bg_a = np.ascontiguousarray(bg, dtype=np.float32) if bg is not None else None
        bg_p = bg_a.ctypes.data if bg_a is not None else None
        lib = self.ctx.lib
        if tree is None:
            tree = not scene.is_flat()
        if not tree:
            s, keep = scene.pack()
            if canvas is not None:
                self.ctx.check(lib.rz_render_scene(self.ctx.ptr, ctypes.byref(s), self.flatness, bg_p,
                                                   canvas.ctypes.data, width, height))
            else:
                self.ctx.check(lib.rz_render_scene_rgba8(self.ctx.ptr, ctypes.byref(s), self.flatness, bg_p,
                                                         rgba8.ctypes.data, width, height))
            return
        if scene._tree is None or scene._tree[0] != Scene._version:
            entries, nodes, n_nodes = scene.entries_and_nodes()
            s, keep = _pack_entries(entries)
            scene._tree = (Scene._version, s, keep, nodes, n_nodes)
        _, s, keep, nodes, n_nodes = scene._tree
        self.ctx.check(lib.rz_render_scene_tree(self.ctx.ptr, ctypes.byref(s), ctypes.addressof(nodes), n_nodes,
                                                self.flatness, bg_p,
                                                canvas.ctypes.data if canvas is not None else None,
                                                rgba8.ctypes.data if rgba8 is not None else None, width, height))

    def encode_rgba8(self, canvas: np.ndarray) -> np.ndarray:
        """`to_rgba` of premultiplied linear RGBA f32 pixels (..., 4) -> uint8 (..., 4)."""
        c = np.ascontiguousarray(canvas, dtype=np.float32)
        if c.shape[-1] != 4:
            raise ValueError("canvas must end in 4 channels")
        out = np.zeros(c.shape, dtype=np.uint8)
        lib = self.ctx.lib
        self.ctx.check(lib.rz_encode_rgba8(self.ctx.ptr, c.ctypes.data, c.size // 4, out.ctypes.data, 0))
        return out

    def encode_mask_rgba8(self, mask: np.ndarray) -> np.ndarray:
        """`to_rgba` of a mask (f64 or f32): grey sRGB of 1 - m, opaque; shape (..., 4) uint8."""
        m = np.ascontiguousarray(mask)
        if m.dtype not in (np.float32, np.float64):
            m = m.astype(np.float64)
        out = np.zeros(m.shape + (4,), dtype=np.uint8)
        lib = self.ctx.lib
        self.ctx.check(lib.rz_encode_mask_rgba8(self.ctx.ptr, m.ctypes.data, m.itemsize, m.size, out.ctypes.data, 0))
        return out

    def flatten_counts(self, path: Path, tr: Transform) -> np.ndarray:
        """Lines per input segment, then one entry per subpath (closing line)."""
        ps, keep = _path_struct(path)
        tr_a = _tr_array(tr)
        n = path.n_segments + path.n_subpaths
        out = np.zeros(max(n, 1), dtype=np.uint32)
        got = ctypes.c_uint64(0)
        lib = self.ctx.lib
        self.ctx.check(lib.rz_flatten_counts(self.ctx.ptr, ctypes.byref(ps), tr_a.ctypes.data, self.flatness,
                                             out.ctypes.data, n, ctypes.byref(got)))
        return out[:n]

    def mask_batch(self, batch: MaskBatch, out: np.ndarray | None = None, per_path: bool = False) -> np.ndarray:
        """Renders every path of ``batch`` into its own mask (host memory)."""
        if out is None:
            out = np.zeros(max(batch.out_len, 1), dtype=np.float32)
        s = batch.struct()
        lib = self.ctx.lib
        fn = lib.rz_mask_batch_per_path if per_path else lib.rz_mask_batch
        self.ctx.check(fn(self.ctx.ptr, ctypes.byref(s), self.flatness, out.ctypes.data, batch.out_len))
        return out

    def plan(self, batch: MaskBatch, device_ptrs: dict, out_ptr: int) -> BatchPlan:
        return BatchPlan(self.ctx, batch, device_ptrs, out_ptr, self.flatness)

    # ---- batch autotuner
    def tune(self, batch: MaskBatch, device_ptrs: dict, out_ptr: int, cache: str | None = None,
             retune: bool = False) -> dict:
        """Chooses the band-height cap and resident CTAs per SM for batches
        like ``batch`` (device memory) by timing every candidate, and applies
        it to this context.  Results are stored in a JSON file (``cache``,
        default $RZ_TUNE_CACHE or ~/.cache/rasterize_gb300/tune.json) keyed by
        the GPU and the batch's shape, so later processes apply them without
        re-timing."""
        import json
        lib = self.ctx.lib
        path = cache or os.environ.get("RZ_TUNE_CACHE") or os.path.join(
            os.path.expanduser("~"), ".cache", "rasterize_gb300", "tune.json")
        key = _tune_key(lib.rz_device_name(self.ctx.ptr).decode(), batch, self.flatness)
        try:
            with open(path) as f:
                table = json.load(f)
        except (OSError, ValueError):
            table = {}
        if not retune and key in table:
            e = table[key]
            self.ctx.check(lib.rz_set_tuning(self.ctx.ptr, int(e["band_rows_cap"]), int(e["ctas_per_sm"]),
                                             int(e.get("walk_slots", 0))))
            return dict(e, cached=True)
        s = batch.struct(_ffi.RZ_MEM_DEVICE, device_ptrs)
        res = _ffi.RzTuneResult()
        self.ctx.check(lib.rz_tune_batch(self.ctx.ptr, ctypes.byref(s), self.flatness, out_ptr, batch.out_len,
                                         ctypes.byref(res)))
        entry = {"band_rows_cap": res.band_rows_cap, "ctas_per_sm": res.ctas_per_sm, "walk_slots": res.walk_slots,
                 "ms": res.ms,
                 "candidates": [[e.band_rows_cap, e.ctas_per_sm, e.walk_slots, e.ms]
                                for e in res.entries[:res.n_entries]]}
        table[key] = entry
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            tmp = path + ".tmp.%d" % os.getpid()
            with open(tmp, "w") as f:
                json.dump(table, f, indent=1, sort_keys=True)
            os.replace(tmp, path)
        except OSError:
            pass
        return dict(entry, cached=False)

    def set_tuning(self, band_rows_cap: int = 0, ctas_per_sm: int = 0, walk_slots: int = 0) -> None:
        self.ctx.check(self.ctx.lib.rz_set_tuning(self.ctx.ptr, int(band_rows_cap), int(ctas_per_sm),
                                                  int(walk_slots)))

    # ---- differentiable batch (device pointers)
    def diff_forward(self, batch: DiffBatch, image_ptr: int) -> None:
        """Renders every image of ``batch`` into ``image_ptr`` (device f32)."""
        s = batch.struct()
        self.ctx.check(self.ctx.lib.rz_diff_forward(self.ctx.ptr, ctypes.byref(s), self.flatness, image_ptr))

    def l2_loss(self, image_ptr: int, target_ptr: int, n: int, dl_ptr: int | None = None) -> float:
        """sum (image - target)^2 (binary64); ``dl_ptr`` receives 2 (image - target)."""
        out = ctypes.c_double(0.0)
        self.ctx.check(self.ctx.lib.rz_l2_loss(self.ctx.ptr, image_ptr, target_ptr, n, ctypes.byref(out), dl_ptr))
        return float(out.value)

    def diff_backward(self, batch: DiffBatch, image_ptr: int, dl_ptr: int, out_ptr: int) -> None:
        """d loss / d control points into ``out_ptr`` (device f32, the layout
        of the control points) from d loss / d image, tree held fixed."""
        s = batch.struct()
        self.ctx.check(self.ctx.lib.rasterize_backward(self.ctx.ptr, ctypes.byref(s), self.flatness, image_ptr,
                                                       dl_ptr, out_ptr))

    def mask_batch_device(self, batch: MaskBatch, device_ptrs: dict, out_ptr: int, per_path: bool = False):
        """Same with inputs and output already in device memory (no copies)."""
        s = batch.struct(_ffi.RZ_MEM_DEVICE, device_ptrs)
        lib = self.ctx.lib
        fn = lib.rz_mask_batch_per_path if per_path else lib.rz_mask_batch
        self.ctx.check(fn(self.ctx.ptr, ctypes.byref(s), self.flatness, out_ptr, batch.out_len))
