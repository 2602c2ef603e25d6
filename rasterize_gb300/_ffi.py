"""ctypes binding of the C ABI (include/rasterize_gb300.h).

The library is built in-tree (``python -m rasterize_gb300.build``) and loaded
from ``rasterize_gb300/_lib``.  There is no fallback: if the library is
missing or no CUDA device is present, the calls raise.
"""
from __future__ import annotations

import ctypes
import os
import re
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "librasterize_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "rasterize_gb300.h")

RZ_OK = 0
STATUS_NAMES = {0: "RZ_OK", 1: "RZ_ERR_NAN", 2: "RZ_ERR_INVALID", 3: "RZ_ERR_CUDA", 4: "RZ_ERR_NO_DEVICE",
                5: "RZ_ERR_DEPTH", 6: "RZ_ERR_ARC", 7: "RZ_ERR_CAPACITY"}
RZ_MEM_HOST, RZ_MEM_DEVICE = 0, 1


class RasterizeError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), message))
        self.status = status


class NanError(RasterizeError):
    """Raised where the reference panics: 'cannot flatten segment with NaN'."""


class RzPath(ctypes.Structure):
    _fields_ = [("seg_kind", ctypes.c_void_p), ("seg_pts", ctypes.c_void_p), ("subpath_off", ctypes.c_void_p),
                ("closed", ctypes.c_void_p), ("n_segments", ctypes.c_uint32), ("n_subpaths", ctypes.c_uint32)]


class RzShape(ctypes.Structure):
    _fields_ = [("start", ctypes.c_uint64), ("width", ctypes.c_uint64), ("height", ctypes.c_uint64),
                ("row_stride", ctypes.c_uint64), ("col_stride", ctypes.c_uint64)]


class RzPixel(ctypes.Structure):
    _fields_ = [("x", ctypes.c_uint64), ("y", ctypes.c_uint64), ("alpha", ctypes.c_double)]


class RzMaskDesc(ctypes.Structure):
    _fields_ = [("offset", ctypes.c_uint64), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("row_stride", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class RzPathBatch(ctypes.Structure):
    _fields_ = [("n_paths", ctypes.c_uint32), ("n_segments", ctypes.c_uint32), ("n_subpaths", ctypes.c_uint32),
                ("memory", ctypes.c_int32), ("seg_kind", ctypes.c_void_p), ("seg_pts", ctypes.c_void_p),
                ("subpath_off", ctypes.c_void_p), ("path_subpath_off", ctypes.c_void_p),
                ("transforms", ctypes.c_void_p), ("fill_rules", ctypes.c_void_p), ("masks", ctypes.c_void_p)]


class RzScene(ctypes.Structure):
    _fields_ = [("n_fills", ctypes.c_uint32), ("n_segments", ctypes.c_uint32), ("n_subpaths", ctypes.c_uint32),
                ("n_paints", ctypes.c_uint32), ("seg_kind", ctypes.c_void_p), ("seg_pts", ctypes.c_void_p),
                ("subpath_off", ctypes.c_void_p), ("fill_subpath_off", ctypes.c_void_p),
                ("transforms", ctypes.c_void_p), ("fill_rules", ctypes.c_void_p), ("fill_paint", ctypes.c_void_p),
                ("paints", ctypes.c_void_p), ("subpath_closed", ctypes.c_void_p)]


class RzStrokeStyle(ctypes.Structure):
    _fields_ = [("width", ctypes.c_double), ("miter_limit", ctypes.c_double), ("line_join", ctypes.c_int32),
                ("line_cap", ctypes.c_int32)]


class RzSceneNode(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("arg", ctypes.c_uint32), ("units", ctypes.c_int32),
                ("line_join", ctypes.c_int32), ("line_cap", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("opacity", ctypes.c_double), ("width", ctypes.c_double), ("miter_limit", ctypes.c_double),
                ("tr", ctypes.c_double * 6)]


NODE_FILL, NODE_GROUP, NODE_TRANSFORM, NODE_OPACITY, NODE_CLIP, NODE_STROKE = 0, 1, 2, 3, 4, 5


class RzDiffBatch(ctypes.Structure):
    _fields_ = [("n_images", ctypes.c_uint32), ("paths_per_image", ctypes.c_uint32), ("segs_per_path", ctypes.c_uint32),
                ("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("fill_rule", ctypes.c_int32),
                ("paint_alpha", ctypes.c_float), ("ctrl", ctypes.c_void_p)]


class RzTuneEntry(ctypes.Structure):
    _fields_ = [("band_rows_cap", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32), ("ms", ctypes.c_float),
                ("walk_slots", ctypes.c_int32)]


class RzTuneResult(ctypes.Structure):
    _fields_ = [("band_rows_cap", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32), ("ms", ctypes.c_float),
                ("n_entries", ctypes.c_uint32), ("entries", RzTuneEntry * 24), ("walk_slots", ctypes.c_int32)]


_lock = threading.Lock()
_lib = None

P = ctypes.c_void_p
_SIGNATURES = {
    "rz_version": (ctypes.c_char_p, []),
    "rz_create": (P, [ctypes.c_int, ctypes.POINTER(ctypes.c_int32)]),
    "rz_destroy": (None, [P]),
    "rz_last_error": (ctypes.c_char_p, [P]),
    "rz_set_stream": (ctypes.c_int32, [P, P]),
    "rz_get_stream": (P, [P]),
    "rz_synchronize": (ctypes.c_int32, [P]),
    "rz_mask": (ctypes.c_int32, [P, ctypes.POINTER(RzPath), P, ctypes.c_int32, ctypes.c_double, P, RzShape]),
    "rz_mask_iter": (ctypes.c_int32, [P, ctypes.POINTER(RzPath), P, ctypes.c_int32, ctypes.c_double,
                                      ctypes.c_uint64, ctypes.c_uint64, P, ctypes.c_uint64,
                                      ctypes.POINTER(ctypes.c_uint64)]),
    "rz_mask_batch": (ctypes.c_int32, [P, ctypes.POINTER(RzPathBatch), ctypes.c_double, P, ctypes.c_uint64]),
    "rz_mask_batch_per_path": (ctypes.c_int32, [P, ctypes.POINTER(RzPathBatch), ctypes.c_double, P,
                                                ctypes.c_uint64]),
    "rz_flatten_counts": (ctypes.c_int32, [P, ctypes.POINTER(RzPath), P, ctypes.c_double, P, ctypes.c_uint64,
                                           ctypes.POINTER(ctypes.c_uint64)]),
    "rz_batch_plan_create": (P, [P, ctypes.POINTER(RzPathBatch), ctypes.c_double, P, ctypes.c_uint64,
                                 ctypes.POINTER(ctypes.c_int32)]),
    "rz_batch_plan_launch": (ctypes.c_int32, [P]),
    "rz_batch_plan_status": (ctypes.c_int32, [P]),
    "rz_batch_plan_info": (ctypes.c_int32, [P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]),
    "rz_batch_plan_destroy": (None, [P]),
    "rz_mask_batch_noalloc": (ctypes.c_int32, [ctypes.POINTER(RzPathBatch), ctypes.c_double, P, ctypes.c_uint64, P]),
    "rz_fill": (ctypes.c_int32, [P, ctypes.POINTER(RzPath), P, ctypes.c_int32, ctypes.c_double, P, P, RzShape]),
    "rz_render_scene": (ctypes.c_int32, [P, ctypes.POINTER(RzScene), ctypes.c_double, P, P, ctypes.c_uint32,
                                         ctypes.c_uint32]),
    "rz_render_scene_rgba8": (ctypes.c_int32, [P, ctypes.POINTER(RzScene), ctypes.c_double, P, P, ctypes.c_uint32,
                                               ctypes.c_uint32]),
    "rz_render_scene_tree": (ctypes.c_int32, [P, ctypes.POINTER(RzScene), P, ctypes.c_uint32, ctypes.c_double, P, P,
                                              P, ctypes.c_uint32, ctypes.c_uint32]),
    "rz_encode_rgba8": (ctypes.c_int32, [P, P, ctypes.c_uint64, P, ctypes.c_int32]),
    "rz_encode_mask_rgba8": (ctypes.c_int32, [P, P, ctypes.c_int32, ctypes.c_uint64, P, ctypes.c_int32]),
    "rz_stroke_path": (ctypes.c_int32, [ctypes.POINTER(RzPath), ctypes.POINTER(RzStrokeStyle), P, P, ctypes.c_uint32,
                                        P, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32),
                                        ctypes.POINTER(ctypes.c_uint32)]),
    "rz_write_image": (ctypes.c_int32, [P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int32, P, ctypes.c_uint64,
                                        ctypes.POINTER(ctypes.c_uint64)]),
    "rz_diff_forward": (ctypes.c_int32, [P, ctypes.POINTER(RzDiffBatch), ctypes.c_double, P]),
    "rz_l2_loss": (ctypes.c_int32, [P, P, P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double), P]),
    "rasterize_backward": (ctypes.c_int32, [P, ctypes.POINTER(RzDiffBatch), ctypes.c_double, P, P, P]),
    "rz_tune_batch": (ctypes.c_int32, [P, ctypes.POINTER(RzPathBatch), ctypes.c_double, P, ctypes.c_uint64,
                                       ctypes.POINTER(RzTuneResult)]),
    "rz_set_tuning": (ctypes.c_int32, [P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    "rz_device_name": (ctypes.c_char_p, [P]),
}


def header_symbols():
    """Function names declared in include/rasterize_gb300.h."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b((?:rz_|rasterize_)[a-z0-9_]+)\s*\(", text)) - {"rz_ctx"})


def load(path: str = LIB_PATH):
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(path):
                raise RasterizeError(4, "CUDA library not built: %s (run python -m rasterize_gb300.build)" % path)
            L = ctypes.CDLL(path)
            for name, (res, args) in _SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(lib, ctx, status):
    if status == RZ_OK:
        return
    msg = lib.rz_last_error(ctx)
    msg = msg.decode() if msg else ""
    if status == 1:
        raise NanError(status, msg)
    raise RasterizeError(status, msg)
