#!/usr/bin/env python
"""Benchmark of the rasterize hot path on GB300.

Workload (default, ``glyphs``): 10,000 independent closed glyph outlines,
10-400 segments each (log-uniform, 70 % cubic / 30 % quad), square boxes of
16-256 px (log-uniform), each rendered to its own f32 mask with NonZero fill
and flatness 0.05 (synthetic, seeded; ~1.07 M segments, ~118 Mpx per step).
One step = one pass of flatten + coverage + fill rule over the whole batch.

* ``value``      Mpx/s with inputs resident in HBM: the batch plan (the glyph
  pipeline's kernels replayed from a CUDA graph) launched back to back.
* ``e2e``        the same metric through the C ABI with host buffers
  (``rz_mask_batch``, pinned inputs in, masks back to pinned host memory).
* ``roofline``   one plan launch against the measured HBM copy bandwidth.
* ``cpu_baseline``  the CPU f64 oracle on a bounded sample, 1 thread.

``--impl reference`` times the reference's CPU algorithm (the oracle port,
the reference crate is Rust and cannot be built here) on all host cores.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mpx/s + segments/s, batched vs per-path GPU at ≤1e-4 err; backward ms/step"
WORKLOAD = "glyph_batch: 10000 closed glyphs, 10-400 segs (70% cubic/30% quad), 16-256 px masks, NonZero, f=0.05"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--glyphs", type=int, default=10000)
    ap.add_argument("--cpu-seconds", type=float, default=8.0, help="bounded CPU baseline sample")
    ap.add_argument("--load-seconds", type=float, default=1.0,
                    help="back-to-back launches just before the timed region, under the clock sampler")
    ap.add_argument("--no-per-path", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the C1/C2/C4/C5 legs")
    ap.add_argument("--workload", default="glyphs", choices=["glyphs", "small_path", "large_path", "scene", "diff", "encode", "scene_tree", "link"],
                    help="glyphs: the headline line; the others run one configuration leg alone")
    ap.add_argument("--diff-images", type=int, default=64, help="images of the diff workload")
    ap.add_argument("--fd-coords", type=int, default=100, help="finite-difference coordinates of the diff workload")
    ap.add_argument("--scene-fills", type=int, default=2000, help="fills of the scene workload")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.first = 0

    def mark(self):
        """Samples before this call (the sampler's own start-up) are left out."""
        self.first = len(self.lines)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines[self.first:]:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(ms, device=None):
    """The slowest rank's time (replicas: every rank renders its own batch)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return ms
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(name: str):
    """Per-launch DRAM bytes from the committed ncu summary (profiles/<name>.md)."""
    p = os.path.join(ROOT, "profiles", name + ".md")
    try:
        for line in open(p):
            if line.strip().startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1].strip().split()[0])
    except Exception:
        pass
    return None


def scan_launches(n):
    """Kernels of one exclusive scan of n words (rz_scan.cu: 1024-word blocks, recursive carries)."""
    blocks = (n + 1023) // 1024
    return 1 if blocks <= 1 else 2 + scan_launches(blocks)


def plan_kernels(batch):
    """Our kernels in one glyph-pipeline plan launch: records, walk, the chain-offset scan, emit, paths, cover."""
    slots = batch.n_segments + len(batch.sub_off) - 1
    return 5 + scan_launches(slots + 1)


def make_workload(n):
    from rasterize_gb300 import MaskBatch
    from rasterize_gb300 import workloads as W
    paths, sizes, rules = W.glyph_batch(seed=2, n=n)
    return paths, sizes, rules, MaskBatch(paths, sizes, fill_rules=rules)


# --------------------------------------------------------------------------- CPU
_WORKER = {}


def _oracle_init(n):
    """Pool initializer: the glyph batch, built once per worker process."""
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    from rasterize_gb300 import Transform
    from rasterize_gb300 import workloads as W
    O.build()
    _WORKER["paths"], _WORKER["sizes"], _WORKER["rules"] = W.glyph_batch(seed=2, n=n)
    _WORKER["O"], _WORKER["id"] = O, Transform.identity()


def _oracle_chunk(args):
    """Worker: renders glyphs start, start + stride, ... with the binary64
    oracle's SignedDifferenceRasterizer (rasterizer "sd") or
    ActiveEdgeRasterizer ("ae"); returns pixels."""
    start, stride = args[:2]
    rasterizer = args[2] if len(args) > 2 else "sd"
    O, tr = _WORKER["O"], _WORKER["id"]
    fn = O.mask if rasterizer == "sd" else O.mask_ae
    px = 0
    for i in range(start, len(_WORKER["paths"]), stride):
        w, h = _WORKER["sizes"][i]
        fn(_WORKER["paths"][i], tr, _WORKER["rules"][i], w, h)
        px += w * h
    return px


def headline_config(n_glyphs, segments, pixels, world):
    """The `config` of the headline line, the same for both arms."""
    return {"workload": WORKLOAD, "glyphs": n_glyphs, "segments": segments, "pixels_per_step": pixels,
            "flatness": 0.05, "parallelism": "replicas" if world > 1 else "single",
            "l2": "masks written per step (%.0f MB) exceed the 129 MB L2" % (pixels * 4 / 1e6)}


def cpu_baseline_single(paths, sizes, rules, seconds, gpu_masks=None):
    """The oracle (reference algorithm restated in C, f64) on 1 thread over a
    bounded prefix sample of the same batch.  With ``gpu_masks(i)`` it also
    returns the max / mean absolute difference of the GPU masks of that
    sample against the oracle's."""
    import numpy as np
    from oracle import oracle as O
    from rasterize_gb300 import Transform
    O.build()
    px, segs, n, dt = 0, 0, 0, 0.0
    emax, esum, en = 0.0, 0.0, 0
    for i in range(len(paths)):
        w, h = sizes[i]
        t = time.perf_counter()
        ref = O.mask(paths[i], Transform.identity(), rules[i], w, h)
        dt += time.perf_counter() - t
        px += w * h
        segs += paths[i].n_segments
        n += 1
        if gpu_masks is not None:
            e = np.abs(gpu_masks(i).astype(np.float64) - ref)
            emax = max(emax, float(e.max()))
            esum += float(e.sum())
            en += e.size
        if dt > seconds:
            break
    out = {"value": round(px / dt / 1e6, 3), "unit": "Mpx/s", "cores": 1, "kind": "port",
           "sample": "first %d of 10000 glyphs (%.1f Mpx, %d segments) in %.2f s" % (n, px / 1e6, segs, dt),
           "masks_per_s": round(n / dt, 2)}
    err = None
    if gpu_masks is not None:
        err = {"max_abs": emax, "mean_abs": esum / max(en, 1), "tolerance": 1e-4, "glyphs_checked": n}
    return out, err


def _event_ms(stream, fn, steps):
    """Median CUDA-event time of ``fn`` on ``stream`` (host buffers in and out)."""
    import torch
    ts = []
    for _ in range(steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    return statistics.median(ts)


def _config_err(gpu, ref):
    import numpy as np
    e = np.abs(gpu.astype(np.float64) - ref.astype(np.float64))
    return {"max_abs": float(e.max()), "mean_abs": float(e.mean()), "tolerance": 1e-4}


def run_configs(R, stream):
    """The other single-GPU configurations, each through the public API with
    host buffers (the ``gpu`` timing) and a CPU-baseline leg that times the
    oracle on the same input once and reports the GPU's error against it."""
    return {"C1_small_path": run_small(R, stream), "C2_large_path": run_large(R, stream),
            "C4_scene": run_scene(R, stream), "C5_diff": run_diff(R, stream), "encode": run_encode(R, stream),
            "scene_tree": run_scene_tree(R, stream)}


def run_small(R, stream):
    """C1: one closed path of 200 cubics in [0,512]^2, NonZero, 512x512 f64 mask."""
    import numpy as np
    from oracle import oracle as O
    from rasterize_gb300 import FillRule, Transform
    from rasterize_gb300 import workloads as W
    path, _, _ = W.small_path(seed=0, n_cubics=200, size=512)
    img = np.zeros((512, 512))

    def c1():
        img[:] = 0.0
        R.mask(path, Transform.identity(), img, FillRule.NonZero)
    c1()
    ms = _event_ms(stream, c1, 10)
    t = time.perf_counter()
    ref = O.mask(path, Transform.identity(), FillRule.NonZero, 512, 512)
    cpu_s = time.perf_counter() - t
    return {"ms": round(ms, 4), "mpx_per_s": round(512 * 512 / ms / 1e3, 1),
            "segments_per_s": round(200 / ms * 1e3, 1), "err": _config_err(img, ref),
            "cpu_baseline_ms": round(cpu_s * 1e3, 3), "cores": 1}


def run_large(R, stream):
    """C2: 20,000 mixed segments in [0,4096]^2 (10 % arcs, 1 % degenerate cubics), EvenOdd, 4096^2."""
    import numpy as np
    from oracle import oracle as O
    from rasterize_gb300 import Transform
    from rasterize_gb300 import workloads as W
    path, rule, _ = W.large_path(seed=1, n_segments=20000, size=4096)
    img = np.zeros((4096, 4096))

    def c2():
        img[:] = 0.0
        R.mask(path, Transform.identity(), img, rule)
    c2()
    ms = _event_ms(stream, c2, 5)
    t = time.perf_counter()
    ref = O.mask(path, Transform.identity(), rule, 4096, 4096)
    cpu_s = time.perf_counter() - t
    return {"ms": round(ms, 3), "mpx_per_s": round(4096 * 4096 / ms / 1e3, 1),
            "segments_per_s": round(20000 / ms * 1e3, 1), "err": _config_err(img, ref),
            "cpu_baseline_ms": round(cpu_s * 1e3, 1), "cores": 1,
            "note": "host f64 image in and out; the time includes the 128 MiB copies"}


def run_scene(R, stream, n=2000, size=2048):
    """C4: 2000 filled paths, affine transforms, 50 % solid / 25 % linear / 25 % radial, 2048^2 RGBA f32."""
    from rasterize_gb300 import workloads as W
    sc = W.scene(seed=3, n=n, size=size)
    canvas = {}

    def c4():
        canvas["c"] = R.render_scene(sc, size, size, bg=(0.0, 0.0, 0.0, 1.0))
    c4()
    ms = _event_ms(stream, c4, 5)
    paths_ = [f[0] for f in sc.fills]
    t = time.perf_counter()
    from tests.paint_oracle import oracle_scene
    ref = oracle_scene(sc, size, size, bg=(0.0, 0.0, 0.0, 1.0))
    cpu_s = time.perf_counter() - t
    nseg = sum(p.n_segments for p in paths_)
    # the same scene straight to sRGB8 bytes (encode fused into the composite)
    import numpy as np
    from oracle import oracle as O

    def c4_rgba8():
        canvas["b"] = R.render_scene_rgba8(sc, size, size, bg=(0.0, 0.0, 0.0, 1.0))
    c4_rgba8()
    ms8 = _event_ms(stream, c4_rgba8, 5)
    lsb = np.abs(canvas["b"].astype(np.int32) - O.encode_rgba8(ref.astype(np.float32)).astype(np.int32))
    return {"ms": round(ms, 3), "mpx_per_s": round(size * size / ms / 1e3, 1),
            "segments_per_s": round(nseg / ms * 1e3, 1), "err": _config_err(canvas["c"], ref),
            "rgba8_ms": round(ms8, 3), "rgba8_err_lsb": {"max": int(lsb.max()), "frac_off": float((lsb > 0).mean())},
            "cpu_baseline_ms": round(cpu_s * 1e3, 1), "cores": 1,
            "note": "error per colour channel; host canvas in and out; rgba8: sRGB8 bytes out, encode fused"}


def run_scene_tree(R, stream, n_groups=200, fills_per_group=10, size=2048):
    """Layered scene: 200 groups of 10 fills on a 2048^2 RGBA f32 canvas, a
    quarter plain, a quarter under Opacity, a quarter clipped, a quarter a clip
    inside an opacity (every third group under a Transform node)."""
    from rasterize_gb300 import workloads as W
    from tests.paint_oracle import oracle_scene_tree
    st = W.scene_tree(seed=6, n_groups=n_groups, fills_per_group=fills_per_group, size=size,
                      seg_range=(20, 2000), radius_range=(8, 128))
    out = {}

    def run():
        out["c"] = R.render_scene(st, size, size, bg=(0.0, 0.0, 0.0, 1.0))
    run()
    ms = _event_ms(stream, run, 5)
    t = time.perf_counter()
    ref = oracle_scene_tree(st, size, size, bg=(0.0, 0.0, 0.0, 1.0))
    cpu_s = time.perf_counter() - t
    return {"ms": round(ms, 3), "mpx_per_s": round(size * size / ms / 1e3, 1), "err": _config_err(out["c"], ref),
            "cpu_baseline_ms": round(cpu_s * 1e3, 1), "cores": 1, "layers": n_groups // 2 + n_groups // 4,
            "workload": "%d groups x %d fills, opacity / clip layers, %dx%d RGBA f32, host canvas in and out" %
                        (n_groups, fills_per_group, size, size)}


def run_encode(R, stream, size=8192):
    """Output encode (to_rgba of every pixel): a size x size premultiplied linear
    RGBA f32 canvas in device memory (1 GiB at 8192^2, larger than L2, so no
    flush is needed) to sRGB8 RGBA; 20 algorithmic bytes a pixel."""
    import numpy as np
    import torch
    from oracle import oracle as O
    dev = torch.device("cuda", torch.cuda.current_device())
    n = size * size
    g = torch.Generator(device=dev)
    g.manual_seed(9)
    a = torch.rand(n, 1, generator=g, device=dev)
    canvas = torch.cat([torch.rand(n, 3, generator=g, device=dev) * a, a], dim=1).contiguous()
    out = torch.empty(n * 4, dtype=torch.uint8, device=dev)
    lib = R.ctx.lib

    def enc():
        R.ctx.check(lib.rz_encode_rgba8(R.ctx.ptr, canvas.data_ptr(), n, out.data_ptr(), 1))
    enc()
    ms = _event_ms(stream, enc, 10)
    sample = 1 << 20
    c_host = canvas[:sample].cpu().numpy()
    exact = bool((out[:4 * sample].cpu().numpy().reshape(-1, 4) == O.encode_rgba8(c_host)).all())
    t = time.perf_counter()
    O.encode_rgba8(c_host)
    cpu_s = time.perf_counter() - t
    gbs = 20.0 * n / ms / 1e6
    peak, kind = measured_peak_hbm()
    del canvas, out
    return {"ms": round(ms, 4), "gpx_per_s": round(n / ms / 1e6, 2), "achieved_gbs": round(gbs, 1),
            "roofline_frac": round(gbs / peak, 3), "peak_gbs": peak, "peak_kind": kind, "bit_exact_sample_px": sample,
            "bit_exact": exact, "cpu_baseline_mpx_per_s": round(sample / cpu_s / 1e6, 1), "cores": 1,
            "workload": "%dx%d RGBA f32 canvas -> sRGB8, device memory" % (size, size)}


def run_diff(R, stream, n_images=64, paths=256, segs=32, size=1024, fd_coords=100):
    """Differentiable batch: 64 images of 1024^2, 256 closed cubic paths x 32
    segments each (FP32 control points uniform in the canvas), solid paint of
    alpha 0.5; target rendered from the control points jittered by N(0, 2 px);
    L2 loss; forward and adjoint timed on device-resident inputs.  Central
    finite differences (h = 1e-3 px) of the GPU loss on 100 random coordinates
    of image 0, and the CPU-baseline leg's binary64 gradient of image 0."""
    import numpy as np
    import torch
    from oracle import oracle as O
    from rasterize_gb300 import DiffBatch
    from rasterize_gb300 import workloads as W
    dev = torch.device("cuda", torch.cuda.current_device())
    ctrl, tctrl = W.diff_batch(seed=4, n_images=n_images, paths=paths, segs=segs, size=size)
    d_ctrl = torch.from_numpy(ctrl).to(dev)
    d_tctrl = torch.from_numpy(tctrl).to(dev)
    npx = n_images * size * size
    img = torch.empty(npx, dtype=torch.float32, device=dev)
    tgt = torch.empty_like(img)
    dl = torch.empty_like(img)
    grad = torch.empty(d_ctrl.numel(), dtype=torch.float32, device=dev)
    batch = DiffBatch(n_images, paths, segs, size, size, d_ctrl.data_ptr())
    R.diff_forward(DiffBatch(n_images, paths, segs, size, size, d_tctrl.data_ptr()), tgt.data_ptr())

    def fwd():
        R.diff_forward(batch, img.data_ptr())
        return R.l2_loss(img.data_ptr(), tgt.data_ptr(), npx, dl.data_ptr())

    def bwd():
        R.diff_backward(batch, img.data_ptr(), dl.data_ptr(), grad.data_ptr())

    loss = fwd()
    bwd()
    fwd_ms = _event_ms(stream, fwd, 3)
    bwd_ms = _event_ms(stream, bwd, 3)
    g = grad.cpu().numpy().reshape(ctrl.shape)
    # finite differences of the GPU loss of image 0 alone
    rng = np.random.default_rng(11)
    c0 = ctrl[:1].copy()
    d_c0 = torch.from_numpy(c0).to(dev)
    img0 = torch.empty(size * size, dtype=torch.float32, device=dev)
    b0 = DiffBatch(1, paths, segs, size, size, d_c0.data_ptr())

    def loss0(c):
        d_c0.copy_(torch.from_numpy(c))
        R.diff_forward(b0, img0.data_ptr())
        return R.l2_loss(img0.data_ptr(), tgt.data_ptr(), size * size)

    coords = [(int(rng.integers(paths)), int(rng.integers(3 * segs)), int(rng.integers(2))) for _ in range(fd_coords)]
    an_l, fd_l = [], []
    for p, j, k in coords:
        cp, cm = c0.copy(), c0.copy()
        cp[0, p, j, k] += np.float32(1e-3)
        cm[0, p, j, k] -= np.float32(1e-3)
        hsum = float(cp[0, p, j, k]) - float(cm[0, p, j, k])
        fd_l.append((loss0(cp) - loss0(cm)) / hsum)
        an_l.append(float(g[0, p, j, k]))
    an_a, fd_a = np.array(an_l), np.array(fd_l)
    rel = np.abs(an_a - fd_a) / np.maximum(np.abs(fd_a), 1e-2) if coords else np.zeros(1)
    rel01 = np.abs(an_a - fd_a) / np.maximum(np.abs(fd_a), 0.1) if coords else np.zeros(1)
    # the same coordinates against central differences of the binary64 oracle's forward (tree held fixed at the
    # unperturbed control points, as the adjoint holds it), evaluated on every host core
    f64 = fd_f64(ctrl[0], tgt[: size * size].cpu().numpy().reshape(size, size), paths, segs, size, coords,
                 an_a) if coords else None
    # CPU-baseline leg: the binary64 forward + adjoint of image 0 (timed), and the GPU gradient's error against it
    t = time.perf_counter()
    A = O.diff_forward(ctrl[0].astype(np.float64), paths, segs, size, size)
    T0 = tgt[: size * size].cpu().numpy().reshape(size, size).astype(np.float64)
    ref = O.diff_backward(ctrl[0].astype(np.float64), paths, segs, size, size, A, 2.0 * (A - T0))
    cpu_s = time.perf_counter() - t
    gerr = np.abs(g[0] - ref)
    return {"forward_ms": round(fwd_ms, 3), "backward_ms_per_step": round(bwd_ms, 3),
            "mpx_per_s_forward": round(npx / fwd_ms / 1e3, 1), "loss": loss,
            "fd": {"coords": fd_coords, "h_px": 1e-3,
                   "vs_f64_forward": f64,
                   "vs_gpu_forward": {
                       "median_rel_err": float(np.median(rel)), "p90_rel_err": float(np.percentile(rel, 90)),
                       "max_rel_err": float(rel.max()), "within_1e-3": int((rel <= 1e-3).sum()),
                       "within_1e-2": int((rel <= 1e-2).sum()),
                       "max_abs_err": float(np.abs(an_a - fd_a).max()) if coords else 0.0,
                       "max_rel_err_floor_0.1": float(rel01.max()),
                       "note": "relative to max(|fd|, 1e-2) unless named; the FP32 forward quantises coverage to "
                               "2^-22 per winding unit, so a 1e-3 px step resolves the derivative to ~1e-4"}},
            "grad_vs_f64": {"max_abs": float(gerr.max()), "max_ref": float(np.abs(ref).max()),
                            "rel_to_max": float(gerr.max() / max(np.abs(ref).max(), 1e-30)), "image": 0},
            "cpu_baseline_ms_per_image": round(cpu_s * 1e3, 1), "cores": 1,
            "workload": "%d images %dx%d, %d closed cubic paths x %d segs, alpha 0.5, NonZero" %
                        (n_images, size, size, paths, segs)}


_FD = {}


def _fd_init(ctrl, target, paths, segs, size):
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    O.build()
    _FD.update(O=O, c=ctrl.astype("float64"), T=target.astype("float64"), P=paths, S=segs, n=size)


def _fd_coord(args):
    """Central difference (h = 1e-3 px) of the binary64 loss at one coordinate, tree frozen."""
    p, j, k = args
    O, c = _FD["O"], _FD["c"]
    cp, cm = c.copy(), c.copy()
    cp[p, j, k] += 1e-3
    cm[p, j, k] -= 1e-3
    n = _FD["n"]
    lp = float(((O.diff_forward(cp, _FD["P"], _FD["S"], n, n, frozen=c) - _FD["T"]) ** 2).sum())
    lm = float(((O.diff_forward(cm, _FD["P"], _FD["S"], n, n, frozen=c) - _FD["T"]) ** 2).sum())
    return (lp - lm) / 2e-3


def fd_f64(ctrl0, target0, paths, segs, size, coords, an):
    """The GPU adjoint `an` at `coords` against central differences of the
    binary64 oracle's forward, on a spawn pool of every host core."""
    import multiprocessing as mp
    import numpy as np
    t = time.perf_counter()
    cores = os.cpu_count() or 1
    with mp.get_context("spawn").Pool(cores, initializer=_fd_init,
                                      initargs=(ctrl0, target0, paths, segs, size)) as pool:
        fd = np.array(pool.map(_fd_coord, coords, chunksize=1))
    rel = np.abs(an - fd) / np.maximum(np.abs(fd), 1e-2)
    return {"max_rel_err": float(rel.max()), "median_rel_err": float(np.median(rel)),
            "within_1e-3": int((rel <= 1e-3).sum()), "max_abs_err": float(np.abs(an - fd).max()),
            "cores": cores, "seconds": round(time.perf_counter() - t, 1),
            "note": "relative to max(|fd|, 1e-2); image 0, tree held at the unperturbed control points"}


def run_link(size_mb=476):
    """Host link: page-locked buffers of the C3 masks' size placed on each NUMA
    node that has CPUs (process-level placement: the memory policy of this
    process while the buffer is allocated and first touched), device->host and
    host->device copy bandwidth (best of 5, CUDA events), and where the GPU
    and this process sit (sysfs, nvidia-smi topo)."""
    import ctypes
    import glob
    import torch
    out = {}
    nodes = sorted(int(p.rsplit("node", 1)[1]) for p in glob.glob("/sys/devices/system/node/node[0-9]*"))
    cpus = {n: open("/sys/devices/system/node/node%d/cpulist" % n).read().strip() for n in nodes}
    out["numa_nodes"] = cpus
    out["process_cpus"] = len(os.sched_getaffinity(0))
    try:
        pci = subprocess.run(["nvidia-smi", "--query-gpu=pci.bus_id", "--format=csv,noheader"], capture_output=True,
                             text=True, timeout=30).stdout.strip().splitlines()[0].lower()
        node_file = "/sys/bus/pci/devices/%s/numa_node" % pci[4:]
        out["gpu_pci"] = pci
        out["gpu_numa_node"] = open(node_file).read().strip() if os.path.exists(node_file) else None
    except Exception as e:  # noqa: BLE001 - informational only
        out["gpu_numa_node"] = "unknown (%s)" % e
    libc = ctypes.CDLL("libc.so.6", use_errno=True)
    nr = 237 if os.uname().machine == "aarch64" else 238  # set_mempolicy

    def policy(node):
        if node is None:
            return libc.syscall(nr, 0, None, 0)
        mask = ctypes.c_ulong(1 << node)
        return libc.syscall(nr, 2, ctypes.byref(mask), 64)  # MPOL_BIND

    n = size_mb * (1 << 20) // 4
    dev = torch.full((n,), 1.0, dtype=torch.float32, device="cuda")
    res = {}
    for node in [None] + [m for m in nodes if cpus[m]]:
        if node is not None and policy(node) != 0:
            res[str(node)] = "set_mempolicy failed (errno %d)" % ctypes.get_errno()
            continue
        host = torch.empty(n, dtype=torch.float32).pin_memory()
        host.fill_(0.0)
        policy(None)
        torch.cuda.synchronize()
        d2h, h2d = [], []
        for _ in range(5):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(); host.copy_(dev, non_blocking=True); b.record(); torch.cuda.synchronize()
            d2h.append(a.elapsed_time(b))
            a.record(); dev.copy_(host, non_blocking=True); b.record(); torch.cuda.synchronize()
            h2d.append(a.elapsed_time(b))
        gb = n * 4 / 1e9
        res["default" if node is None else str(node)] = {"d2h_gbs": round(gb / (min(d2h) / 1e3), 1),
                                                          "h2d_gbs": round(gb / (min(h2d) / 1e3), 1)}
        del host
    out["bandwidth"] = res
    out["bytes"] = n * 4
    return out


def run_reference(args, rank, world):
    """The reference's algorithm (the binary64 oracle port: the Rust crate has
    no toolchain here) on every host core: one process per core, each
    rendering an interleaved share of the whole glyph batch per step."""
    if rank != 0:
        return
    import multiprocessing as mp
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    from rasterize_gb300 import workloads as W
    paths, sizes, _ = W.glyph_batch(seed=2, n=args.glyphs)
    px_step = sum(w * h for w, h in sizes)
    segments = sum(p.n_segments for p in paths)
    ctx = mp.get_context("spawn")

    def timed(pool, rasterizer, steps, warmup):
        times = []
        for s in range(warmup + steps):
            t = time.perf_counter()
            done = sum(pool.map(_oracle_chunk, [(c, cores, rasterizer) for c in range(cores)], chunksize=1))
            dt = time.perf_counter() - t
            assert done == px_step
            if s >= warmup:
                times.append(dt)
        return sum(times) / len(times)

    with ctx.Pool(cores, initializer=_oracle_init, initargs=(args.glyphs,)) as pool:
        pool.map(_oracle_chunk, [(c, cores) for c in range(cores)])  # every worker has built its batch
        dt = timed(pool, "sd", args.steps, args.warmup)
        # the reference's other CPU rasterizer, on the same batch and cores (fewer steps: it is slower)
        ae_steps = max(1, min(args.steps, 3))
        dt_ae = timed(pool, "ae", ae_steps, 1)
    value = px_step / dt / 1e6
    out = {"metric": METRIC, "value": round(value, 3), "unit": "Mpx/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(dt * 1e3, 3), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "impl": "reference",
           "config": headline_config(args.glyphs, segments, px_step, world),
           "cpu_baseline": {"value": round(value, 3), "unit": "Mpx/s", "cores": cores, "kind": "port",
                            "sample": "the whole batch (%d glyphs, %.2f Mpx) per step, interleaved over a spawn "
                                      "pool of %d processes" % (args.glyphs, px_step / 1e6, cores)},
           "rasterizer": "SignedDifferenceRasterizer (src/rasterize.rs:279-507), binary64 port",
           "active_edge": {"value": round(px_step / dt_ae / 1e6, 3), "unit": "Mpx/s", "steps": ae_steps,
                           "ms_per_step": round(dt_ae * 1e3, 3), "cores": cores, "kind": "port",
                           "rasterizer": "ActiveEdgeRasterizer (src/rasterize.rs:517-937), binary64 port"},
           "e2e": {"value": round(value, 3), "unit": "Mpx/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


# --------------------------------------------------------------------------- GPU
def main():
    args = parse()
    rank, world, local = dist_info()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import numpy as np
    import torch

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if args.workload != "glyphs":
        from rasterize_gb300 import GpuRasterizer
        R = GpuRasterizer(device=local)
        stream = torch.cuda.Stream(dev)
        torch.cuda.set_stream(stream)
        R.ctx.set_stream(stream.cuda_stream)
        leg = {"small_path": lambda: run_small(R, stream), "large_path": lambda: run_large(R, stream),
               "scene": lambda: run_scene(R, stream, n=args.scene_fills),
               "diff": lambda: run_diff(R, stream, n_images=args.diff_images, fd_coords=args.fd_coords),
               "encode": lambda: run_encode(R, stream),
               "scene_tree": lambda: run_scene_tree(R, stream),
               "link": lambda: run_link()}[args.workload]()
        if rank == 0:
            print(json.dumps({"metric": METRIC, "workload": args.workload, "n_gpus": world, **leg}))
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    from rasterize_gb300 import GpuRasterizer, Transform

    paths, sizes, rules, batch = make_workload(args.glyphs)
    R = GpuRasterizer(device=local)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    R.ctx.set_stream(stream.cuda_stream)

    # ---- device-resident inputs / output
    d_kind = torch.from_numpy(batch.kind).to(dev)
    d_pts = torch.from_numpy(batch.pts.reshape(-1)).to(dev)
    d_sub = torch.from_numpy(batch.sub_off.view(np.int32)).to(dev)
    d_psub = torch.from_numpy(batch.path_sub.view(np.int32)).to(dev)
    d_rule = torch.from_numpy(batch.fill_rules).to(dev)
    d_out = torch.empty(batch.out_len, dtype=torch.float32, device=dev)
    ptrs = dict(kind=d_kind.data_ptr(), pts=d_pts.data_ptr(), sub_off=d_sub.data_ptr(), path_sub=d_psub.data_ptr(),
                fill_rules=d_rule.data_ptr())
    tuning = R.tune(batch, ptrs, d_out.data_ptr())  # band-height cap and CTAs per SM, before the timed region
    plan = R.plan(batch, ptrs, d_out.data_ptr())
    for _ in range(args.warmup):
        plan.launch()
    plan.status()
    torch.cuda.synchronize(dev)

    out_host = d_out.cpu().numpy()

    # ---- timed region: device-resident batch, graph replay
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    clocks.mark()
    # the sampler's period (200 ms) is far longer than a step: keep the GPU under the same load for
    # --load-seconds before the timed region so the clock record describes this workload, not idle time
    t_load = time.perf_counter()
    load_launches = 0
    while time.perf_counter() - t_load < args.load_seconds:
        for _ in range(64):
            plan.launch()
        load_launches += 64
        torch.cuda.synchronize(dev)
    load_s = time.perf_counter() - t_load
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for s in range(args.steps):
        ev[s][0].record(stream)
        plan.launch()
        ev[s][1].record(stream)
    t_end.record(stream)
    torch.cuda.synchronize(dev)
    clk = clocks.stop()
    clk["window"] = "%d back-to-back plan launches (%.2f s) just before the timed region, then the timed region" % (
        load_launches, load_s)
    plan.status()
    total_ms = max_over_ranks(t_start.elapsed_time(t_end), dev)
    launch_ms = [a.elapsed_time(b) for a, b in ev]
    kernel_ms = statistics.mean(launch_ms)
    ms_per_step = total_ms / args.steps
    px = batch.pixels
    value = px * world / (ms_per_step / 1e3) / 1e6
    n_items, fallbacks = plan.info()

    # ---- plain per-path launches (same batch, one launch per glyph)
    per_path = None
    if not args.no_per_path:
        R.mask_batch_device(batch, ptrs, d_out.data_ptr(), per_path=True)
        torch.cuda.synchronize(dev)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        R.mask_batch_device(batch, ptrs, d_out.data_ptr(), per_path=True)
        b.record(stream)
        torch.cuda.synchronize(dev)
        pp_ms = a.elapsed_time(b)
        per_path = {"ms_per_step": round(pp_ms, 3), "masks_per_s": round(len(paths) / (pp_ms / 1e3), 1),
                    "launches": len(paths)}

    # ---- e2e through the C ABI with host buffers (pinned)
    h_kind = torch.from_numpy(batch.kind).pin_memory().numpy()
    h_pts = torch.from_numpy(batch.pts).pin_memory().numpy()
    h_out = torch.empty(batch.out_len, dtype=torch.float32).pin_memory().numpy()
    batch.kind, batch.pts = h_kind, h_pts
    for _ in range(2):
        R.mask_batch(batch, out=h_out)
    e_ms = []
    for _ in range(max(3, min(args.steps, 10))):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        R.mask_batch(batch, out=h_out)
        b.record(stream)
        torch.cuda.synchronize(dev)
        e_ms.append(a.elapsed_time(b))
    e2e_ms = statistics.median(e_ms)
    h2d = batch.kind.nbytes + batch.pts.nbytes + batch.sub_off.nbytes + batch.path_sub.nbytes + batch.fill_rules.nbytes
    d2h = batch.out_len * 4

    if rank != 0:
        return
    peak, peak_kind = measured_peak_hbm()
    algo_bytes = px * 4 + batch.n_segments * (64 + 1) + (len(batch.sub_off) + len(batch.path_sub)) * 4
    achieved = algo_bytes / (kernel_ms / 1e3) / 1e9
    traffic = profile_traffic("glyph_pipeline_glyph_batch")
    cpu, err = cpu_baseline_single(paths, sizes, rules, args.cpu_seconds, gpu_masks=lambda i: batch.mask(out_host, i))
    configs = None if args.no_configs else run_configs(R, stream)
    out = {
        "metric": METRIC, "value": round(value, 2), "unit": "Mpx/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded glyph outlines)",
        "config": headline_config(len(paths), batch.n_segments, px, world),
        "segments_per_s": round(batch.n_segments * world / (ms_per_step / 1e3), 1),
        "masks_per_s": round(len(paths) * world / (ms_per_step / 1e3), 1),
        "per_path": per_path,
        "batched_vs_per_path": round(per_path["ms_per_step"] / ms_per_step, 2) if per_path else None,
        "err": err,
        "work_items": n_items, "f64_fallbacks_total": fallbacks,
        "e2e": {"value": round(px / (e2e_ms / 1e3) / 1e6, 2), "unit": "Mpx/s", "ms_per_step": round(e2e_ms, 3),
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": peak_kind,
                     "kernel": "glyph pipeline, one plan launch: k_glyph_records, k_glyph_walk, chain-offset scan, "
                               "k_glyph_emit, k_glyph_cover",
                     "algorithmic_bytes_per_launch": int(algo_bytes), "kernel_ms": round(kernel_ms, 4)},
        "cpu_baseline": cpu,
        "gpu_launches": plan_kernels(batch) * args.steps,
        "clocks": clk,
        "configs": configs,
        "tuning": {k: tuning[k] for k in ("band_rows_cap", "ctas_per_sm", "walk_slots", "ms", "cached", "candidates")
                   if k in tuning},
    }
    print(json.dumps(out))


if __name__ == "__main__":
    main()
