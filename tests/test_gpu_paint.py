"""GPU parity of Rasterizer::fill, Scene::render and the large-path line
pipeline against the CPU f64 oracle (through the C ABI).

Coverage is within 1e-4 per pixel of the f64 rasterizer; colours are
compared per channel within COLOR_TOL (the paint math runs in FP32 on the
GPU, in f64 coordinates with f32 colours in the reference).
"""
import math

import numpy as np
import pytest

from oracle import oracle as O
from rasterize_gb300 import (FillRule, GpuRasterizer, GradLinear, GradRadial, GradSpread, GradStop, LinColor, Path,
                             PathBuilder, Transform, Units)
from rasterize_gb300 import workloads as W
from tests.paint_oracle import oracle_paint, oracle_scene

pytestmark = pytest.mark.gpu

TOL = 1e-4
COLOR_TOL = 2e-4


@pytest.fixture(scope="module")
def R():
    return GpuRasterizer()


def assert_close(gpu, ref, tol):
    err = np.abs(gpu.astype(np.float64) - ref.astype(np.float64))
    i = np.unravel_index(err.argmax(), err.shape)
    assert err.max() <= tol, "max err %.3g at %s: gpu %r ref %r (mean %.3g)" % (err.max(), i, gpu[i], ref[i], err.mean())


def blob(seed, r=40.0, c=(60.0, 50.0), n=24):
    rng = np.random.default_rng(seed)
    return W.contour(rng, n, r), Transform.new_translate(*c)


STOPS = [GradStop(0.0, LinColor(0.9, 0.1, 0.1, 1.0)), GradStop(0.4, LinColor(0.1, 0.45, 0.1, 0.5)),
         GradStop(1.0, LinColor(0.0, 0.1, 0.6, 0.8))]


@pytest.mark.parametrize("which", ["solid", "linear", "radial", "linear_bbox_srgb", "radial_reflect", "linear_repeat",
                                   "radial_repeat_far", "linear_reflect_far", "radial_focal_outside"])
def test_fill_paints(R, which):
    path, tr = blob(1)
    paint = {
        "solid": LinColor(0.2, 0.3, 0.4, 0.7),
        "linear": GradLinear(STOPS, (30, 20), (90, 80)),
        "radial": GradRadial(STOPS, (60, 50), 45.0, (70, 45), 5.0),
        "linear_bbox_srgb": GradLinear(STOPS, (0.1, 0.2), (0.9, 0.7), Units.BoundingBox, False),
        "radial_reflect": GradRadial(STOPS, (60, 50), 15.0, (62, 49), 2.0, spread=GradSpread.Reflect),
        "linear_repeat": GradLinear(STOPS, (50, 40), (65, 52), spread=GradSpread.Repeat,
                                    tr=Transform.new_rotate(0.3)),
        # offsets of 50-200 periods: the fraction must survive FP32 evaluation
        "radial_repeat_far": GradRadial(STOPS, (300, 250), 3.0, (296, 247), 0.5, spread=GradSpread.Repeat),
        "linear_reflect_far": GradLinear(STOPS, (-900, -700), (-899.5, -699.6), spread=GradSpread.Reflect),
        # focal circle not inside the end circle: cone edge, no-root regions
        "radial_focal_outside": GradRadial(STOPS, (60, 50), 20.0, (95, 60), 10.0),
    }[which]
    bg = np.zeros((100, 120, 4), dtype=np.float32)
    bg[..., :] = (0.05, 0.1, 0.15, 0.5)
    gpu = bg.copy()
    R.fill(path, tr, FillRule.NonZero, paint, gpu)
    ref = bg.copy()
    O.fill(path, tr, FillRule.NonZero, oracle_paint(paint), ref)
    assert_close(gpu, ref, COLOR_TOL)


def test_fill_strided_view_and_evenodd(R):
    path, tr = blob(2, r=30, c=(40, 30), n=40)
    big = np.full((90, 150, 4), 0.25, dtype=np.float32)
    view = big[10:70, 20:140:2]
    R.fill(path, tr, FillRule.EvenOdd, LinColor(0.5, 0.2, 0.1, 0.9), view)
    ref = np.full((60, 60, 4), 0.25, dtype=np.float32)
    O.fill(path, tr, FillRule.EvenOdd, oracle_paint(LinColor(0.5, 0.2, 0.1, 0.9)), ref)
    assert_close(view, ref, COLOR_TOL)
    assert np.all(big[:10] == 0.25) and np.all(big[:, 21:140:2] == 0.25)


def test_scene_small(R):
    sc = W.scene(seed=5, n=40, size=256, seg_range=(20, 200), radius_range=(8, 64))
    bg = (0.1, 0.1, 0.12, 1.0)
    gpu = R.render_scene(sc, 256, 256, bg=bg)
    ref = oracle_scene(sc, 256, 256, bg=bg)
    assert_close(gpu, ref, COLOR_TOL)


def test_scene_paths_off_canvas(R):
    """Fills partly outside the canvas on every side (view clamping, align)."""
    sc = W.scene(seed=8, n=30, size=128, seg_range=(20, 80), radius_range=(20, 90))
    gpu = R.render_scene(sc, 128, 96)
    ref = oracle_scene(sc, 128, 96)
    assert_close(gpu, ref, COLOR_TOL)


def test_scene_empty(R):
    from rasterize_gb300 import Scene
    gpu = R.render_scene(Scene(), 17, 9, bg=(0.5, 0.25, 0.0, 1.0))
    assert np.all(gpu == np.array([0.5, 0.25, 0.0, 1.0], dtype=np.float32))


def test_large_path_pipeline(R):
    """A path big enough for the line pipeline (flatten once, bin by band)."""
    path, rule, _ = W.large_path(seed=4, n_segments=20000, size=1024)
    img = np.zeros((1024, 1024))
    R.mask(path, Transform.identity(), img, rule)
    ref = O.mask(path, Transform.identity(), rule, 1024, 1024)
    assert_close(img, ref, TOL)


def test_scene_many_tall_fills(R):
    """300 thin fills nearly as tall as the canvas, a few lines each: the line blocks of the flatten and
    scatter passes span more (fill, band) entries than their shared-memory histograms hold, so the global
    counting route runs; the canvas must still match the oracle."""
    from rasterize_gb300 import Scene
    rng = np.random.default_rng(21)
    sc = Scene()
    for i in range(300):
        x = rng.uniform(2, 1000)
        y0, y1 = rng.uniform(0, 20), rng.uniform(990, 1020)
        w = rng.uniform(0.5, 4.0)
        p = PathBuilder().move_to((x, y0)).line_to((x + w, y0 + 3)).line_to((x + w, y1)).line_to((x, y1 - 2)).close().build()
        sc.fill(p, LinColor(rng.uniform(0, 1), rng.uniform(0, 1), rng.uniform(0, 1), rng.uniform(0.2, 1.0)))
    bg = (0.0, 0.0, 0.0, 1.0)
    gpu = R.render_scene(sc, 1024, 1024, bg=bg)
    ref = oracle_scene(sc, 1024, 1024, bg=bg)
    assert_close(gpu, ref, COLOR_TOL)
