"""GPU parity of scene trees (rz_render_scene_tree): Opacity and Clip layers,
Transform and Group nodes, against the oracle's restatement of
Pipeline::build_rec / render_rec / Layer::compose (src/scene.rs:153-565)."""
import numpy as np
import pytest

from oracle import oracle as O
from rasterize_gb300 import FillRule, GpuRasterizer, LinColor, RasterizeError, Scene, Transform, Units
from rasterize_gb300 import workloads as W
from tests.paint_oracle import oracle_scene_tree

pytestmark = pytest.mark.gpu

TOL = 2e-4  # per colour channel, as the flat scenes (clip masks add their own 1e-4 at most)


@pytest.fixture(scope="module")
def R():
    return GpuRasterizer()


def assert_close(gpu, ref, tol=TOL):
    err = np.abs(gpu.astype(np.float64) - ref.astype(np.float64))
    i = np.unravel_index(err.argmax(), err.shape)
    assert err.max() <= tol, "max err %.3g at %s: gpu %r ref %r" % (err.max(), i, gpu[i], ref[i])


def test_flat_group_through_the_tree_path_is_identical(R):
    sc = W.scene(seed=5, n=40, size=256, seg_range=(20, 200), radius_range=(8, 64))
    bg = (0.1, 0.1, 0.12, 1.0)
    assert np.array_equal(R.render_scene(sc, 256, 200, bg=bg, tree=True), R.render_scene(sc, 256, 200, bg=bg))


@pytest.mark.parametrize("seed", [6, 7])
def test_layered_scene_matches_oracle(R, seed):
    st = W.scene_tree(seed=seed, n_groups=16, fills_per_group=6, size=256)
    bg = (0.0, 0.0, 0.0, 1.0)
    assert_close(R.render_scene(st, 256, 256, bg=bg), oracle_scene_tree(st, 256, 256, bg=bg))


def test_concurrent_and_in_order_layers_are_identical(R, monkeypatch):
    """The concurrent layer path (a stream per layer sequence, every layer in
    its own arena buffer) and the in-order path with per-depth buffers (taken
    for plans whose arena would be too large) render the same canvas bit for
    bit, nested clips and opacities included."""
    st = W.scene_tree(seed=8, n_groups=24, fills_per_group=5, size=256)
    bg = (0.05, 0.0, 0.1, 1.0)
    concurrent = R.render_scene(st, 256, 256, bg=bg)
    monkeypatch.setenv("RZ_SCENE_LAYERS", "serial")
    in_order = R.render_scene(st, 256, 256, bg=bg)
    assert np.array_equal(concurrent, in_order)


def test_opacity_clip_nesting_and_units(R):
    rng = np.random.default_rng(3)
    paint = [LinColor(0.8, 0.2, 0.1, 1.0), LinColor(0.1, 0.5, 0.2, 0.7), LinColor(0.0, 0.2, 0.6, 0.9)]
    inner = Scene()
    for i in range(3):
        inner.fill(W.contour(rng, 20, 30.0, center=(40.0 + 25 * i, 50.0)), paint[i])
    clip_u = W.contour(rng, 16, 35.0, center=(70.0, 55.0))
    clip_b = W.contour(rng, 16, 0.45, center=(0.5, 0.5))
    root = Scene()
    root.fill(W.contour(rng, 30, 60.0, center=(64.0, 64.0)), LinColor(0.2, 0.2, 0.2, 1.0))
    root.add(inner.clip(clip_u, Units.UserSpaceOnUse, FillRule.NonZero).opacity(0.6))
    root.add(inner.clip(clip_b, Units.BoundingBox, FillRule.EvenOdd)
             .transform(Transform.new_translate(10, 30)))
    root.add(inner.opacity(0.5).clip(clip_u, fill_rule=FillRule.EvenOdd).opacity(0.8))
    bg = (1.0, 1.0, 1.0, 1.0)
    assert_close(R.render_scene(root, 160, 128, bg=bg), oracle_scene_tree(root, 160, 128, bg=bg))


def test_nodes_out_of_view_and_empty_groups(R):
    far = Scene().fill(W.contour(np.random.default_rng(0), 8, 5.0, center=(900.0, 900.0)), LinColor(1, 1, 1, 1))
    root = Scene().add(far.opacity(0.5)).add(Scene()).add(
        Scene().fill(W.contour(np.random.default_rng(1), 8, 10.0, center=(16.0, 8.0)), LinColor(1, 0, 0, 1))
        .clip(W.contour(np.random.default_rng(2), 8, 3.0, center=(500.0, 8.0))))
    bg = (0.25, 0.0, 0.0, 1.0)
    got = R.render_scene(root, 32, 16, bg=bg)
    assert (got == np.float32(bg)).all()
    assert_close(got, oracle_scene_tree(root, 32, 16, bg=bg))


def test_tree_rgba8_is_the_encoded_canvas(R):
    st = W.scene_tree(seed=8, n_groups=8, fills_per_group=4, size=128)
    canvas = R.render_scene(st, 128, 100, bg=(0, 0, 0, 1))
    assert (R.render_scene_rgba8(st, 128, 100, bg=(0, 0, 0, 1)) == O.encode_rgba8(canvas)).all()


def test_invalid_trees_are_rejected(R):
    import ctypes
    from rasterize_gb300 import _ffi
    from rasterize_gb300.rasterizer import _pack_entries
    s, keep = _pack_entries([(W.contour(np.random.default_rng(0), 8, 5.0, center=(8.0, 8.0)), Transform.identity(),
                              FillRule.NonZero, LinColor(1, 1, 1, 1))])
    canvas = np.zeros((16, 16, 4), dtype=np.float32)
    lib = R.ctx.lib

    def call(nodes):
        arr = (_ffi.RzSceneNode * len(nodes))()
        for i, (k, a) in enumerate(nodes):
            arr[i].kind, arr[i].arg = k, a
        return lib.rz_render_scene_tree(R.ctx.ptr, ctypes.byref(s), ctypes.addressof(arr), len(nodes), 0.05, None,
                                        canvas.ctypes.data, None, 16, 16)

    assert call([(_ffi.NODE_FILL, 0)]) == 0
    assert call([(_ffi.NODE_FILL, 1)]) == 2          # entry out of range
    assert call([(_ffi.NODE_GROUP, 2), (_ffi.NODE_FILL, 0)]) == 2  # children run past the array
    assert call([(_ffi.NODE_FILL, 0), (_ffi.NODE_FILL, 0)]) == 2   # nodes after the root's subtree
    assert call([(9, 0)]) == 2
    assert call([(_ffi.NODE_OPACITY, 0)]) == 2       # opacity without its child


def test_line_only_strokes_match_oracle(R):
    """Stroke nodes whose paths hold only lines: the device stroker's curve
    stages have nothing to do and every offset is a line's."""
    from rasterize_gb300 import LineCap, LineJoin, PathBuilder, StrokeStyle
    rng = np.random.default_rng(77)
    root = Scene()
    for t in range(5):
        b = PathBuilder().move_to(tuple(rng.uniform(10, 118, 2)))
        for _ in range(6):
            b.line_to(tuple(rng.uniform(10, 118, 2)))
        if t % 2:
            b.close()
        style = StrokeStyle(float(rng.uniform(1.0, 6.0)), LineJoin(t % 3), 4.0, LineCap(t % 3))
        root.stroke(b.build(), LinColor(*rng.uniform(0, 1, 3), 1.0), style)
    bg = (0.0, 0.0, 0.0, 1.0)
    assert_close(R.render_scene(root, 128, 128, bg=bg), oracle_scene_tree(root, 128, 128, bg=bg))


@pytest.mark.parametrize("join,cap", [(0, 0), (1, 1), (2, 2)])
def test_strokes_match_oracle(R, join, cap):
    """Stroke nodes (the outline filled NonZero): open and closed paths with
    lines, quads, cubics and arcs, under an opacity layer and a clip."""
    from rasterize_gb300 import LineCap, LineJoin, PathBuilder, StrokeStyle
    rng = np.random.default_rng(20 + join)
    root = Scene()
    for t in range(6):
        b = PathBuilder().move_to(tuple(rng.uniform(10, 118, 2)))
        for _ in range(5):
            k = rng.integers(4)
            p = [tuple(rng.uniform(10, 118, 2)) for _ in range(3)]
            [lambda: b.line_to(p[0]), lambda: b.quad_to(p[0], p[1]), lambda: b.cubic_to(*p),
             lambda: b.arc_to((20.0, 12.0), 30.0, bool(t % 2), True, p[0])][k]()
        if t % 2:
            b.close()
        style = StrokeStyle(float(rng.uniform(1.0, 8.0)), LineJoin(join), 4.0, LineCap(cap))
        root.stroke(b.build(), LinColor(*rng.uniform(0, 1, 3), 1.0), style)
    layered = Scene().add(root.opacity(0.7)).add(
        root.clip(W.contour(rng, 16, 40.0, center=(64.0, 64.0))).transform(Transform.new_translate(5, 3)))
    bg = (0.0, 0.0, 0.0, 1.0)
    for sc in (root, layered):
        assert_close(R.render_scene(sc, 128, 128, bg=bg), oracle_scene_tree(sc, 128, 128, bg=bg))
