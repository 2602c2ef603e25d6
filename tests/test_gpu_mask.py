"""GPU parity of the mask path against the CPU f64 oracle (through the C ABI).

Bars: the bisection tree is exact (per-segment line counts equal the
oracle's), and coverage is within 1e-4 absolute per pixel of the f64
SignedDifferenceRasterizer restatement.
"""
import json
import math
import os

import numpy as np
import pytest

from oracle import oracle as O
from rasterize_gb300 import FillRule, GpuRasterizer, MaskBatch, Path, PathBuilder, Size, Transform
from rasterize_gb300 import workloads as W
from rasterize_gb300._ffi import NanError, RasterizeError

pytestmark = pytest.mark.gpu

TOL = 1e-4  # max abs coverage error per pixel vs the f64 oracle
FIX = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_fixtures.json")))


@pytest.fixture(scope="module")
def R():
    return GpuRasterizer()


def gpu_mask(R, path, tr, rule, w, h):
    img = np.zeros((h, w), dtype=np.float64)
    R.mask(path, tr, img, rule)
    return img


def assert_close(gpu, ref, tol=TOL):
    err = np.abs(gpu - ref)
    assert err.max() <= tol, "max err %.3g at %s (mean %.3g)" % (err.max(), np.unravel_index(err.argmax(), err.shape),
                                                              err.mean())


def test_kat_polygon_9x4(R):
    """src/rasterize.rs:1065-1110 expected values, on the GPU."""
    from tests.test_oracle_kat import RASTERIZER_EXPECTED, polygon_9x4
    img = gpu_mask(R, polygon_9x4(), Transform.identity(), FillRule.EvenOdd, 9, 4)
    assert np.abs(img - RASTERIZER_EXPECTED).max() < 1e-6


def test_kat_fill_rule_areas(R):
    """src/rasterize.rs:1122-1161 areas and point values, on the GPU."""
    from tests.test_oracle_kat import path_size
    path = Path.parse(FIX["fill_rule_star_boxes"])
    w, h, tr = path_size(path, Transform.identity())
    img = gpu_mask(R, path, tr, FillRule.EvenOdd, w, h)
    assert abs(img[50, 50]) < 1e-6 and abs(img[50, 150]) < 1e-6 and abs(img[50, 250]) < 1e-6
    assert abs(img.sum() - 13130.0) < 1.0
    img = gpu_mask(R, path, tr, FillRule.NonZero, w, h)
    assert abs(img[50, 50] - 1) < 1e-6 and abs(img[50, 150] - 1) < 1e-6 and abs(img[50, 250]) < 1e-6
    assert abs(img.sum() - 16492.5) < 1.0
    for rule in (FillRule.EvenOdd, FillRule.NonZero):
        assert_close(gpu_mask(R, path, tr, rule, w, h), O.mask(path, tr, rule, w, h))


def test_small_path_config(R):
    """200 cubics, control points U[0,512]^2, NonZero, 512x512."""
    path, rule, (w, h) = W.small_path(seed=0)
    assert_close(gpu_mask(R, path, Transform.identity(), rule, w, h),
                 O.mask(path, Transform.identity(), rule, w, h))


@pytest.mark.parametrize("seed,w,h", [(1, 512, 512), (2, 509, 257), (3, 384, 130)])
def test_small_route_rules_and_transforms(R, seed, w, h):
    """Single masks of a few hundred curves (the two-launch route for small
    masks: one flatten pass into a counter-reserved line buffer, every band
    reading every line) under a rotation and a shear, both fill rules, odd
    mask sizes whose last band is short."""
    path, _, _ = W.small_path(seed=seed, n_cubics=300, size=512)
    tr = Transform.new_translate(w / 2, h / 2) * Transform.new_rotate(0.3 * seed) * Transform.new_translate(-256, -256)
    tr = tr.pre_scale(1.0, 0.6)
    for rule in (FillRule.NonZero, FillRule.EvenOdd):
        assert_close(gpu_mask(R, path, tr, rule, w, h), O.mask(path, tr, rule, w, h))


@pytest.mark.parametrize("seed", range(6))
def test_random_paths_both_rules(R, seed):
    rng = np.random.default_rng(100 + seed)
    b = PathBuilder()
    for s in range(3):
        b.move_to(rng.uniform(-20, 140, 2))
        for _ in range(int(rng.integers(3, 25))):
            k = rng.integers(4)
            if k == 0:
                b.line_to(rng.uniform(-20, 140, 2))
            elif k == 1:
                b.quad_to(rng.uniform(-20, 140, 2), rng.uniform(-20, 140, 2))
            elif k == 2:
                b.cubic_to(rng.uniform(-20, 140, 2), rng.uniform(-20, 140, 2), rng.uniform(-20, 140, 2))
            else:
                b.arc_to(rng.uniform(3, 60, 2), rng.uniform(0, 360), bool(rng.integers(2)), bool(rng.integers(2)),
                         rng.uniform(-20, 140, 2))
        if s != 1:
            b.close()
    path = b.build()
    tr = Transform.new_rotate(rng.uniform(0, 2 * math.pi)).pre_scale(0.9, 1.1) * Transform.identity()
    tr = Transform.new_translate(60, 50) * tr * Transform.new_translate(-60, -50)
    for rule in (FillRule.NonZero, FillRule.EvenOdd):
        w, h = 131, 97
        assert_close(gpu_mask(R, path, tr, rule, w, h), O.mask(path, tr, rule, w, h))


def test_tree_parity_counts(R):
    """Per-segment line counts equal PathFlattenIter's (exact bisection tree)."""
    for seed in range(3):
        path, rule, (w, h) = W.small_path(seed=seed)
        tr = Transform.new_rotate(0.3 * seed).pre_translate(-5.0 * seed, 3.0)
        assert np.array_equal(R.flatten_counts(path, tr), O.flatten_counts_per_input(path, tr))
    path, rule, _ = W.large_path(seed=5, n_segments=3000)
    assert np.array_equal(R.flatten_counts(path, Transform.identity()),
                          O.flatten_counts_per_input(path, Transform.identity()))


def test_squirrel_and_data_fixtures(R):
    """The reference's own path fixtures (src/path.rs SQUIRREL, data/*.path)."""
    for name, text in [("squirrel", FIX["squirrel"])] + sorted(FIX["data"].items()):
        path = Path.parse(text)
        bb = O.path_bbox(path, Transform.identity())
        scale = 200.0 / max(bb[2] - bb[0], bb[3] - bb[1])
        tr = Transform.new_scale(scale, scale) * Transform.new_translate(-bb[0] + 1, -bb[1] + 1)
        w = int(math.ceil((bb[2] - bb[0] + 2) * scale)) + 2
        h = int(math.ceil((bb[3] - bb[1] + 2) * scale)) + 2
        for rule in (FillRule.NonZero, FillRule.EvenOdd):
            assert_close(gpu_mask(R, path, tr, rule, w, h), O.mask(path, tr, rule, w, h))
        assert np.array_equal(R.flatten_counts(path, tr), O.flatten_counts_per_input(path, tr))


def test_strided_view(R):
    """mask writes through an arbitrary Shape (start, row_stride, col_stride)."""
    path, rule, _ = W.small_path(seed=3, n_cubics=20, size=64)
    big = np.full((80, 200), 7.0)
    view = big[5:69:1, 10:138:2]  # col_stride 2
    R.mask(path, Transform.identity(), view, rule)
    ref = O.mask(path, Transform.identity(), rule, 64, 64)
    assert_close(view, ref)
    assert np.all(big[:5] == 7.0) and np.all(big[:, 139:] == 7.0)


def test_mask_iter(R):
    path, rule, _ = W.small_path(seed=4, n_cubics=30, size=100)
    size = Size(90, 80)
    dense = R.mask_iter_dense(path, Transform.identity(), size, rule)
    ref, n = O.mask_iter(path, Transform.identity(), rule, 90, 80)
    assert_close(dense, ref)
    pix = list(R.mask_iter(path, Transform.identity(), size, rule))
    assert all(abs(p.alpha) >= 1e-6 for p in pix)
    assert [(p.y, p.x) for p in pix] == sorted((p.y, p.x) for p in pix)


def test_edges_and_outside(R):
    """Geometry beyond every image edge (the x rules of src/rasterize.rs:372-393)."""
    b = PathBuilder().move_to((-50, -30)).line_to((90, 10)).cubic_to((200, 40), (-80, 70), (30, 200))
    b.line_to((75, 45)).quad_to((500, 60), (-10, 20)).close()
    b.move_to((63.5, 5)).line_to((64.2, 60)).line_to((10, 30)).close()
    path = b.build()
    for rule in (FillRule.NonZero, FillRule.EvenOdd):
        assert_close(gpu_mask(R, path, Transform.identity(), rule, 64, 48),
                     O.mask(path, Transform.identity(), rule, 64, 48))


def test_empty_and_degenerate(R):
    empty = Path.empty()
    img = gpu_mask(R, empty, Transform.identity(), FillRule.NonZero, 16, 16)
    assert not img.any()
    # zero-size image: nothing to do
    R.mask(empty, Transform.identity(), np.zeros((0, 5)), FillRule.NonZero)
    # all-degenerate segments
    b = PathBuilder().move_to((3, 3)).cubic_to((3, 3), (3, 3), (3, 3)).quad_to((5, 5), (5, 5)).close()
    path = b.build()
    assert_close(gpu_mask(R, path, Transform.identity(), FillRule.NonZero, 8, 8),
                 O.mask(path, Transform.identity(), FillRule.NonZero, 8, 8))


def test_nan_is_an_error(R):
    bad = PathBuilder().move_to((0, 0)).line_to((float("nan"), 1)).line_to((3, 3)).close().build()
    with pytest.raises(NanError):
        gpu_mask(R, bad, Transform.identity(), FillRule.NonZero, 8, 8)
    # the context stays usable
    path, rule, _ = W.small_path(seed=1, n_cubics=10, size=32)
    assert_close(gpu_mask(R, path, Transform.identity(), rule, 32, 32),
                 O.mask(path, Transform.identity(), rule, 32, 32))


def test_invalid_flatness(R):
    path, rule, _ = W.small_path(seed=1, n_cubics=3, size=16)
    bad = GpuRasterizer(flatness=0.0, context=R.ctx)
    with pytest.raises(RasterizeError):
        gpu_mask(bad, path, Transform.identity(), rule, 16, 16)


def test_batch_matches_oracle_and_per_path(R):
    paths, sizes, rules = W.glyph_batch(seed=9, n=300)
    batch = MaskBatch(paths, sizes, fill_rules=rules)
    out = R.mask_batch(batch)
    out_pp = R.mask_batch(batch, per_path=True)
    for i in range(0, 300, 7):
        w, h = sizes[i]
        ref = O.mask(paths[i], Transform.identity(), rules[i], w, h)
        assert_close(batch.mask(out, i), ref)
    # fixed-point integer atomics: the order of accumulation does not matter
    assert np.array_equal(out, out_pp)


def test_batch_into_page_locked_host_memory(R):
    """Masks written by the kernel straight into page-locked host memory
    (no device copy of the output) equal the staged path's bit for bit."""
    torch = pytest.importorskip("torch")
    paths, sizes, rules = W.glyph_batch(seed=21, n=120)
    batch = MaskBatch(paths, sizes, fill_rules=rules)
    staged = R.mask_batch(batch)
    pinned = torch.full((max(batch.out_len, 1),), -7.0, dtype=torch.float32).pin_memory().numpy()
    R.mask_batch(batch, out=pinned)
    for i in range(len(paths)):
        assert np.array_equal(batch.mask(pinned, i), batch.mask(staged, i))


def _arc_glyph(w, h):
    cx, cy, r = w / 2, h / 2, 0.4 * min(w, h)
    b = PathBuilder()
    b.move_to((cx - r, cy)).arc_to((r, 0.7 * r), 0.3, False, True, (cx + r, cy))
    b.arc_to((r, 0.5 * r), 0.0, True, True, (cx - r, cy)).close()
    return b.build()


@pytest.mark.parametrize("with_arcs", [False, True])
def test_large_batch_in_chunks_into_page_locked_memory(R, with_arcs):
    """A host batch above 64 MB of masks with page-locked output is rendered in
    chunks of paths (uploads, band kernels and downloads on three streams);
    its masks equal the one-launch path's bit for bit, with transforms, both
    fill rules and (expanded on the host) arcs."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(41)
    paths, sizes, _ = W.glyph_batch(seed=43, n=1700)
    # a few empty masks, the first one among them: chunks skip or absorb them
    sizes = [(0, 0) if i % 61 == 0 else (w, 0) if i % 89 == 3 else (w, h) for i, (w, h) in enumerate(sizes)]
    trs, rules = [], []
    for i, (w, h) in enumerate(sizes):
        if with_arcs and i % 37 == 5 and w and h:
            paths[i] = _arc_glyph(w, h)
        a = rng.uniform(-0.3, 0.3)
        c = (w / 2, h / 2)
        trs.append(Transform.new_translate(*c) * Transform.new_rotate(a) * Transform.new_translate(-c[0], -c[1]))
        rules.append(FillRule(i % 2))
    batch = MaskBatch(paths, sizes, transforms=trs, fill_rules=rules)
    assert batch.out_len * 4 >= 64 << 20
    one = R.mask_batch(batch)  # pageable output: one launch
    pinned = torch.full((batch.out_len,), -7.0, dtype=torch.float32).pin_memory().numpy()
    R.mask_batch(batch, out=pinned)
    for i in range(len(paths)):
        assert np.array_equal(batch.mask(pinned, i), batch.mask(one, i)), i
    for i in range(1, len(paths), 97):
        w, h = sizes[i]
        if w and h:
            assert_close(batch.mask(pinned, i), O.mask(paths[i], trs[i], rules[i], w, h))


def test_batch_with_transforms_and_rules(R):
    rng = np.random.default_rng(5)
    paths, sizes, _ = W.glyph_batch(seed=11, n=40, side_range=(16, 300))
    trs, rules = [], []
    for i, (w, h) in enumerate(sizes):
        a = rng.uniform(0, 2 * math.pi)
        c = (w / 2, h / 2)
        trs.append(Transform.new_translate(*c) * Transform.new_rotate(a) * Transform.new_translate(-c[0], -c[1]))
        rules.append(FillRule(i % 2))
    batch = MaskBatch(paths, sizes, transforms=trs, fill_rules=rules)
    out = R.mask_batch(batch)
    for i in range(len(paths)):
        w, h = sizes[i]
        assert_close(batch.mask(out, i), O.mask(paths[i], trs[i], rules[i], w, h))


def test_lines_kernel_matches_band_kernel(R, monkeypatch):
    """The two batch kernels (the band kernel that walks the trees per band,
    the default, and flatten once + k_mask_lines) render the same masks."""
    paths, sizes, rules = W.glyph_batch(seed=31, n=200, side_range=(16, 400))
    batch = MaskBatch(paths, sizes, fill_rules=rules)
    bands = R.mask_batch(batch)
    monkeypatch.setenv("RZ_BATCH_KERNEL", "lines")
    lines = R.mask_batch(batch)
    assert np.abs(lines - bands).max() <= 1e-6
    for i in range(0, 200, 9):
        w, h = sizes[i]
        assert_close(batch.mask(lines, i), O.mask(paths[i], Transform.identity(), rules[i], w, h))


def _far_swinging_path():
    """Ten cubics swinging 5e4 px left of a 512 x 512 view: beyond the 16.16
    range (binary64 leaves, two lines each), trees 12 levels deep at flatness
    0.005 (512 subtree tasks each, under the task cap), about 80 K lines; the
    x < 0 parts become vertical lines on column 0.  And a 200-gon inside the
    view."""
    pb = PathBuilder()
    pb.move_to((300.0, 4.0))
    for k in range(10):
        y0, y1 = 4.0 + 24.0 * k, 4.0 + 24.0 * (k + 1)
        pb.cubic_to((-5.0e4, y0 + 6.0), (-5.0e4, y1 - 6.0), (300.0, y1))
    pb.close()
    pb.move_to((90.0, 60.0))
    for i in range(1, 200):
        a = 2.0 * math.pi * i / 200.0
        pb.line_to((60.0 + 30.0 * math.cos(a), 60.0 + 30.0 * math.sin(a)))
    pb.close()
    return pb.build()


def test_small_route_line_buffer_grows():
    """A path whose task estimate is small (it takes the two-launch route for
    small masks) but whose binary64 leaves take two line slots each: its
    lines overflow what that route takes, so the call falls back to the
    binned pipeline (which sizes its own buffers from the device's counts);
    the mask matches the oracle, call after call."""
    R2 = GpuRasterizer(flatness=0.005)
    path = _far_swinging_path()
    for rule in (FillRule.NonZero, FillRule.EvenOdd):
        ref = O.mask(path, Transform.identity(), rule, 512, 512, flatness=0.005)
        first = gpu_mask(R2, path, Transform.identity(), rule, 512, 512)
        assert_close(first, ref)
        assert np.array_equal(gpu_mask(R2, path, Transform.identity(), rule, 512, 512), first)


def test_pipeline_line_buffers_grow():
    """The line pipeline sizes its buffers without a host round trip: a fresh
    context starts small, so its first large path runs out of room, is
    re-rendered with buffers sized from the device's counts, and every later
    call (large or small) renders the same masks."""
    R2 = GpuRasterizer()
    path, rule, _ = W.large_path(seed=4, n_segments=5000, size=1024)
    ref = O.mask(path, Transform.identity(), rule, 1024, 1024)
    first = gpu_mask(R2, path, Transform.identity(), rule, 1024, 1024)
    assert_close(first, ref)
    assert np.array_equal(gpu_mask(R2, path, Transform.identity(), rule, 1024, 1024), first)
    small, srule, (w, h) = W.small_path(seed=0)
    assert_close(gpu_mask(R2, small, Transform.identity(), srule, w, h),
                 O.mask(small, Transform.identity(), srule, w, h))
    assert np.array_equal(gpu_mask(R2, path, Transform.identity(), rule, 1024, 1024), first)
