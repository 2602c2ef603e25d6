"""The glyph pipeline (rz_glyph.cu: records, walk, emit, cover) behind batch
plans, against the band kernel (RZ_BATCH_KERNEL=bands) and the binary64 oracle.

Both kernels quantise every segment through the same fixed-point record and
accumulate int32 signed areas, so their masks agree to the last bits; the
oracle bounds them to 1e-4 per pixel.
"""
import numpy as np
import pytest

from oracle import oracle as O
from rasterize_gb300 import GpuRasterizer, MaskBatch, Path, PathBuilder, Transform
from rasterize_gb300 import workloads as W
from rasterize_gb300._ffi import NanError, RasterizeError

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = 1e-4


@pytest.fixture(scope="module")
def R():
    return GpuRasterizer()


def device_arrays(batch):
    dev = torch.device("cuda", 0)
    keep = dict(kind=torch.from_numpy(batch.kind).to(dev), pts=torch.from_numpy(batch.pts.reshape(-1)).to(dev),
                sub_off=torch.from_numpy(batch.sub_off.view(np.int32)).to(dev),
                path_sub=torch.from_numpy(batch.path_sub.view(np.int32)).to(dev))
    if batch.fill_rules is not None:
        keep["fill_rules"] = torch.from_numpy(batch.fill_rules).to(dev)
    if batch.transforms is not None:
        keep["transforms"] = torch.from_numpy(batch.transforms.reshape(-1)).to(dev)
    return keep, {k: v.data_ptr() for k, v in keep.items()}


def plan_render(R, batch, ptrs, kernel, monkeypatch, launches=2):
    if kernel == "bands":
        monkeypatch.setenv("RZ_BATCH_KERNEL", "bands")
    else:
        monkeypatch.delenv("RZ_BATCH_KERNEL", raising=False)
    out = torch.full((max(batch.out_len, 1),), -2.0, dtype=torch.float32, device=torch.device("cuda", 0))
    plan = R.plan(batch, ptrs, out.data_ptr())
    try:
        for _ in range(launches):
            plan.launch()
        plan.status()
        return out.cpu().numpy()
    finally:
        plan.close()


def affine(p, sx, sy, tx, ty):
    """The path with every control point mapped by x -> sx x + tx, y -> sy y + ty (no arcs)."""
    pts = np.array(p.pts, dtype=np.float64, copy=True)
    pts[:, 0::2] = pts[:, 0::2] * sx + tx
    pts[:, 1::2] = pts[:, 1::2] * sy + ty
    return Path(p.kind, pts, p.subpath_off, p.closed)


def arc_glyph(w, h):
    cx, cy, r = w / 2, h / 2, 0.4 * min(w, h)
    b = PathBuilder()
    b.move_to((cx - r, cy)).arc_to((r, 0.7 * r), 0.3, False, True, (cx + r, cy))
    b.arc_to((r, 0.5 * r), 0.0, True, True, (cx - r, cy)).close()
    return b.build()


def far_glyph(w, h):
    """A subpath beyond the 16.16 range (x ~ 20000 px) next to one inside the mask."""
    b = PathBuilder()
    b.move_to((2, 2)).cubic_to((w, 0), (w, h), (2, h - 2)).close()
    b.move_to((20000.0, 3)).line_to((20010.0, h - 3)).quad_to((-30000.0, h / 2), (20000.0, 3)).close()
    return b.build()


def mixed_batch():
    rng = np.random.default_rng(77)
    paths, sizes, _ = W.glyph_batch(seed=78, n=600, side_range=(8, 300))
    sizes = [(0, 0) if i % 97 == 5 else (w, 0) if i % 89 == 3 else (w, h) for i, (w, h) in enumerate(sizes)]
    trs, rules = [], []
    for i, (w, h) in enumerate(sizes):
        if i % 41 == 7 and w and h:
            paths[i] = arc_glyph(w, h)
        if i % 53 == 11 and w > 8 and h > 8:
            paths[i] = far_glyph(w, h)
        c = (w / 2, h / 2)
        a = rng.uniform(-0.4, 0.4)
        trs.append(Transform.new_translate(*c) * Transform.new_rotate(a) * Transform.new_translate(-c[0], -c[1]))
        rules.append(i % 2)
    return paths, sizes, trs, rules


def test_glyph_equals_bands_mixed_batch(R, monkeypatch):
    """Transforms, both rules, raw arcs on the device, coordinates beyond the
    fixed-point range, empty masks.  With the same bands the glyph pipeline
    and the band kernel agree bit for bit; with their own band heights long
    lines are clipped at other rows, which may move a last bit."""
    paths, sizes, trs, rules = mixed_batch()
    batch = MaskBatch(paths, sizes, transforms=trs, fill_rules=rules)
    assert (batch.kind == 3).any()  # raw arcs reach the device
    keep, ptrs = device_arrays(batch)
    R.set_tuning(16, 0)  # both kernels cut every mask of this batch (at most 300 px wide) into 16-row bands
    try:
        glyph = plan_render(R, batch, ptrs, "glyph", monkeypatch)
        bands = plan_render(R, batch, ptrs, "bands", monkeypatch)
    finally:
        R.set_tuning(0, 0)
    for i in range(batch.n_paths):
        assert np.array_equal(batch.mask(glyph, i), batch.mask(bands, i)), i
    glyph_own = plan_render(R, batch, ptrs, "glyph", monkeypatch)
    assert float(np.abs(glyph_own - glyph).max()) <= 1e-6
    for i in range(0, batch.n_paths, 13):
        w, h = sizes[i]
        if w and h:
            ref = O.mask(paths[i], trs[i], rules[i], w, h)
            assert float(np.abs(batch.mask(glyph_own, i) - ref).max()) <= TOL, i


def test_glyph_plan_rewritten_inputs(R):
    """A plan's inputs rewritten between launches (same sizes): the next launch
    renders the new geometry; geometry beyond the vertex buffer's slack is an
    RZ_ERR_CAPACITY status, not an overrun."""
    dev = torch.device("cuda", 0)
    paths, sizes, rules = W.glyph_batch(seed=5, n=300)
    batch = MaskBatch(paths, sizes, fill_rules=rules)
    keep, ptrs = device_arrays(batch)
    out = torch.zeros(batch.out_len, dtype=torch.float32, device=dev)
    plan = R.plan(batch, ptrs, out.data_ptr())
    try:
        plan.launch()
        plan.status()
        # mirror every glyph in x inside its own mask: about the same number of lines
        flipped = [affine(p, -1.0, 1.0, float(sizes[i][0]), 0.0) for i, p in enumerate(paths)]
        b2 = MaskBatch(flipped, sizes, fill_rules=rules)
        keep["pts"].copy_(torch.from_numpy(b2.pts.reshape(-1)))
        plan.launch()
        plan.status()
        got = out.cpu().numpy()
        ref = R.mask_batch(b2)
        for i in range(batch.n_paths):
            assert float(np.abs(batch.mask(got, i) - b2.mask(ref, i)).max()) <= 1e-6, i
        # 16x larger control polygons: many more lines than the buffer's slack
        big = [affine(p, 16.0, 16.0, 0.0, 0.0) for p in paths]
        b3 = MaskBatch(big, sizes, fill_rules=rules)
        keep["pts"].copy_(torch.from_numpy(b3.pts.reshape(-1)))
        plan.launch()
        with pytest.raises(RasterizeError):
            plan.status()
        # the same plan renders again once the inputs fit
        keep["pts"].copy_(torch.from_numpy(batch.pts.reshape(-1)))
        plan.launch()
        plan.status()
        again = out.cpu().numpy()
        first = R.mask_batch(batch)
        for i in range(batch.n_paths):
            assert float(np.abs(batch.mask(again, i) - batch.mask(first, i)).max()) <= 1e-6, i
    finally:
        plan.close()


def test_glyph_plan_nan_is_an_error(R):
    dev = torch.device("cuda", 0)
    paths, sizes, rules = W.glyph_batch(seed=6, n=50)
    paths[17] = PathBuilder().move_to((1, 1)).line_to((float("nan"), 4)).line_to((5, 5)).close().build()
    batch = MaskBatch(paths, sizes, fill_rules=rules)
    keep, ptrs = device_arrays(batch)
    out = torch.zeros(batch.out_len, dtype=torch.float32, device=dev)
    plan = R.plan(batch, ptrs, out.data_ptr())
    try:
        plan.launch()
        with pytest.raises(NanError):
            plan.status()
        plan.launch()  # the error word was cleared: the next launch reports it again
        with pytest.raises(NanError):
            plan.status()
    finally:
        plan.close()
    # the context stays usable
    ok_paths, ok_sizes, ok_rules = W.glyph_batch(seed=7, n=20)
    b2 = MaskBatch(ok_paths, ok_sizes, fill_rules=ok_rules)
    out2 = R.mask_batch(b2)
    for i in range(0, 20, 3):
        w, h = ok_sizes[i]
        ref = O.mask(ok_paths[i], Transform.identity(), ok_rules[i], w, h)
        assert float(np.abs(b2.mask(out2, i) - ref).max()) <= TOL
