"""Parity at the benchmark's own shapes, through the C ABI.

* The batch plan (``rz_batch_plan_create`` / ``launch`` / ``status`` /
  ``info``: a captured CUDA graph of the record pass and the persistent band
  kernel) is the code path the headline throughput times.  Its masks must
  equal ``rz_mask_batch`` and the per-path launches bit for bit, launch after
  launch, and every glyph of the full 10,000-glyph batch must be within 1e-4
  of the binary64 oracle.
* The large single path (20,000 mixed segments with arcs and degenerate
  cubics, 4096 x 4096, EvenOdd) is where FP32 coordinates are weakest (an
  FP32 ulp at 4096 px is 4.9e-4 px): coverage within 1e-4 and the bisection
  tree's line counts equal to the oracle's.
* The scene composite (2,000 painted fills on a 2048 x 2048 RGBA f32 canvas)
  within 1e-4 per colour channel.
* The differentiable batch (64 images of 1024 x 1024, 256 closed cubic paths
  x 32 segments each): the first and last images within 1e-4 of the binary64
  forward, their gradients within 2e-3 of the binary64 adjoint's scale.
"""
import numpy as np
import pytest

from oracle import oracle as O
from rasterize_gb300 import DiffBatch, GpuRasterizer, MaskBatch, Transform
from rasterize_gb300 import workloads as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = 1e-4  # max abs coverage error per pixel (per colour channel for scenes) vs the binary64 oracle


@pytest.fixture(scope="module")
def R():
    return GpuRasterizer()


def _device_batch(batch, dev):
    d = dict(kind=torch.from_numpy(batch.kind).to(dev), pts=torch.from_numpy(batch.pts.reshape(-1)).to(dev),
             sub_off=torch.from_numpy(batch.sub_off.view(np.int32)).to(dev),
             path_sub=torch.from_numpy(batch.path_sub.view(np.int32)).to(dev))
    if batch.fill_rules is not None:
        d["fill_rules"] = torch.from_numpy(batch.fill_rules).to(dev)
    if batch.transforms is not None:
        d["transforms"] = torch.from_numpy(batch.transforms.reshape(-1)).to(dev)
    return d, {k: v.data_ptr() for k, v in d.items()}


def test_batch_plan_full_glyph_batch(R):
    """The timed path: 10,000 glyphs (seed 2, the benchmark's batch)."""
    dev = torch.device("cuda", 0)
    paths, sizes, rules = W.glyph_batch(seed=2, n=10000)
    batch = MaskBatch(paths, sizes, fill_rules=rules)
    keep, ptrs = _device_batch(batch, dev)
    out = torch.full((batch.out_len,), -3.0, dtype=torch.float32, device=dev)
    plan = R.plan(batch, ptrs, out.data_ptr())
    plan.launch()
    plan.status()
    first = out.cpu().numpy()
    out.fill_(-5.0)
    plan.launch()
    plan.launch()
    plan.status()
    again = out.cpu().numpy()
    n_items, fallbacks = plan.info()
    plan.close()
    assert n_items >= batch.n_paths and fallbacks >= 0
    ref_dev = torch.zeros(batch.out_len, dtype=torch.float32, device=dev)
    R.mask_batch_device(batch, ptrs, ref_dev.data_ptr())
    R.ctx.synchronize()
    one = ref_dev.cpu().numpy()
    ref_dev.zero_()
    R.mask_batch_device(batch, ptrs, ref_dev.data_ptr(), per_path=True)
    R.ctx.synchronize()
    per_path = ref_dev.cpu().numpy()
    worst = 0.0
    for i in range(batch.n_paths):
        m = batch.mask(first, i)
        assert np.array_equal(m, batch.mask(again, i)), "plan launches differ at glyph %d" % i
        assert np.array_equal(m, batch.mask(one, i)), "plan != rz_mask_batch at glyph %d" % i
        assert np.array_equal(m, batch.mask(per_path, i)), "plan != per-path launch at glyph %d" % i
        w, h = sizes[i]
        ref = O.mask(paths[i], Transform.identity(), rules[i], w, h)
        worst = max(worst, float(np.abs(m - ref).max()) if m.size else 0.0)
    assert worst <= TOL, worst


def test_batch_plan_transforms_and_device_rules(R):
    """A plan over a batch with per-path transforms and both fill rules."""
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(12)
    paths, sizes, _ = W.glyph_batch(seed=13, n=500)
    trs, rules = [], []
    for i, (w, h) in enumerate(sizes):
        c = (w / 2, h / 2)
        a = rng.uniform(0, 2 * np.pi)
        trs.append(Transform.new_translate(*c) * Transform.new_rotate(a) * Transform.new_translate(-c[0], -c[1]))
        rules.append(i % 2)
    batch = MaskBatch(paths, sizes, transforms=trs, fill_rules=rules)
    keep, ptrs = _device_batch(batch, dev)
    out = torch.zeros(batch.out_len, dtype=torch.float32, device=dev)
    plan = R.plan(batch, ptrs, out.data_ptr())
    for _ in range(2):
        plan.launch()
    plan.status()
    got = out.cpu().numpy()
    plan.close()
    one = R.mask_batch(batch)
    for i in range(batch.n_paths):
        assert np.array_equal(batch.mask(got, i), batch.mask(one, i)), i
        if i % 5 == 0:
            w, h = sizes[i]
            ref = O.mask(paths[i], trs[i], rules[i], w, h)
            assert float(np.abs(batch.mask(got, i) - ref).max()) <= TOL, i


def test_large_path_full_shape(R):
    """20,000 segments (40 % lines, 20 % quads, 30 % cubics with 1 % degenerate,
    10 % arcs) in [0, 4096]^2, EvenOdd, 4096 x 4096: the benchmark's input."""
    path, rule, _ = W.large_path(seed=1, n_segments=20000, size=4096)
    img = np.zeros((4096, 4096))
    R.mask(path, Transform.identity(), img, rule)
    ref = O.mask(path, Transform.identity(), rule, 4096, 4096)
    err = np.abs(img - ref)
    assert err.max() <= TOL, "max %.3g mean %.3g" % (err.max(), err.mean())
    assert np.array_equal(R.flatten_counts(path, Transform.identity()),
                          O.flatten_counts_per_input(path, Transform.identity()))


def test_scene_full_shape(R):
    """2,000 fills (20-2,000 segments each, affine transforms, 50 % solid, 25 %
    linear and 25 % radial gradients) over a 2048^2 canvas: the benchmark's input."""
    from tests.paint_oracle import oracle_scene
    sc = W.scene(seed=3, n=2000, size=2048)
    bg = (0.0, 0.0, 0.0, 1.0)
    gpu = R.render_scene(sc, 2048, 2048, bg=bg)
    ref = oracle_scene(sc, 2048, 2048, bg=bg)
    err = np.abs(gpu.astype(np.float64) - ref.astype(np.float64))
    assert err.max() <= TOL, "max %.3g mean %.3g" % (err.max(), err.mean())


def test_diff_full_shape(R):
    """The benchmark's differentiable batch: forward, L2 loss against targets
    rendered from jittered control points, adjoint; images 0 and 63 and their
    gradients against the oracle (each image's paths are independent of the
    other images')."""
    n, P, S, size = 64, 256, 32, 1024
    ctrl, tctrl = W.diff_batch(seed=4, n_images=n, paths=P, segs=S, size=size)
    dev = torch.device("cuda", 0)
    c = torch.from_numpy(ctrl).to(dev)
    t = torch.from_numpy(tctrl).to(dev)
    img = torch.empty(n * size * size, dtype=torch.float32, device=dev)
    tgt = torch.empty_like(img)
    dl = torch.empty_like(img)
    g = torch.empty(c.numel(), dtype=torch.float32, device=dev)
    R.diff_forward(DiffBatch(n, P, S, size, size, t.data_ptr()), tgt.data_ptr())
    b = DiffBatch(n, P, S, size, size, c.data_ptr())
    R.diff_forward(b, img.data_ptr())
    R.l2_loss(img.data_ptr(), tgt.data_ptr(), img.numel(), dl.data_ptr())
    R.diff_backward(b, img.data_ptr(), dl.data_ptr(), g.data_ptr())
    torch.cuda.synchronize()
    A = img.cpu().numpy().reshape(n, size, size)
    T = tgt.cpu().numpy().reshape(n, size, size)
    G = g.cpu().numpy().reshape(ctrl.shape)
    assert np.isfinite(A).all() and np.isfinite(G).all()
    for i in (0, n - 1):
        ref = O.diff_forward(ctrl[i].astype(np.float64), P, S, size, size)
        err = np.abs(A[i] - ref)
        assert err.max() <= TOL, "image %d: max %.3g mean %.3g" % (i, err.max(), err.mean())
        ref_t = O.diff_forward(tctrl[i].astype(np.float64), P, S, size, size)
        assert np.abs(T[i] - ref_t).max() <= TOL
        ref_g = O.diff_backward(ctrl[i].astype(np.float64), P, S, size, size, ref,
                                2.0 * (ref - T[i].astype(np.float64)))
        scale = np.abs(ref_g).max()
        gerr = np.abs(G[i] - ref_g).max()
        assert gerr <= 2e-3 * scale, "image %d: gradient max err %.3g, scale %.3g" % (i, gerr, scale)
