"""GPU parity of the differentiable batch (rz_diff_forward, rz_l2_loss,
rasterize_backward) against the CPU binary64 oracle, and of the adjoint
against central finite differences (h = 1e-3 px)."""
import numpy as np
import pytest

from oracle import oracle as O
from rasterize_gb300 import DiffBatch, FillRule, GpuRasterizer
from rasterize_gb300 import workloads as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = 1e-4  # per pixel against the binary64 forward


@pytest.fixture(scope="module")
def R():
    return GpuRasterizer()


def run(R, ctrl, target, n, P, S, w, h, rule, alpha=0.5):
    dev = torch.device("cuda", 0)
    c = torch.from_numpy(np.ascontiguousarray(ctrl, dtype=np.float32)).to(dev)
    t = torch.from_numpy(np.ascontiguousarray(target, dtype=np.float32)).to(dev)
    img = torch.empty(n * h * w, dtype=torch.float32, device=dev)
    dl = torch.empty_like(img)
    g = torch.empty(c.numel(), dtype=torch.float32, device=dev)
    b = DiffBatch(n, P, S, w, h, c.data_ptr(), alpha=alpha, fill_rule=rule)
    R.diff_forward(b, img.data_ptr())
    loss = R.l2_loss(img.data_ptr(), t.data_ptr(), img.numel(), dl.data_ptr())
    R.diff_backward(b, img.data_ptr(), dl.data_ptr(), g.data_ptr())
    torch.cuda.synchronize()
    return (img.cpu().numpy().reshape(n, h, w), loss, g.cpu().numpy().reshape(np.shape(ctrl)))


def oracle_images(ctrl, n, P, S, w, h, rule, alpha=0.5):
    return np.stack([O.diff_forward(ctrl[i].astype(np.float64), P, S, w, h, alpha=alpha, rule=int(rule))
                     for i in range(n)])


@pytest.mark.parametrize("rule,margin,w", [(FillRule.NonZero, 0.0, 96), (FillRule.EvenOdd, 0.0, 96),
                                           (FillRule.NonZero, 15.0, 96), (FillRule.EvenOdd, 15.0, 101)])
def test_forward_loss_and_gradient_match_oracle(R, rule, margin, w):
    """Paths inside the image and crossing all four edges; a width that is not
    a multiple of 4 (the row scan's ragged end, lines written past it)."""
    n, P, S, h = 3, 6, 8, 72
    ctrl, _ = W.diff_batch(seed=1, n_images=n, paths=P, segs=S, size=72, margin=margin)
    ctrl[..., 0] *= w / 72.0
    target_imgs = oracle_images(ctrl + np.float32(1.5), n, P, S, w, h, rule)
    img, loss, grad = run(R, ctrl, target_imgs.astype(np.float32), n, P, S, w, h, rule)
    ref = oracle_images(ctrl, n, P, S, w, h, rule)
    err = np.abs(img - ref)
    assert err.max() <= TOL, err.max()
    ref_loss = float(((ref - target_imgs.astype(np.float32).astype(np.float64)) ** 2).sum())
    assert abs(loss - ref_loss) <= 1e-3 * max(1.0, ref_loss)
    ref_grad = np.stack([O.diff_backward(ctrl[i].astype(np.float64), P, S, w, h, ref[i],
                                         2.0 * (ref[i] - target_imgs[i].astype(np.float32)), rule=int(rule))
                         for i in range(n)])
    scale = np.abs(ref_grad).max()
    gerr = np.abs(grad - ref_grad)
    assert gerr.max() <= 2e-3 * scale, (gerr.max(), scale)


@pytest.mark.parametrize("w,h", [(1, 5), (3, 4), (7, 6), (33, 9)])
def test_tiny_images(R, w, h):
    """Images narrower than one 128-pixel scan step and than a word of the
    adjoint's bitmask (the row spans and marked words clamp at the edges),
    heights not multiples of the 8-row CTAs."""
    n, P, S = 2, 3, 4
    ctrl, _ = W.diff_batch(seed=9, n_images=n, paths=P, segs=S, size=h, margin=2.0)
    ctrl[..., 0] *= w / float(h)
    target = oracle_images(ctrl + np.float32(0.7), n, P, S, w, h, FillRule.NonZero).astype(np.float32)
    img, loss, grad = run(R, ctrl, target, n, P, S, w, h, FillRule.NonZero)
    ref = oracle_images(ctrl, n, P, S, w, h, FillRule.NonZero)
    assert np.abs(img - ref).max() <= TOL
    ref_grad = np.stack([O.diff_backward(ctrl[i].astype(np.float64), P, S, w, h, ref[i],
                                         2.0 * (ref[i] - target[i].astype(np.float64)))
                         for i in range(n)])
    scale = max(np.abs(ref_grad).max(), 1e-6)
    assert np.abs(grad - ref_grad).max() <= 2e-3 * scale


def _fd_setup(seed=2, P=8, S=8, w=128, h=96):
    ctrl, target = W.diff_batch(seed=seed, n_images=1, paths=P, segs=S, size=h)
    ctrl[..., 0] *= w / float(h)
    target[..., 0] *= w / float(h)
    T = oracle_images(target, 1, P, S, w, h, FillRule.NonZero).astype(np.float32)
    return ctrl, T, P, S, w, h


def _coords(rng, P, S, n=100):
    return [(int(rng.integers(P)), int(rng.integers(3 * S)), int(rng.integers(2))) for _ in range(n)]


def test_adjoint_matches_f64_finite_differences(R):
    """The GPU adjoint against central differences (h = 1e-3 px) of the
    reference's binary64 forward (the oracle) with the bisection tree held at
    the unperturbed control points, as the adjoint holds it: at most 1e-3
    relative error on 100 random coordinates (relative to max(|fd|, 1e-2))."""
    ctrl, T, P, S, w, h = _fd_setup()
    _, _, grad = run(R, ctrl, T, 1, P, S, w, h, FillRule.NonZero)
    c64 = ctrl[0].astype(np.float64)
    T64 = T[0].astype(np.float64)
    worst = 0.0
    for p, j, c in _coords(np.random.default_rng(7), P, S):
        cp, cm = c64.copy(), c64.copy()
        cp[p, j, c] += 1e-3
        cm[p, j, c] -= 1e-3
        lp = float(((O.diff_forward(cp, P, S, w, h, frozen=c64) - T64) ** 2).sum())
        lm = float(((O.diff_forward(cm, P, S, w, h, frozen=c64) - T64) ** 2).sum())
        fd = (lp - lm) / 2e-3
        worst = max(worst, abs(float(grad[0, p, j, c]) - fd) / max(abs(fd), 1e-2))
    assert worst <= 1e-3, worst


def test_gradient_matches_gpu_finite_differences(R):
    """Central differences (h = 1e-3 px) of the GPU's own FP32 forward.  The
    forward quantises coverage to 2^-22 per winding unit, so a 1e-3 px step
    resolves the loss derivative only to a few 1e-4 (the FD noise, not the
    adjoint: against the binary64 forward the adjoint matches to 1e-4, see
    the test above).  Bar: every coordinate within 1e-3 of the gradient's
    scale (max |d loss / d ctrl|), the median within 1e-3 relative."""
    ctrl, T, P, S, w, h = _fd_setup()
    _, _, grad = run(R, ctrl, T, 1, P, S, w, h, FillRule.NonZero)
    scale = float(np.abs(grad).max())
    hstep = np.float32(1e-3)
    errs, rels = [], []
    for p, j, c in _coords(np.random.default_rng(8), P, S, 60):
        cp, cm = ctrl.copy(), ctrl.copy()
        cp[0, p, j, c] += hstep
        cm[0, p, j, c] -= hstep
        dsum = float(cp[0, p, j, c]) - float(cm[0, p, j, c])
        lp = run(R, cp, T, 1, P, S, w, h, FillRule.NonZero)[1]
        lm = run(R, cm, T, 1, P, S, w, h, FillRule.NonZero)[1]
        fd = (lp - lm) / dsum
        an = float(grad[0, p, j, c])
        errs.append(abs(an - fd))
        rels.append(abs(an - fd) / max(abs(fd), 1e-2))
    assert max(errs) <= 1e-3 * scale, (max(errs), scale)
    assert float(np.median(rels)) <= 1e-3, float(np.median(rels))


def test_empty_and_invalid(R):
    dev = torch.device("cuda", 0)
    c = torch.zeros(2 * 3 * 4 * 2, dtype=torch.float32, device=dev)
    img = torch.full((2 * 8 * 8,), 5.0, dtype=torch.float32, device=dev)
    R.diff_forward(DiffBatch(2, 0, 4, 8, 8, c.data_ptr()), img.data_ptr())
    torch.cuda.synchronize()
    assert float(img.abs().max()) == 0.0
    from rasterize_gb300 import RasterizeError
    with pytest.raises(RasterizeError):
        R.diff_forward(DiffBatch(1, 1, 4, 8, 8, c.data_ptr(), alpha=1.5), img.data_ptr())
