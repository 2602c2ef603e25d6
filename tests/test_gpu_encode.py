"""GPU parity of the output encode (sRGB8 RGBA, `Color::to_rgba`) against the
oracle: bit-exact on the same f32 inputs, host and device memory, f32 and
f64 masks, and the composite's fused encode against the standalone kernel."""
import numpy as np
import pytest

from oracle import oracle as O
from rasterize_gb300 import GpuRasterizer
from rasterize_gb300 import workloads as W
from tests.paint_oracle import oracle_scene

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def R():
    return GpuRasterizer()


def random_canvas(rng, n):
    """Premultiplied colours with alpha spread over [0, 1] (and the 1e-6 cut),
    plus values outside [0, 1], NaN and infinities."""
    a = rng.uniform(0, 1, n).astype(np.float32)
    a[rng.random(n) < 0.05] = np.float32(1e-6)
    a[rng.random(n) < 0.05] = 0.0
    rgb = (rng.uniform(0, 1, (n, 3)) * a[:, None]).astype(np.float32)
    c = np.concatenate([rgb, a[:, None]], axis=1)
    odd = rng.random(n) < 0.02
    c[odd] = rng.uniform(-2, 3, (int(odd.sum()), 4)).astype(np.float32)
    c[rng.random(n) < 0.002, 0] = np.nan
    c[rng.random(n) < 0.002, 1] = np.inf
    return c


@pytest.mark.parametrize("n", [1, 3, 4, 1023, 100_003])
def test_encode_rgba8_bit_exact(R, n):
    c = random_canvas(np.random.default_rng(n), n)
    assert (R.encode_rgba8(c) == O.encode_rgba8(c)).all()


def test_encode_rgba8_every_byte_roundtrip(R):
    """RGBA -> LinColor (oracle) -> RGBA (GPU) is the identity for every byte."""
    v = np.arange(256)
    lin = np.stack([O.lin_from_rgba8(np.array([x, 255 - x, x // 3, 255], dtype=np.uint8)) for x in v])
    out = R.encode_rgba8(lin)
    assert (out[:, 0] == v).all() and (out[:, 1] == 255 - v).all() and (out[:, 2] == v // 3).all()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_encode_mask_bit_exact(R, dtype):
    rng = np.random.default_rng(11)
    m = rng.uniform(-0.25, 1.25, 50_001)
    m[:5] = [0.0, 1.0, 0.5, np.nan, 1e-9]
    m = m.astype(dtype)
    assert (R.encode_mask_rgba8(m) == O.encode_mask_rgba8(m.astype(np.float64))).all()


def test_encode_mask_of_a_rendered_mask(R):
    """A path's f64 mask, encoded the way the reference writes mask images."""
    from rasterize_gb300 import FillRule, Transform
    path = W.contour(np.random.default_rng(2), 60, 40.0)
    img = np.zeros((96, 96))
    R.mask(path, Transform.new_translate(48, 48), img, FillRule.NonZero)
    assert (R.encode_mask_rgba8(img) == O.encode_mask_rgba8(img)).all()


def test_encode_device_memory(R):
    torch = pytest.importorskip("torch")
    c = random_canvas(np.random.default_rng(5), 4099)
    dev = torch.device("cuda", 0)
    src = torch.from_numpy(c).to(dev)
    dst = torch.zeros(4099 * 4, dtype=torch.uint8, device=dev)
    lib = R.ctx.lib
    R.ctx.check(lib.rz_encode_rgba8(R.ctx.ptr, src.data_ptr(), 4099, dst.data_ptr(), 1))
    R.ctx.check(lib.rz_synchronize(R.ctx.ptr))
    assert (dst.cpu().numpy().reshape(-1, 4) == O.encode_rgba8(c)).all()


def test_scene_rgba8_fused_equals_encode_of_canvas(R):
    """The composite's fused epilogue writes exactly the standalone encode of
    the f32 canvas; against the oracle's scene the bytes stay within the
    canvas tolerance carried through the encode."""
    sc = W.scene(seed=5, n=40, size=256, seg_range=(20, 200), radius_range=(8, 64))
    bg = (0.1, 0.1, 0.12, 1.0)
    canvas = R.render_scene(sc, 256, 200, bg=bg)
    fused = R.render_scene_rgba8(sc, 256, 200, bg=bg)
    assert (fused == R.encode_rgba8(canvas)).all()
    ref = O.encode_rgba8(oracle_scene(sc, 256, 200, bg=bg).astype(np.float32))
    diff = np.abs(fused.astype(np.int32) - ref.astype(np.int32))
    # opaque background: alpha ~1, so a 6.5e-5 canvas error moves a byte by at most 1
    assert diff.max() <= 1, diff.max()
    assert (diff > 0).mean() < 0.01


def test_scene_rgba8_empty(R):
    from rasterize_gb300 import Scene
    out = R.render_scene_rgba8(Scene(), 9, 5, bg=(0.5, 0.25, 0.0, 1.0))
    want = O.encode_rgba8(np.array([[0.5, 0.25, 0.0, 1.0]], dtype=np.float32))[0]
    assert (out == want).all()


def test_encode_at_every_byte_threshold(R):
    """Channel values a few ulps either side of every place the byte changes
    (the oracle's scan of every f32 in [0, 1]), where the hardware square
    roots and the IEEE route could disagree: opaque and through the division."""
    T, mono = O.l2s_byte_thresholds()
    assert not mono  # the rounded fit steps back by one byte in a dozen places
    vals = []
    for t in T[1:]:
        b = int(np.float32(t).view(np.uint32))
        vals += [np.uint32(b + d).view(np.float32) for d in range(-64, 65)]
    v = np.array(vals, dtype=np.float32)
    v = v[(v >= 0) & (v <= 1)]
    for a in (np.float32(1.0), np.float32(0.5), np.float32(0.7)):
        c = np.stack([v * a, v[::-1] * a, np.full_like(v, 0.25) * a, np.full_like(v, a)], axis=1).astype(np.float32)
        assert (R.encode_rgba8(c) == O.encode_rgba8(c)).all()
    m = (np.float32(1.0) - v).astype(np.float32)
    assert (R.encode_mask_rgba8(m) == O.encode_mask_rgba8(m.astype(np.float64))).all()


def test_encode_strided_sweep_of_unit_interval(R):
    """Every 64th f32 in [0, 1] as an opaque channel (16.6 M values)."""
    bits = np.arange(0, 0x3F800001, 64, dtype=np.uint32)
    v = bits.view(np.float32)
    n = (len(v) + 2) // 3 * 3
    v = np.concatenate([v, np.zeros(n - len(v), dtype=np.float32)]).reshape(-1, 3)
    c = np.concatenate([v, np.ones((len(v), 1), dtype=np.float32)], axis=1)
    assert (R.encode_rgba8(c) == O.encode_rgba8(c)).all()
