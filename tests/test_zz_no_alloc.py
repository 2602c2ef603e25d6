"""The allocation-free batch entry point, through the C ABI.

rz_mask_batch_noalloc serves callers that cannot allocate device memory
while rendering (a host framework's memory pool, real-time loops, device
memory reserved up front): its scratch is a static device array inside the
library.  This test checks it against rz_mask_batch on the same device-memory
batch, on two calls in a row (the second call reuses the array left by the
first).  Coverage is accumulated in int32 fixed point, whose sums do not
depend on the order of the atomics, and the record pass of rz_mask_batch and
the per-band loads of this entry point quantise every segment the same way,
so the masks must be equal bit for bit.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_matches_mask_batch():
    torch = pytest.importorskip("torch")
    from rasterize_gb300 import GpuRasterizer, MaskBatch, _ffi
    from rasterize_gb300 import workloads as W

    dev = torch.device("cuda", 0)
    paths, sizes, rules = W.glyph_batch(seed=21, n=400)
    batch = MaskBatch(paths, sizes, fill_rules=rules)
    d = dict(kind=torch.from_numpy(batch.kind).to(dev), pts=torch.from_numpy(batch.pts.reshape(-1)).to(dev),
             sub_off=torch.from_numpy(batch.sub_off.view(np.int32)).to(dev),
             path_sub=torch.from_numpy(batch.path_sub.view(np.int32)).to(dev),
             fill_rules=torch.from_numpy(batch.fill_rules).to(dev))
    ptrs = {k: v.data_ptr() for k, v in d.items()}
    torch.cuda.synchronize(dev)

    # existing entry point (allocates its scratch through a context)
    R = GpuRasterizer()
    ref = torch.zeros(batch.out_len, dtype=torch.float32, device=dev)
    R.mask_batch_device(batch, ptrs, ref.data_ptr())
    R.ctx.synchronize()
    ref_h = ref.cpu().numpy()
    assert ref_h.any()

    lib = _ffi.load()
    s = batch.struct(_ffi.RZ_MEM_DEVICE, ptrs)
    for call in range(2):
        out = torch.full((batch.out_len,), 7.0, dtype=torch.float32, device=dev)
        torch.cuda.synchronize(dev)
        st = lib.rz_mask_batch_noalloc(ctypes.byref(s), R.flatness, out.data_ptr(), batch.out_len, None)
        assert st == 0, "rz_mask_batch_noalloc returned %d on call %d" % (st, call)
        got = out.cpu().numpy()
        for i in range(batch.n_paths):
            a = batch.mask(got, i)
            e = batch.mask(ref_h, i)
            assert np.array_equal(a, e), "call %d, path %d: max difference %.3g" % (call, i, float(np.abs(a - e).max()))


def _small_device_batch(torch, n, seed):
    """A real device-memory batch: whatever the entry point does with it stays in bounds."""
    from rasterize_gb300 import MaskBatch, _ffi
    from rasterize_gb300 import workloads as W

    dev = torch.device("cuda", 0)
    paths, sizes, _ = W.glyph_batch(seed=seed, n=n)
    batch = MaskBatch(paths, sizes)
    keep = dict(kind=torch.from_numpy(batch.kind).to(dev), pts=torch.from_numpy(batch.pts.reshape(-1)).to(dev),
                sub_off=torch.from_numpy(batch.sub_off.view(np.int32)).to(dev),
                path_sub=torch.from_numpy(batch.path_sub.view(np.int32)).to(dev),
                out=torch.zeros(max(batch.out_len, 1), dtype=torch.float32, device=dev))
    s = batch.struct(_ffi.RZ_MEM_DEVICE, {k: v.data_ptr() for k, v in keep.items()})
    return batch, s, keep


def test_noalloc_rejects_oversized_batch():
    torch = pytest.importorskip("torch")
    from rasterize_gb300 import _ffi

    batch, s, keep = _small_device_batch(torch, 2, 22)
    s.n_paths = 16385  # beyond the static scratch; rejected before any memory is touched
    big = (_ffi.RzMaskDesc * 16385)()  # zero-size masks: nothing to render even if it were accepted
    s.masks = ctypes.addressof(big)
    lib = _ffi.load()
    st = lib.rz_mask_batch_noalloc(ctypes.byref(s), 0.05, keep["out"].data_ptr(), batch.out_len, None)
    torch.cuda.synchronize()
    assert st == 7  # RZ_ERR_CAPACITY


def test_noalloc_rejects_bad_flatness():
    """Flatness must make 16 f^2 finite and positive, as for rz_mask_batch."""
    torch = pytest.importorskip("torch")
    from rasterize_gb300 import _ffi

    batch, s, keep = _small_device_batch(torch, 2, 22)
    lib = _ffi.load()
    for f in (float("inf"), float("-inf"), float("nan"), 0.0, 1e-200):
        st = lib.rz_mask_batch_noalloc(ctypes.byref(s), f, keep["out"].data_ptr(), batch.out_len, None)
        assert st == 2, (f, st)  # RZ_ERR_INVALID
    torch.cuda.synchronize()
