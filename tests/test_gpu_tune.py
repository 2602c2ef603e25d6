"""The batch autotuner: candidates timed on a device-memory batch, the best
applied to the context and stored in a JSON cache; masks rendered under any
tuning equal the default ones."""
import json

import numpy as np
import pytest

from rasterize_gb300 import GpuRasterizer, MaskBatch
from rasterize_gb300 import workloads as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def device_batch(n=300, seed=13):
    paths, sizes, rules = W.glyph_batch(seed=seed, n=n)
    batch = MaskBatch(paths, sizes, fill_rules=rules)
    dev = torch.device("cuda", 0)
    keep = dict(kind=torch.from_numpy(batch.kind).to(dev), pts=torch.from_numpy(batch.pts.reshape(-1)).to(dev),
                sub_off=torch.from_numpy(batch.sub_off.view(np.int32)).to(dev),
                path_sub=torch.from_numpy(batch.path_sub.view(np.int32)).to(dev),
                fill_rules=torch.from_numpy(batch.fill_rules).to(dev))
    out = torch.zeros(max(batch.out_len, 1), dtype=torch.float32, device=dev)
    return batch, {k: v.data_ptr() for k, v in keep.items()}, out, keep


def test_tune_applies_and_caches(tmp_path):
    R = GpuRasterizer()
    batch, ptrs, out, _keep = device_batch()
    R.mask_batch_device(batch, ptrs, out.data_ptr())
    torch.cuda.synchronize()
    ref = out.cpu().numpy().copy()
    cache = str(tmp_path / "tune.json")
    res = R.tune(batch, ptrs, out.data_ptr(), cache=cache)
    assert not res["cached"] and res["ms"] > 0
    assert [res["band_rows_cap"], res["ctas_per_sm"]] in [c[:2] for c in res["candidates"]]
    assert len(res["candidates"]) >= 5
    # the glyph pipeline's walk: slots per lane tried at the chosen band shape
    assert res["walk_slots"] in (1, 2, 4, 8)
    assert {c[2] for c in res["candidates"]} >= {1, 2, 4, 8}
    out.zero_()
    R.mask_batch_device(batch, ptrs, out.data_ptr())  # under the tuned shape
    torch.cuda.synchronize()
    assert np.abs(out.cpu().numpy() - ref).max() <= 1e-6
    table = json.load(open(cache))
    assert len(table) == 1
    R2 = GpuRasterizer()
    again = R2.tune(batch, ptrs, out.data_ptr(), cache=cache)
    assert again["cached"] and again["band_rows_cap"] == res["band_rows_cap"]


def test_set_tuning_rejects_bad_values():
    from rasterize_gb300 import RasterizeError
    R = GpuRasterizer()
    with pytest.raises(RasterizeError):
        R.set_tuning(1000, 0)
    with pytest.raises(RasterizeError):
        R.set_tuning(0, 0, 17)
    R.set_tuning(32, 2, 2)
    R.set_tuning(0, 0)


def test_walk_slots_render_the_same():
    """Slots per lane of the glyph pipeline's tree walk only change which lane walks which tree: plans made
    under every setting render the same masks, bit for bit."""
    R = GpuRasterizer()
    batch, ptrs, out, _keep = device_batch(n=500, seed=17)
    results = []
    try:
        for w in (0, 1, 2, 8, 16):
            R.set_tuning(0, 0, w)
            out.fill_(-1.0)
            plan = R.plan(batch, ptrs, out.data_ptr())
            try:
                plan.launch()
                plan.status()
            finally:
                plan.close()
            results.append(out.cpu().numpy().copy())
    finally:
        R.set_tuning(0, 0)
    for r in results[1:]:
        assert np.array_equal(r, results[0])
