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
    R.set_tuning(32, 2)
    R.set_tuning(0, 0)
