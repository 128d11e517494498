"""downsample_depth on the GPU: depths and the index map bit-identical to the oracle (both keep
equal depths in their region scan order), for the ratios the reference application uses and
for invalid regions, ties and NaN."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ratio", [1, 2, 4, 8])
def test_downsample_bit_identical_to_oracle(oracle, gpu, ratio):
    import torch
    from supereight2_gb300 import synthetic as syn
    spec, scene, poses, frames = syn.dataset("tsdf640", 1)
    depth = frames[0].copy()
    depth[:ratio, :ratio] = 0.0
    depth[16:16 + ratio, 16:16 + ratio] = 1.25
    depth[40, 40] = np.nan
    want, wmap = oracle.downsample_depth(depth, ratio)
    d = torch.from_numpy(depth).cuda()
    out = torch.empty((480 // ratio, 640 // ratio), dtype=torch.float32, device="cuda")
    mp = torch.empty(out.shape, dtype=torch.int64, device="cuda")
    gpu.downsample_depth(d, out, mp)
    assert np.array_equal(out.cpu().numpy().view(np.uint32), want.view(np.uint32))
    assert np.array_equal(mp.cpu().numpy(), wmap)


def test_downsample_rejects_bad_shapes(gpu):
    import torch
    d = torch.zeros((480, 640), device="cuda")
    with pytest.raises(gpu.SeGpuError):
        gpu.downsample_depth(d, torch.zeros((240, 300), device="cuda"))
    with pytest.raises(gpu.SeGpuError):
        gpu.downsample_depth(d, torch.zeros((30, 40), device="cuda"))  # ratio 16 > 8
