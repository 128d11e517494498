"""The persistent ICP (all levels and iterations of a track() in one cooperative launch, CTAs
meeting at a bounded grid barrier) against the one-launch-per-iteration ICP: poses, final
reductions and iteration counts bit-identical, on a converging and on a non-converging
(threshold 0) configuration."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("icp_threshold", [1e-5, 0.0])
def test_persistent_equals_per_iteration(gpu, icp_threshold):
    import torch
    from supereight2_gb300 import synthetic as syn
    spec, scene, poses, frames = syn.dataset("tsdf640", 3)
    sensor = gpu.PinholeCamera.from_spec(spec)
    m = gpu.Map(10.24, 0.01, max_blocks=1 << 19)
    integ = gpu.MapIntegrator(m)
    T0 = poses[0].astype(np.float32)
    integ.integrateDepth(0, torch.from_numpy(frames[0]).cuda(), sensor, T0)
    pts = torch.zeros((sensor.height, sensor.width, 3), device="cuda")
    nrm = torch.zeros_like(pts)
    gpu.raycast_volume(m, sensor, T0, pts, nrm)
    d = gpu.bilateral_filter(torch.from_numpy(frames[1]).cuda())
    out = []
    for persistent in (True, False):
        tr = gpu.Tracker(m, sensor, gpu.TrackerConfig(icp_threshold=icp_threshold))
        tr.set_persistent(persistent)
        T = T0.copy()
        acc = tr.track(d, T, pts, nrm)
        red, its = tr.last_reduction()
        out.append((acc, T, np.asarray(red), tuple(its)))
    (a1, T1, r1, i1), (a2, T2, r2, i2) = out
    assert a1 == a2 and i1 == i2
    assert np.array_equal(T1, T2)
    assert np.array_equal(r1.view(np.uint32), r2.view(np.uint32))
    if icp_threshold == 0.0:
        assert i1 == (10, 5, 4)
    assert np.linalg.norm(T1[:3, 3] - poses[1][:3, 3]) < 0.01
