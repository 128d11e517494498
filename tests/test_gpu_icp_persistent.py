"""The persistent ICP (all levels and iterations of a track() in one cooperative launch, CTAs
waiting, bounded, for each iteration's merged totals) against the one-launch-per-iteration ICP:
poses, final reductions and iteration counts bit-identical, on a converging and on a
non-converging (threshold 0) configuration."""
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


@pytest.mark.parametrize("persistent", [True, False])
def test_merge_overflow_is_reported(gpu, persistent):
    """A partial sum outside the exact merge's range (here: a fronto-parallel plane 3e5 m from
    the world origin, so that |p_W x n|^2 summed over a CTA's 256 pixels exceeds 2^38) is not
    silently wrapped: the call reports an error and the pose stays the input pose."""
    import torch
    W, H = 128, 96
    sensor = gpu.PinholeCamera(width=W, height=H, fx=100.0, fy=100.0, cx=63.5, cy=47.5,
                               near_plane=0.1, far_plane=10.0)
    depth = np.full((H, W), 2.0, np.float32)
    T = np.eye(4, dtype=np.float32)
    T[0, 3] = 3.0e5
    v, u = np.meshgrid(np.arange(H, dtype=np.float32), np.arange(W, dtype=np.float32), indexing="ij")
    p_S = np.stack([(u - np.float32(63.5)) / np.float32(100.0) * depth,
                    (v - np.float32(47.5)) / np.float32(100.0) * depth, depth], -1).astype(np.float32)
    p_W = (p_S + T[:3, 3]).astype(np.float32)
    n_ref = np.zeros_like(p_W)
    n_ref[..., 2] = -1.0
    m = gpu.Map(10.24, 0.02, max_blocks=1 << 10)
    tr = gpu.Tracker(m, sensor)
    tr.set_persistent(persistent)
    T_in = T.copy()
    with pytest.raises(gpu.SeGpuError, match="exact merge"):
        tr.track(torch.from_numpy(depth).cuda(), T, torch.from_numpy(p_W).cuda(), torch.from_numpy(n_ref).cuda())
    assert np.array_equal(T, T_in)
    # the same plane near the origin stays within range: no error (a single plane leaves the
    # system rank-deficient, so only the absence of the overflow report is checked)
    T2 = np.eye(4, dtype=np.float32)
    tr.track(torch.from_numpy(depth).cuda(), T2, torch.from_numpy(p_S.copy()).cuda(), torch.from_numpy(n_ref).cuda())


def test_barrier_timeout_is_reported(gpu):
    """The persistent ICP's wait for the merged totals is bounded: made to wait for a CTA that
    does not exist, it gives up after half a second, the pose is rejected and the call reports the
    timeout; the context stays usable and the next track succeeds."""
    import time
    import torch
    from supereight2_gb300 import synthetic as syn
    spec, scene, poses, frames = syn.dataset("tsdf320", 2)
    sensor = gpu.PinholeCamera.from_spec(spec)
    m = gpu.Map(10.24, 0.02, max_blocks=1 << 16)
    integ = gpu.MapIntegrator(m)
    T0 = poses[0].astype(np.float32)
    integ.integrateDepth(0, torch.from_numpy(frames[0]).cuda(), sensor, T0)
    pts = torch.zeros((sensor.height, sensor.width, 3), device="cuda")
    nrm = torch.zeros_like(pts)
    gpu.raycast_volume(m, sensor, T0, pts, nrm)
    d = torch.from_numpy(frames[1]).cuda()
    tr = gpu.Tracker(m, sensor)
    tr.set_persistent(True)
    tr.test_barrier_timeout(True)
    T = T0.copy()
    t0 = time.perf_counter()
    with pytest.raises(gpu.SeGpuError, match="timed out"):
        tr.track(d, T, pts, nrm)
    assert time.perf_counter() - t0 < 30.0
    assert np.array_equal(T, T0)
    tr.test_barrier_timeout(False)
    T = T0.copy()
    assert tr.track(d, T, pts, nrm)
    assert np.linalg.norm(T[:3, 3] - poses[1][:3, 3]) < 0.01
