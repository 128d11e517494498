"""The bilateral pre-filter on the GPU: bit-identical to the oracle (both evaluate the same float
operations, including the exponential), and the captured frame pipeline that tracks on the
filtered input equals the blocking calls with the filter applied explicitly; the ICP on filtered
input matches the oracle's within the pose bar."""
import numpy as np
import pytest

from tests.test_gpu_parity import POSE_TOL_M, POSE_TOL_RAD, _gpu_raycast, _rot_angle, seq320  # noqa: F401

pytestmark = pytest.mark.gpu


def test_filter_bit_identical_to_oracle(oracle, gpu):
    import torch
    from supereight2_gb300 import synthetic as syn
    for cfg, n in (("tsdf640", 2), ("tsdf320", 2)):
        spec, scene, poses, frames = syn.dataset(cfg, n)
        for d in frames:
            d = d.copy()
            d[5, 7] = np.nan
            want = oracle.bilateral_filter(d)
            got = gpu.bilateral_filter(torch.from_numpy(d).cuda()).cpu().numpy()
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # other radii and sigmas
    d = frames[0]
    for r, ss, sr in ((0, 1.0, 0.01), (1, 2.0, 0.05), (7, 3.0, 0.02)):
        want = oracle.bilateral_filter(d, r, ss, sr)
        got = gpu.bilateral_filter(torch.from_numpy(d).cuda(), radius=r, sigma_space=ss,
                                   sigma_range=sr).cpu().numpy()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    with pytest.raises(gpu.SeGpuError):
        gpu.bilateral_filter(torch.from_numpy(d).cuda(), radius=8)


def test_track_on_filtered_input_matches_oracle(seq320, oracle, gpu):  # noqa: F811
    import torch
    k = len(seq320["poses"]) - 2
    T_ref = seq320["poses"][k].astype(np.float32)
    op, on, _ = seq320["om"].raycast(seq320["os"], T_ref)
    gp, gn, _ = _gpu_raycast(gpu, seq320["gm"], seq320["gs"], T_ref)
    depth = seq320["frames"][k + 1]
    acc_o, T_o, _ = oracle.track(seq320["os"], oracle.tracker_config(), oracle.bilateral_filter(depth), T_ref,
                                 op, on)
    tracker = gpu.Tracker(seq320["gm"], seq320["gs"], gpu.TrackerConfig())
    T_g = T_ref.copy()
    filt = gpu.bilateral_filter(torch.from_numpy(depth).cuda())
    acc_g = tracker.track(filt, T_g, torch.from_numpy(gp).cuda(), torch.from_numpy(gn).cuda())
    assert acc_g == acc_o
    assert np.max(np.abs(T_g[:3, 3] - T_o[:3, 3])) <= POSE_TOL_M
    dR = T_g[:3, :3].astype(np.float64) @ T_o[:3, :3].astype(np.float64).T
    assert _rot_angle(dR) <= POSE_TOL_RAD


def test_frame_pipeline_with_filter_equals_blocking_calls(gpu):
    import torch
    from supereight2_gb300 import synthetic as syn
    spec, scene, poses, frames = syn.dataset("tsdf320", 6)
    sensor = gpu.PinholeCamera.from_spec(spec)
    H, W = sensor.height, sensor.width
    # blocking calls: filter, track on the filtered depth, integrate and raycast the raw depth
    m1 = gpu.Map(10.24, 0.02, max_blocks=1 << 16)
    integ = gpu.MapIntegrator(m1)
    tr1 = gpu.Tracker(m1, sensor)
    pts = torch.zeros((H, W, 3), device="cuda")
    nrm = torch.zeros_like(pts)
    T = poses[0].astype(np.float32).copy()
    out1 = []
    for i, d in enumerate(frames):
        dd = torch.from_numpy(d).cuda()
        if i > 0:
            tr1.track(gpu.bilateral_filter(dd), T, pts, nrm)
        integ.integrateDepth(i, dd, sensor, T)
        gpu.raycast_volume(m1, sensor, T, pts, nrm)
        out1.append(T.copy())
    # the captured pipeline
    m2 = gpu.Map(10.24, 0.02, max_blocks=1 << 16)
    tr2 = gpu.Tracker(m2, sensor)
    fp = gpu.FramePipeline(m2, sensor, tr2)
    fp.set_bilateral(**gpu.BILATERAL_DEFAULTS)
    fp.set_pose(poses[0].astype(np.float32), 0)
    out2 = []
    for i, d in enumerate(frames):
        fp.depth.copy_(torch.from_numpy(d).cuda())
        fp.run(track=i > 0)
        out2.append(fp.pose()[0])
    torch.cuda.synchronize()
    for a, b in zip(out1, out2):
        assert np.array_equal(a[:3], b[:3])
    assert np.array_equal(pts.cpu().numpy(), fp.points_W.cpu().numpy())
    # filtering changed the poses (the filter is in the loop)
    m3 = gpu.Map(10.24, 0.02, max_blocks=1 << 16)
    fp3 = gpu.FramePipeline(m3, sensor, gpu.Tracker(m3, sensor))
    fp3.set_pose(poses[0].astype(np.float32), 0)
    for i, d in enumerate(frames):
        fp3.depth.copy_(torch.from_numpy(d).cuda())
        fp3.run(track=i > 0)
    assert not np.array_equal(fp3.pose()[0], out2[-1])
