"""se_gpu_track_noalloc, the tracking entry point that allocates no device memory.

It runs one full-resolution ICP level with its scratch in a static device array of the
library. Its poses must agree with se_gpu_track configured for the same single level (within
1e-5 m / 1e-5 rad, the ICP parity bar) on consecutive calls, which share that scratch.
This file is collected last so that it also runs after every other GPU test in one process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

POSE_TOL_M = 1e-5
POSE_TOL_RAD = 1e-5


def _rot_angle(R):
    """Rotation angle of R: atan2 of the skew part's norm and (trace - 1) / 2. Near the identity
    arccos((trace - 1) / 2) is dominated by the rounding of float32 rotation matrices (a trace
    off by 1e-7 reads as 4.5e-4 rad); the skew part carries the small angle itself."""
    s = 0.5 * float(np.linalg.norm([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]]))
    c = (float(np.trace(R)) - 1.0) / 2.0
    return float(np.arctan2(s, c))


@pytest.fixture(scope="module")
def scene(gpu):
    """320x240 sequence integrated into a 512^3 map at 2 cm, with the raycasts at poses 3, 4."""
    import torch
    from supereight2_gb300 import synthetic as syn
    sensor, _, poses, frames = syn.dataset("tsdf320", 6)
    gs = gpu.PinholeCamera.from_spec(sensor)
    gm = gpu.Map(10.24, 0.02, max_blocks=1 << 16)
    integ = gpu.MapIntegrator(gm)
    for i, (T, d) in enumerate(zip(poses, frames)):
        integ.integrateDepth(i, torch.from_numpy(d).cuda(), gs, T.astype(np.float32))
    gm.check()
    refs = {}
    for k in (3, 4):
        T = poses[k].astype(np.float32)
        pts = torch.zeros((gs.height, gs.width, 3), dtype=torch.float32, device="cuda")
        nrm = torch.zeros_like(pts)
        sc = torch.zeros((gs.height, gs.width), dtype=torch.int8, device="cuda")
        gpu.raycast_volume(gm, gs, T, pts, nrm, sc)
        refs[k] = (T, pts, nrm, torch.from_numpy(frames[k + 1]).cuda())
    torch.cuda.synchronize()
    return dict(gm=gm, gs=gs, poses=poses, refs=refs)


def _check_close(T_a, T_b):
    assert np.max(np.abs(T_a[:3, 3] - T_b[:3, 3])) <= POSE_TOL_M
    dR = T_a[:3, :3].astype(np.float64) @ T_b[:3, :3].astype(np.float64).T
    assert _rot_angle(dR) <= POSE_TOL_RAD


def test_noalloc_matches_tracker_on_consecutive_calls(scene, gpu):
    cfg = gpu.TrackerConfig(iterations=(10,))
    tracker = gpu.Tracker(scene["gm"], scene["gs"], cfg)
    results = []
    for k in (3, 4, 3):  # two calls in a row on different inputs, then the first again
        T_ref, pts, nrm, depth = scene["refs"][k]
        T_t = T_ref.copy()
        acc_t = tracker.track(depth, T_t, pts, nrm)
        red_t, _ = tracker.last_reduction()
        T_n = T_ref.copy()
        acc_n, red_n = gpu.track_noalloc(scene["gs"], cfg, depth, T_n, pts, nrm)
        assert acc_n == acc_t
        _check_close(T_n, T_t)
        assert abs(red_n[28] - red_t[28]) <= 2           # inlier count
        # the tracked pose is near the ground truth of the tracked frame
        assert np.linalg.norm(T_n[:3, 3] - scene["poses"][k + 1][:3, 3]) < 0.01
        results.append((T_n.copy(), red_n.copy()))
    # the shared scratch carries nothing from one call into the next
    assert np.array_equal(results[0][0], results[2][0])
    assert np.array_equal(results[0][1], results[2][1])


def test_noalloc_rejects_what_it_cannot_hold(scene, gpu):
    import torch
    L = gpu.library()
    T = np.eye(4, dtype=np.float32)
    T_p = T.ctypes.data_as(C.POINTER(C.c_float))
    # a pyramid needs scratch images: more than one level is refused
    _, pts, nrm, depth = scene["refs"][3]
    s = scene["gs"]._c()
    c3 = gpu.TrackerConfig()._c()
    st = L.se_gpu_track_noalloc(C.byref(s), C.byref(c3), C.c_void_p(depth.data_ptr()),
                                C.c_void_p(pts.data_ptr()), C.c_void_p(nrm.data_ptr()), T_p,
                                None, None, None)
    assert st != 0 and b"one full-resolution level" in L.se_gpu_last_error()
    # a 4097 x 4096 image is past the pixel limit; the buffers cover it, so nothing is read out
    # of bounds even if the check were missing
    w, h = 4097, 4096
    big_d = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    big_p = torch.zeros((h, w, 3), dtype=torch.float32, device="cuda")
    big_n = torch.zeros((h, w, 3), dtype=torch.float32, device="cuda")
    sb = gpu.PinholeCamera(w, h, 500.0, 500.0, w / 2, h / 2, 0.4, 6.0)._c()
    c1 = gpu.TrackerConfig(iterations=(10,))._c()
    st = L.se_gpu_track_noalloc(C.byref(sb), C.byref(c1), C.c_void_p(big_d.data_ptr()),
                                C.c_void_p(big_p.data_ptr()), C.c_void_p(big_n.data_ptr()), T_p,
                                None, None, None)
    assert st != 0 and b"allocation-free limit" in L.se_gpu_last_error()
    del big_d, big_p, big_n
    torch.cuda.synchronize()


def test_noalloc_repeat_call_leaves_free_device_memory_unchanged(scene, gpu):
    """After a first call on the device (which loads this part of the library there), further
    calls allocate nothing: the device's free memory is the same before and after them."""
    import torch
    cfg = gpu.TrackerConfig(iterations=(10,))
    T_ref, pts, nrm, depth = scene["refs"][3]
    gpu.track_noalloc(scene["gs"], cfg, depth, T_ref.copy(), pts, nrm)  # warm-up call
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for k in (3, 4):
        T_k, pts_k, nrm_k, depth_k = scene["refs"][k]
        gpu.track_noalloc(scene["gs"], cfg, depth_k, T_k.copy(), pts_k, nrm_k)
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
