"""The FP64 run of the oracle (the same restatement compiled with every float a double): it
loads beside the FP32 oracle without interference and agrees with it to float precision on a
short sequence, which is what makes it the reference for the precision reports."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def seq():
    from supereight2_gb300 import synthetic as syn
    return syn.dataset("tsdf320", 4)


def test_f64_integration_and_raycast_agree_with_f32(oracle, seq):
    from oracle import pyoracle64 as o64
    spec, scene, poses, frames = seq
    args = (spec.width, spec.height, spec.fx, spec.fy, spec.cx, spec.cy, spec.near_plane, spec.far_plane)
    m32 = oracle.OracleMap(10.24, 0.02)
    m64 = o64.OracleMap64(10.24, 0.02)
    s32, s64 = oracle.pinhole(*args), o64.pinhole(*args)
    for i, (T, d) in enumerate(zip(poses, frames)):
        a = m32.integrate_depth(d, s32, T.astype(np.float32), i)
        b = m64.integrate_depth(d, s64, T.astype(np.float32).astype(np.float64), i)
        assert abs(a.n_updated_voxels - b.n_updated_voxels) <= 1e-4 * a.n_updated_voxels
    k32, _, t32, w32, _ = m32.blocks()
    k64, _, t64, w64, _ = m64.blocks()
    common, i32, i64 = np.intersect1d(k32, k64, return_indices=True)
    assert len(common) >= 0.999 * max(len(k32), len(k64))
    both = (w32[i32] > 0) & (w64[i64] > 0)
    assert np.mean(w32[i32][both] == w64[i64][both]) > 0.999
    err = np.abs(t32[i32][both] - t64[i64][both])
    # rounding differences except where a decision flips (a projection on a pixel border, the
    # truncation bound): those few voxels see another depth
    assert np.median(err) < 1e-6 and np.quantile(err, 0.99) < 1e-5
    assert (err > 1e-4).mean() < 5e-3
    T = poses[-1]
    p32, _, _ = m32.raycast(s32, T.astype(np.float32))
    p64, _, _ = m64.raycast(s64, T.astype(np.float32).astype(np.float64))
    hit = (p32 != 0).any(-1) & (p64 != 0).any(-1)
    assert hit.mean() > 0.5
    # the march's bracketing samples move with rounding on a few rays (mm-level there)
    e = np.abs(p32[hit] - p64[hit]).max(-1)
    assert np.quantile(e, 0.9) < 1e-5 and np.quantile(e, 0.99) < 5e-3


def test_f64_track_agrees_with_f32(oracle, seq):
    from oracle import pyoracle64 as o64
    spec, scene, poses, frames = seq
    args = (spec.width, spec.height, spec.fx, spec.fy, spec.cx, spec.cy, spec.near_plane, spec.far_plane)
    m32 = oracle.OracleMap(10.24, 0.02)
    s32, s64 = oracle.pinhole(*args), o64.pinhole(*args)
    for i in range(3):
        m32.integrate_depth(frames[i], s32, poses[i].astype(np.float32), i)
    T_ref = poses[2].astype(np.float32)
    pts, nrm, _ = m32.raycast(s32, T_ref)
    acc32, T32, _ = oracle.track(s32, oracle.tracker_config(), frames[3], T_ref, pts, nrm)
    acc64, T64, _ = o64.track(s64, o64.tracker_config(), frames[3], T_ref.astype(np.float64),
                              pts.astype(np.float64), nrm.astype(np.float64))
    assert acc32 == acc64
    assert np.max(np.abs(T32[:3, 3] - T64[:3, 3])) < 1e-5
    assert np.max(np.abs(T32[:3, :3] - T64[:3, :3])) < 1e-5
