"""Parity of the multi-resolution TSDF map on the GPU with the CPU oracle.

Bars (as for the single-res map): block keys, integration scales and integer weights (data and
past data, every level of the voxel pyramid) bit-exact; TSDF values within 1e-5 * truncation
(FP32 storage); raycast depth within 1e-4 m on >= 99.9 % of the pixels both hit, with the same
surface scale; batched interpolation / gradient queries as the oracle answers them.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TSDF_TOL = 1e-5
DEPTH_TOL_M = 1e-4
DEPTH_FRAC = 0.999


def _spec(sensor):
    return dict(width=sensor.width, height=sensor.height, fx=sensor.fx, fy=sensor.fy,
                cx=sensor.cx, cy=sensor.cy, near_plane=sensor.near_plane,
                far_plane=sensor.far_plane)


def _by_key(keys, *arrays):
    order = np.argsort(keys)
    return (keys[order],) + tuple(a[order] for a in arrays)


def _run(oracle, gpu, config, n_frames, storage="f32"):
    import torch
    from supereight2_gb300 import synthetic as syn
    sensor, _, poses, frames = syn.dataset(config, n_frames)
    spec = _spec(sensor)
    om = oracle.OracleMap(10.24, 0.02, multires=True)
    os_ = oracle.pinhole(**spec)
    gm = gpu.Map(10.24, 0.02, max_blocks=1 << 16, res_type="multi", storage=storage)
    gs = gpu.PinholeCamera(**spec)
    integ = gpu.MapIntegrator(gm)
    stats = []
    for i, (T, d) in enumerate(zip(poses, frames)):
        T32 = T.astype(np.float32)
        ost = om.integrate_depth(d, os_, T32, i)
        integ.integrateDepth(i, torch.from_numpy(d).cuda(), gs, T32)
        stats.append((ost, gm.integrate_stats()))
    gm.check()
    return dict(om=om, gm=gm, os=os_, gs=gs, poses=poses, stats=stats)


@pytest.fixture(scope="module")
def dolly(oracle, gpu):
    return _run(oracle, gpu, "mr160", 14)


def test_counters_match(dolly):
    for ost, gst in dolly["stats"]:
        assert gst["n_valid_pixels"] == ost.n_valid_pixels
        assert gst["n_new_blocks"] == ost.n_new_blocks
        assert gst["n_updated_voxels"] == ost.n_updated_voxels


def test_pyramids_match(dolly):
    o = _by_key(*dolly["om"].mr_blocks())
    g = _by_key(*dolly["gm"].download_multires())
    ok, oc, ot, ow, opt, opw, osc = o
    gk, gc, gt, gw, gpt, gpw, gsc = g
    assert len(gk) == len(ok) > 0
    assert np.array_equal(gk, ok) and np.array_equal(gc, oc)
    assert np.array_equal(gsc, osc)                       # current and min scales
    assert len(np.unique(osc[:, 0])) >= 2
    assert np.array_equal(gw, ow) and np.array_equal(gpw, opw)   # integer weights, all levels
    assert np.max(np.abs(gt - ot)) <= TSDF_TOL
    assert np.max(np.abs(gpt - opt)) <= TSDF_TOL


def _cam_depth(pts, T_WS):
    Tinv = np.linalg.inv(T_WS.astype(np.float64))
    p = pts.reshape(-1, 3).astype(np.float64) @ Tinv[:3, :3].T + Tinv[:3, 3]
    return p[:, 2].reshape(pts.shape[:2])


def test_raycast_matches(dolly, gpu):
    import torch
    gs = dolly["gs"]
    for k in (4, 11):
        T = dolly["poses"][k].astype(np.float32)
        op, on, osc = dolly["om"].raycast(dolly["os"], T)
        pts = torch.zeros((gs.height, gs.width, 3), dtype=torch.float32, device="cuda")
        nrm = torch.zeros_like(pts)
        sc = torch.zeros((gs.height, gs.width), dtype=torch.int8, device="cuda")
        gpu.raycast_volume(dolly["gm"], gs, T, pts, nrm, sc)
        gp, gn, gsc = pts.cpu().numpy(), nrm.cpu().numpy(), sc.cpu().numpy()
        ohit, ghit = (op != 0).any(-1), (gp != 0).any(-1)
        assert (ohit == ghit).mean() >= DEPTH_FRAC
        both = ohit & ghit
        assert both.mean() > 0.5
        dz = np.abs(_cam_depth(gp, T) - _cam_depth(op, T))[both]
        assert (dz <= DEPTH_TOL_M).mean() >= DEPTH_FRAC
        assert (gsc[both] == osc[both]).mean() >= DEPTH_FRAC
        on_ok = (on != 0).any(-1) & both
        assert (np.sum(gn[on_ok] * on[on_ok], -1) > 1 - 1e-6).mean() >= DEPTH_FRAC


def test_field_queries_match(dolly, oracle, gpu):
    import torch
    from oracle import pyoracle as po
    rng = np.random.default_rng(7)
    T = dolly["poses"][6].astype(np.float32)
    op, _, _ = dolly["om"].raycast(dolly["os"], T)
    hits = op[(op != 0).any(-1)]
    pts = (hits[rng.choice(len(hits), 2000)] + rng.normal(0, 0.03, (2000, 3))).astype(np.float32)
    dp = torch.from_numpy(pts).cuda()
    gv, gvalid = dolly["gm"].getFieldInterp(dp)
    gg, ggvalid = dolly["gm"].getFieldGrad(dp)
    gv, gvalid, gg, ggvalid = [t.cpu().numpy() for t in (gv, gvalid, gg, ggvalid)]
    L = po.lib()
    import ctypes as C
    n_ok = 0
    for i, p in enumerate(pts):
        v = C.c_float()
        ok = L.so_map_get_field_interp(dolly["om"].h, np.ascontiguousarray(p), C.byref(v))
        assert bool(ok) == bool(gvalid[i])
        if ok:
            assert abs(v.value - gv[i]) <= TSDF_TOL
            n_ok += 1
        g = np.zeros(3, np.float32)
        okg = L.so_map_get_field_grad(dolly["om"].h, np.ascontiguousarray(p), g)
        assert bool(okg) == bool(ggvalid[i])
        if okg:
            assert np.allclose(g, gg[i], rtol=1e-4, atol=1e-3)
    assert n_ok > 500


def test_scale0_maps_equal_single_res(gpu):
    """All blocks at scale 0: the multi-res map's finest level equals the single-res map."""
    import torch
    from supereight2_gb300 import synthetic as syn
    sensor, _, poses, frames = syn.dataset("tsdf320", 4)
    gs = gpu.PinholeCamera(**_spec(sensor))
    maps = [gpu.Map(10.24, 0.02, max_blocks=1 << 16, res_type=r) for r in ("single", "multi")]
    for m in maps:
        integ = gpu.MapIntegrator(m)
        for i, (T, d) in enumerate(zip(poses, frames)):
            integ.integrateDepth(i, torch.from_numpy(d).cuda(), gs, T.astype(np.float32))
        m.check()
    a = _by_key(*maps[0].download_blocks()[:4])
    b = _by_key(*maps[1].download_blocks()[:4])
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_fp16_multires_weights_exact(oracle, gpu):
    r = _run(oracle, gpu, "mr160", 8, storage="f16")
    o = _by_key(*r["om"].mr_blocks())
    g = _by_key(*r["gm"].download_multires())
    assert np.array_equal(g[0], o[0]) and np.array_equal(g[6], o[6])
    assert np.array_equal(g[3], o[3])      # weights do not depend on the TSDF values
    # FP16 rounding of a running mean: |error| <= ((w + 1) / 2) * 2^-11 after w updates,
    # plus the down-propagated deltas
    assert np.max(np.abs(g[2] - o[2])) <= 1e-2
