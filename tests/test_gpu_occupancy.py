"""Parity of the GPU multi-resolution occupancy integration with the CPU oracle.

Every live block must match: coordinates, (current, min, buffer) scales, the four integration /
observation counters, and the mean / min / max pyramids (occupancy, integer weight, observed
flag); every node reachable from the root (depth first) must match in coordinates, size, leaf
flag and min / max data. Occupancy values are compared within 1e-6 (the arithmetic follows the
oracle's operation order; the tolerance only absorbs a different summation order nowhere used).

Scenarios: the reference's occupancy system test (config.yaml field parameters, 320x240 sensor
with fy < 0, split and flat walls, and the delete-children run long enough to prune), and the
synthetic room seen by the wide dolly camera at 2 cm with the default field parameters (blocks
move between scales in both directions).
"""
import numpy as np
import pytest

from tests.test_oracle_occupancy import CFG

pytestmark = pytest.mark.gpu

OCC_TOL = 1e-6


def _pinhole_spec():
    return dict(width=320, height=240, fx=481.2 / 2, fy=-480.0 / 2, cx=(319.5 + 0.5) / 2 - 0.5,
                cy=(239.5 + 0.5) / 2 - 0.5, near_plane=0.4, far_plane=6.0)


def _by_coords(coords, *arrays):
    key = (coords[:, 0].astype(np.int64) << 40) | (coords[:, 1].astype(np.int64) << 20) | coords[:, 2]
    order = np.argsort(key)
    return (coords[order],) + tuple(a[order] for a in arrays)


def _compare(om, gm):
    o = _by_coords(*om.blocks())
    g = _by_coords(*gm.download_occupancy())
    assert len(o[0]) == len(g[0]) > 0
    assert np.array_equal(o[0], g[0])                     # block coordinates
    assert np.array_equal(o[1], g[1])                     # scales
    assert np.array_equal(o[2], g[2])                     # counters
    for a, b in zip(o[3:], g[3:]):                        # mean, min, max pyramids
        assert np.array_equal(a[..., 1], b[..., 1])       # weights
        assert np.array_equal(a[..., 2], b[..., 2])       # observed flags
        assert np.max(np.abs(a[..., 0] - b[..., 0])) <= OCC_TOL
    on = om.nodes()
    gn = gm.download_nodes()
    assert np.array_equal(on[0], gn[0]) and np.array_equal(on[3], gn[3])
    for a, b in zip(on[1:3], gn[1:3]):
        assert np.array_equal(a[:, 1:], b[:, 1:])
        assert np.max(np.abs(a[:, 0] - b[:, 0])) <= OCC_TOL


def _run(oracle, gpu, frames, spec, poses, cfg, dim=10.24, res=0.01, max_blocks=1 << 17):
    import torch
    om = oracle.OracleOccMap(dim, res, **cfg) if cfg else oracle.OracleOccMap(dim, res)
    gm = gpu.Map(dim, res, res_type="multi", field="occupancy", occupancy=cfg or None, max_blocks=max_blocks)
    s = oracle.pinhole(**spec)
    integ = gpu.MapIntegrator(gm)
    gs = gpu.PinholeCamera(**spec)
    stats = []
    for i, (d, T) in enumerate(zip(frames, poses)):
        ost = om.integrate_depth(d, s, T, i)
        integ.integrateDepth(i, torch.from_numpy(np.ascontiguousarray(d, np.float32)).cuda(), gs, T)
        gst = gm.occupancy_stats()
        stats.append(((ost.n_blocks_listed, ost.n_nodes_listed, ost.n_blocks_freed, ost.n_nodes_pruned), gst))
    gm.check()
    return om, gm, stats


def test_system_test_split_wall(oracle, gpu):
    x = np.arange(320)[None, :]
    depth = (np.where(x < 160, 2.0, 4.0) * np.ones((240, 1))).astype(np.float32)
    om, gm, stats = _run(oracle, gpu, [depth], _pinhole_spec(), [np.eye(4, dtype=np.float32)], CFG)
    assert stats[0][0] == stats[0][1]
    _compare(om, gm)


def test_delete_children_run(oracle, gpu):
    x = np.arange(320)[None, :]
    noisy = (np.where((x < 120) | (x > 200), 2.0, 4.0) * np.ones((240, 1))).astype(np.float32)
    wall = np.full((240, 320), 4.0, np.float32)
    frames = [noisy] + [wall] * 19
    om, gm, stats = _run(oracle, gpu, frames, _pinhole_spec(), [np.eye(4, dtype=np.float32)] * 20, CFG)
    for o, g in stats:
        assert o == g
    assert sum(o[3] for o, _ in stats) > 0                # nodes were pruned
    _compare(om, gm)


def test_room_dolly_default_config(oracle, gpu):
    from supereight2_gb300 import synthetic as syn
    sensor, _, poses, frames = syn.dataset("mr160", 10)
    spec = dict(width=sensor.width, height=sensor.height, fx=sensor.fx, fy=sensor.fy, cx=sensor.cx,
                cy=sensor.cy, near_plane=sensor.near_plane, far_plane=sensor.far_plane)
    om, gm, stats = _run(oracle, gpu, frames, spec, [T.astype(np.float32) for T in poses], None,
                         res=0.02, max_blocks=1 << 18)
    for o, g in stats:
        assert o == g
    _compare(om, gm)
    scales = om.blocks()[1]
    assert len(np.unique(scales[:, 0])) >= 2


def _gpu_raycast(gpu, gm, spec, T):
    import torch
    gs = gpu.PinholeCamera(**spec)
    pts = torch.zeros((gs.height, gs.width, 3), dtype=torch.float32, device="cuda")
    nrm = torch.zeros_like(pts)
    sc = torch.zeros((gs.height, gs.width), dtype=torch.int8, device="cuda")
    gpu.raycast_volume(gm, gs, T, pts, nrm, sc)
    torch.cuda.synchronize()
    return pts.cpu().numpy(), nrm.cpu().numpy(), sc.cpu().numpy()


def _compare_raycast(om, gm, gpu, oracle, spec, T):
    op, on, osc = om.raycast(oracle.pinhole(**spec), T)
    gp, gn, gsc = _gpu_raycast(gpu, gm, spec, T)
    ohit, ghit = (op != 0).any(-1), (gp != 0).any(-1)
    assert (ohit == ghit).mean() >= 0.999
    both = ohit & ghit
    assert both.mean() > 0.5
    assert (np.abs(op - gp)[both].max(-1) <= 1e-4).mean() >= 0.999
    assert (osc[both] == gsc[both]).mean() >= 0.999
    on_ok = (on != 0).any(-1) & both
    assert (np.sum(on[on_ok] * gn[on_ok], -1) > 1 - 1e-5).mean() >= 0.999


def test_raycast_room_dolly(oracle, gpu):
    from supereight2_gb300 import synthetic as syn
    sensor, _, poses, frames = syn.dataset("mr160", 8)
    spec = dict(width=sensor.width, height=sensor.height, fx=sensor.fx, fy=sensor.fy, cx=sensor.cx,
                cy=sensor.cy, near_plane=sensor.near_plane, far_plane=sensor.far_plane)
    om, gm, _ = _run(oracle, gpu, frames, spec, [T.astype(np.float32) for T in poses], None,
                     res=0.02, max_blocks=1 << 18)
    for k in (3, 7):
        _compare_raycast(om, gm, gpu, oracle, spec, poses[k].astype(np.float32))


def test_raycast_system_test_wall(oracle, gpu):
    wall = np.full((240, 320), 4.0, np.float32)
    om, gm, _ = _run(oracle, gpu, [wall] * 3, _pinhole_spec(), [np.eye(4, dtype=np.float32)] * 3, CFG)
    _compare_raycast(om, gm, gpu, oracle, _pinhole_spec(), np.eye(4, dtype=np.float32))
