"""Parity of the GPU LiDAR occupancy integration and of the batched integration with the CPU
oracle: every live block (coordinates, scales, counters, mean / min / max pyramids) and every
node reachable from the root must match, as in the pinhole occupancy tests.

Scenes: the seeded outdoor scene (ground plane, 100 boxes and 100 cylinders over 100 x 100 m)
seen by the 64 x 1024 LiDAR (+-22.5 degrees, 0.5-60 m) driving along three roads with 40 %, 64 %
and 95 % of the returns kept, at 0.4 m in a 256^3 map; and the room dolly of the pinhole tests
for the batched pinhole path.
"""
import numpy as np
import pytest

from supereight2_gb300 import synthetic as syn
from tests.test_gpu_occupancy import _compare

pytestmark = pytest.mark.gpu

T_MW = np.eye(4, dtype=np.float32)
T_MW[:3, 3] = (51.2, 51.2, 12.8)


def _oracle_lidar(oracle, spec):
    return oracle.lidar(spec.width, spec.height, spec.elevation_min_deg, spec.elevation_max_deg,
                        spec.near_plane, spec.far_plane)


def _lidar_data(n_frames, roads=(0, 3, 7)):
    spec = syn.LIDAR_64
    scene = syn.make_outdoor_scene(1004)
    keep = [0.40 + 0.55 * k / 7 for k in roads]
    poses = [syn.road_trajectory(k, n_frames, phase=0.7 * k) for k in roads]
    ranges = [[syn.render_range(scene, spec, T, 7919 + 1000 * k + i, keep=kp)
               for i, T in enumerate(P)] for k, kp, P in zip(roads, keep, poses)]
    return spec, poses, ranges


def _gpu_map(gpu):
    return gpu.Map(102.4, 0.4, res_type="multi", field="occupancy", max_blocks=1 << 15, T_MW=T_MW)


def test_lidar_single_map_matches_oracle(oracle, gpu):
    import torch
    spec, poses, ranges = _lidar_data(4, roads=(2,))
    om = oracle.OracleOccMap(102.4, 0.4, T_MW=T_MW)
    gm = _gpu_map(gpu)
    integ = gpu.MapIntegrator(gm)
    gs = gpu.OusterLidar.from_spec(spec)
    for i, (r, T) in enumerate(zip(ranges[0], poses[0])):
        T = T.astype(np.float32)
        ost = om.integrate_lidar(r, _oracle_lidar(oracle, spec), T, i)
        integ.integrateDepth(i, torch.from_numpy(r).cuda(), gs, T)
        assert (ost.n_blocks_listed, ost.n_nodes_listed, ost.n_blocks_freed, ost.n_nodes_pruned) \
            == tuple(gm.occupancy_stats())
    gm.check()
    _compare(om, gm)


@pytest.mark.parametrize("graph,autotune,persistent", [(False, False, False), (True, False, False),
                                                        (True, True, False), (False, False, True),
                                                        (True, True, True)])
def test_lidar_batch_matches_oracle(oracle, gpu, graph, autotune, persistent):
    import torch
    spec, poses, ranges = _lidar_data(4)
    n = len(poses)
    oms = [oracle.OracleOccMap(102.4, 0.4, T_MW=T_MW) for _ in range(n)]
    gms = [_gpu_map(gpu) for _ in range(n)]
    batch = gpu.OccupancyBatch(gms, gpu.OusterLidar.from_spec(spec), graph=graph, autotune=autotune,
                               persistent=persistent)
    ol = _oracle_lidar(oracle, spec)
    for i in range(len(poses[0])):
        imgs = torch.from_numpy(np.stack([ranges[k][i] for k in range(n)])).cuda()
        Ts = np.stack([poses[k][i] for k in range(n)]).astype(np.float32)
        batch.integrate(imgs, Ts, i)
        for k in range(n):
            oms[k].integrate_lidar(ranges[k][i], ol, Ts[k], i)
    if autotune:
        assert batch.tiles()[1] == 16 - len(poses[0])  # still tuning (its first calls are untimed)
    counts = []
    for om, gm in zip(oms, gms):
        gm.check()
        _compare(om, gm)
        counts.append(len(om.blocks()[0]))
    assert len(set(counts)) == n          # uneven work across the batch


@pytest.mark.parametrize("persistent", [False, True])
def test_pinhole_batch_matches_oracle(oracle, gpu, persistent):
    import torch
    sensor, _, poses, frames = syn.dataset("mr160", 6)
    spec = dict(width=sensor.width, height=sensor.height, fx=sensor.fx, fy=sensor.fy, cx=sensor.cx,
                cy=sensor.cy, near_plane=sensor.near_plane, far_plane=sensor.far_plane)
    s = oracle.pinhole(**spec)
    oms = [oracle.OracleOccMap(10.24, 0.02) for _ in range(2)]
    gms = [gpu.Map(10.24, 0.02, res_type="multi", field="occupancy", max_blocks=1 << 18) for _ in range(2)]
    batch = gpu.OccupancyBatch(gms, gpu.PinholeCamera(**spec), graph=True, persistent=persistent)
    for i in range(len(frames)):
        # the second map sees the frames in reverse order
        idx = [i, len(frames) - 1 - i]
        imgs = [torch.from_numpy(np.ascontiguousarray(frames[j], np.float32)).cuda() for j in idx]
        Ts = np.stack([poses[j] for j in idx]).astype(np.float32)
        batch.integrate(imgs, Ts, i)
        for k in range(2):
            oms[k].integrate_depth(frames[idx[k]], s, Ts[k], i)
    for om, gm in zip(oms, gms):
        gm.check()
        _compare(om, gm)


@pytest.mark.parametrize("persistent", [False, True])
def test_lidar_batch_after_tuning_matches_oracle(oracle, gpu, persistent):
    """Eighteen scans: sixteen tuning calls (four untimed), then the graph captured with the
    chosen geometry."""
    import torch
    spec, poses, ranges = _lidar_data(18, roads=(5,))
    om = oracle.OracleOccMap(102.4, 0.4, T_MW=T_MW)
    gm = _gpu_map(gpu)
    batch = gpu.OccupancyBatch([gm], gpu.OusterLidar.from_spec(spec), graph=True, autotune=True,
                               persistent=persistent)
    ol = _oracle_lidar(oracle, spec)
    for i, (r, T) in enumerate(zip(ranges[0], poses[0])):
        T = T.astype(np.float32)
        batch.integrate([torch.from_numpy(r).cuda()], T[None], i)
        om.integrate_lidar(r, ol, T, i)
    tiles, left = batch.tiles()
    assert left == 0 and all(t in (1, 2, 4, 8, 16) for t in tiles)
    if persistent:
        assert tiles[0] in (1, 2)
    gm.check()
    _compare(om, gm)


def test_batch_stats_async_equals_map_stats(gpu):
    import torch
    spec, poses, ranges = _lidar_data(2, roads=(0, 3))
    gms = [_gpu_map(gpu) for _ in range(2)]
    batch = gpu.OccupancyBatch(gms, gpu.OusterLidar.from_spec(spec), graph=True)
    out = torch.zeros((2, 4), dtype=torch.int32).pin_memory()
    for i in range(2):
        imgs = torch.from_numpy(np.stack([ranges[k][i] for k in range(2)])).cuda()
        batch.integrate(imgs, np.stack([poses[k][i] for k in range(2)]).astype(np.float32), i)
        batch.stats_async(out)
        torch.cuda.synchronize()
        for k, gm in enumerate(gms):
            assert tuple(int(v) for v in out[k]) == tuple(gm.occupancy_stats())
    assert int(out[:, 0].min()) > 0
