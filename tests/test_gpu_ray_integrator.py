"""Parity of the GPU ray-batch integration (se_gpu_occ_integrate_ray_batch) with the oracle's
serial restatement of se::RayIntegrator / MapIntegrator::integrateRayBatch.

The map after a batch must equal the oracle's: every live block (coordinates, current / min
scale, the mean / min / max pyramids bit for bit), every node reachable from the root (coordinates,
leaf flag, min / max data bit for bit) and the set of updated octants. Scenarios: the reference's
SingleRay and Propagation tests (test/integrator/ray_integrator_unittest.cpp), and a scanner moving
through a box room with a pose per ray over several batches (blocks refine and coarsen, and one
timestamp repeats), with rays inside the near plane, past the far plane and out of the map.
"""
import numpy as np
import pytest

from supereight2_gb300.synthetic import wall_rays

pytestmark = pytest.mark.gpu


def _by_coords(coords, *arrays):
    key = (coords[:, 0].astype(np.int64) << 40) | (coords[:, 1].astype(np.int64) << 20) | coords[:, 2]
    order = np.argsort(key)
    return (coords[order],) + tuple(a[order] for a in arrays)


def _compare(om, gm):
    oc, osc, _, *opyr = om.blocks()
    gc, gsc, _, *gpyr = gm.download_occupancy()
    o = _by_coords(oc, osc[:, :2], *opyr)
    g = _by_coords(gc, gsc[:, :2], *gpyr)
    assert len(o[0]) == len(g[0]) > 0
    assert np.array_equal(o[0], g[0])              # block coordinates
    assert np.array_equal(o[1], g[1])              # current and min scale
    for a, b in zip(o[2:], g[2:]):                 # mean, min, max pyramids, bit for bit
        assert np.array_equal(a, b)
    on, gn = om.nodes(), gm.download_nodes()
    for a, b in zip(on, gn):
        assert np.array_equal(a, b)


def _octant_set(a):
    return {tuple(int(v) for v in r) for r in np.asarray(a)}


def _maps(oracle, gpu, dim, res):
    T_MW = np.eye(4, dtype=np.float32)
    T_MW[:3, 3] = dim / 2
    om = oracle.OracleOccMap(dim, res, T_MW=T_MW)
    gm = gpu.Map(dim, res, res_type="multi", field="occupancy", T_MW=T_MW, max_blocks=1 << 17)
    return om, gm


def _batch(oracle, gpu, om, gm, leica, poses, rays, ts):
    import torch
    poses = np.array(np.broadcast_to(np.asarray(poses, np.float32), (len(rays), 4, 4)), order="C")
    o_upd = om.integrate_ray_batch(oracle.leica(**leica), poses, rays, ts)
    g_upd = gpu.integrate_ray_batch(gm, ts, torch.from_numpy(poses).cuda(), torch.from_numpy(rays).cuda(),
                                    gpu.LeicaLidar(**leica))
    torch.cuda.synchronize()
    gm.check()
    return _octant_set(o_upd), _octant_set(g_upd.cpu().numpy())


def test_single_ray(oracle, gpu):
    leica = dict(width=360, height=180, near_plane=0.2, far_plane=30.0, elevation_resolution_deg=1.0,
                 azimuth_resolution_deg=1.0)
    om, gm = _maps(oracle, gpu, 25.6, 0.05)
    o, g = _batch(oracle, gpu, om, gm, leica, np.eye(4), np.array([[10.0, 0.0, 0.0]], np.float32), 0)
    assert o == g and len(o) > 0
    _compare(om, gm)


def test_propagation_wall(oracle, gpu):
    leica = dict(width=360, height=180, near_plane=0.6, far_plane=30.0, elevation_resolution_deg=0.1,
                 azimuth_resolution_deg=0.1)
    om, gm = _maps(oracle, gpu, 25.6, 0.05)
    o, g = _batch(oracle, gpu, om, gm, leica, np.eye(4), wall_rays(), 0)
    assert o == g and len(o) > 1000
    _compare(om, gm)


def room_scan(n, seed, t0=0.0):
    """A scanner moving along x through a box room (|x| < 4, |y| < 3, -1.5 < z < 2.5 m), one pose
    per ray; ranges to the walls with noise, a few below the near plane and past the far plane,
    and some rays whose scanner position lies outside the map."""
    rng = np.random.default_rng(seed)
    poses = np.zeros((n, 4, 4), np.float32)
    rays = np.zeros((n, 3), np.float32)
    lo, hi = np.array([-4.0, -3.0, -1.5]), np.array([4.0, 3.0, 2.5])
    for i in range(n):
        s = t0 + i / n
        yaw = 0.3 * np.sin(2.0 * s) + 0.01 * i
        c, si = np.cos(yaw), np.sin(yaw)
        R = np.array([[c, -si, 0.0], [si, c, 0.0], [0.0, 0.0, 1.0]])
        p = np.array([-2.0 + 3.0 * s, 0.5 * np.sin(3.0 * s), 0.2])
        T = np.eye(4)
        T[:3, :3] = R
        T[:3, 3] = p
        az = 2 * np.pi * ((i * 0.618034) % 1.0)
        el = np.deg2rad(-40 + 80 * ((i * 0.41421) % 1.0))
        d_S = np.array([np.cos(el) * np.cos(az), np.cos(el) * np.sin(az), np.sin(el)])
        d_W = R @ d_S
        t = np.min(np.where(d_W > 0, (hi - p) / np.where(d_W > 0, d_W, 1), (lo - p) / np.where(d_W < 0, d_W, -1)))
        r = t + rng.normal(0, 0.02)
        if i % 97 == 0:
            r = 0.1          # inside the near plane
        if i % 89 == 0:
            r = 45.0         # past the far plane
        poses[i] = T.astype(np.float32)
        rays[i] = (r * d_S).astype(np.float32)
    return poses, rays


def test_moving_scanner_batches(oracle, gpu):
    leica = dict(width=360, height=180, near_plane=0.3, far_plane=12.0, elevation_resolution_deg=0.5,
                 azimuth_resolution_deg=0.4)
    om, gm = _maps(oracle, gpu, 12.8, 0.05)
    for k, ts in enumerate((0, 1, 1, 2)):
        poses, rays = room_scan(6000, seed=k, t0=0.25 * k)
        o, g = _batch(oracle, gpu, om, gm, leica, poses, rays, ts)
        assert o == g and len(o) > 0
        _compare(om, gm)
    sc = gm.download_occupancy()[1][:, 0]
    assert len(np.unique(sc)) >= 3               # blocks at several integration scales


def test_edge_cases(oracle, gpu):
    import torch
    leica = dict(width=360, height=180, near_plane=0.5, far_plane=5.0)
    om, gm = _maps(oracle, gpu, 6.4, 0.05)
    empty = torch.zeros((0, 3), dtype=torch.float32, device="cuda")
    assert gpu.integrate_ray_batch(gm, 0, torch.zeros((0, 4, 4), dtype=torch.float32, device="cuda"), empty,
                                   gpu.LeicaLidar(**leica)).shape[0] == 0
    # rays inside the near plane allocate only the root's children; a ray leaving the map stops
    # at its edge (the map spans [-3.2, 3.2) m); a ray that starts outside samples nothing
    poses = np.tile(np.eye(4, dtype=np.float32), (4, 1, 1))
    poses[2, :3, 3] = (2.0, 0.0, 0.0)
    poses[3, :3, 3] = (2.9, 0.0, 0.0)
    rays = np.array([[0.2, 0.0, 0.0], [0.0, 0.3, 0.0], [4.0, 0.0, 0.0], [4.0, 0.0, 0.0]], np.float32)
    o, g = _batch(oracle, gpu, om, gm, leica, poses, rays, 5)
    assert o == g
    _compare(om, gm)
