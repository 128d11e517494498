"""The ray integrator (se::RayIntegrator with a LeicaLidar, MapIntegrator::integrateRayBatch) in
the oracle, against the reference's own tests (test/integrator/ray_integrator_unittest.cpp):

- SingleRay: one 10 m ray along x into a 25.6 m map at 5 cm; every point along the ray lies in an
  allocated block whose current scale is the LeicaLidar integration scale of the block centre,
  raised to 1 in free space.
- Propagation: 300 x 300 rays at 0.1 degree onto a wall 10 m away; every node's min / max data
  bound its children's. The reference's block-level check (expect_valid_scale_data) reads parent
  and "child" at the same scale, so it compares each entry with itself; here the max data of every
  coarser block scale is checked against the finer scale's. The min side does not hold across
  scales: propagate_block_to_scale sets a parent's minimum from the mean data only for children
  that did not raise the maximum (ray_integrator_core_impl.hpp:262-272), so a parent with one
  valid child keeps a zero minimum; the oracle keeps that behaviour.
- And the map's box after the wall batch on either side of the scanner
  (test/map/map/map_aabb_unittest.cpp, aabb_ray_batch).
"""
import numpy as np
import pytest

from supereight2_gb300.synthetic import wall_rays

RES, DIM = 0.05, 25.6


def _map(oracle):
    T_MW = np.eye(4, dtype=np.float32)
    T_MW[:3, 3] = DIM / 2  # Map(dim, res): the world origin at the map centre
    return oracle.OracleOccMap(DIM, RES, T_MW=T_MW), T_MW


def _block_of(coords, v):
    hit = np.nonzero(np.all((coords <= v) & (v < coords + 8), axis=1))[0]
    return int(hit[0]) if len(hit) else -1


def test_single_ray(oracle):
    m, T_MW = _map(oracle)
    L = oracle.leica(360, 180, 0.2, 30.0, 1.0, 1.0)
    upd = m.integrate_ray_batch(L, np.eye(4, dtype=np.float32), np.array([[10.0, 0.0, 0.0]], np.float32), 0)
    assert len(upd) > 0
    coords, scales = m.blocks()[:2]
    d = 10.0
    tau = np.clip(np.float32(0.026) * np.float32(d), np.float32(6 * RES), np.float32(16 * RES))
    three_sigma = 3 * np.clip(np.float32(0.052) * np.float32(d), np.float32(1.5 * RES), np.float32(6 * RES))
    di = np.float32(0.2)
    checked = 0
    while di <= d:
        v = ((np.array([di, 0, 0], np.float32) + T_MW[:3, 3]) / np.float32(RES)).astype(np.int32)
        b = _block_of(coords, v)
        assert b >= 0
        centre = (coords[b].astype(np.float32) + 4.0) * np.float32(RES) - T_MW[:3, 3]
        s = oracle.leica_integration_scale(L, centre, RES, -1, -1)
        if np.float32(di - d) < -three_sigma and s < 1:
            s = 1
        assert scales[b, 0] == s, (di, v, s, scales[b])
        di = np.float32(di + np.float32(0.01))
        checked += 1
    assert checked > 900
    assert tau > 0


def _child_bounds(parent_min, parent_max, child_min, child_max, min_side=True):
    """expect_valid_node_data: field = occupancy * weight."""
    ok = True
    if min_side and child_min[2]:
        ok &= parent_min[0] * parent_min[1] <= child_min[0] * child_min[1]
    if child_max[2]:
        ok &= parent_max[0] * parent_max[1] >= child_max[0] * child_max[1]
    return ok


@pytest.fixture(scope="module")
def wall_map(oracle):
    m, _ = _map(oracle)
    L = oracle.leica(360, 180, 0.6, 30.0, 0.1, 0.1)
    upd = m.integrate_ray_batch(L, np.eye(4, dtype=np.float32), wall_rays(), 0)
    return m, upd


def test_propagation_nodes(wall_map):
    m, upd = wall_map
    assert len(upd) > 0
    c, mn, mx, leaf = m.nodes()
    coords, scales, _, mean, bmin, bmax = m.blocks()
    key = {tuple(x): i for i, x in enumerate(c.tolist())}
    bkey = {tuple(x): i for i, x in enumerate(coords.tolist())}
    checked = 0
    for i, (x, y, z, s) in enumerate(c.tolist()):
        h = s // 2
        for k in range(8):
            cc = (x + h * (k & 1), y + h * ((k >> 1) & 1), z + h * (k >> 2))
            if h == 8:
                if cc not in bkey:
                    continue
                b = bkey[cc]
                cmin, cmax = bmin[b, 584], bmax[b, 584]
            else:
                j = key.get(cc + (h,))
                if j is None:
                    continue
                cmin, cmax = mn[j], mx[j]
            assert _child_bounds(mn[i], mx[i], cmin, cmax), (c[i], cc)
            checked += 1
    assert checked > 1000


def test_propagation_blocks(wall_map):
    m, _ = wall_map
    coords, scales, _, mean, bmin, bmax = m.blocks()
    off = [0, 512, 576, 584]
    checked = 0
    for b in range(len(coords)):
        for s in range(3, scales[b, 0], -1):
            n, nc = 8 >> s, 8 >> (s - 1)
            for p in range(n ** 3):
                px, py, pz = p % n, (p // n) % n, p // (n * n)
                for k in range(8):
                    ci = off[s - 1] + (2 * px + (k & 1)) + nc * (2 * py + ((k >> 1) & 1)) + nc * nc * (2 * pz + (k >> 2))
                    assert _child_bounds(bmin[b, off[s] + p], bmax[b, off[s] + p], bmin[b, ci], bmax[b, ci],
                                         min_side=False)
                    checked += 1
    assert checked > 10000


def test_aabb_of_ray_batches(oracle):
    """map_aabb_unittest.cpp:88-214 (TEST(Map, aabb_ray_batch)): the wall batch at x = +10 m, then
    the same wall at x = -10 m, into a fresh 25.6 m map at 5 cm. The map's box reaches from the
    block of the near plane to the block past the wall plus tau (3 res), and one block more
    than the wall's half width on either side in y and z."""
    from tests.reference_cases import dim_to_blocks, world_aabb
    m, T_MW = _map(oracle)
    L = oracle.leica(1, 1, 0.6, 30.0, 0.1, 0.1)
    f = np.float32
    d, res = 10.0, f(RES)
    block_dim = f(res * f(8))
    half_wall_blocks = dim_to_blocks(float(f(d) * np.tan(f(15.0) * f(np.pi / 180.0))), block_dim)
    n_blocks_x = int(np.ceil(f(f(d) + f(3) * res) / block_dim))
    rays = wall_rays(d)
    for side in (1, -1):
        r = rays.copy()
        r[:, 0] *= side
        m.integrate_ray_batch(L, np.eye(4, dtype=np.float32), r, 0)
        lo, hi = world_aabb(*m.aabb(), res, T_MW[:3, 3])
        if side == 1:
            assert abs(float(lo[0]) - float(block_dim * np.floor(f(0.6) / (f(2) * block_dim)))) <= 1e-2, lo
        else:
            assert np.isclose(lo[0], np.floor(-f(f(d) + f(3) * res) / block_dim) * block_dim, rtol=0, atol=4e-6), lo
        assert np.isclose(hi[0], n_blocks_x * block_dim, rtol=0, atol=4e-6), hi
        assert np.isclose(lo[2], lo[1], rtol=0, atol=4e-6) and np.isclose(hi[2], hi[1], rtol=0, atol=4e-6)
        assert dim_to_blocks(float(lo[1]), block_dim) == -half_wall_blocks - 1
        assert dim_to_blocks(float(hi[1]), block_dim) == half_wall_blocks + 1
