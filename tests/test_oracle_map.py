"""Pin the oracle's map, allocation and interpolation to the reference's map tests."""
import numpy as np
import pytest

from tests import reference_cases as rc


@pytest.mark.parametrize("dim,res,size", rc.MAP_SIZES)
def test_octree_size(oracle, dim, res, size):
    # map_unittest.cpp:210-236
    m = oracle.OracleMap(dim, res)
    assert m.size == size
    assert m.dim >= np.float32(dim) * (1 - 1e-6)


def test_interpolation_known_answers(oracle):
    # map_unittest.cpp:127-208
    m = oracle.OracleMap(rc.INTERP_DIM, rc.INTERP_RES)
    for i, c in enumerate(rc.INTERP_BLOCKS):
        m.set_block(c, float(i), 1.0)
    for p, want in rc.INTERP_CASES:
        got = m.field_interp(np.array(p, np.float32))
        if want is None:
            assert got is None
        else:
            assert got == want


def test_wall_aabb(oracle):
    # map_aabb_unittest.cpp:37-60 (TEST(Map, aabbTSDF))
    spec, T_WC = rc.wall_sensor()
    m = oracle.OracleMap(rc.WALL_MAP_DIM, rc.WALL_MAP_RES)
    s = oracle.pinhole(**spec)
    depth = np.full((spec["height"], spec["width"]), rc.WALL_DEPTH, np.float32)
    m.integrate_depth(depth, s, T_WC, 0)
    mn, mx = m.aabb()
    rc.check_wall_aabb(mn, mx)


def test_wall_aabb_occupancy(oracle):
    # map_aabb_unittest.cpp:62-86 (TEST(Map, aabbOccupancy))
    spec, T_WC = rc.wall_sensor()
    m = oracle.OracleOccMap(rc.WALL_MAP_DIM, rc.WALL_MAP_RES)
    assert m.aabb() is None
    s = oracle.pinhole(**spec)
    depth = np.full((spec["height"], spec["width"]), rc.WALL_DEPTH, np.float32)
    m.integrate_depth(depth, s, T_WC, 0)
    mn, mx = m.aabb()
    rc.check_wall_aabb_occupancy(mn, mx)


def test_empty_and_invalid_depth_allocates_nothing(oracle):
    m = oracle.OracleMap(10.24, 0.02)
    s = oracle.pinhole(64, 48, 50.0, 50.0, 31.5, 23.5, 0.4, 6.0)
    T = np.eye(4, dtype=np.float32)
    for d in (np.zeros((48, 64), np.float32), np.full((48, 64), 0.1, np.float32),
              np.full((48, 64), 50.0, np.float32)):
        st = m.integrate_depth(d, s, T, 0)
        assert st.n_valid_pixels == 0 and st.n_new_blocks == 0 and st.n_updated_voxels == 0
    assert m.num_blocks() == 0 and m.aabb() is None


def test_first_block_tmin_matches_block_entry(oracle):
    # VoxelBlockRayIterator::tcmin() of the first block along axis-aligned rays through a
    # single allocated block: the entry distance of that block.
    m = oracle.OracleMap(8.0, 0.5)  # 16^3 voxels, T_MW = (4, 4, 4)
    m.set_block((8, 8, 8), 0.5, 1.0)  # block covering world [0, 4)^3
    found, t = m.first_block_tmin([-2.0, 1.0, 1.0], [1.0, 0.0, 0.0], 0.1, 100.0)
    assert found and abs(t - 2.0) < 1e-6
    found, t = m.first_block_tmin([-2.0, -3.0, 1.0], [1.0, 0.0, 0.0], 0.1, 100.0)
    assert not found


def test_se3_exp_small_and_general(oracle):
    import math
    T = oracle.se3_exp([0, 0, 0, 0, 0, 0])
    assert np.allclose(T, np.eye(4), atol=0)
    tw = np.array([0.1, -0.2, 0.3, 0.05, -0.1, 0.2], np.float64)
    T = oracle.se3_exp(tw.astype(np.float32)).astype(np.float64)
    # closed form (Rodrigues + V) in float64
    w = tw[3:]
    th = np.linalg.norm(w)
    K = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    R = np.eye(3) + math.sin(th) / th * K + (1 - math.cos(th)) / th ** 2 * K @ K
    V = np.eye(3) + (1 - math.cos(th)) / th ** 2 * K + (th - math.sin(th)) / th ** 3 * K @ K
    assert np.allclose(T[:3, :3], R, atol=2e-6)
    assert np.allclose(T[:3, 3], V @ tw[:3], atol=2e-6)


def test_multires_interpolation_known_answers(oracle):
    # octree_visitor_unittest.cpp:114-200 (TEST(VisitorTSDFMultiRes, Interpolation)): a 32^3 octree
    # whose eight blocks of the 16^3 corner hold, at their current scale 1, the value of their
    # index; interpolation at scale 1 across block borders gives the reference's answers, and
    # outside the allocated blocks nothing. Voxel coordinates are the map's (1 m voxels, the
    # world origin at the map centre).
    m = oracle.OracleMap(32.0, 1.0, multires=True)
    for i, c in enumerate(rc.INTERP_BLOCKS):
        tsdf = np.ones(585, np.float32)
        weight = np.zeros(585, np.float32)
        tsdf[512:576] = float(i)
        weight[512:576] = 1.0
        m.set_mr_block(c, tsdf, weight, 1, -1)
    cases = [((2, 2, 2), 0.0), ((8, 2, 2), 0.5), ((2, 8, 2), 1.0), ((8, 8, 2), 1.5), ((2, 2, 8), 2.0),
             ((8, 2, 8), 2.5), ((2, 8, 8), 3.0), ((8, 8, 8), 3.5), ((16, 16, 16), None)]
    for v, want in cases:
        got = m.field_interp(np.array(v, np.float32) - np.float32(16.0))
        if want is None:
            assert got is None, v
        else:
            assert got == want, (v, got, want)
