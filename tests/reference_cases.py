"""Inputs and expected values of the reference's map tests, shared by the oracle pins and the
GPU tests. Each constant cites the supereight2 test it re-expresses."""
import math

import numpy as np

# test/map/map/map_unittest.cpp:210-236 (Map.initialization): (dim, res, octree size)
MAP_SIZES = [(12.8, 0.1, 128), (25.6, 0.1, 256), (51.2, 0.1, 512), (10.24, 0.01, 1024),
             (20.48, 0.01, 2048), (10.24, 0.02, 512), (20.48, 0.02, 1024), (10.0, 0.05, 256),
             (100.0, 0.05, 2048)]

# test/map/map/map_unittest.cpp:127-208 (Map.Interpolation): a 32^3 map at 1 m with the 8
# blocks of the 16^3 corner set to tsdf = block index, weight 1, and the expected
# getFieldInterp values at world points (None = nullopt).
INTERP_DIM = 32.0
INTERP_RES = 1.0
INTERP_BLOCKS = [(0, 0, 0), (8, 0, 0), (0, 8, 0), (8, 8, 0), (0, 0, 8), (8, 0, 8), (0, 8, 8),
                 (8, 8, 8)]
INTERP_CASES = [((-12, -12, -12), 0.0), ((-8, -12, -12), 0.5), ((-12, -8, -12), 1.0),
                ((-8, -8, -12), 1.5), ((-12, -12, -8), 2.0), ((-8, -12, -8), 2.5),
                ((-12, -8, -8), 3.0), ((-8, -8, -8), 3.5), ((2, 2, 2), None)]


def _angle_axis_f32(axis, angle):
    """Eigen::AngleAxisf(angle, axis).toRotationMatrix() evaluated in float32."""
    a = np.float32(angle)
    c, s = np.float32(math.cos(a)), np.float32(math.sin(a))
    x, y, z = (np.float32(v) for v in axis)
    t = np.float32(1) - c
    return np.array([[t * x * x + c, t * x * y - s * z, t * x * z + s * y],
                     [t * x * y + s * z, t * y * y + c, t * y * z - s * x],
                     [t * x * z - s * y, t * y * z + s * x, t * z * z + c]], np.float32)


def wall_sensor():
    """test/map/map/map_aabb_unittest.cpp:12-20: 100x100, f = 100, near 0.1, far 10, and
    T_BS = AngleAxis(pi/2, Y) * AngleAxis(-pi/2, Z) (z-forward camera to x-forward body)."""
    R = (_angle_axis_f32((0, 1, 0), math.pi / 2) @ _angle_axis_f32((0, 0, 1), -math.pi / 2)).astype(np.float32)
    T = np.eye(4, dtype=np.float32)
    T[:3, :3] = R
    return dict(width=100, height=100, fx=100.0, fy=100.0, cx=49.5, cy=49.5, near_plane=0.1,
                far_plane=10.0), T


WALL_DEPTH = 4.0
WALL_MAP_DIM = 12.8
WALL_MAP_RES = 0.1


def dim_to_blocks(dim, block_dim):
    """map_aabb_unittest.cpp:32-35, in float32 like the reference."""
    f = np.float32
    v = f(abs(f(dim))) / f(block_dim) + f(0.5)
    return int(math.copysign(float(v), float(dim)))


def world_aabb(vmin, vmax, res, t_MW):
    """Map::aabb() (include/se/map/impl/map_impl.hpp:635-664) for a translation-only T_MW."""
    lo = np.asarray(vmin, np.float32)
    hi = (np.asarray(vmax, np.int64) + 1).astype(np.float32)
    hi = np.nextafter(hi, lo).astype(np.float32)
    t = -np.asarray(t_MW, np.float32)
    return lo * np.float32(res) + t, hi * np.float32(res) + t


def check_wall_aabb(vmin, vmax, truncation_boundary_factor=8.0):
    """The assertions of TEST(Map, aabbTSDF), map_aabb_unittest.cpp:37-60."""
    res = WALL_MAP_RES
    lo, hi = world_aabb(vmin, vmax, res, [WALL_MAP_DIM / 2] * 3)
    f = np.float32
    trunc = f(res) * f(truncation_boundary_factor)
    block_dim = f(res) * f(8)
    hfov = f(2.0) * f(math.atan(f(100) / (f(2.0) * f(100.0))))
    half_wall_dim = f(WALL_DEPTH) * f(math.tan(hfov / f(2)))
    half_wall_blocks = dim_to_blocks(half_wall_dim, block_dim)
    assert np.isclose(lo[0], WALL_DEPTH - trunc, rtol=0, atol=4e-6), lo
    assert np.isclose(hi[0], WALL_DEPTH + trunc, rtol=0, atol=4e-6), hi
    assert np.isclose(lo[2], lo[1], rtol=0, atol=4e-6)
    assert np.isclose(hi[2], hi[1], rtol=0, atol=4e-6)
    assert dim_to_blocks(float(lo[1]), block_dim) == -half_wall_blocks
    assert dim_to_blocks(float(hi[1]), block_dim) == half_wall_blocks


def check_wall_aabb_occupancy(vmin, vmax):
    """The assertions of TEST(Map, aabbOccupancy), map_aabb_unittest.cpp:62-86: from the sensor
    (x = 0) to three blocks behind the wall, and one block more than the wall's half width on
    either side in y and z."""
    res = WALL_MAP_RES
    lo, hi = world_aabb(vmin, vmax, res, [WALL_MAP_DIM / 2] * 3)
    f = np.float32
    block_dim = f(res) * f(8)
    hfov = f(2.0) * f(math.atan(f(100) / (f(2.0) * f(100.0))))
    half_wall_dim = f(WALL_DEPTH) * f(math.tan(hfov / f(2)))
    half_wall_blocks = dim_to_blocks(half_wall_dim, block_dim)
    assert abs(float(lo[0])) <= 1e-6, lo
    assert np.isclose(hi[0], f(WALL_DEPTH) + f(3) * block_dim, rtol=0, atol=4e-6), hi
    assert np.isclose(lo[2], lo[1], rtol=0, atol=4e-6)
    assert np.isclose(hi[2], hi[1], rtol=0, atol=4e-6)
    assert dim_to_blocks(float(lo[1]), block_dim) == -half_wall_blocks - 1
    assert dim_to_blocks(float(hi[1]), block_dim) == half_wall_blocks + 1
