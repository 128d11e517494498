"""The oracle's spinning-LiDAR path (the reference's OusterLidar with the occupancy map).

The reference leaves the Ouster projection to the un-vendored srl_projection module, so the
model here is project-defined (equiangular columns, rows linear in elevation) and its parity
with the reference is unpinned; what the reference itself fixes is checked against its own
formulas: the integration scale from the chord between neighbouring rays
(src/sensor/ouster_lidar.cpp:107-146), the wrap-around pooling image
(dense_pooling_image_impl.hpp:395-598), and the occupancy update with range measurements.
"""
import math

import numpy as np
import pytest

from supereight2_gb300 import synthetic as syn


def _lidar(oracle, spec=syn.LIDAR_64):
    return oracle.lidar(spec.width, spec.height, spec.elevation_min_deg, spec.elevation_max_deg,
                        spec.near_plane, spec.far_plane)


def test_atan2_accuracy(oracle):
    rng = np.random.default_rng(3)
    pts = rng.standard_normal((4000, 2)).astype(np.float32)
    pts[:8] = [[0, 1], [0, -1], [1, 0], [-1, 0], [1, 1], [-1, -1], [1e-30, -1], [-1, 1e-30]]
    err = [abs(float(oracle.atan2(y, x)) - math.atan2(float(y), float(x))) for x, y in pts]
    assert max(err) < 1.2e-5
    assert oracle.atan2(0.0, 0.0) == 0.0


def test_projection_round_trips_pixel_centres(oracle):
    spec = syn.LIDAR_64
    L = _lidar(oracle)
    dirs = syn.lidar_directions(spec)
    for v in (0, 1, 31, 32, 62, 63):
        for u in (0, 1, 255, 511, 512, 1022, 1023):
            ok, uv = oracle.lidar_project(L, (dirs[v, u] * 7.5).astype(np.float32))
            assert ok
            du = (uv[0] - u + spec.width / 2) % spec.width - spec.width / 2
            assert abs(du) < 0.02 and abs(uv[1] - v) < 0.01
    # above the top beam by more than half a row: not projected
    el = math.radians(22.5 + 0.5 * 45 / 63 + 0.05)
    ok, _ = oracle.lidar_project(L, np.array([math.cos(el), 0, math.sin(el)], np.float32))
    assert not ok


def test_integration_scale_from_ray_chord(oracle):
    L = _lidar(oracle)
    tan_half = float(oracle.lib().so_lidar_tan_half_min_angle(oracle.C.byref(L)))
    # min_ray_angle = min(45 / 63, 360 / 1024) degrees
    assert tan_half == pytest.approx(math.tan(math.radians(min(45 / 63, 360 / 1024)) / 2), rel=1e-6)
    res = 0.4
    for dist in np.linspace(1.0, 800.0, 60):
        pv = 2 * dist * tan_half / (math.sqrt(3) * res)
        want = sum(pv >= r for r in (1.5, 3.0, 6.0))
        got = oracle.lidar_integration_scale(L, np.array([dist, 0, 0], np.float32), res, 0, -1)
        if min(abs(pv - r) for r in (1.5, 3.0, 6.0)) > 1e-3:
            assert got == want


def test_pooling_image_wraps_columns(oracle):
    h, w = 16, 64
    depth = np.full((h, w), 5.0, np.float32)
    depth[7, 0] = 2.0                   # seen by column w - 1's window through the wrap
    depth[3, 40] = 0.0                  # a hole
    lid, mv = oracle.pooling_image_lidar(depth)
    pin, _ = oracle.pooling_image(depth)
    assert lid[1, 7, w - 1, 0] == 2.0 and pin[1, 7, w - 1, 0] == 5.0
    # level 1: columns at the border are not crossing in the LiDAR image
    assert lid[1, 7, 0, 2] == 0.0 and pin[1, 7, 0, 2] == 1.0
    assert lid[1, 3, 40, 3] == 1.0      # partly known window
    assert mv == pytest.approx(5.0)
    # windows of every level hold the min / max of the wrapped neighbourhood
    for level in range(2, lid.shape[0]):
        half = 1 << (level - 1)
        x, y = 1, 7
        cols = [(x + dx) % w for dx in range(-half, half + 1)]
        rows = [min(max(y + dy, 0), h - 1) for dy in range(-half, half + 1)]
        win = depth[np.ix_(rows, cols)]
        assert lid[level, y, x, 0] == win[win > 0].min()


def test_lidar_scan_carves_free_space_and_occupies_hits(oracle):
    spec = syn.LIDAR_64
    scene = syn.make_outdoor_scene(1004)
    T = syn.road_trajectory(0, 1)[0].astype(np.float32)
    rng_img = syn.render_range(scene, spec, T, 5, keep=1.0, noise=False)
    T_MW = np.eye(4, dtype=np.float32)
    T_MW[:3, 3] = (51.2, 51.2, 12.8)
    m = oracle.OracleOccMap(102.4, 0.4, T_MW=T_MW)
    st = m.integrate_lidar(rng_img, _lidar(oracle), T, 0)
    assert st.n_blocks_listed > 100
    dirs = syn.lidar_directions(spec)
    R, o = T[:3, :3].astype(np.float64), T[:3, 3].astype(np.float64)
    rs = np.random.default_rng(0)
    free = occ = n = 0
    for _ in range(300):
        v, u = rs.integers(28, 64), rs.integers(0, spec.width)
        r = float(rng_img[v, u])
        if r < 3.0 or r > 40.0:
            continue
        d = R @ dirs[v, u]
        n += 1
        free += m.get_data((o + d * 0.5 * r).astype(np.float32))[0] < 0
        occ += m.get_data((o + d * (r + 0.1)).astype(np.float32))[0] > 0
    assert n > 50
    assert free / n > 0.85
    assert occ / n > 0.6
