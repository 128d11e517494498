"""The oracle's multi-resolution occupancy map pinned to the reference's own system test
(test/system/multires_ofusion/multires_ofusion_systemtest.cpp with its config.yaml): the
field configuration of that YAML, the 640x480 sensor (fx 481.2, fy -480) downsampled by 2, an
identity pose and a synthetic wall.

Pins (values the reference's test asserts with EXPECT_EQ / EXPECT_FLOAT_EQ):
  GetField (2 m / 4 m split wall): voxels (688,500,933) and (256,166,338) unknown (occupancy 0),
  voxels (578,500,737) and (477,500,618) free (-5.015).
  GetFieldInterpolation (4 m wall): interpolation at (639,511,799), (600,520,811) and
  (575,511,615) is -5.015 (node neighbours of different size, all inside a node, node and
  block neighbours).
DeleteChildren (the first frame a 2 m / 4 m / 2 m wall, then the 4 m wall) has no assertion in
the reference and runs 15 frames; free-space nodes reach the pruning threshold (max data
observed with occupancy * weight <= -95, i.e. weight 19 of at most 20) at frame 18, so the run
here is 20 frames long and must prune and keep the pyramid invariants.
"""
import numpy as np
import pytest

CFG = dict(log_odd_min=-5.015, log_odd_max=5.015, fs_integr_scale=1, tau_min_factor=3,
           tau_max_factor=12, k_tau=0.05, sigma_min_factor=1, sigma_max_factor=3, k_sigma=0.05)


def _sensor(oracle):
    # se::PinholeCamera(config.sensor, 2): w, h / 2; f / 2; c' = (c + 0.5) / 2 - 0.5
    return oracle.pinhole(width=320, height=240, fx=481.2 / 2, fy=-480.0 / 2,
                          cx=(319.5 + 0.5) / 2 - 0.5, cy=(239.5 + 0.5) / 2 - 0.5,
                          near_plane=0.4, far_plane=6.0)


def _voxel_point(c):
    # Map::voxelToPoint: T_WM * ((c + 0.5) * res), T_MW = translation(dim / 2)
    return ((np.asarray(c, np.float32) + np.float32(0.5)) * np.float32(0.01) - np.float32(5.12)).astype(np.float32)


def _float_eq(a, b, ulps=4):
    a32, b32 = np.float32(a), np.float32(b)
    ia, ib = np.array(a32).view(np.int32), np.array(b32).view(np.int32)
    return abs(int(ia) - int(ib)) <= ulps


def test_get_field_pins(oracle):
    m = oracle.OracleOccMap(10.24, 0.01, **CFG)
    x = np.arange(320)[None, :]
    depth = (np.where(x < 160, 2.0, 4.0) * np.ones((240, 1))).astype(np.float32)
    m.integrate_depth(depth, _sensor(oracle), np.eye(4, dtype=np.float32), 0)
    for c in [(688, 500, 933), (256, 166, 338)]:
        assert m.get_data(_voxel_point(c))[0] == 0.0
    for c in [(578, 500, 737), (477, 500, 618)]:
        assert _float_eq(m.get_data(_voxel_point(c))[0], -5.015)


def test_get_field_interpolation_pins(oracle):
    m = oracle.OracleOccMap(10.24, 0.01, **CFG)
    m.integrate_depth(np.full((240, 320), 4.0, np.float32), _sensor(oracle), np.eye(4, dtype=np.float32), 0)
    for c in [(639, 511, 799), (600, 520, 811), (575, 511, 615)]:
        r = m.get_field_interp(_voxel_point(c))
        assert r is not None and _float_eq(r[0], -5.015)


def test_delete_children_run_prunes_and_keeps_invariants(oracle):
    m = oracle.OracleOccMap(10.24, 0.01, **CFG)
    x = np.arange(320)[None, :]
    noisy = (np.where((x < 120) | (x > 200), 2.0, 4.0) * np.ones((240, 1))).astype(np.float32)
    wall = np.full((240, 320), 4.0, np.float32)
    pruned = 0
    for f in range(20):
        st = m.integrate_depth(noisy if f == 0 else wall, _sensor(oracle), np.eye(4, dtype=np.float32), f)
        pruned += st.n_nodes_pruned
    assert pruned > 0
    coords, scales, counts, mean, mn, mx = m.blocks()
    cur, mins = scales[:, 0], scales[:, 1]
    assert ((mins == -1) | (mins <= cur)).all()
    w = mean[..., 1]
    assert np.array_equal(w, np.round(w)) and (w >= 0).all() and (w <= 20).all()
    # the min and max pyramids bracket the mean wherever both are valid
    offs = [0, 512, 576, 584]
    for b in range(len(coords)):
        for s in range(max(cur[b], 0) + 1, 4):
            sl = slice(offs[s], offs[s] + (8 >> s) ** 3)
            ok = (mean[b, sl, 1] > 0) & (mn[b, sl, 1] > 0) & (mx[b, sl, 1] > 0)
            f_mean = mean[b, sl, 0] * mean[b, sl, 1]
            assert (mn[b, sl, 0][ok] * mn[b, sl, 1][ok] <= mx[b, sl, 0][ok] * mx[b, sl, 1][ok]).all()
            assert np.isfinite(f_mean).all()
    nc, nmin, nmax, leaf = m.nodes()
    assert (nmin[:, 1] >= 0).all() and leaf.sum() > 0


def test_raycast_finds_the_wall(oracle):
    m = oracle.OracleOccMap(10.24, 0.01, **CFG)
    wall = np.full((240, 320), 4.0, np.float32)
    for f in range(3):
        m.integrate_depth(wall, _sensor(oracle), np.eye(4, dtype=np.float32), f)
    pts, nrm, sc = m.raycast(_sensor(oracle), np.eye(4, dtype=np.float32))
    hit = (pts != 0).any(-1)
    assert hit.mean() > 0.9
    # the occupancy zero crossing lies within the surface thickness in front of the wall
    assert np.median(np.abs(pts[hit][:, 2] - 4.0)) < 0.05
    n_ok = (nrm != 0).any(-1) & hit
    assert n_ok.mean() > 0.5
    assert np.median(nrm[n_ok][:, 2]) < -0.9   # normals face the camera (-z)


def test_map_gradient_reference_cases(oracle):
    """map_unittest.cpp:11-113 (TEST(Map, Gradient)): a 32 m occupancy map at 3 cm, a 640x480
    pinhole downsampled by 2 (fx 262.5, near 0.4 m, far 20 m) at the identity pose integrates a
    uniform 15 m depth image with the test's field parameters. In free space (z = 4, 6, 8 m) the
    interpolated occupancy is log_odd_min and the gradient zero; in the linear part of the inverse
    sensor model (z = 14.85 ... 15 m) the gradient matches central differences of the
    interpolation (step res / 10) within 1e-2; behind the surface (z = 15.35 m) the occupancy is
    positive and the gradient zero."""
    def float_eq(a, b):
        # googletest's EXPECT_FLOAT_EQ: within 4 units in the last place
        ia, ib = (int(np.array(x, np.float32).view(np.int32)) for x in (a, b))
        ia, ib = (x if x >= 0 else -(x & 0x7fffffff) for x in (ia, ib))
        return abs(ia - ib) <= 4

    cfg = dict(tau_min_factor=20.0, tau_max_factor=20.0, k_tau=1.0, sigma_min_factor=1.0,
               sigma_max_factor=3.0, k_sigma=0.05)
    res = 0.03
    m = oracle.OracleOccMap(32.0, res, **cfg)
    s = oracle.pinhole(320, 240, 262.5, 262.5, (319.5 + 0.5) / 2 - 0.5, (239.5 + 0.5) / 2 - 0.5, 0.4, 20.0)
    m.integrate_depth(np.full((240, 320), 15.0, np.float32), s, np.eye(4, dtype=np.float32), 0)
    for z in (4.0, 6.0, 8.0):
        p = np.array([0.0, 0.0, z], np.float32)
        v = m.get_field_interp(p)
        assert v is not None and float_eq(v[0], -5.015), v
        g = m.get_field_grad(p)
        assert g is not None and float_eq(np.linalg.norm(g), 0.0), g
    delta = np.float32(res / 10)
    for z in (14.85, 14.90, 14.95, 15.00):
        p = np.array([0.0, 0.0, z], np.float32)
        num = np.zeros(3, np.float32)
        for i in range(3):
            d = np.zeros(3, np.float32)
            d[i] = delta
            vm, vp = m.get_field_interp(p - d), m.get_field_interp(p + d)
            assert vm is not None and vp is not None
            if abs(vp[0] - vm[0]) > 1e-6:
                num[i] = (vp[0] - vm[0]) / (2 * delta)
        g = m.get_field_grad(p)
        assert g is not None
        assert np.all(np.abs(num - g) <= 1e-2), (z, num, g)
    p = np.array([0.0, 0.0, 15.35], np.float32)
    v = m.get_field_interp(p)
    assert v is not None and v[0] > 0.0
    g = m.get_field_grad(p)
    assert g is not None and float_eq(np.linalg.norm(g), 0.0), g


def test_block_allocation_keeps_the_octree_path(oracle):
    """octree_allocator_unittest.cpp:40-233 (SingleResAllocation.BlockKey) for 8^3 blocks, on the
    occupancy map's pointer octree: allocating the block of a voxel gives the block at the
    voxel's coordinates rounded down to 8, and its ancestors are the nodes at the voxel's
    coordinates rounded down to 2^s at every scale s up to the root (a 256^3 octree)."""
    m = oracle.OracleOccMap(25.6, 0.1)
    assert m.size == 256
    voxels = [(253, 74, 135), (114, 244, 65), (38, 104, 85)]
    mean = np.zeros((585, 3), np.float32)
    for v in voxels:
        m.set_block(tuple(((np.array(v) >> 3) << 3).tolist()), 0, 0, mean)
    coords = {tuple(c) for c in m.blocks()[0].tolist()}
    nodes = {tuple(c) for c in m.nodes()[0].tolist()}
    for v in voxels:
        v = np.array(v)
        assert tuple(((v >> 3) << 3).tolist()) in coords
        for s in range(4, 9):
            assert tuple(((v >> s) << s).tolist()) + (1 << s,) in nodes, (v, s)
