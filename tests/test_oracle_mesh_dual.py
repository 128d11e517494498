"""Dual marching cubes (se::algorithms::marching_cube for Res::Multi maps) in the oracle.

- The partition of a boundary primal corner's 8 dual corners into blocks, and the rank of each
  neighbouring block, equal what the reference tabulates in meshing::norm_dual_corner_idxs
  (extracted from its source into tests/golden/reference_pins.json) for all 26 positions.
- The reference's meshing test EqualScaleNeighbour2 (test/map/meshing/meshing_unittest.cpp):
  four multi-res TSDF blocks at scale 1, tsdf 1 for local x < 4 else -1; the reference asserts a
  non-empty mesh. The construction gives exactly 2 x 7 x 7 faces on the plane x = 12, at scale 1.
- A map whose blocks all integrate at scale 0 meshes exactly like the single-res marching cubes
  of the same voxels (the dual grid at scale 0 is the voxel-centre grid), bit for bit.
- Mixed scales: every face carries its block's scale, clamp(min_desired_scale, current, 3).
- Occupancy: faces between occupied (occupancy * weight > 0) and free space, away from occupied.
"""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
OFF = [0, 512, 576, 584]


def _pins():
    with open(os.path.join(HERE, "golden", "reference_pins.json")) as f:
        return json.load(f)["dual_corner_partition"]


def _rel(mask):
    # crossmask bits: upper x (32), y (16), z (8), lower x (4), y (2), z (1)
    return [8 if mask & (32 >> a) else (0 if mask & (4 >> a) else 3) for a in range(3)]


def test_dual_partition_matches_reference_table(oracle):
    pins = _pins()
    assert len(pins) == 26
    for mask, ref in pins.items():
        g, above = oracle.dual_groups(_rel(int(mask)))
        groups = {}
        for i, k in enumerate(g):
            groups.setdefault(int(k), set()).add(i)
        assert groups[0] == set(ref["groups"][0]), mask
        assert {frozenset(v) for k, v in groups.items() if k} == {frozenset(v) for v in ref["groups"][1:]}, mask
        rank = {i: int(above[k]) for i, k in enumerate(g) if k}
        assert all(rank[i] == 0 for i in ref["lower"]) and all(rank[i] == 1 for i in ref["higher"]), mask
        assert len(ref["lower"]) + len(ref["higher"]) == len(groups) - 1, mask


def _pyramid(bc, fn):
    """585-entry (tsdf, weight) of the block at bc from fn(voxel centres [N, 3], scale)."""
    t = np.ones(585, np.float32)
    w = np.zeros(585, np.float32)
    for s in range(4):
        n, st = 8 >> s, 1 << s
        i = np.arange(n ** 3)
        lx, ly, lz = i % n, (i // n) % n, i // (n * n)
        p = np.stack([bc[0] + st * lx, bc[1] + st * ly, bc[2] + st * lz], -1) + 0.5 * st
        v, ww = fn(p, s)
        t[OFF[s]:OFF[s] + n ** 3] = v
        w[OFF[s]:OFF[s] + n ** 3] = ww
    return t, w


def reference_scale1_map(oracle):
    m = oracle.OracleMap(0.16, 0.01, multires=True)
    for y in (0, 8):
        for z in (0, 8):
            def fn(p, s):
                if s != 1:
                    return np.ones(len(p)), np.zeros(len(p))
                return np.where(p[:, 0] - 8 < 4, 1.0, -1.0), np.ones(len(p))
            t, w = _pyramid((8, y, z), fn)
            m.set_mr_block((8, y, z), t, w, 1, 1)
    return m


def sphere_maps(oracle, scale_of=lambda b: 0, n=64, c=(31.3, 32.6, 30.9), r=17.2):
    c = np.asarray(c)
    mr = oracle.OracleMap(n * 0.01, 0.01, multires=True)
    sr = oracle.OracleMap(n * 0.01, 0.01)
    for bx in range(0, n, 8):
        for by in range(0, n, 8):
            for bz in range(0, n, 8):
                t, w = _pyramid((bx, by, bz), lambda p, s: (np.clip((np.linalg.norm(p - c, axis=-1) - r) / 3.0, -1, 1),
                                                            np.ones(len(p))))
                s = scale_of((bx, by, bz))
                mr.set_mr_block((bx, by, bz), t, w, s, s)
                sr.set_block((bx, by, bz), t[:512], w[:512])
    return mr, sr


def mixed_scale(b):
    return (b[0] // 8 + b[1] // 8 + b[2] // 8) % 3


def occupancy_plane_map(oracle, mixed=False):
    m = oracle.OracleOccMap(0.32, 0.01)
    for bx in range(0, 32, 8):
        for by in range(0, 32, 8):
            for bz in range(0, 32, 8):
                s = mixed_scale((bx, by, bz)) if mixed else 0
                mean = np.zeros((585, 3), np.float32)
                for sc in range(4):
                    k, st = 8 >> sc, 1 << sc
                    i = np.arange(k ** 3)
                    x = bx + st * (i % k) + 0.5 * st
                    y = by + st * ((i // k) % k) + 0.5 * st
                    occ = np.where(x + 0.3 * y > 17.0, 2.0, -3.0)
                    mean[OFF[sc]:OFF[sc] + k ** 3, 0] = occ
                    mean[OFF[sc]:OFF[sc] + k ** 3, 1] = 4.0
                    mean[OFF[sc]:OFF[sc] + k ** 3, 2] = 1.0
                m.set_block((bx, by, bz), s, s, mean)
    return m


def _sorted(f):
    f = np.asarray(f, np.float32).reshape(-1, 9)
    return f[np.lexsort(f.T[::-1])]


def test_reference_equal_scale_neighbour2(oracle):
    f, sc = reference_scale1_map(oracle).dual_marching_cubes(0)
    assert len(f) == 2 * 7 * 7
    assert np.all(f[:, :, 0] == 12.0) and np.all(sc == 1)
    n = np.cross(f[:, 1] - f[:, 0], f[:, 2] - f[:, 0])
    assert np.all(n[:, 0] < 0)                      # away from the inside (x > 12)


def test_scale0_equals_single_res(oracle):
    mr, sr = sphere_maps(oracle)
    fd, sc = mr.dual_marching_cubes(0)
    fs = sr.marching_cubes()
    assert len(fd) == len(fs) > 1000 and np.all(sc == 0)
    assert np.array_equal(_sorted(fd).view(np.uint32), _sorted(fs).view(np.uint32))


def test_mixed_scales_and_min_desired(oracle):
    mr, _ = sphere_maps(oracle, mixed_scale)
    f0, s0 = mr.dual_marching_cubes(0)
    assert set(np.unique(s0)) == {0, 1, 2}
    # the surface stays on the sphere within a voxel of the coarsest scale used
    d = np.linalg.norm(f0.reshape(-1, 3) - np.array([31.3, 32.6, 30.9]), axis=-1) - 17.2
    assert np.max(np.abs(d)) < 4.0
    f2, s2 = mr.dual_marching_cubes(2)
    assert len(f2) < len(f0) and np.all(s2 >= 2)
    f3, s3 = mr.dual_marching_cubes(3)
    assert np.all(s3 == 3)


def test_occupancy_plane(oracle):
    f, sc = occupancy_plane_map(oracle).dual_marching_cubes(0)
    assert len(f) > 100 and np.all(sc == 0)
    v = f.reshape(-1, 3)
    assert np.max(np.abs(v[:, 0] + 0.3 * v[:, 1] - 17.0)) < 1.0
    n = np.cross(f[:, 1] - f[:, 0], f[:, 2] - f[:, 0])
    area = np.linalg.norm(n, axis=-1) > 1e-6
    assert np.all(n[area, 0] < 0)                   # away from occupied space (larger x)
    fm, sm = occupancy_plane_map(oracle, mixed=True).dual_marching_cubes(0)
    assert len(fm) > 0 and set(np.unique(sm)) <= {0, 1, 2}


def test_integrated_maps(oracle):
    """Multi-res TSDF and occupancy maps integrated from the dolly sequence mesh at the scales
    their blocks integrate at."""
    from supereight2_gb300 import synthetic as syn
    sensor, _, poses, frames = syn.dataset("mr160", 6)
    spec = dict(width=sensor.width, height=sensor.height, fx=sensor.fx, fy=sensor.fy, cx=sensor.cx,
                cy=sensor.cy, near_plane=sensor.near_plane, far_plane=sensor.far_plane)
    s = oracle.pinhole(**spec)
    mr = oracle.OracleMap(10.24, 0.02, multires=True)
    occ = oracle.OracleOccMap(10.24, 0.02)
    for i, (T, d) in enumerate(zip(poses, frames)):
        mr.integrate_depth(d, s, T.astype(np.float32), i)
        occ.integrate_depth(d, s, T.astype(np.float32), i)
    f, sc = mr.dual_marching_cubes(0)
    assert len(f) > 10000 and np.all(sc >= 0) and np.all(sc <= 3)
    fo, so = occ.dual_marching_cubes(0)
    assert len(fo) > 10000 and np.all(so >= 0) and np.all(so <= 3)
    with pytest.raises(ValueError):
        oracle.OracleMap(1.28, 0.02).dual_marching_cubes(0)
