"""Marching cubes (se::algorithms::marching_cube, single-res) in the oracle: its case table (the
reference's triTable, include/se/map/algorithms/edge_tables.hpp, pinned in
tests/golden/reference_pins.json and identical to the GPU library's), the reference's
meshing test configuration (test/map/meshing/meshing_unittest.cpp: EqualScaleNeighbour, where
the reference only asserts a non-empty mesh; the plane it meshes gives exactly 2 x 15 x 15 faces
at x = 12), and a closed, outward-facing surface around a sphere."""
import json
import os

import numpy as np
import pytest

PINS = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_pins.json")))


def _faces_normals(f):
    n = np.cross(f[:, 1] - f[:, 0], f[:, 2] - f[:, 0])
    return n


def _reference_test_map(oracle):
    # 16^3 voxels (size 16), blocks at x = 8 for y, z in {0, 8}: tsdf 1 for local x < 4, else -1
    m = oracle.OracleMap(0.16, 0.01)
    assert m.size == 16
    t = np.where((np.arange(512) % 8) < 4, 1.0, -1.0).astype(np.float32)
    for y in (0, 8):
        for z in (0, 8):
            m.set_block((8, y, z), t, np.ones(512, np.float32))
    return m


def _sphere_map(oracle, n=32, r=9.3, c=(15.7, 16.2, 16.9)):
    m = oracle.OracleMap(n * 0.01, 0.01)
    idx = np.arange(512)
    lx, ly, lz = idx % 8, (idx // 8) % 8, idx // 64
    for bx in range(0, n, 8):
        for by in range(0, n, 8):
            for bz in range(0, n, 8):
                p = np.stack([bx + lx + 0.5, by + ly + 0.5, bz + lz + 0.5], -1)
                d = np.linalg.norm(p - np.asarray(c), axis=-1) - r
                m.set_block((bx, by, bz), np.clip(d / 3.0, -1, 1).astype(np.float32), np.ones(512, np.float32))
    return m, np.asarray(c)


def test_case_table_is_the_reference_table(oracle):
    ref = np.asarray(PINS["mc_tri_table"])
    ntri, tri = oracle.mc_table()
    assert ntri.max() <= 5
    for cfg in range(256):
        n = int(np.argmax(ref[cfg] < 0)) if (ref[cfg] < 0).any() else 16
        assert ntri[cfg] * 3 == n
        assert np.array_equal(tri[cfg][:n], ref[cfg][:n]) and np.all(tri[cfg][n:] == -1)


def test_case_table_vertices_on_crossed_edges(oracle):
    ntri, tri = oracle.mc_table()
    corner_edges = [(0, 1), (1, 2), (2, 3), (0, 3), (4, 5), (5, 6), (6, 7), (4, 7), (0, 4), (1, 5), (2, 6), (3, 7)]
    for cfg in range(256):
        inside = [(cfg >> c) & 1 for c in range(8)]
        crossed = {e for e, (a, b) in enumerate(corner_edges) if inside[a] != inside[b]}
        assert set(tri[cfg][: 3 * ntri[cfg]].tolist()) == crossed


def test_case_table_equals_gpu_library_table(oracle):
    se = pytest.importorskip("supereight2_gb300")
    ntri_o, tri_o = oracle.mc_table()
    ntri_g, tri_g = se.mc_case_table()
    assert np.array_equal(ntri_o, ntri_g)
    assert np.array_equal(tri_o[:, :15], tri_g)


def test_reference_meshing_configuration(oracle):
    f = _reference_test_map(oracle).marching_cubes()
    assert len(f) == 2 * 15 * 15
    assert np.all(f[:, :, 0] == 12.0)
    n = _faces_normals(f)
    assert np.all(n[:, 0] < 0) and np.allclose(n[:, 1:], 0)   # away from the inside (x >= 12)


def _sim_topology(ntri, tri, f):
    """Faces of the case table on a sampled field, vertices named by their lattice edge."""
    C = [(0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1), (0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1)]
    E = [(0, 1), (1, 2), (2, 3), (0, 3), (4, 5), (5, 6), (6, 7), (4, 7), (0, 4), (1, 5), (2, 6), (3, 7)]
    n = f.shape[0]
    faces = []
    for x in range(n - 1):
        for y in range(n - 1):
            for z in range(n - 1):
                cfg = sum(1 << k for k, (a, b, c) in enumerate(C) if f[x + a, y + b, z + c] < 0)
                for t in range(ntri[cfg]):
                    v = []
                    for j in range(3):
                        a, b = E[tri[cfg][3 * t + j]]
                        pa = (x + C[a][0], y + C[a][1], z + C[a][2])
                        pb = (x + C[b][0], y + C[b][1], z + C[b][2])
                        v.append(min(pa, pb) + max(pa, pb))
                    faces.append(tuple(v))
    return faces


def test_sphere_is_closed_and_outward(oracle):
    m, c = _sphere_map(oracle)
    f = m.marching_cubes()
    assert len(f) > 500
    # closed and consistently oriented: every directed lattice edge of the mesh appears once and
    # its reverse appears once (vertex floats of one lattice edge differ in the last bits between
    # cubes that list its corners in opposite order, as in the reference's edge_to_corners)
    n = 32
    g = np.stack(np.meshgrid(*[np.arange(n) + 0.5] * 3, indexing="ij"), -1)
    field = np.clip((np.linalg.norm(g - c, axis=-1) - 9.3) / 3.0, -1, 1).astype(np.float32)
    ntri, tri = oracle.mc_table()
    topo = _sim_topology(ntri, tri, field)
    assert len(topo) == len(f)
    directed = {}
    for t in topo:
        for j in range(3):
            directed[(t[j], t[(j + 1) % 3])] = directed.get((t[j], t[(j + 1) % 3]), 0) + 1
    assert all(v == 1 for v in directed.values())
    assert all((b, a) in directed for (a, b) in directed)
    nrm = _faces_normals(f)
    area = np.linalg.norm(nrm, axis=-1)
    ok = area > 0  # fans over loops with collinear vertices leave zero-area faces
    assert ok.mean() > 0.95
    cosr = np.sum(nrm[ok] * (f.mean(1)[ok] - c), -1) / (area[ok] * np.linalg.norm(f.mean(1)[ok] - c, axis=-1))
    assert np.all(cosr > 0.9)
    # vertices lie near the sphere (linear interpolation of a clamped distance field)
    assert np.max(np.abs(np.linalg.norm(f.reshape(-1, 3) - c, axis=-1) - 9.3)) < 0.1
