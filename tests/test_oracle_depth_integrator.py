"""The reference's integrateDepth.occupancy unit test (test/integrator/depth_integrator_unittest.cpp)
re-expressed on the oracle: a 640x480 pinhole (PinholeCamera::testInstance,
src/sensor/pinhole_camera.cpp:228-242: f = 315, principal point at the image centre, 0.1-10 m,
T_BS turning its z-forward frame to the body's x-forward, z-up frame) integrates a uniform depth
image of 10 m from a body at (-5, 0, 0) into a 12.8 m occupancy map at 0.1 m, then 9 m from one
metre closer; before and after each integration every octant passes the reference's validity
checks (expect_valid_octree):
  - every octant lies inside the octree;
  - nodes: min and max data agree on valid (weight > 0) and observed; a leaf with valid data is
    observed; a parent's children are half its size, an observed child's min field
    (occupancy x weight) is >= the parent's and an observed child's max field <= the parent's,
    and the parent is observed exactly when all 8 children are (by their min data);
  - blocks: each has a parent node, and at every scale above its current one each voxel's
    min / max pyramids bound those of its 8 children the same way."""
import numpy as np

DIM, RES = 12.8, 0.1
W, H, F = 640, 480, 315.0


def _rot(axis, angle):
    """Eigen::AngleAxisf's rotation matrix in float arithmetic."""
    a = np.asarray(axis, np.float32)
    c, s = np.float32(np.cos(np.float32(angle))), np.float32(np.sin(np.float32(angle)))
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]], np.float32)
    return (c * np.eye(3, dtype=np.float32) + s * K + (np.float32(1) - c) * np.outer(a, a)).astype(np.float32)


def _T_BS():
    T = np.eye(4, dtype=np.float32)
    T[:3, :3] = _rot([0, 1, 0], np.pi / 2) @ _rot([0, 0, 1], np.pi / 2)
    return T


def _field(d):
    return d[..., 0] * d[..., 1]


def _check_octree(m):
    size = m.size
    coords, scales, counts, mean, mn, mx = m.blocks()
    nc, nmin, nmax, leaf = m.nodes()
    assert ((coords >= 0) & (coords < size)).all()
    assert ((nc[:, :3] >= 0) & (nc[:, :3] < size)).all()
    # octants by (coordinate, size): nodes, then blocks (size 8)
    nodes = {tuple(c): i for i, c in enumerate(nc)}
    blocks = {tuple(c) + (8,): i for i, c in enumerate(coords)}
    # blocks: a parent node of twice their size holds each of them
    for c in coords:
        p = tuple((c // 16) * 16) + (16,)
        assert p in nodes, tuple(c)
    # nodes
    for i, c in enumerate(nc):
        dmin, dmax = nmin[i], nmax[i]
        assert (dmin[1] > 0) == (dmax[1] > 0)
        assert dmin[2] == dmax[2]
        half = c[3] // 2
        kids = []
        for k in range(8):
            cc = (c[0] + half * (k & 1), c[1] + half * ((k >> 1) & 1), c[2] + half * (k >> 2), half)
            if cc in nodes:
                j = nodes[cc]
                kids.append((nmin[j], nmax[j]))
            elif half == 8 and cc in blocks:
                j = blocks[cc]
                kids.append((mn[j, 584], mx[j, 584]))   # the block's min / max data (scale 3)
        if leaf[i]:
            assert not kids
            if dmin[1] > 0:
                assert dmin[2] == 1
            if dmax[1] > 0:
                assert dmax[2] == 1
            continue
        assert kids
        observed = 0
        for kmin, kmax in kids:
            if kmin[2]:
                assert _field(kmin) >= _field(dmin)
                observed += 1
            if kmax[2]:
                assert _field(kmax) <= _field(dmax)
        assert dmin[2] == (observed == 8) and dmax[2] == (observed == 8)
    # blocks: the min / max pyramids above the current scale
    offs = [0, 512, 576, 584]
    for b in range(len(coords)):
        cur = scales[b, 0]
        for s in range(3, max(cur, 0), -1):
            n, nc_ = 8 >> s, 8 >> (s - 1)
            for z in range(n):
                for y in range(n):
                    for x in range(n):
                        pmin = mn[b, offs[s] + x + n * y + n * n * z]
                        pmax = mx[b, offs[s] + x + n * y + n * n * z]
                        observed = 0
                        for k in range(8):
                            cx, cy, cz = 2 * x + (k & 1), 2 * y + ((k >> 1) & 1), 2 * z + (k >> 2)
                            ci = offs[s - 1] + cx + nc_ * cy + nc_ * nc_ * cz
                            if mn[b, ci, 2]:
                                assert _field(mn[b, ci]) >= _field(pmin)
                                observed += 1
                            if mx[b, ci, 2]:
                                assert _field(mx[b, ci]) <= _field(pmax)
                        assert pmin[2] == (observed == 8) and pmax[2] == (observed == 8)
    return len(coords), len(nc)


def test_integrate_depth_occupancy_keeps_a_valid_octree(oracle):
    sensor = oracle.pinhole(W, H, F, F, W / 2 - 0.5, H / 2 - 0.5, 0.1, 10.0)
    m = oracle.OracleOccMap(DIM, RES)
    _check_octree(m)
    T_WB = np.eye(4, dtype=np.float32)
    T_WB[0, 3] = -5.0
    depth = np.full((H, W), 10.0, np.float32)
    m.integrate_depth(depth, sensor, (T_WB @ _T_BS()).astype(np.float32), 0)
    nb1, nn1 = _check_octree(m)
    assert nb1 > 0 and nn1 > 1
    depth -= np.float32(1.0)
    T_WB[0, 3] += np.float32(1.0)
    m.integrate_depth(depth, sensor, (T_WB @ _T_BS()).astype(np.float32), 1)
    nb2, nn2 = _check_octree(m)
    assert nb2 > 0 and nn2 > 1
