"""Marching cubes on the GPU: the face set equals the oracle's bit for bit (faces sorted), on the
reference's meshing test configuration, a sphere, and a map integrated from the synthetic room;
the capacity contract (count returned, partial write) holds."""
import numpy as np
import pytest

from tests.test_oracle_mesh import _reference_test_map, _sphere_map

pytestmark = pytest.mark.gpu


def _gpu_copy(gpu, om, dim, res):
    keys, coords, tsdf, weight, _ = om.blocks()
    gm = gpu.Map(dim, res, max_blocks=max(1024, 2 * len(keys)))
    gm.upload_blocks(keys, tsdf, weight)
    return gm


def _sorted(f):
    f = np.asarray(f, np.float32).reshape(-1, 9)
    return f[np.lexsort(f.T[::-1])]


def _compare(gpu, om, gm):
    fo = om.marching_cubes()
    fg = gpu.marching_cube(gm).cpu().numpy()
    assert len(fo) == len(fg) > 0
    assert np.array_equal(_sorted(fo).view(np.uint32), _sorted(fg).view(np.uint32))
    return fo


def test_reference_configuration(oracle, gpu):
    om = _reference_test_map(oracle)
    f = _compare(gpu, om, _gpu_copy(gpu, om, 0.16, 0.01))
    assert len(f) == 450


def test_sphere(oracle, gpu):
    om, _ = _sphere_map(oracle)
    _compare(gpu, om, _gpu_copy(gpu, om, 0.32, 0.01))


def test_integrated_room(oracle, gpu):
    import torch
    from supereight2_gb300 import synthetic as syn
    spec, scene, poses, frames = syn.dataset("tsdf320", 4)
    args = dict(width=spec.width, height=spec.height, fx=spec.fx, fy=spec.fy, cx=spec.cx, cy=spec.cy,
                near_plane=spec.near_plane, far_plane=spec.far_plane)
    om = oracle.OracleMap(10.24, 0.02)
    gm = gpu.Map(10.24, 0.02, max_blocks=1 << 16)
    integ = gpu.MapIntegrator(gm)
    for i, (T, d) in enumerate(zip(poses, frames)):
        om.integrate_depth(d, oracle.pinhole(**args), T.astype(np.float32), i)
        integ.integrateDepth(i, torch.from_numpy(d).cuda(), gpu.PinholeCamera(**args), T.astype(np.float32))
    f = _compare(gpu, om, gm)
    assert len(f) > 10000
    # capacity contract: a short buffer gets a prefix, the count is the total
    L = gpu.library()
    import ctypes as C
    buf = torch.empty((100, 3, 3), dtype=torch.float32, device="cuda")
    n = C.c_int64()
    assert L.se_gpu_marching_cube(gm.h, C.c_void_p(buf.data_ptr()), 100, C.byref(n), None) == 0
    assert n.value == len(f)
