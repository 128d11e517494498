"""Dual marching cubes on the GPU (se_gpu_dual_marching_cube) against the oracle, bit for bit:
the oracle meshes a copy of the GPU map's blocks (coordinates, scales, data pyramid), so the two
meshes must hold the same faces (sorted) with the same scales. Maps: multi-res TSDF (FP32 and
FP16 storage) and occupancy maps integrated from the dolly sequence (blocks at scales 0-2), at
min_desired_scale 0 and 2; plus the capacity contract and Map::saveMesh of a multi-res map."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _spec(sensor):
    return dict(width=sensor.width, height=sensor.height, fx=sensor.fx, fy=sensor.fy, cx=sensor.cx,
                cy=sensor.cy, near_plane=sensor.near_plane, far_plane=sensor.far_plane)


def _integrate(gpu, gm, n_frames=8):
    import torch
    from supereight2_gb300 import synthetic as syn
    sensor, _, poses, frames = syn.dataset("mr160", n_frames)
    gs = gpu.PinholeCamera(**_spec(sensor))
    integ = gpu.MapIntegrator(gm)
    for i, (T, d) in enumerate(zip(poses, frames)):
        integ.integrateDepth(i, torch.from_numpy(d).cuda(), gs, T.astype(np.float32))
    return gm


def _sorted(f, s):
    f = np.asarray(f, np.float32).reshape(-1, 9)
    order = np.lexsort(np.concatenate([f, s.reshape(-1, 1).astype(np.float32)], 1).T[::-1])
    return f[order], s[order]


def _compare(gpu, gm, om, min_scale):
    fg, sg = gpu.dual_marching_cube(gm, min_scale)
    fo, so = om.dual_marching_cubes(min_scale)
    fg, sg = _sorted(fg.cpu().numpy(), sg.cpu().numpy())
    fo, so = _sorted(fo, so)
    assert len(fg) == len(fo) > 1000
    assert np.array_equal(fg.view(np.uint32), fo.view(np.uint32))
    assert np.array_equal(sg, so) and np.all(sg >= min_scale)
    return fg, sg


def _tsdf_copy(oracle, gm):
    keys, coords, tsdf, weight, _, _, scales = gm.download_multires()
    om = oracle.OracleMap(10.24, 0.02, multires=True)
    for c, t, w, s in zip(coords, tsdf, weight, scales):
        om.set_mr_block(c, t, w, int(s[0]), int(s[1]))
    return om


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_multires_tsdf(oracle, gpu, storage):
    gm = _integrate(gpu, gpu.Map(10.24, 0.02, max_blocks=1 << 16, res_type="multi", storage=storage))
    om = _tsdf_copy(oracle, gm)
    _, s0 = _compare(gpu, gm, om, 0)
    assert len(np.unique(s0)) >= 2
    _compare(gpu, gm, om, 2)
    # marching_cube on a multi-res map is the dual mesh at min_desired_scale 0
    f = gpu.marching_cube(gm).cpu().numpy()
    assert len(f) == len(s0)


def test_occupancy(oracle, gpu):
    gm = _integrate(gpu, gpu.Map(10.24, 0.02, res_type="multi", field="occupancy", max_blocks=1 << 17))
    coords, scales, _, mean, _, _ = gm.download_occupancy()
    om = oracle.OracleOccMap(10.24, 0.02)
    for c, s, m in zip(coords, scales, mean):
        om.set_block(c, int(s[0]), int(s[1]), m)
    assert len(om.blocks()[0]) == len(coords)
    _, s0 = _compare(gpu, gm, om, 0)
    assert len(np.unique(s0)) >= 2
    _compare(gpu, gm, om, 2)


def test_capacity_and_errors(gpu, tmp_path):
    import ctypes as C
    import torch
    gm = _integrate(gpu, gpu.Map(10.24, 0.02, max_blocks=1 << 16, res_type="multi"), 3)
    f, s = gpu.dual_marching_cube(gm, 0)
    L = gpu.library()
    buf = torch.empty((50, 3, 3), dtype=torch.float32, device="cuda")
    sb = torch.empty(50, dtype=torch.int8, device="cuda")
    n = C.c_int64()
    assert L.se_gpu_dual_marching_cube(gm.h, 0, C.c_void_p(buf.data_ptr()), C.c_void_p(sb.data_ptr()), 50,
                                       C.byref(n), None) == 0
    assert n.value == len(f) > 50
    assert L.se_gpu_dual_marching_cube(gm.h, 4, None, None, 0, C.byref(n), None) != 0
    single = gpu.Map(1.28, 0.02, max_blocks=1 << 10)
    assert L.se_gpu_dual_marching_cube(single.h, 0, None, None, 0, C.byref(n), None) != 0
    gm.saveMesh(tmp_path / "mr.vtk", min_desired_scale=1)
    txt = (tmp_path / "mr.vtk").read_text().splitlines()
    i = txt.index("SCALARS scale unsigned_char")
    npoly = int([l for l in txt if l.startswith("POLYGONS")][0].split()[1])
    vals = np.array([int(v) for v in txt[i + 2:i + 2 + npoly]])
    assert npoly > 0 and vals.min() >= 1
