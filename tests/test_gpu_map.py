"""The reference's map tests and the error paths, run on the GPU through the C ABI."""
import numpy as np
import pytest

from tests import reference_cases as rc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim,res,size", rc.MAP_SIZES)
def test_octree_size(gpu, dim, res, size):
    # map_unittest.cpp:210-236
    m = gpu.Map(dim, res, max_blocks=64)
    assert m.size == size
    assert m.dim >= np.float32(dim) * (1 - 1e-6)


def _key(x, y, z, scale=3):
    from oracle import pyoracle
    import ctypes
    k = ctypes.c_uint64()
    pyoracle.lib().so_encode_key(x & ~7, y & ~7, z & ~7, scale, ctypes.byref(k))
    return k.value


def test_interpolation_known_answers(gpu):
    # map_unittest.cpp:127-208 through Map::getFieldInterp
    import torch
    m = gpu.Map(rc.INTERP_DIM, rc.INTERP_RES, max_blocks=64)
    keys = np.array([_key(*c) for c in rc.INTERP_BLOCKS], np.uint64)
    tsdf = np.repeat(np.arange(8, dtype=np.float32)[:, None], 512, 1)
    m.upload_blocks(keys, tsdf, np.ones((8, 512), np.float32))
    pts = torch.tensor([p for p, _ in rc.INTERP_CASES], dtype=torch.float32, device="cuda")
    vals, valid = m.getFieldInterp(pts)
    vals, valid = vals.cpu().numpy(), valid.cpu().numpy()
    for i, (_, want) in enumerate(rc.INTERP_CASES):
        if want is None:
            assert not valid[i]
        else:
            assert valid[i] and vals[i] == want


def test_wall_aabb(gpu):
    # map_aabb_unittest.cpp:37-60 (TEST(Map, aabbTSDF))
    import torch
    spec, T_WC = rc.wall_sensor()
    m = gpu.Map(rc.WALL_MAP_DIM, rc.WALL_MAP_RES, max_blocks=4096)
    depth = torch.full((spec["height"], spec["width"]), rc.WALL_DEPTH, dtype=torch.float32,
                       device="cuda")
    gpu.MapIntegrator(m).integrateDepth(0, depth, gpu.PinholeCamera(**spec), T_WC)
    m.check()
    mn, mx = m.aabb()
    rc.check_wall_aabb(mn, mx)


def test_empty_invalid_and_nan_depth(gpu):
    import torch
    m = gpu.Map(10.24, 0.02, max_blocks=1024)
    s = gpu.PinholeCamera(64, 48, 50.0, 50.0, 31.5, 23.5, 0.4, 6.0)
    integ = gpu.MapIntegrator(m)
    for v in (0.0, 0.1, 50.0, float("nan")):
        integ.integrateDepth(0, torch.full((48, 64), v, device="cuda"), s, np.eye(4))
        st = m.integrate_stats()
        assert st["n_new_blocks"] == 0 and st["n_updated_voxels"] == 0
    m.check()
    assert m.num_blocks() == 0 and m.aabb() is None


def test_camera_outside_map_is_safe(gpu):
    import torch
    m = gpu.Map(2.56, 0.02, max_blocks=4096)  # 128^3 voxels, world [-1.28, 1.28)
    s = gpu.PinholeCamera(64, 48, 50.0, 50.0, 31.5, 23.5, 0.4, 6.0)
    T = np.eye(4, dtype=np.float32)
    T[:3, 3] = (0.0, 0.0, -3.0)  # 3 m behind the map, looking at it along +z
    gpu.MapIntegrator(m).integrateDepth(0, torch.full((48, 64), 3.0, device="cuda"), s, T)
    m.check()
    keys, coords, tsdf, w, _ = m.download_blocks()
    assert len(keys) > 0 and (coords >= 0).all() and (coords < 128).all()
    pts = torch.zeros((48, 64, 3), device="cuda")
    nrm = torch.zeros_like(pts)
    gpu.raycast_volume(m, s, T, pts, nrm)
    torch.cuda.synchronize()
    hit = (pts != 0).any(-1)
    # the wall at z = 0 is inside the map for |x| < 1.28 of +-1.92 and |y| < 1.28 of +-1.44
    assert hit.float().mean() > 0.5
    z = pts[..., 2][hit]
    # an oblique ray crosses the along-ray TSDF of a 2 cm grid within a quarter voxel
    assert torch.allclose(z, torch.zeros_like(z), atol=5e-3)


def test_pool_full_is_reported(gpu):
    import torch
    m = gpu.Map(10.24, 0.02, max_blocks=8)
    s = gpu.PinholeCamera(64, 48, 50.0, 50.0, 31.5, 23.5, 0.4, 6.0)
    gpu.MapIntegrator(m).integrateDepth(0, torch.full((48, 64), 2.0, device="cuda"), s, np.eye(4))
    with pytest.raises(gpu.SeGpuError, match="pool"):
        m.check()
    assert m.num_blocks() == 8
    m.check()  # the latched error was cleared


def test_downloaded_keys_are_morton_block_keys(gpu):
    import torch
    m = gpu.Map(10.24, 0.02, max_blocks=1 << 14)
    s = gpu.PinholeCamera(64, 48, 50.0, 50.0, 31.5, 23.5, 0.4, 6.0)
    gpu.MapIntegrator(m).integrateDepth(3, torch.full((48, 64), 2.0, device="cuda"), s, np.eye(4))
    keys, coords, _, _, ts = m.download_blocks(voxels=False)
    assert len(keys) > 0 and (ts == 3).all()
    for k, c in zip(keys[:200], coords[:200]):
        assert int(k) == _key(*[int(v) for v in c])


def test_bad_arguments_raise(gpu):
    import torch
    with pytest.raises(gpu.SeGpuError):
        gpu.Map(10.24, -1.0)
    m = gpu.Map(10.24, 0.02, max_blocks=64)
    s = gpu.PinholeCamera(64, 48, 50.0, 50.0, 31.5, 23.5, 0.4, 6.0)
    with pytest.raises(gpu.SeGpuError):
        gpu.MapIntegrator(m).integrateDepth(0, torch.zeros((10, 10), device="cuda"), s, np.eye(4))
    with pytest.raises(gpu.SeGpuError):
        gpu.MapIntegrator(m).integrateDepth(0, torch.zeros((48, 64)), s, np.eye(4))
