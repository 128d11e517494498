"""Small runs of the oracle's paths, for the sanitizer build (tests/test_oracle_sanitized.py runs
this script with SE_ORACLE_LIB pointing at an AddressSanitizer / UndefinedBehaviorSanitizer build
of the oracle): TSDF integration, raycast and tracking (single- and multi-res), the bilateral
filter, marching cubes, occupancy integration from a pinhole camera and a LiDAR,
the occupancy raycast and dual marching cubes, ray batches, downsampling and the tracker's
pyramid."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import pyoracle as o  # noqa: E402

o.set_num_threads(2)
W, H = 80, 60
s = o.pinhole(W, H, 65.0, 65.0, W / 2 - 0.5, H / 2 - 0.5, 0.1, 6.0)
v, u = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
depth = (2.0 + 0.3 * np.sin(u / 9.0) + 0.2 * np.cos(v / 7.0)).astype(np.float32)
depth[::7, ::5] = 0.0
T0 = np.eye(4, dtype=np.float32)
T1 = T0.copy()
T1[0, 3] = 0.01

for multires in (False, True):
    m = o.OracleMap(6.4, 0.02, multires=multires)
    m.integrate_depth(depth, s, T0, 0)
    m.integrate_depth(depth, s, T1, 1)
    pts, nrm, _ = m.raycast(s, T1)
    f = o.bilateral_filter(depth, radius=2, sigma_space=4.0, sigma_range=0.03)
    o.track(s, o.tracker_config(), f, T1, pts, nrm)
    m.field_interp(np.array([0.0, 0.0, 2.0], np.float32))
    m.field_grad(np.array([0.0, 0.0, 2.0], np.float32))
    if multires:
        m.dual_marching_cubes()
        m.mr_blocks()
    else:
        m.marching_cubes()
        m.blocks()

om = o.OracleOccMap(6.4, 0.05)
om.integrate_depth(depth, s, T0, 0)
om.integrate_depth(depth, s, T1, 1)
om.raycast(s, T1)
om.dual_marching_cubes()
om.blocks()
om.nodes()

lid = o.lidar(64, 16, -15.0, 15.0, 0.5, 20.0)
rng = np.full((16, 64), 5.0, np.float32)
rng[::3, ::4] = 0.0
ol = o.OracleOccMap(25.6, 0.4)
ol.integrate_lidar(rng, lid, T0, 0)
ol.integrate_lidar(rng, lid, T1, 1)
ol.blocks()

# a ray batch (LeicaLidar): a fan of rays onto a wall, then a second batch from another pose
L = o.leica(360, 180, 0.2, 30.0, 1.0, 1.0)
az = np.radians(np.linspace(-10.0, 10.0, 21, dtype=np.float32))
rays = np.stack([6.0 * np.cos(az), 6.0 * np.sin(az), np.zeros_like(az)], 1).astype(np.float32)
ob = o.OracleOccMap(25.6, 0.1)
ob.integrate_ray_batch(L, np.eye(4, dtype=np.float32), rays, 0)
ob.integrate_ray_batch(L, T1, rays, 1)
ob.blocks()
ob.nodes()

o.downsample_depth(depth, 2)
o.tracker_pyramid(s, depth, 3)
print("workload ok")
