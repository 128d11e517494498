"""ctypes binding of the CPU oracle (test infrastructure only).

Only the tests, the smoke check and the benchmark's CPU-baseline leg import this module. It
wraps ``libse_oracle.so`` (built by ``oracle/build.py``), the CPU restatement of the
supereight2 hot path that the GPU product is checked against.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


class Pinhole(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("fx", C.c_float), ("fy", C.c_float),
                ("cx", C.c_float), ("cy", C.c_float), ("near_plane", C.c_float),
                ("far_plane", C.c_float)]


class Lidar(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("elevation_min_deg", C.c_float),
                ("elevation_max_deg", C.c_float), ("near_plane", C.c_float), ("far_plane", C.c_float)]


class Leica(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("near_plane", C.c_float), ("far_plane", C.c_float),
                ("elevation_resolution_deg", C.c_float), ("azimuth_resolution_deg", C.c_float)]


class TrackerConfig(C.Structure):
    _fields_ = [("num_levels", C.c_int), ("iterations", C.c_int * 3),
                ("dist_threshold", C.c_float), ("normal_threshold", C.c_float),
                ("track_threshold", C.c_float), ("icp_threshold", C.c_float)]


class IntegrateStats(C.Structure):
    _fields_ = [("n_valid_pixels", C.c_longlong), ("n_new_blocks", C.c_longlong),
                ("n_frustum_blocks", C.c_longlong), ("n_updated_voxels", C.c_longlong)]


class TrackStats(C.Structure):
    _fields_ = [("converged_iterations", C.c_int * 3), ("accepted", C.c_int),
                ("reduction", C.c_float * 32)]


def lib():
    global _lib
    if _lib is None:
        # SE_ORACLE_LIB: another build of the same sources (the sanitizer test's)
        path = os.environ.get("SE_ORACLE_LIB") or _build.build()
        L = C.CDLL(path)
        f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
        u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
        i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        i8p = np.ctypeslib.ndpointer(np.int8, flags="C_CONTIGUOUS")
        f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        vp = C.c_void_p
        sig = {
            "so_set_num_threads": (None, [C.c_int]),
            "so_get_num_threads": (C.c_int, []),
            "so_map_create": (vp, [f32p, C.c_float, C.c_float, C.c_float, vp]),
            "so_map_create_multires": (vp, [f32p, C.c_float, C.c_float, C.c_float, vp]),
            "so_map_is_multires": (C.c_int, [vp]),
            "so_map_mr_blocks": (None, [vp, vp, vp, vp, vp, vp, vp, vp]),
            "so_map_destroy": (None, [vp]),
            "so_occ_map_create": (vp, [f32p, C.c_float, vp]),
            "so_occ_map_destroy": (None, [vp]),
            "so_occ_map_create_cfg": (vp, [f32p, C.c_float, vp, vp]),
            "so_occ_get_data": (None, [vp, f32p, f32p]),
            "so_occ_get_field_interp": (C.c_int, [vp, f32p, C.POINTER(C.c_float), C.POINTER(C.c_int)]),
            "so_occ_get_field_grad": (C.c_int, [vp, f32p, f32p]),
            "so_occ_map_size": (C.c_int, [vp]),
            "so_occ_integrate_depth": (None, [vp, f32p, C.POINTER(Pinhole), f32p, C.c_int,
                                              C.POINTER(OccStats)]),
            "so_occ_num_blocks": (C.c_longlong, [vp]),
            "so_occ_num_nodes": (C.c_longlong, [vp]),
            "so_occ_blocks": (None, [vp, vp, vp, vp, vp, vp, vp]),
            "so_occ_nodes": (C.c_longlong, [vp, vp, vp, vp, vp]),
            "so_occ_aabb": (C.c_int, [vp, i32p, i32p]),
            "so_occ_raycast_volume": (None, [vp, C.POINTER(Pinhole), f32p, f32p, f32p, i8p]),
            "so_occ_depth_sigma": (None, [f32p, C.c_int, C.c_float, f32p]),
            "so_occ_pooling_image": (C.c_int, [f32p, C.c_int, C.c_int, vp, C.POINTER(C.c_float)]),
            "so_occ_pooling_image_lidar": (C.c_int, [f32p, C.c_int, C.c_int, vp, C.POINTER(C.c_float)]),
            "so_occ_integrate_lidar": (None, [vp, f32p, C.POINTER(Lidar), f32p, C.c_int, vp]),
            "so_lidar_project": (C.c_int, [C.POINTER(Lidar), f32p, f32p]),
            "so_occ_integrate_ray_batch": (C.c_longlong, [vp, C.POINTER(Leica), f32p, f32p, C.c_longlong, C.c_int,
                                                          vp, C.c_longlong]),
            "so_leica_integration_scale": (C.c_int, [C.POINTER(Leica), f32p, C.c_float, C.c_int, C.c_int]),
            "so_occ_block_timestamps": (None, [vp, vp]),
            "so_atan2": (C.c_float, [C.c_float, C.c_float]),
            "so_lidar_tan_half_min_angle": (C.c_float, [C.POINTER(Lidar)]),
            "so_occ_lidar_integration_scale": (C.c_int, [C.POINTER(Lidar), f32p, C.c_float, C.c_int, C.c_int]),
            "so_render_depth_f64": (None, [vp, C.POINTER(Pinhole), f64p, f64p]),
            "so_raycast_adjoint_f64": (None, [vp, C.POINTER(Pinhole), f64p, vp, f64p, vp, vp]),
            "so_map_set_voxel": (None, [vp, i32p, C.c_float, C.c_float]),
            "so_map_size": (C.c_int, [vp]),
            "so_map_dim": (C.c_float, [vp]),
            "so_integrate_depth": (None, [vp, f32p, C.POINTER(Pinhole), f32p, C.c_int,
                                          C.POINTER(IntegrateStats)]),
            "so_raycast_volume": (None, [vp, C.POINTER(Pinhole), f32p, f32p, f32p, i8p]),
            "so_track": (C.c_int, [C.POINTER(Pinhole), C.POINTER(TrackerConfig), f32p, f32p,
                                   f32p, f32p, C.POINTER(TrackStats)]),
            "so_map_num_blocks": (C.c_longlong, [vp]),
            "so_map_blocks": (None, [vp, vp, vp, vp, vp, vp]),
            "so_map_aabb": (C.c_int, [vp, i32p, i32p]),
            "so_map_set_block": (None, [vp, i32p, f32p, f32p]),
            "so_map_get_data": (C.c_int, [vp, f32p, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
            "so_map_get_field_interp": (C.c_int, [vp, f32p, C.POINTER(C.c_float)]),
            "so_map_get_field_grad": (C.c_int, [vp, f32p, f32p]),
            "so_first_block_tmin": (C.c_int, [vp, f32p, f32p, C.c_float, C.c_float,
                                              C.POINTER(C.c_float)]),
            "so_expand": (C.c_uint64, [C.c_uint64]),
            "so_compact": (C.c_uint64, [C.c_uint64]),
            "so_encode_code": (C.c_uint64, [C.c_int32, C.c_int32, C.c_int32]),
            "so_decode_code": (None, [C.c_uint64, i32p]),
            "so_encode_key": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_uint64,
                                        C.POINTER(C.c_uint64)]),
            "so_decode_key": (None, [C.c_uint64, i32p, C.POINTER(C.c_uint64)]),
            "so_code_to_child_idx": (C.c_uint64, [C.c_uint64, C.c_uint64]),
            "so_parent_key": (C.c_uint64, [C.c_uint64]),
            "so_key_at_scale": (C.c_int, [C.c_uint64, C.c_uint64, C.POINTER(C.c_uint64)]),
            "so_code_at_scale": (C.c_int, [C.c_uint64, C.c_uint64, C.POINTER(C.c_uint64)]),
            "so_block_key": (C.c_uint64, [C.c_uint64, C.c_uint64]),
            "so_block_code": (C.c_uint64, [C.c_uint64, C.c_uint64]),
            "so_is_child": (C.c_int, [C.c_uint64, C.c_uint64]),
            "so_is_siblings": (C.c_int, [C.c_uint64, C.c_uint64]),
            "so_unique_keys": (C.c_longlong, [u64p, C.c_longlong, u64p]),
            "so_unique_codes": (C.c_longlong, [u64p, C.c_longlong, u64p]),
            "so_unique_allocation": (C.c_longlong, [u64p, C.c_longlong, C.c_uint64, u64p]),
            "so_unique_at_scale": (C.c_longlong, [u64p, C.c_longlong, C.c_uint64, u64p]),
            "so_se3_exp": (None, [f32p, f32p]),
            "so_half_sample_robust": (None, [f32p, C.c_int, C.c_int, C.c_float, C.c_int, f32p]),
            "so_depth_to_point_cloud": (None, [f32p, C.POINTER(Pinhole), f32p]),
            "so_bilateral_weights": (None, [C.c_int, C.c_float, f32p]),
            "so_bilateral_filter": (None, [f32p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, f32p]),
            "so_exp_cw": (C.c_float, [C.c_float]),
            "so_marching_cubes": (C.c_longlong, [vp, vp, C.c_longlong]),
            "so_mc_table": (None, [i32p, i32p]),
            "so_dual_marching_cubes": (C.c_longlong, [vp, C.c_int, vp, vp, C.c_longlong]),
            "so_occ_dual_marching_cubes": (C.c_longlong, [vp, C.c_int, vp, vp, C.c_longlong]),
            "so_dual_groups": (None, [i32p, i32p, i32p, i32p]),
            "so_raycast_touched": (C.c_longlong, [vp, C.POINTER(Pinhole), f32p]),
            "so_map_set_mr_block": (None, [vp, i32p, f32p, f32p, C.c_int, C.c_int]),
            "so_occ_set_block": (None, [vp, i32p, C.c_int, C.c_int, f32p]),
            "so_downsample_depth": (None, [f32p, C.c_int, C.c_int, f32p, C.c_int, C.c_int, vp]),
            "so_point_cloud_to_normal": (None, [f32p, C.c_int, C.c_int, C.c_int, f32p]),
            "so_tracker_pyramid": (None, [C.POINTER(Pinhole), f32p, C.c_int, f32p, f32p, f32p]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def set_num_threads(n: int) -> None:
    lib().so_set_num_threads(int(n))


def num_threads() -> int:
    return lib().so_get_num_threads()


def pinhole(width, height, fx, fy, cx, cy, near_plane, far_plane) -> Pinhole:
    return Pinhole(int(width), int(height), float(fx), float(fy), float(cx), float(cy),
                   float(near_plane), float(far_plane))


def _m16(T):
    return np.ascontiguousarray(np.asarray(T, dtype=np.float32).reshape(16))


class OccStats(C.Structure):
    _fields_ = [("n_blocks_listed", C.c_longlong), ("n_nodes_listed", C.c_longlong),
                ("n_blocks_freed", C.c_longlong), ("n_nodes_pruned", C.c_longlong)]


class OracleOccMap:
    """se::OccupancyMap<Res::Multi> restated on the CPU (pinhole integration)."""

    # the field configuration of a YAML "data" node, in so_occ_map_create_cfg's order
    CFG_KEYS = ("k_sigma", "sigma_min_factor", "sigma_max_factor", "k_tau", "tau_min_factor",
                "tau_max_factor", "log_odd_min", "log_odd_max", "fs_integr_scale")

    def __init__(self, dim, res, T_MW=None, **cfg):
        d = np.ascontiguousarray(np.broadcast_to(np.asarray(dim, np.float32), (3,)))
        self._tmw = None if T_MW is None else _m16(T_MW)
        tmw = None if self._tmw is None else self._tmw.ctypes.data
        if cfg:
            defaults = dict(k_sigma=0.052, sigma_min_factor=1.5, sigma_max_factor=6.0, k_tau=0.026,
                            tau_min_factor=6.0, tau_max_factor=16.0, log_odd_min=-5.015,
                            log_odd_max=5.015, fs_integr_scale=1)
            defaults.update(cfg)
            self._cfg = np.array([defaults[k] for k in self.CFG_KEYS], np.float32)
            self.h = lib().so_occ_map_create_cfg(d, float(res), tmw, self._cfg.ctypes.data)
        else:
            self.h = lib().so_occ_map_create(d, float(res), tmw)
        self.res = float(res)

    def raycast(self, sensor, T_WS):
        n = sensor.width * sensor.height
        pts = np.zeros((sensor.height, sensor.width, 3), np.float32)
        nrm = np.zeros((sensor.height, sensor.width, 3), np.float32)
        scale = np.zeros((sensor.height, sensor.width), np.int8)
        lib().so_occ_raycast_volume(self.h, C.byref(sensor), _m16(T_WS), pts.reshape(n * 3),
                                    nrm.reshape(n * 3), scale.reshape(n))
        return pts, nrm, scale

    def get_data(self, p):
        out = np.zeros(3, np.float32)
        lib().so_occ_get_data(self.h, np.ascontiguousarray(p, np.float32), out)
        return out

    def get_field_interp(self, p):
        v, sc = C.c_float(), C.c_int()
        ok = lib().so_occ_get_field_interp(self.h, np.ascontiguousarray(p, np.float32), C.byref(v), C.byref(sc))
        return (v.value, sc.value) if ok else None

    def get_field_grad(self, p):
        """Map::getFieldGrad(point): f32[3] or None."""
        g = np.zeros(3, np.float32)
        ok = lib().so_occ_get_field_grad(self.h, np.ascontiguousarray(p, np.float32), g)
        return g if ok else None

    def __del__(self):
        if getattr(self, "h", None):
            lib().so_occ_map_destroy(self.h)
            self.h = None

    @property
    def size(self):
        return lib().so_occ_map_size(self.h)

    def integrate_depth(self, depth, sensor, T_WC, timestamp=0):
        st = OccStats()
        depth = np.ascontiguousarray(depth, dtype=np.float32)
        lib().so_occ_integrate_depth(self.h, depth, C.byref(sensor), _m16(T_WC), int(timestamp), C.byref(st))
        return st

    def integrate_lidar(self, rng, sensor, T_WS, timestamp=0):
        rng = np.ascontiguousarray(rng, np.float32).reshape(-1)
        st = OccStats()
        lib().so_occ_integrate_lidar(self.h, rng, C.byref(sensor), _m16(T_WS), int(timestamp), C.byref(st))
        return st

    def blocks(self):
        """(coords i32[N,3], scales i32[N,3] (current, min, buffer), counts i64[N,4],
        mean / min / max f32[N,585,3] (occupancy, weight, observed))."""
        n = int(lib().so_occ_num_blocks(self.h))
        coords = np.zeros((n, 3), np.int32)
        scales = np.zeros((n, 3), np.int32)
        counts = np.zeros((n, 4), np.int64)
        arrs = [np.zeros((n, 585, 3), np.float32) for _ in range(3)]
        if n:
            lib().so_occ_blocks(self.h, coords.ctypes.data, scales.ctypes.data, counts.ctypes.data,
                                *[a.ctypes.data for a in arrs])
        return (coords, scales, counts, *arrs)

    def nodes(self):
        """(coords+size i32[N,4], min f32[N,3], max f32[N,3], leaf i32[N]) depth first."""
        n = int(lib().so_occ_nodes(self.h, None, None, None, None))
        c = np.zeros((n, 4), np.int32)
        mn = np.zeros((n, 3), np.float32)
        mx = np.zeros((n, 3), np.float32)
        lf = np.zeros(n, np.int32)
        lib().so_occ_nodes(self.h, c.ctypes.data, mn.ctypes.data, mx.ctypes.data, lf.ctypes.data)
        return c, mn, mx, lf

    def aabb(self):
        mn = np.zeros(3, np.int32)
        mx = np.zeros(3, np.int32)
        return (mn, mx) if lib().so_occ_aabb(self.h, mn, mx) else None

    def set_block(self, coord, current_scale, min_scale, mean):
        """Test set-up: the block at voxel coord with its scales and mean pyramid f32[585, 3]."""
        lib().so_occ_set_block(self.h, np.asarray(coord, np.int32), int(current_scale), int(min_scale),
                               np.ascontiguousarray(mean, np.float32).reshape(-1))

    def dual_marching_cubes(self, min_desired_scale=0):
        """(faces [N, 3, 3] float32 in voxel units, scales [N] int8) between occupied and free."""
        return _dual_mc(lib().so_occ_dual_marching_cubes, self.h, min_desired_scale)

    def integrate_ray_batch(self, sensor, poses, rays, timestamp=0):
        """MapIntegrator::integrateRayBatch: rays f32[N,3] (sensor frame) with poses f32[N,4,4]
        (T_WS); returns the updated octants i32[K,4] (x, y, z, size), sorted."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 3)
        poses = np.ascontiguousarray(np.broadcast_to(np.asarray(poses, np.float32), (len(rays), 4, 4)))
        cap = 1 << 20
        out = np.zeros((cap, 4), np.int32)
        k = int(lib().so_occ_integrate_ray_batch(self.h, C.byref(sensor), poses.reshape(-1), rays.reshape(-1),
                                                 len(rays), int(timestamp), out.ctypes.data, cap))
        if k > cap:
            raise RuntimeError("more updated octants than the buffer holds: %d" % k)
        return out[:k]

    def block_timestamps(self):
        n = int(lib().so_occ_num_blocks(self.h))
        ts = np.zeros(n, np.int32)
        if n:
            lib().so_occ_block_timestamps(self.h, ts.ctypes.data)
        return ts


def occ_depth_sigma(depth, res):
    depth = np.ascontiguousarray(depth, np.float32)
    out = np.zeros_like(depth)
    lib().so_occ_depth_sigma(depth.reshape(-1), depth.size, float(res), out.reshape(-1))
    return out


def lidar(width, height, elevation_min_deg, elevation_max_deg, near_plane, far_plane) -> Lidar:
    return Lidar(int(width), int(height), float(elevation_min_deg), float(elevation_max_deg),
                 float(near_plane), float(far_plane))


def lidar_project(sensor, p_S):
    uv = np.zeros(2, np.float32)
    ok = lib().so_lidar_project(C.byref(sensor), np.ascontiguousarray(p_S, np.float32), uv)
    return bool(ok), uv


def atan2(y, x):
    return np.float32(lib().so_atan2(float(y), float(x)))


def lidar_integration_scale(sensor, c_S, res, last_scale, min_scale):
    return int(lib().so_occ_lidar_integration_scale(C.byref(sensor), np.ascontiguousarray(c_S, np.float32),
                                                    float(res), int(last_scale), int(min_scale)))


def leica(width, height, near_plane, far_plane, elevation_resolution_deg=1.0, azimuth_resolution_deg=1.0) -> Leica:
    return Leica(int(width), int(height), float(near_plane), float(far_plane), float(elevation_resolution_deg),
                 float(azimuth_resolution_deg))


def leica_integration_scale(sensor, c_S, res, last_scale, min_scale):
    return int(lib().so_leica_integration_scale(C.byref(sensor), np.ascontiguousarray(c_S, np.float32),
                                                float(res), int(last_scale), int(min_scale)))


def pooling_image_lidar(depth):
    depth = np.ascontiguousarray(depth, np.float32)
    h, w = depth.shape
    mv = C.c_float()
    L = lib().so_occ_pooling_image_lidar(depth.reshape(-1), w, h, None, C.byref(mv))
    out = np.zeros((L + 1, h, w, 4), np.float32)
    lib().so_occ_pooling_image_lidar(depth.reshape(-1), w, h, out.ctypes.data, C.byref(mv))
    return out, float(mv.value)


def pooling_image(depth):
    """(levels f32[L+1, h, w, 4] of (min, max, crossing, known), max_value)."""
    depth = np.ascontiguousarray(depth, np.float32)
    h, w = depth.shape
    mv = C.c_float()
    L = lib().so_occ_pooling_image(depth.reshape(-1), w, h, None, C.byref(mv))
    out = np.zeros((L + 1, h, w, 4), np.float32)
    lib().so_occ_pooling_image(depth.reshape(-1), w, h, out.ctypes.data, C.byref(mv))
    return out, mv.value


class OracleMap:
    """se::TSDFMap<Res::Single> (or, with multires=True, se::TSDFMap<Res::Multi>) restated on
    the CPU."""

    def __init__(self, dim, res, truncation_boundary_factor=8.0, max_weight=100.0, T_MW=None,
                 multires=False):
        d = np.ascontiguousarray(np.broadcast_to(np.asarray(dim, np.float32), (3,)))
        self._tmw = None if T_MW is None else _m16(T_MW)
        create = lib().so_map_create_multires if multires else lib().so_map_create
        self.h = create(d, float(res), float(truncation_boundary_factor), float(max_weight),
                        None if self._tmw is None else self._tmw.ctypes.data)
        self.res = float(res)
        self.multires = bool(multires)

    def __del__(self):
        if getattr(self, "h", None):
            lib().so_map_destroy(self.h)
            self.h = None

    @property
    def size(self) -> int:
        return lib().so_map_size(self.h)

    @property
    def dim(self) -> float:
        return lib().so_map_dim(self.h)

    def integrate_depth(self, depth, sensor: Pinhole, T_WC, timestamp=0) -> IntegrateStats:
        st = IntegrateStats()
        depth = np.ascontiguousarray(depth, dtype=np.float32)
        lib().so_integrate_depth(self.h, depth, C.byref(sensor), _m16(T_WC), int(timestamp),
                                 C.byref(st))
        return st

    def raycast(self, sensor: Pinhole, T_WS):
        n = sensor.width * sensor.height
        pts = np.zeros((sensor.height, sensor.width, 3), np.float32)
        nrm = np.zeros((sensor.height, sensor.width, 3), np.float32)
        scale = np.zeros((sensor.height, sensor.width), np.int8)
        lib().so_raycast_volume(self.h, C.byref(sensor), _m16(T_WS), pts.reshape(n * 3),
                                nrm.reshape(n * 3), scale.reshape(n))
        return pts, nrm, scale

    def raycast_touched(self, sensor: Pinhole, T_WS) -> int:
        """Distinct voxels the raycast at T_WS reads (single-res maps)."""
        return int(lib().so_raycast_touched(self.h, C.byref(sensor), _m16(T_WS)))

    def num_blocks(self) -> int:
        return int(lib().so_map_num_blocks(self.h))

    def blocks(self):
        """Return (keys u64[N], coords i32[N,3], tsdf f32[N,512], weight f32[N,512], ts i32[N])."""
        n = self.num_blocks()
        keys = np.zeros(n, np.uint64)
        coords = np.zeros((n, 3), np.int32)
        tsdf = np.zeros((n, 512), np.float32)
        weight = np.zeros((n, 512), np.float32)
        ts = np.zeros(n, np.int32)
        if n:
            lib().so_map_blocks(self.h, keys.ctypes.data, coords.ctypes.data, tsdf.ctypes.data,
                                weight.ctypes.data, ts.ctypes.data)
        return keys, coords, tsdf, weight, ts

    def render_depth_f64(self, sensor: Pinhole, T_WS):
        """Differentiable depth render in FP64: z of the trilinear root per pixel, 0 if none."""
        d = np.zeros((sensor.height, sensor.width), np.float64)
        T = np.ascontiguousarray(np.asarray(T_WS, np.float64).reshape(16))
        lib().so_render_depth_f64(self.h, C.byref(sensor), T, d.reshape(-1))
        return d

    def adjoint_f64(self, sensor: Pinhole, T_WS, grad_depth=None, voxel_grad=False, jac=False):
        """(twist_grad[6], voxel_grad[N, 512] or None, jac[H, W, 6] or None) in FP64."""
        T = np.ascontiguousarray(np.asarray(T_WS, np.float64).reshape(16))
        g = None if grad_depth is None else np.ascontiguousarray(grad_depth, np.float64)
        tw = np.zeros(6, np.float64)
        vg = np.zeros((self.num_blocks(), 512), np.float64) if voxel_grad else None
        jc = np.zeros((sensor.height, sensor.width, 6), np.float64) if jac else None
        lib().so_raycast_adjoint_f64(self.h, C.byref(sensor), T, None if g is None else g.ctypes.data,
                                     tw, None if vg is None else vg.ctypes.data,
                                     None if jc is None else jc.ctypes.data)
        return tw, vg, jc

    def set_voxel(self, voxel_coord, tsdf, weight):
        lib().so_map_set_voxel(self.h, np.ascontiguousarray(voxel_coord, np.int32), float(tsdf),
                               float(weight))

    def mr_blocks(self):
        """Multi-res blocks: (keys u64[N], coords i32[N,3], tsdf f32[N,585], weight f32[N,585],
        past_tsdf f32[N,585], past_weight f32[N,585], scales i32[N,2] = (current, min))."""
        n = self.num_blocks()
        keys = np.zeros(n, np.uint64)
        coords = np.zeros((n, 3), np.int32)
        arrs = [np.zeros((n, 585), np.float32) for _ in range(4)]
        scales = np.zeros((n, 2), np.int32)
        if n:
            lib().so_map_mr_blocks(self.h, keys.ctypes.data, coords.ctypes.data,
                                   *[a.ctypes.data for a in arrs], scales.ctypes.data)
        return (keys, coords, *arrs, scales)

    def marching_cubes(self):
        """Faces [N, 3, 3] (float32, voxel units of the map frame)."""
        n = int(lib().so_marching_cubes(self.h, None, 0))
        f = np.zeros((n, 3, 3), np.float32)
        if n:
            lib().so_marching_cubes(self.h, f.ctypes.data, n)
        return f

    def set_mr_block(self, coord, tsdf, weight, current_scale, min_scale):
        """Test set-up of a multi-res block: data pyramid f32[585] x 2 and its scales."""
        lib().so_map_set_mr_block(self.h, np.asarray(coord, np.int32), np.ascontiguousarray(tsdf, np.float32),
                                  np.ascontiguousarray(weight, np.float32), int(current_scale), int(min_scale))

    def dual_marching_cubes(self, min_desired_scale=0):
        """Multi-res maps: (faces [N, 3, 3] float32 in voxel units, scales [N] int8)."""
        return _dual_mc(lib().so_dual_marching_cubes, self.h, min_desired_scale)

    def aabb(self):
        mn = np.zeros(3, np.int32)
        mx = np.zeros(3, np.int32)
        ok = lib().so_map_aabb(self.h, mn, mx)
        return (mn, mx) if ok else None

    def set_block(self, voxel_coord, tsdf512, weight512):
        lib().so_map_set_block(self.h, np.asarray(voxel_coord, np.int32),
                               np.ascontiguousarray(np.broadcast_to(np.float32(tsdf512), (512,))),
                               np.ascontiguousarray(np.broadcast_to(np.float32(weight512), (512,))))

    def get_data(self, p_W):
        t, w = C.c_float(), C.c_float()
        lib().so_map_get_data(self.h, np.asarray(p_W, np.float32), C.byref(t), C.byref(w))
        return t.value, w.value

    def field_interp(self, p_W):
        v = C.c_float()
        ok = lib().so_map_get_field_interp(self.h, np.asarray(p_W, np.float32), C.byref(v))
        return v.value if ok else None

    def field_grad(self, p_W):
        g = np.zeros(3, np.float32)
        ok = lib().so_map_get_field_grad(self.h, np.asarray(p_W, np.float32), g)
        return g if ok else None

    def first_block_tmin(self, origin, direction, t_near, t_far):
        t = C.c_float()
        found = lib().so_first_block_tmin(self.h, np.asarray(origin, np.float32),
                                          np.asarray(direction, np.float32), float(t_near),
                                          float(t_far), C.byref(t))
        return bool(found), t.value


def bilateral_filter(depth, radius=2, sigma_space=4.0, sigma_range=0.03):
    depth = np.ascontiguousarray(depth, np.float32)
    h, w = depth.shape
    out = np.zeros_like(depth)
    lib().so_bilateral_filter(depth.reshape(-1), w, h, int(radius), float(sigma_space), float(sigma_range),
                              out.reshape(-1))
    return out


def _dual_mc(fn, h, min_desired_scale):
    n = int(fn(h, int(min_desired_scale), None, None, 0))
    if n < 0:
        raise ValueError("dual marching cubes needs a multi-res map")
    f = np.zeros((n, 3, 3), np.float32)
    sc = np.zeros(n, np.int8)
    if n:
        fn(h, int(min_desired_scale), f.ctypes.data, sc.ctypes.data, n)
    return f, sc


def dual_groups(rel):
    """The partition of a block-relative primal corner's 8 dual corners: (group_of[8], above[n])."""
    r = np.asarray(rel, np.int32)
    g = np.zeros(8, np.int32)
    a = np.zeros(8, np.int32)
    n = np.zeros(1, np.int32)
    lib().so_dual_groups(r, g, a, n)
    return g, a[:int(n[0])]


def mc_table():
    ntri = np.zeros(256, np.int32)
    tri = np.zeros(256 * 24, np.int32)
    lib().so_mc_table(ntri, tri)
    return ntri, tri.reshape(256, 24)


def downsample_depth(depth, ratio):
    """preprocessor::downsample_depth: (out [h/ratio, w/ratio] float32, map int64 of input indices)."""
    depth = np.ascontiguousarray(depth, np.float32)
    h, w = depth.shape
    out = np.zeros((h // ratio, w // ratio), np.float32)
    mp = np.zeros(out.shape, np.int64)
    lib().so_downsample_depth(depth.reshape(-1), w, h, out.reshape(-1), w // ratio, h // ratio, mp.ctypes.data)
    return out, mp


def exp_cw(x):
    return np.float32(lib().so_exp_cw(float(x)))


def tracker_config(iterations=(10, 5, 4), dist_threshold=0.1, normal_threshold=0.8,
                   track_threshold=0.15, icp_threshold=1e-5) -> TrackerConfig:
    it = (C.c_int * 3)(*([int(i) for i in iterations] + [0] * (3 - len(iterations))))
    return TrackerConfig(len(iterations), it, dist_threshold, normal_threshold,
                         track_threshold, icp_threshold)


def track(sensor: Pinhole, config: TrackerConfig, depth, T_WS, ref_pts, ref_nrm):
    """Tracker::track(depth, T_WS, pts, nrm); returns (accepted, T_WS_new, stats)."""
    T = _m16(T_WS).copy()
    st = TrackStats()
    acc = lib().so_track(C.byref(sensor), C.byref(config),
                         np.ascontiguousarray(depth, np.float32).reshape(-1), T,
                         np.ascontiguousarray(ref_pts, np.float32).reshape(-1),
                         np.ascontiguousarray(ref_nrm, np.float32).reshape(-1), C.byref(st))
    return bool(acc), T.reshape(4, 4), st


def tracker_pyramid(sensor: Pinhole, depth, levels=3):
    """The tracker's input pyramid as track() forms it: [(depth, points, normals)] per level,
    level l of size (H >> l, W >> l) (half_sample_robust_image, depth_to_point_cloud,
    point_cloud_to_normal)."""
    W, H = sensor.width, sensor.height
    sizes = [(H >> l, W >> l) for l in range(levels)]
    n = sum(h * w for h, w in sizes)
    d = np.zeros(n, np.float32)
    p = np.zeros(3 * n, np.float32)
    q = np.zeros(3 * n, np.float32)
    lib().so_tracker_pyramid(C.byref(sensor), np.ascontiguousarray(depth, np.float32).reshape(-1),
                             int(levels), d, p, q)
    out, off = [], 0
    for h, w in sizes:
        out.append((d[off:off + h * w].reshape(h, w), p[3 * off:3 * (off + h * w)].reshape(h, w, 3),
                    q[3 * off:3 * (off + h * w)].reshape(h, w, 3)))
        off += h * w
    return out


def se3_exp(twist):
    T = np.zeros(16, np.float32)
    lib().so_se3_exp(np.asarray(twist, np.float32), T)
    return T.reshape(4, 4)
