"""supereight2_gb300 — GB300 (sm_103a) implementation of supereight2's per-frame mapping path.

The compute lives in ``libse_gpu.so`` (hand-written CUDA kernels behind the C ABI of
``include/se_gpu.h``). This module is the Python mirror of the reference's interface for that
path, with the reference's names and argument meaning:

    Map(dim, res, ...)                                  se::TSDFMap<se::Res::Single>
    MapIntegrator(map).integrateDepth(ts, depth, sensor, T_WC)
                                                        se::MapIntegrator::integrateDepth
    raycast_volume(map, sensor, T_WS, pts, nrm, scale)  se::raycaster::raycast_volume
    Tracker(map, sensor, config).track(depth, T_WS, pts, nrm) -> bool
                                                        se::Tracker::track

Device images are torch CUDA tensors (float32 depth [H, W], float32 points/normals [H, W, 3],
int8 scale [H, W]); poses are 4x4 arrays (T_WC maps camera to world). There is no CPU
fallback: without the built library or a GPU every call raises.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

__all__ = ["Map", "MapIntegrator", "Tracker", "TrackerConfig", "PinholeCamera", "OusterLidar", "LeicaLidar",
           "integrate_ray_batch",
           "OccupancyBatch", "raycast_volume",
           "render_depth", "raycast_adjoint", "track_noalloc", "bilateral_filter", "downsample_depth", "marching_cube",
           "dual_marching_cube", "save_mesh",
           "FramePipeline", "SeGpuError", "library", "library_path"]


class SeGpuError(RuntimeError):
    """A libse_gpu call returned a status other than SE_GPU_OK."""


class _MapConfig(C.Structure):
    _fields_ = [("dim", C.c_float * 3), ("res", C.c_float), ("T_MW", C.c_float * 16),
                ("has_T_MW", C.c_int), ("field", C.c_int), ("res_type", C.c_int),
                ("storage", C.c_int), ("truncation_boundary_factor", C.c_float),
                ("max_weight", C.c_float), ("max_blocks", C.c_int64)]


class _OccupancyConfig(C.Structure):
    _fields_ = [("k_sigma", C.c_float), ("sigma_min_factor", C.c_float), ("sigma_max_factor", C.c_float),
                ("k_tau", C.c_float), ("tau_min_factor", C.c_float), ("tau_max_factor", C.c_float),
                ("log_odd_min", C.c_float), ("log_odd_max", C.c_float), ("fs_integr_scale", C.c_int)]


OCCUPANCY_DEFAULTS = dict(k_sigma=0.052, sigma_min_factor=1.5, sigma_max_factor=6.0, k_tau=0.026,
                          tau_min_factor=6.0, tau_max_factor=16.0, log_odd_min=-5.015,
                          log_odd_max=5.015, fs_integr_scale=1)


class _Pinhole(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("fx", C.c_float), ("fy", C.c_float),
                ("cx", C.c_float), ("cy", C.c_float), ("near_plane", C.c_float),
                ("far_plane", C.c_float)]


class _Lidar(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("elevation_min_deg", C.c_float),
                ("elevation_max_deg", C.c_float), ("near_plane", C.c_float),
                ("far_plane", C.c_float)]


class _LeicaLidar(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("near_plane", C.c_float),
                ("far_plane", C.c_float), ("elevation_resolution_deg", C.c_float),
                ("azimuth_resolution_deg", C.c_float)]


class _BilateralConfig(C.Structure):
    _fields_ = [("radius", C.c_int), ("sigma_space_px", C.c_float), ("sigma_range_m", C.c_float)]


# The bilateral pre-filter of the tracked TSDF benchmark configuration: 5x5, 4 px, 0.03 m.
BILATERAL_DEFAULTS = dict(radius=2, sigma_space=4.0, sigma_range=0.03)


class _TrackerConfig(C.Structure):
    _fields_ = [("num_levels", C.c_int), ("iterations", C.c_int * 3),
                ("dist_threshold", C.c_float), ("normal_threshold", C.c_float),
                ("track_threshold", C.c_float), ("icp_threshold", C.c_float)]


class _IntegrateStats(C.Structure):
    _fields_ = [("n_new_blocks", C.c_int64), ("n_listed_blocks", C.c_int64),
                ("n_updated_voxels", C.c_int64), ("n_valid_pixels", C.c_int64)]


# Every symbol include/se_gpu.h declares, with its ctypes signature.
_VP = C.c_void_p
_F16 = C.POINTER(C.c_float)
SIGNATURES = {
    "se_gpu_last_error": (C.c_char_p, []),
    "se_gpu_status_string": (C.c_char_p, [C.c_int]),
    "se_gpu_abi_version": (C.c_int, []),
    "se_gpu_map_create": (C.c_int, [C.POINTER(_MapConfig), C.POINTER(_VP)]),
    "se_gpu_map_destroy": (C.c_int, [_VP]),
    "se_gpu_map_create_occupancy": (C.c_int, [C.POINTER(_MapConfig), C.POINTER(_OccupancyConfig),
                                              C.POINTER(_VP)]),
    "se_gpu_map_occupancy_stats": (C.c_int, [_VP, C.POINTER(C.c_int64)]),
    "se_gpu_map_download_occupancy": (C.c_int, [_VP, C.c_int64, _VP, _VP, _VP, _VP, _VP, _VP,
                                                C.POINTER(C.c_int64)]),
    "se_gpu_map_download_nodes": (C.c_int, [_VP, C.c_int64, _VP, _VP, _VP, _VP, C.POINTER(C.c_int64)]),
    "se_gpu_map_size": (C.c_int, [_VP, C.POINTER(C.c_int), C.POINTER(C.c_float)]),
    "se_gpu_map_check": (C.c_int, [_VP]),
    "se_gpu_integrate_depth": (C.c_int, [_VP, _VP, C.POINTER(_Pinhole), _F16, C.c_int, _VP]),
    "se_gpu_integrate_range": (C.c_int, [_VP, _VP, C.POINTER(_Lidar), _F16, C.c_int, _VP]),
    "se_gpu_occ_batch_stats_async": (C.c_int, [_VP, _VP, _VP]),
    "se_gpu_occ_integrate_ray_batch": (C.c_int, [_VP, C.POINTER(_LeicaLidar), _VP, _VP, C.c_int64, C.c_int32,
                                                 _VP, C.c_int64, C.POINTER(C.c_int64), _VP]),
    "se_gpu_bilateral_filter": (C.c_int, [_VP, _VP, C.c_int, C.c_int, C.POINTER(_BilateralConfig), _VP]),
    "se_gpu_tracker_set_persistent": (C.c_int, [_VP, C.c_int]),
    "se_gpu_tracker_test_barrier_timeout": (C.c_int, [_VP, C.c_int]),
    "se_gpu_marching_cube": (C.c_int, [_VP, _VP, C.c_int64, C.POINTER(C.c_int64), _VP]),
    "se_gpu_dual_marching_cube": (C.c_int, [_VP, C.c_int, _VP, _VP, C.c_int64, C.POINTER(C.c_int64), _VP]),
    "se_gpu_mc_case_table": (C.c_int, [_VP, _VP]),
    "se_gpu_save_mesh": (C.c_int, [_VP, _VP, C.c_int64, _F16, C.c_char_p]),
    "se_gpu_map_mesh_transform": (C.c_int, [_VP, _F16, _F16]),
    "se_gpu_map_save_mesh": (C.c_int, [_VP, _F16, C.c_int, C.c_char_p, _VP]),
    "se_gpu_save_point_cloud_vtk": (C.c_int, [_VP, C.c_int64, _F16, C.c_char_p]),
    "se_gpu_map_field_box": (C.c_int, [_VP, _VP, _VP, _VP]),
    "se_gpu_map_save_field_slices": (C.c_int, [_VP, C.c_char_p, C.c_char_p, C.c_char_p, _F16]),
    "se_gpu_downsample_depth": (C.c_int, [_VP, C.c_int, C.c_int, _VP, C.c_int, C.c_int, _VP, _VP]),
    "se_gpu_frame_set_bilateral": (C.c_int, [_VP, C.POINTER(_BilateralConfig)]),
    "se_gpu_occ_batch_create": (C.c_int, [_VP, C.c_int, C.POINTER(_Pinhole), C.POINTER(_Lidar),
                                          C.c_int, C.POINTER(_VP)]),
    "se_gpu_occ_batch_integrate": (C.c_int, [_VP, _VP, _F16, _VP, _VP]),
    "se_gpu_occ_batch_destroy": (C.c_int, [_VP]),
    "se_gpu_occ_batch_tiles": (C.c_int, [_VP, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "se_gpu_map_integrate_stats": (C.c_int, [_VP, C.POINTER(_IntegrateStats)]),
    "se_gpu_raycast": (C.c_int, [_VP, C.POINTER(_Pinhole), _F16, _VP, _VP, _VP, _VP]),
    "se_gpu_map_download_blocks": (C.c_int, [_VP, C.c_int64, _VP, _VP, _VP, _VP, _VP,
                                             C.POINTER(C.c_int64)]),
    "se_gpu_map_upload_blocks": (C.c_int, [_VP, C.c_int64, _VP, _VP, _VP]),
    "se_gpu_map_download_multires": (C.c_int, [_VP, C.c_int64, _VP, _VP, _VP, _VP, _VP, _VP, _VP,
                                               C.POINTER(C.c_int64)]),
    "se_gpu_map_field_interp": (C.c_int, [_VP, C.c_int64, _VP, _VP, _VP, _VP]),
    "se_gpu_map_field_grad": (C.c_int, [_VP, C.c_int64, _VP, _VP, _VP, _VP]),
    "se_gpu_map_aabb": (C.c_int, [_VP, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                  C.POINTER(C.c_int)]),
    "se_gpu_render_depth": (C.c_int, [_VP, C.POINTER(_Pinhole), _F16, _VP, _VP]),
    "se_gpu_raycast_adjoint": (C.c_int, [_VP, C.POINTER(_Pinhole), _F16, _VP, _VP, _VP, _VP, _VP]),
    "se_gpu_tracker_create": (C.c_int, [C.POINTER(_Pinhole), C.POINTER(_TrackerConfig),
                                        C.POINTER(_VP)]),
    "se_gpu_tracker_destroy": (C.c_int, [_VP]),
    "se_gpu_track": (C.c_int, [_VP, _VP, _VP, _VP, _F16, C.POINTER(C.c_int), _VP]),
    "se_gpu_tracker_last_reduction": (C.c_int, [_VP, _F16, C.POINTER(C.c_int)]),
    "se_gpu_frame_autotune": (C.c_int, [_VP, C.c_int]),
    "se_gpu_frame_tiles": (C.c_int, [_VP, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "se_gpu_tracker_level_images": (C.c_int, [_VP, C.c_int, _VP, _VP, _VP, _VP]),
    "se_gpu_track_noalloc": (C.c_int, [C.POINTER(_Pinhole), C.POINTER(_TrackerConfig), _VP, _VP,
                                       _VP, _F16, C.POINTER(C.c_int), _F16, _VP]),
    "se_gpu_frame_create": (C.c_int, [_VP, _VP, C.POINTER(_Pinhole), C.POINTER(_VP)]),
    "se_gpu_frame_destroy": (C.c_int, [_VP]),
    "se_gpu_frame_buffers": (C.c_int, [_VP, C.POINTER(_VP), C.POINTER(_VP), C.POINTER(_VP),
                                       C.POINTER(_VP)]),
    "se_gpu_frame_set_pose": (C.c_int, [_VP, _F16, C.c_int]),
    "se_gpu_frame_run": (C.c_int, [_VP, C.c_int, _VP]),
    "se_gpu_frame_run_host": (C.c_int, [_VP, _VP, C.c_int, _VP]),
    "se_gpu_frame_get_pose": (C.c_int, [_VP, _F16, C.POINTER(C.c_int), _VP]),
    "se_gpu_frame_get_pose_async": (C.c_int, [_VP, _VP, _VP, _VP]),
    "se_gpu_profiling_enable": (C.c_int, [C.c_int]),
    "se_gpu_profiling_read": (C.c_int, [C.c_int, _VP, _VP, C.c_int]),
    "se_gpu_profiling_name": (C.c_char_p, [C.c_int]),
    "se_gpu_profiling_count": (C.c_int, []),
}

_lib = None


def library_path() -> str:
    return _build.LIB_PATH


def library(build_if_missing: bool = True):
    """Load libse_gpu.so (building it with nvcc if it is missing or stale)."""
    global _lib
    if _lib is None:
        path = _build.build() if build_if_missing else _build.LIB_PATH
        if not os.path.exists(path):
            raise SeGpuError(f"libse_gpu.so not found at {path}: run supereight2_gb300/build.py")
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(status: int, what: str):
    if status != 0:
        L = library()
        raise SeGpuError(f"{what}: {L.se_gpu_status_string(status).decode()} "
                         f"({L.se_gpu_last_error().decode()})")


def _m16(T):
    a = np.ascontiguousarray(np.asarray(T, dtype=np.float32).reshape(16))
    return a, a.ctypes.data_as(_F16)


def _stream(stream):
    if stream is not None:
        return C.c_void_p(int(stream))
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dptr(t, dtype, shape=None, name="tensor"):
    import torch
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise SeGpuError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype or not t.is_contiguous():
        raise SeGpuError(f"{name} must be a contiguous {dtype} tensor")
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise SeGpuError(f"{name} has shape {tuple(t.shape)}, expected {tuple(shape)}")
    return C.c_void_p(t.data_ptr())


class PinholeCamera:
    """se::PinholeCamera::Config: width, height, fx, fy, cx, cy, near_plane, far_plane."""

    def __init__(self, width, height, fx, fy, cx, cy, near_plane=0.01, far_plane=10.0):
        self.width, self.height = int(width), int(height)
        self.fx, self.fy, self.cx, self.cy = float(fx), float(fy), float(cx), float(cy)
        self.near_plane, self.far_plane = float(near_plane), float(far_plane)

    @classmethod
    def from_spec(cls, s):
        return cls(s.width, s.height, s.fx, s.fy, s.cx, s.cy, s.near_plane, s.far_plane)

    def downsampled(self, dsf):
        """se::PinholeCamera(config, dsf) (src/sensor/pinhole_camera.cpp:29-39), in float32."""
        f = np.float32
        d = f(dsf)
        return PinholeCamera(int(f(self.width) / d), int(f(self.height) / d), f(self.fx) / d, f(self.fy) / d,
                             (f(self.cx) + f(0.5)) / d - f(0.5), (f(self.cy) + f(0.5)) / d - f(0.5),
                             self.near_plane, self.far_plane)

    def _c(self) -> _Pinhole:
        return _Pinhole(self.width, self.height, self.fx, self.fy, self.cx, self.cy,
                        self.near_plane, self.far_plane)


class OusterLidar:
    """se::OusterLidar::Config of an equiangular spinning LiDAR: width columns over 360 degrees,
    height beams linear in elevation from elevation_max_deg (row 0) to elevation_min_deg.
    Range images hold metres (<= 0: no return)."""

    def __init__(self, width, height, elevation_min_deg, elevation_max_deg, near_plane=0.5,
                 far_plane=60.0):
        self.width, self.height = int(width), int(height)
        self.elevation_min_deg, self.elevation_max_deg = float(elevation_min_deg), float(elevation_max_deg)
        self.near_plane, self.far_plane = float(near_plane), float(far_plane)

    @classmethod
    def from_spec(cls, s):
        return cls(s.width, s.height, s.elevation_min_deg, s.elevation_max_deg, s.near_plane,
                   s.far_plane)

    def _c(self) -> _Lidar:
        return _Lidar(self.width, self.height, self.elevation_min_deg, self.elevation_max_deg,
                      self.near_plane, self.far_plane)


class LeicaLidar:
    """se::LeicaLidar::Config: the ray-batch sensor (angular resolutions in degrees)."""

    def __init__(self, width=360, height=180, near_plane=0.2, far_plane=30.0, elevation_resolution_deg=1.0,
                 azimuth_resolution_deg=1.0):
        self.width, self.height = int(width), int(height)
        self.near_plane, self.far_plane = float(near_plane), float(far_plane)
        self.elevation_resolution_deg = float(elevation_resolution_deg)
        self.azimuth_resolution_deg = float(azimuth_resolution_deg)

    def _c(self) -> _LeicaLidar:
        return _LeicaLidar(self.width, self.height, self.near_plane, self.far_plane,
                           self.elevation_resolution_deg, self.azimuth_resolution_deg)


class TrackerConfig:
    """se::TrackerConfig (include/se/tracker/tracker.hpp:22-33) defaults."""

    def __init__(self, iterations=(10, 5, 4), dist_threshold=0.1, normal_threshold=0.8,
                 track_threshold=0.15, icp_threshold=1e-5):
        self.iterations = tuple(int(i) for i in iterations)
        self.dist_threshold = float(dist_threshold)
        self.normal_threshold = float(normal_threshold)
        self.track_threshold = float(track_threshold)
        self.icp_threshold = float(icp_threshold)

    def _c(self) -> _TrackerConfig:
        it = list(self.iterations) + [0] * (3 - len(self.iterations))
        return _TrackerConfig(len(self.iterations), (C.c_int * 3)(*it), self.dist_threshold,
                              self.normal_threshold, self.track_threshold, self.icp_threshold)


class Map:
    """se::TSDFMap<se::Res::Single> (or, with res="multi", se::TSDFMap<se::Res::Multi>) on the
    GPU: block hash + block pool of 8^3 voxels (585-entry voxel pyramids for multi-res)."""

    def __init__(self, dim, res, truncation_boundary_factor=8.0, max_weight=100.0,
                 storage="f32", max_blocks=1 << 20, T_MW=None, res_type="single", field="tsdf",
                 occupancy=None):
        cfg = _MapConfig()
        d = np.broadcast_to(np.asarray(dim, np.float32), (3,))
        cfg.dim = (C.c_float * 3)(*[float(v) for v in d])
        cfg.res = float(res)
        if T_MW is not None:
            cfg.T_MW = (C.c_float * 16)(*[float(v) for v in np.asarray(T_MW, np.float32).reshape(16)])
            cfg.has_T_MW = 1
        cfg.field = {"tsdf": 0, "occupancy": 1}[field]
        cfg.res_type = {"single": 0, "multi": 1}[res_type]
        cfg.storage = {"f32": 0, "f16": 1}[storage]
        cfg.truncation_boundary_factor = float(truncation_boundary_factor)
        cfg.max_weight = float(max_weight)
        cfg.max_blocks = int(max_blocks)
        self._L = library()
        h = C.c_void_p()
        self.field = field
        if field == "occupancy":
            oc = dict(OCCUPANCY_DEFAULTS)
            oc.update(occupancy or {})
            occ = _OccupancyConfig(*[oc[k] for k, _ in _OccupancyConfig._fields_])
            _check(self._L.se_gpu_map_create_occupancy(C.byref(cfg), C.byref(occ), C.byref(h)),
                   "se_gpu_map_create_occupancy")
        else:
            _check(self._L.se_gpu_map_create(C.byref(cfg), C.byref(h)), "se_gpu_map_create")
        self.h = h
        self.res = float(res)
        self.storage = storage
        self.res_type = res_type
        self.max_blocks = int(max_blocks)
        self.truncation_boundary_factor = float(truncation_boundary_factor)

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self._L.se_gpu_map_destroy(h)
            self.h = None

    @property
    def size(self) -> int:
        s, d = C.c_int(), C.c_float()
        _check(self._L.se_gpu_map_size(self.h, C.byref(s), C.byref(d)), "se_gpu_map_size")
        return s.value

    @property
    def dim(self) -> float:
        s, d = C.c_int(), C.c_float()
        _check(self._L.se_gpu_map_size(self.h, C.byref(s), C.byref(d)), "se_gpu_map_size")
        return d.value

    def check(self):
        """Synchronise and raise on a latched device-side error (pool full, probe limit)."""
        _check(self._L.se_gpu_map_check(self.h), "se_gpu_map_check")

    def integrate_stats(self) -> dict:
        st = _IntegrateStats()
        _check(self._L.se_gpu_map_integrate_stats(self.h, C.byref(st)), "integrate_stats")
        return {"n_new_blocks": st.n_new_blocks, "n_listed_blocks": st.n_listed_blocks,
                "n_updated_voxels": st.n_updated_voxels, "n_valid_pixels": st.n_valid_pixels}

    def num_blocks(self) -> int:
        n = C.c_int64()
        _check(self._L.se_gpu_map_download_blocks(self.h, 0, None, None, None, None, None,
                                                  C.byref(n)), "download_blocks")
        return n.value

    def download_blocks(self, voxels=True):
        """(keys u64[N], coords i32[N,3], tsdf f32[N,512], weight f32[N,512], ts i32[N])."""
        n = self.num_blocks()
        keys = np.zeros(n, np.uint64)
        coords = np.zeros((n, 3), np.int32)
        ts = np.zeros(n, np.int32)
        tsdf = np.zeros((n, 512), np.float32) if voxels else None
        weight = np.zeros((n, 512), np.float32) if voxels else None
        cnt = C.c_int64()
        if n:
            _check(self._L.se_gpu_map_download_blocks(
                self.h, n, keys.ctypes.data, coords.ctypes.data,
                tsdf.ctypes.data if voxels else None, weight.ctypes.data if voxels else None,
                ts.ctypes.data, C.byref(cnt)), "download_blocks")
        return keys, coords, tsdf, weight, ts

    def occupancy_stats(self):
        """(blocks listed, free-space nodes listed, blocks freed, nodes pruned) of the last frame."""
        st = (C.c_int64 * 4)()
        _check(self._L.se_gpu_map_occupancy_stats(self.h, st), "occupancy_stats")
        return tuple(int(v) for v in st)

    def download_occupancy(self):
        """Live blocks: (coords i32[N,3], scales i32[N,3], counts i64[N,4], mean / min / max
        f32[N,585,3] of (occupancy, weight, observed))."""
        n = C.c_int64()
        _check(self._L.se_gpu_map_download_occupancy(self.h, 0, None, None, None, None, None, None,
                                                     C.byref(n)), "download_occupancy")
        k = n.value
        coords = np.zeros((k, 3), np.int32)
        scales = np.zeros((k, 3), np.int32)
        counts = np.zeros((k, 4), np.int64)
        arrs = [np.zeros((k, 585, 3), np.float32) for _ in range(3)]
        if k:
            _check(self._L.se_gpu_map_download_occupancy(
                self.h, k, coords.ctypes.data, scales.ctypes.data, counts.ctypes.data,
                *[a.ctypes.data for a in arrs], C.byref(n)), "download_occupancy")
        return (coords, scales, counts, *arrs)

    def download_nodes(self):
        """Nodes reachable from the root, depth first: (coords+size i32[N,4], min f32[N,3],
        max f32[N,3], leaf i32[N])."""
        n = C.c_int64()
        _check(self._L.se_gpu_map_download_nodes(self.h, 0, None, None, None, None, C.byref(n)),
               "download_nodes")
        k = n.value
        c = np.zeros((k, 4), np.int32)
        mn = np.zeros((k, 3), np.float32)
        mx = np.zeros((k, 3), np.float32)
        lf = np.zeros(k, np.int32)
        _check(self._L.se_gpu_map_download_nodes(self.h, k, c.ctypes.data, mn.ctypes.data,
                                                 mx.ctypes.data, lf.ctypes.data, C.byref(n)),
               "download_nodes")
        return c, mn, mx, lf

    def download_multires(self):
        """Multi-res maps: (keys u64[N], coords i32[N,3], tsdf, weight, past_tsdf, past_weight
        f32[N,585], scales i32[N,2] = (current, min))."""
        n = self.num_blocks()
        keys = np.zeros(n, np.uint64)
        coords = np.zeros((n, 3), np.int32)
        arrs = [np.zeros((n, 585), np.float32) for _ in range(4)]
        scales = np.zeros((n, 2), np.int32)
        cnt = C.c_int64()
        if n:
            _check(self._L.se_gpu_map_download_multires(
                self.h, n, keys.ctypes.data, coords.ctypes.data, *[a.ctypes.data for a in arrs],
                scales.ctypes.data, C.byref(cnt)), "download_multires")
        return (keys, coords, *arrs, scales)

    def upload_blocks(self, keys, tsdf, weight):
        """Allocate the blocks with these keys (Morton code << 5 | 3) and overwrite their voxels."""
        keys = np.ascontiguousarray(keys, np.uint64)
        tsdf = np.ascontiguousarray(np.broadcast_to(np.asarray(tsdf, np.float32), (len(keys), 512)))
        weight = np.ascontiguousarray(np.broadcast_to(np.asarray(weight, np.float32), (len(keys), 512)))
        _check(self._L.se_gpu_map_upload_blocks(self.h, len(keys), keys.ctypes.data,
                                                tsdf.ctypes.data, weight.ctypes.data),
               "se_gpu_map_upload_blocks")

    def getFieldInterp(self, points_W, stream=None):
        """Map::getFieldInterp for a CUDA [N, 3] float32 tensor: (values [N], valid [N] bool)."""
        return self._field_query(points_W, stream, grad=False)

    def mesh_transform(self, T_OW=None):
        """T_OV = T_OW T_WM Scaling(res): voxel-unit mesh vertices to the output frame."""
        _, tw = _m16(np.eye(4) if T_OW is None else T_OW)
        out = np.zeros(16, np.float32)
        _check(self._L.se_gpu_map_mesh_transform(self.h, tw, out.ctypes.data_as(_F16)), "se_gpu_map_mesh_transform")
        return out.reshape(4, 4)

    def saveMesh(self, filename, T_OW=None, min_desired_scale=0, stream=None):
        """Map::saveMesh: marching cubes (dual for multi-res and occupancy maps, at
        min_desired_scale or coarser) written as .ply / .vtk / .obj in the T_OW frame."""
        _, tw = _m16(np.eye(4) if T_OW is None else T_OW)
        _check(self._L.se_gpu_map_save_mesh(self.h, tw, int(min_desired_scale), str(filename).encode(),
                                            _stream(stream)), "se_gpu_map_save_mesh")

    def saveFieldSlices(self, filename_x, filename_y, filename_z, point_W):
        """Map::saveFieldSlices: VTK rectilinear slices of the field through point_W's voxel."""
        p = np.ascontiguousarray(np.asarray(point_W, np.float32).reshape(3))
        enc = lambda s: str(s).encode() if s else None  # noqa: E731
        _check(self._L.se_gpu_map_save_field_slices(self.h, enc(filename_x), enc(filename_y), enc(filename_z),
                                                    p.ctypes.data_as(_F16)), "se_gpu_map_save_field_slices")

    def field_box(self, lo, hi):
        """get_field(getData(v)) over the voxel box [lo, hi) as an array [z, y, x]."""
        lo = np.ascontiguousarray(lo, np.int32)
        hi = np.ascontiguousarray(hi, np.int32)
        out = np.zeros(tuple(int(v) for v in (hi - lo)[::-1]), np.float32)
        _check(self._L.se_gpu_map_field_box(self.h, lo.ctypes.data, hi.ctypes.data, out.ctypes.data),
               "se_gpu_map_field_box")
        return out

    def getFieldGrad(self, points_W, stream=None):
        """Map::getFieldGrad for a CUDA [N, 3] float32 tensor: (grads [N, 3], valid [N] bool)."""
        return self._field_query(points_W, stream, grad=True)

    def _field_query(self, points_W, stream, grad):
        import torch
        n = points_W.shape[0]
        p = _dptr(points_W, torch.float32, (n, 3), "points_W")
        out = torch.zeros((n, 3) if grad else (n,), dtype=torch.float32, device=points_W.device)
        valid = torch.zeros(n, dtype=torch.int32, device=points_W.device)
        fn = self._L.se_gpu_map_field_grad if grad else self._L.se_gpu_map_field_interp
        _check(fn(self.h, n, p, C.c_void_p(out.data_ptr()), C.c_void_p(valid.data_ptr()),
                  _stream(stream)), "field query")
        return out, valid.bool()

    def aabb(self):
        mn = (C.c_int32 * 3)()
        mx = (C.c_int32 * 3)()
        empty = C.c_int()
        _check(self._L.se_gpu_map_aabb(self.h, mn, mx, C.byref(empty)), "se_gpu_map_aabb")
        return None if empty.value else (np.array(mn[:], np.int32), np.array(mx[:], np.int32))


class MapIntegrator:
    """se::MapIntegrator<TSDFMap<Res::Single>>."""

    def __init__(self, map: Map):
        self.map = map

    def integrateDepth(self, timestamp, depth, sensor, T_WC, stream=None):
        """sensor: PinholeCamera (depth in metres of z) or OusterLidar (occupancy maps; range in
        metres)."""
        import torch
        ptr = _dptr(depth, torch.float32, (sensor.height, sensor.width), "depth")
        s = sensor._c()
        _, tp = _m16(T_WC)
        L = self.map._L
        if isinstance(sensor, OusterLidar):
            _check(L.se_gpu_integrate_range(self.map.h, ptr, C.byref(s), tp, int(timestamp),
                                            _stream(stream)), "se_gpu_integrate_range")
            return
        _check(L.se_gpu_integrate_depth(self.map.h, ptr, C.byref(s), tp, int(timestamp),
                                        _stream(stream)), "se_gpu_integrate_depth")


def integrate_ray_batch(map: Map, timestamp, poses, rays, sensor: LeicaLidar, stream=None,
                        with_octants=True):
    """se::MapIntegrator::integrateRayBatch(timestamp, rayPoseBatch, sensor, updated_octants) for
    an occupancy map: rays (N, 3) float32 CUDA tensor in the sensor frame, poses (N, 4, 4) float32
    CUDA tensor (T_WS per ray). Returns the updated octants as an (K, 4) int32 CUDA tensor of
    (x, y, z, size) in voxels (any order), or their number when with_octants is False."""
    import torch
    n = int(rays.shape[0]) if rays.dim() == 2 else -1
    rp = _dptr(rays, torch.float32, (n, 3), "rays")
    pp = _dptr(poses, torch.float32, (n, 4, 4), "poses")
    cnt = C.c_int64()
    s = sensor._c()
    L = map._L
    if not with_octants:
        _check(L.se_gpu_occ_integrate_ray_batch(map.h, C.byref(s), pp, rp, n, int(timestamp), None, 0,
                                                C.byref(cnt), _stream(stream)), "se_gpu_occ_integrate_ray_batch")
        return cnt.value
    cap = max(4096, 64 * n)
    out = torch.empty((cap, 4), dtype=torch.int32, device=rays.device)
    _check(L.se_gpu_occ_integrate_ray_batch(map.h, C.byref(s), pp, rp, n, int(timestamp),
                                            C.c_void_p(out.data_ptr()), cap, C.byref(cnt), _stream(stream)),
           "se_gpu_occ_integrate_ray_batch")
    if cnt.value > cap:
        raise SeGpuError("more updated octants (%d) than the output holds" % cnt.value)
    return out[: cnt.value]


class OccupancyBatch:
    """Several occupancy maps integrated together, one frame each per call, every pipeline stage
    in one launch over all maps (no counterpart in the reference). graph=True captures the
    launches of a call into a CUDA graph on the first call and replays it afterwards;
    autotune=True runs the default geometry for the first 4 calls, then spends 12 calls timing
    4 launch geometries three times each and keeps per stage the one with the least time in its
    best round (the graph is captured after that). persistent=True runs each call as one
    cooperative launch (every stage a grid-stride loop, grid barriers between them); its tuned
    geometry is the CTAs per SM of that launch."""

    def __init__(self, maps, sensor, graph=True, autotune=False, persistent=False):
        self.maps = list(maps)
        self.sensor = sensor
        self._L = library()
        arr = (_VP * len(self.maps))(*[m.h for m in self.maps])
        s = sensor._c()
        pin = C.byref(s) if isinstance(sensor, PinholeCamera) else None
        lid = C.byref(s) if isinstance(sensor, OusterLidar) else None
        h = _VP()
        flags = (1 if graph else 0) | (2 if autotune else 0) | (4 if persistent else 0)
        _check(self._L.se_gpu_occ_batch_create(arr, len(self.maps), pin, lid, flags, C.byref(h)),
               "se_gpu_occ_batch_create")
        self.h = h

    def stats_async(self, out, stream=None):
        """Enqueue the copy of every map's four per-frame counters into out, a pinned int32 host
        tensor of shape (n, 4); valid once the stream passes this call."""
        import torch
        if out.is_cuda or out.dtype != torch.int32 or tuple(out.shape) != (len(self.maps), 4) or not out.is_contiguous():
            raise SeGpuError("out must be a contiguous (n, 4) int32 host tensor")
        _check(self._L.se_gpu_occ_batch_stats_async(self.h, C.c_void_p(out.data_ptr()), _stream(stream)),
               "se_gpu_occ_batch_stats_async")

    def tiles(self):
        """(CTAs per SM of the carver, list and block stages), tuning calls left."""
        t = (C.c_int * 3)()
        left = C.c_int()
        _check(self._L.se_gpu_occ_batch_tiles(self.h, t, C.byref(left)), "se_gpu_occ_batch_tiles")
        return tuple(t), left.value

    def __del__(self):
        if getattr(self, "h", None):
            self._L.se_gpu_occ_batch_destroy(self.h)
            self.h = None

    def integrate(self, images, T_WS, timestamps, stream=None):
        """images: per map a [height, width] float32 CUDA tensor (or one [n, height, width]
        tensor); T_WS: n 4x4 poses; timestamps: n ints (or one int for all maps)."""
        import torch
        n = len(self.maps)
        if isinstance(images, torch.Tensor) and images.dim() == 3:
            _dptr(images, torch.float32, (n, self.sensor.height, self.sensor.width), "images")
            ptrs = [images.data_ptr() + i * images.stride(0) * 4 for i in range(n)]
        else:
            if len(images) != n:
                raise SeGpuError(f"{len(images)} images for {n} maps")
            ptrs = [_dptr(im, torch.float32, (self.sensor.height, self.sensor.width), "image").value
                    for im in images]
        arr = (_VP * n)(*ptrs)
        T = np.ascontiguousarray(np.asarray(T_WS, np.float32).reshape(n, 16))
        if np.isscalar(timestamps):
            timestamps = [int(timestamps)] * n
        ts = (C.c_int * n)(*[int(t) for t in timestamps])
        _check(self._L.se_gpu_occ_batch_integrate(self.h, arr, T.ctypes.data_as(_F16), ts,
                                                  _stream(stream)), "se_gpu_occ_batch_integrate")


def raycast_volume(map: Map, sensor: PinholeCamera, T_WS, surface_point_cloud_W,
                   surface_normals_W, surface_scale=None, stream=None):
    """se::raycaster::raycast_volume into preallocated device images."""
    import torch
    shp = (sensor.height, sensor.width, 3)
    p = _dptr(surface_point_cloud_W, torch.float32, shp, "surface_point_cloud_W")
    n = _dptr(surface_normals_W, torch.float32, shp, "surface_normals_W")
    sc = None
    if surface_scale is not None:
        sc = _dptr(surface_scale, torch.int8, shp[:2], "surface_scale")
    s = sensor._c()
    _, tp = _m16(T_WS)
    _check(map._L.se_gpu_raycast(map.h, C.byref(s), tp, p, n, sc, _stream(stream)),
           "se_gpu_raycast")


class Tracker:
    """se::Tracker<MapT, PinholeCamera>: 3-level projective point-to-plane ICP."""

    def __init__(self, map: Map, sensor: PinholeCamera, config: TrackerConfig = None):
        self.map = map
        self.sensor = sensor
        self.config = config or TrackerConfig()
        self._L = library()
        h = C.c_void_p()
        s = sensor._c()
        c = self.config._c()
        _check(self._L.se_gpu_tracker_create(C.byref(s), C.byref(c), C.byref(h)),
               "se_gpu_tracker_create")
        self.h = h

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self._L.se_gpu_tracker_destroy(h)
            self.h = None

    def track(self, depth, T_WS, surface_point_cloud_W, surface_normals_W, stream=None):
        """Track depth against the raycast taken at T_WS. T_WS (a float32 4x4 numpy array) is
        updated in place; returns whether the pose was accepted."""
        import torch
        s = self.sensor
        d = _dptr(depth, torch.float32, (s.height, s.width), "depth")
        p = _dptr(surface_point_cloud_W, torch.float32, (s.height, s.width, 3), "points")
        n = _dptr(surface_normals_W, torch.float32, (s.height, s.width, 3), "normals")
        if not (isinstance(T_WS, np.ndarray) and T_WS.dtype == np.float32 and T_WS.shape == (4, 4)
                and T_WS.flags.c_contiguous):
            raise SeGpuError("T_WS must be a C-contiguous float32 4x4 numpy array (updated in place)")
        acc = C.c_int()
        _check(self._L.se_gpu_track(self.h, d, p, n, T_WS.ctypes.data_as(_F16), C.byref(acc),
                                    _stream(stream)), "se_gpu_track")
        return bool(acc.value)

    def set_persistent(self, enable=True):
        """One cooperative launch per track() (default when it fits) or one launch per ICP iteration."""
        _check(self._L.se_gpu_tracker_set_persistent(self.h, 1 if enable else 0), "se_gpu_tracker_set_persistent")

    def test_barrier_timeout(self, enable=True):
        """Test aid: make the persistent ICP's bounded wait for the merged totals time out (the
        frame's pose is rejected and track() raises SeGpuError)."""
        _check(self._L.se_gpu_tracker_test_barrier_timeout(self.h, 1 if enable else 0),
               "se_gpu_tracker_test_barrier_timeout")

    def level_images(self, level, stream=None):
        """The last track()'s input pyramid at one level: (depth or None at level 0, points,
        normals), new CUDA tensors of (H >> level, W >> level) pixels."""
        import torch
        h, w = self.sensor.height >> level, self.sensor.width >> level
        d = torch.zeros((h, w), dtype=torch.float32, device="cuda") if level > 0 else None
        p = torch.zeros((h, w, 3), dtype=torch.float32, device="cuda")
        n = torch.zeros_like(p)
        _check(self._L.se_gpu_tracker_level_images(self.h, int(level), d.data_ptr() if d is not None else None,
                                                   p.data_ptr(), n.data_ptr(), _stream(stream)),
               "se_gpu_tracker_level_images")
        torch.cuda.synchronize()
        return d, p, n

    def last_reduction(self):
        red = (C.c_float * 32)()
        its = (C.c_int * 3)()
        _check(self._L.se_gpu_tracker_last_reduction(self.h, red, its), "last_reduction")
        return np.array(red[:], np.float32), list(its[:])


def render_depth(map: Map, sensor: PinholeCamera, T_WS, out=None, stream=None):
    """Differentiable depth render (no counterpart in the reference): z of the root of the
    trilinear TSDF on each pixel's ray, 0 where there is none. Returns a CUDA [H, W] tensor."""
    import torch
    L = library()
    if out is None:
        out = torch.zeros((sensor.height, sensor.width), dtype=torch.float32, device="cuda")
    d = _dptr(out, torch.float32, (sensor.height, sensor.width), "depth")
    s = sensor._c()
    _, tp = _m16(T_WS)
    _check(L.se_gpu_render_depth(map.h, C.byref(s), tp, d, _stream(stream)), "se_gpu_render_depth")
    return out


def raycast_adjoint(map: Map, sensor: PinholeCamera, T_WS, grad_depth=None, twist_grad=None,
                    voxel_grad=None, jac=None, stream=None):
    """Adjoint of render_depth: accumulates sum_i grad_depth[i] * d depth_i / d xi into
    twist_grad (CUDA float64 [6]; allocated and returned if None) for T = exp(xi) T_WS,
    xi = [rho; omega]; voxel_grad (CUDA float32 [max_blocks, 512], pool order) receives
    d L / d tsdf; jac (CUDA float32 [H, W, 6]) receives d depth_i / d xi."""
    import torch
    L = library()
    if twist_grad is None:
        twist_grad = torch.zeros(6, dtype=torch.float64, device="cuda")
    g = _dptr(grad_depth, torch.float32, (sensor.height, sensor.width), "grad_depth") if grad_depth is not None else None
    tw = _dptr(twist_grad, torch.float64, (6,), "twist_grad")
    vg = _dptr(voxel_grad, torch.float32, (map.max_blocks, 512), "voxel_grad") if voxel_grad is not None else None
    jc = _dptr(jac, torch.float32, (sensor.height, sensor.width, 6), "jac") if jac is not None else None
    s = sensor._c()
    _, tp = _m16(T_WS)
    _check(L.se_gpu_raycast_adjoint(map.h, C.byref(s), tp, g, tw, vg, jc, _stream(stream)),
           "se_gpu_raycast_adjoint")
    return twist_grad


def track_noalloc(sensor: PinholeCamera, config: TrackerConfig, depth, T_WS,
                  surface_point_cloud_W, surface_normals_W, stream=None):
    """One-level ICP that allocates no device memory (no counterpart in the reference).

    For callers that cannot allocate while they track; the scratch is a static device array
    inside the library, shared by all calls, so calls must not overlap on the GPU. The first
    call on a device also loads that part of the library onto the device (lazy module
    loading), which allocates the array: make it at start-up. ``config``
    must have exactly one level. T_WS (float32 4x4 numpy, C-contiguous) is updated in place.
    Returns (accepted, reduction[32])."""
    import torch
    L = library()
    d = _dptr(depth, torch.float32, (sensor.height, sensor.width), "depth")
    p = _dptr(surface_point_cloud_W, torch.float32, (sensor.height, sensor.width, 3), "points")
    n = _dptr(surface_normals_W, torch.float32, (sensor.height, sensor.width, 3), "normals")
    if not (isinstance(T_WS, np.ndarray) and T_WS.dtype == np.float32 and T_WS.shape == (4, 4)
            and T_WS.flags.c_contiguous):
        raise SeGpuError("T_WS must be a C-contiguous float32 4x4 numpy array (updated in place)")
    s = sensor._c()
    c = config._c()
    acc = C.c_int()
    red = (C.c_float * 32)()
    _check(L.se_gpu_track_noalloc(C.byref(s), C.byref(c), d, p, n, T_WS.ctypes.data_as(_F16),
                                  C.byref(acc), red, _stream(stream)), "se_gpu_track_noalloc")
    return bool(acc.value), np.array(red[:], np.float32)


def marching_cube(map: Map, stream=None):
    """se::algorithms::marching_cube(octree): faces [N, 3, 3] (float32 CUDA tensor, vertices in
    voxel units of the map frame; world = T_WM (res v)); multi-res and occupancy maps are meshed
    by the dual marching cubes at their blocks' current scales."""
    import torch
    L = library()
    n = C.c_int64()
    _check(L.se_gpu_marching_cube(map.h, None, 0, C.byref(n), _stream(stream)), "se_gpu_marching_cube")
    out = torch.empty((max(n.value, 1), 3, 3), dtype=torch.float32, device="cuda")
    cap = n.value
    _check(L.se_gpu_marching_cube(map.h, C.c_void_p(out.data_ptr()), cap, C.byref(n), _stream(stream)),
           "se_gpu_marching_cube")
    return out[: n.value]


def dual_marching_cube(map: Map, min_desired_scale=0, stream=None):
    """se::algorithms::marching_cube(octree, min_desired_scale) for a multi-res TSDF or occupancy
    map: (faces [N, 3, 3] float32, scales [N] int8), CUDA tensors."""
    import torch
    L = library()
    n = C.c_int64()
    _check(L.se_gpu_dual_marching_cube(map.h, int(min_desired_scale), None, None, 0, C.byref(n), _stream(stream)),
           "se_gpu_dual_marching_cube")
    out = torch.empty((max(n.value, 1), 3, 3), dtype=torch.float32, device="cuda")
    sc = torch.empty(max(n.value, 1), dtype=torch.int8, device="cuda")
    cap = n.value
    _check(L.se_gpu_dual_marching_cube(map.h, int(min_desired_scale), C.c_void_p(out.data_ptr()),
                                       C.c_void_p(sc.data_ptr()), cap, C.byref(n), _stream(stream)),
           "se_gpu_dual_marching_cube")
    return out[: n.value], sc[: n.value]


def save_mesh(faces, filename, T_OV=None, scales=None):
    """io::save_mesh: faces [N, 3, 3] (numpy or tensor) transformed by T_OV (4x4, default the
    identity), written as .ply, .vtk or .obj; scales [N] (default 0) colour the faces."""
    f = np.ascontiguousarray(faces.cpu().numpy() if hasattr(faces, "cpu") else faces, np.float32).reshape(-1, 9)
    sc = None
    if scales is not None:
        sc = np.ascontiguousarray(scales.cpu().numpy() if hasattr(scales, "cpu") else scales, np.int8).reshape(-1)
        if len(sc) != len(f):
            raise SeGpuError("save_mesh: one scale per face")
    _, tp = _m16(np.eye(4) if T_OV is None else T_OV)
    _check(library().se_gpu_save_mesh(f.ctypes.data, None if sc is None else sc.ctypes.data, len(f), tp,
                                      str(filename).encode()), "se_gpu_save_mesh")


def save_point_cloud_vtk(points, filename, T_WC=None):
    """io::save_point_cloud_vtk: points [..., 3] transformed by T_WC."""
    p = np.ascontiguousarray(points.cpu().numpy() if hasattr(points, "cpu") else points, np.float32).reshape(-1, 3)
    _, tp = _m16(np.eye(4) if T_WC is None else T_WC)
    _check(library().se_gpu_save_point_cloud_vtk(p.ctypes.data, len(p), tp, str(filename).encode()),
           "se_gpu_save_point_cloud_vtk")


def mc_case_table():
    """(ntri[256], tri[256, 15]) of the library's marching-cubes case table (host only)."""
    ntri = np.zeros(256, np.int32)
    tri = np.zeros(256 * 15, np.int32)
    _check(library(build_if_missing=True).se_gpu_mc_case_table(ntri.ctypes.data, tri.ctypes.data),
           "se_gpu_mc_case_table")
    return ntri, tri.reshape(256, 15)


def downsample_depth(depth, out, map=None, stream=None):
    """se::preprocessor::downsample_depth(input, output): median downsampling of a [H, W] float32
    CUDA tensor into out ([H / r, W / r]); map (int64, out's shape, optional) receives the chosen
    input pixel x + y * W. Returns map."""
    import torch
    H, W = depth.shape
    h, w = out.shape
    pin = _dptr(depth, torch.float32, (H, W), "depth")
    pout = _dptr(out, torch.float32, (h, w), "out")
    pmap = _dptr(map, torch.int64, (h, w), "map") if map is not None else None
    _check(library().se_gpu_downsample_depth(pin, W, H, pout, w, h, pmap, _stream(stream)),
           "se_gpu_downsample_depth")
    return map


def bilateral_filter(depth, out=None, radius=2, sigma_space=4.0, sigma_range=0.03, stream=None):
    """The bilateral pre-filter of the tracking input (not in the reference; defined in
    se_gpu.h): a [H, W] float32 CUDA tensor into out (a new tensor when None)."""
    import torch
    H, W = depth.shape
    pin = _dptr(depth, torch.float32, (H, W), "depth")
    if out is None:
        out = torch.empty_like(depth)
    pout = _dptr(out, torch.float32, (H, W), "out")
    cfg = _BilateralConfig(int(radius), float(sigma_space), float(sigma_range))
    L = library()
    _check(L.se_gpu_bilateral_filter(pin, pout, W, H, C.byref(cfg), _stream(stream)), "se_gpu_bilateral_filter")
    return out


class FramePipeline:
    """The reference application's per-frame loop (track, integrate, raycast) as one captured
    CUDA graph with the pose on the device. ``depth`` is the frame's input buffer (write the
    next depth image into it, then call ``run``); ``points_W`` / ``normals_W`` hold the last
    raycast. Not part of the reference's interface: it batches the three blocking calls."""

    def __init__(self, map: Map, sensor: PinholeCamera, tracker: "Tracker" = None):
        import torch
        self.map, self.sensor, self.tracker = map, sensor, tracker
        self._L = library()
        h = C.c_void_p()
        s = sensor._c()
        _check(self._L.se_gpu_frame_create(map.h, tracker.h if tracker else None, C.byref(s),
                                           C.byref(h)), "se_gpu_frame_create")
        self.h = h
        d, p, n, sc = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_void_p()
        _check(self._L.se_gpu_frame_buffers(h, C.byref(d), C.byref(p), C.byref(n), C.byref(sc)),
               "se_gpu_frame_buffers")
        H, W = sensor.height, sensor.width
        self.depth = _wrap_device(d.value, (H, W), torch.float32, self)
        self.points_W = _wrap_device(p.value, (H, W, 3), torch.float32, self)
        self.normals_W = _wrap_device(n.value, (H, W, 3), torch.float32, self)

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self._L.se_gpu_frame_destroy(h)
            self.h = None

    def set_bilateral(self, radius=2, sigma_space=4.0, sigma_range=0.03, enable=True):
        """Track on the bilateral-filtered input (integration keeps the raw depth)."""
        cfg = _BilateralConfig(int(radius), float(sigma_space), float(sigma_range))
        _check(self._L.se_gpu_frame_set_bilateral(self.h, C.byref(cfg) if enable else None),
               "se_gpu_frame_set_bilateral")

    def set_pose(self, T_WS, timestamp=0):
        _, tp = _m16(T_WS)
        _check(self._L.se_gpu_frame_set_pose(self.h, tp, int(timestamp)), "se_gpu_frame_set_pose")

    def run(self, track=True, stream=None, depth=None):
        """One frame: [track] + integrate + raycast, asynchronous on stream. With ``depth`` (a
        host float32 H x W array or CPU tensor, pinned for an asynchronous copy) the frame's
        input is copied from it first; otherwise ``self.depth`` holds it."""
        if depth is None:
            _check(self._L.se_gpu_frame_run(self.h, 1 if track else 0, _stream(stream)), "se_gpu_frame_run")
            return
        if hasattr(depth, "is_cuda"):
            if depth.is_cuda or depth.dtype != self.depth.dtype or not depth.is_contiguous():
                raise SeGpuError("depth must be a contiguous float32 host tensor")
            if tuple(depth.shape) != tuple(self.depth.shape):
                raise SeGpuError("depth has the wrong shape")
            ptr = depth.data_ptr()
        else:
            depth = np.ascontiguousarray(depth, np.float32)
            if depth.shape != tuple(self.depth.shape):
                raise SeGpuError("depth has the wrong shape")
            ptr = depth.ctypes.data
        _check(self._L.se_gpu_frame_run_host(self.h, C.c_void_p(ptr), 1 if track else 0, _stream(stream)),
               "se_gpu_frame_run_host")

    def pose(self, stream=None):
        T = np.zeros(16, np.float32)
        acc = C.c_int()
        _check(self._L.se_gpu_frame_get_pose(self.h, T.ctypes.data_as(_F16), C.byref(acc),
                                             _stream(stream)), "se_gpu_frame_get_pose")
        return T.reshape(4, 4), bool(acc.value)

    def autotune(self, runs=12):
        """Time the next ``runs`` runs with candidate launch geometries of the voxel update and
        the raycast (each run synchronises) and keep the fastest; results are unchanged."""
        _check(self._L.se_gpu_frame_autotune(self.h, int(runs)), "se_gpu_frame_autotune")

    def tiles(self):
        """({"update_ctas_per_sm", "update_voxels_per_lane_round", "raycast_warp_tile"},
        tuning runs left)."""
        t = (C.c_int * 3)()
        left = C.c_int()
        _check(self._L.se_gpu_frame_tiles(self.h, t, C.byref(left)), "se_gpu_frame_tiles")
        return ({"update_ctas_per_sm": t[0], "update_voxels_per_lane_round": t[1],
                 "raycast_warp_tile": "8x4" if t[2] == 0 else "16x2"}, left.value)

    def pose_async(self, pose12, accepted, stream=None):
        """Enqueue the pose read into pinned host tensors: ``pose12`` (12 float32, the row-major
        3x4 T_WS) and ``accepted`` (1 int32); valid once the stream has passed this point."""
        for t, dt, n in ((pose12, "float32", 12), (accepted, "int32", 1)):
            if t.is_cuda or str(t.dtype) != "torch." + dt or t.numel() != n or not t.is_contiguous():
                raise SeGpuError("pose_async wants contiguous host tensors: 12 float32 and 1 int32")
        _check(self._L.se_gpu_frame_get_pose_async(self.h, C.c_void_p(pose12.data_ptr()),
                                                   C.c_void_p(accepted.data_ptr()), _stream(stream)),
               "se_gpu_frame_get_pose_async")


def _wrap_device(ptr, shape, dtype, owner):
    """A torch tensor view of library-owned device memory (kept alive by owner)."""
    import torch

    class _Holder:
        def __init__(self, p, nbytes):
            self.__cuda_array_interface__ = {
                "shape": (nbytes // 4,) if dtype == torch.float32 else (nbytes,),
                "typestr": "<f4" if dtype == torch.float32 else "|i1",
                "data": (p, False), "version": 3}

    n = int(np.prod(shape))
    nbytes = n * (4 if dtype == torch.float32 else 1)
    t = torch.as_tensor(_Holder(ptr, nbytes), device="cuda").view(*shape)
    t._se_owner = owner
    return t
