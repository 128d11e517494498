"""ctypes bindings of the FP64 run of the oracle (``libse_oracle_f64.so``: the TSDF / ICP
restatement with every float a double). Test and report infrastructure only, like the FP32
oracle: the product never loads it."""
import ctypes as C

import numpy as np

from . import build as _build

_lib = None


class Pinhole(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("fx", C.c_double), ("fy", C.c_double),
                ("cx", C.c_double), ("cy", C.c_double), ("near_plane", C.c_double),
                ("far_plane", C.c_double)]


class TrackerConfig(C.Structure):
    _fields_ = [("num_levels", C.c_int), ("iterations", C.c_int * 3),
                ("dist_threshold", C.c_double), ("normal_threshold", C.c_double),
                ("track_threshold", C.c_double), ("icp_threshold", C.c_double)]


class IntegrateStats(C.Structure):
    _fields_ = [("n_valid_pixels", C.c_longlong), ("n_new_blocks", C.c_longlong),
                ("n_frustum_blocks", C.c_longlong), ("n_updated_voxels", C.c_longlong)]


class TrackStats(C.Structure):
    _fields_ = [("converged_iterations", C.c_int * 3), ("accepted", C.c_int),
                ("reduction", C.c_double * 32)]


def lib():
    global _lib
    if _lib is None:
        _build.build()
        L = C.CDLL(_build.LIB64_PATH)
        f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        i8p = np.ctypeslib.ndpointer(np.int8, flags="C_CONTIGUOUS")
        vp = C.c_void_p
        sig = {
            "so_set_num_threads": (None, [C.c_int]),
            "so_map_create": (vp, [f64p, C.c_double, C.c_double, C.c_double, vp]),
            "so_map_create_multires": (vp, [f64p, C.c_double, C.c_double, C.c_double, vp]),
            "so_map_destroy": (None, [vp]),
            "so_map_num_blocks": (C.c_longlong, [vp]),
            "so_map_blocks": (None, [vp, vp, vp, vp, vp, vp]),
            "so_map_mr_blocks": (None, [vp, vp, vp, vp, vp, vp, vp, vp]),
            "so_integrate_depth": (None, [vp, f64p, C.POINTER(Pinhole), f64p, C.c_int,
                                          C.POINTER(IntegrateStats)]),
            "so_raycast_volume": (None, [vp, C.POINTER(Pinhole), f64p, f64p, f64p, i8p]),
            "so_track": (C.c_int, [C.POINTER(Pinhole), C.POINTER(TrackerConfig), f64p, f64p,
                                   f64p, f64p, C.POINTER(TrackStats)]),
            "so_bilateral_filter": (None, [f64p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, f64p]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def set_num_threads(n: int) -> None:
    lib().so_set_num_threads(int(n))


def pinhole(width, height, fx, fy, cx, cy, near_plane, far_plane) -> Pinhole:
    # the parameters are float in the reference's configuration; they enter as their float values
    f = lambda v: float(np.float32(v))  # noqa: E731
    return Pinhole(int(width), int(height), f(fx), f(fy), f(cx), f(cy), f(near_plane), f(far_plane))


def _m16(T):
    return np.ascontiguousarray(np.asarray(T, np.float64).reshape(16))


class OracleMap64:
    """The oracle's TSDF map (single- or multi-res) in FP64."""

    def __init__(self, dim, res, truncation_boundary_factor=8.0, max_weight=100.0, multires=False):
        d = np.ascontiguousarray(np.broadcast_to(np.asarray(dim, np.float64), (3,)))
        create = lib().so_map_create_multires if multires else lib().so_map_create
        self.h = create(d, float(np.float32(res)), float(truncation_boundary_factor), float(max_weight), None)
        self.multires = bool(multires)

    def __del__(self):
        if getattr(self, "h", None):
            lib().so_map_destroy(self.h)
            self.h = None

    def integrate_depth(self, depth, sensor: Pinhole, T_WC, timestamp=0) -> IntegrateStats:
        st = IntegrateStats()
        lib().so_integrate_depth(self.h, np.ascontiguousarray(depth, np.float64).reshape(-1), C.byref(sensor),
                                 _m16(T_WC), int(timestamp), C.byref(st))
        return st

    def raycast(self, sensor: Pinhole, T_WS):
        n = sensor.width * sensor.height
        pts = np.zeros((sensor.height, sensor.width, 3), np.float64)
        nrm = np.zeros((sensor.height, sensor.width, 3), np.float64)
        scale = np.zeros((sensor.height, sensor.width), np.int8)
        lib().so_raycast_volume(self.h, C.byref(sensor), _m16(T_WS), pts.reshape(n * 3), nrm.reshape(n * 3),
                                scale.reshape(n))
        return pts, nrm, scale

    def num_blocks(self) -> int:
        return int(lib().so_map_num_blocks(self.h))

    def blocks(self):
        n = self.num_blocks()
        keys = np.zeros(n, np.uint64)
        coords = np.zeros((n, 3), np.int32)
        tsdf = np.zeros((n, 512), np.float64)
        weight = np.zeros((n, 512), np.float64)
        ts = np.zeros(n, np.int32)
        if n:
            lib().so_map_blocks(self.h, keys.ctypes.data, coords.ctypes.data, tsdf.ctypes.data,
                                weight.ctypes.data, ts.ctypes.data)
        return keys, coords, tsdf, weight, ts

    def mr_blocks(self):
        n = self.num_blocks()
        keys = np.zeros(n, np.uint64)
        coords = np.zeros((n, 3), np.int32)
        arrs = [np.zeros((n, 585), np.float64) for _ in range(4)]
        scales = np.zeros((n, 2), np.int32)
        if n:
            lib().so_map_mr_blocks(self.h, keys.ctypes.data, coords.ctypes.data, *[a.ctypes.data for a in arrs],
                                   scales.ctypes.data)
        return (keys, coords, *arrs, scales)


def tracker_config(iterations=(10, 5, 4), dist_threshold=0.1, normal_threshold=0.8, track_threshold=0.15,
                   icp_threshold=1e-5) -> TrackerConfig:
    it = (C.c_int * 3)(*([int(i) for i in iterations] + [0] * (3 - len(iterations))))
    f = lambda v: float(np.float32(v))  # noqa: E731
    return TrackerConfig(len(iterations), it, f(dist_threshold), f(normal_threshold), f(track_threshold),
                         f(icp_threshold))


def track(sensor: Pinhole, config: TrackerConfig, depth, T_WS, ref_pts, ref_nrm):
    T = _m16(T_WS).copy()
    st = TrackStats()
    acc = lib().so_track(C.byref(sensor), C.byref(config), np.ascontiguousarray(depth, np.float64).reshape(-1),
                         T, np.ascontiguousarray(ref_pts, np.float64).reshape(-1),
                         np.ascontiguousarray(ref_nrm, np.float64).reshape(-1), C.byref(st))
    return bool(acc), T.reshape(4, 4), st


def bilateral_filter(depth, radius=2, sigma_space=4.0, sigma_range=0.03):
    d = np.ascontiguousarray(depth, np.float64)
    h, w = d.shape
    out = np.zeros_like(d)
    lib().so_bilateral_filter(d.reshape(-1), w, h, int(radius), float(sigma_space), float(sigma_range),
                              out.reshape(-1))
    return out
