"""Host-side calls of libse_gpu.so that need no GPU, for the sanitizer test
(tests/test_abi_sanitized.py runs this script on an AddressSanitizer / UndefinedBehaviorSanitizer
build of the library, path in argv[1]): every entry point of include/se_gpu.h called with null
pointers and zero sizes returns a status (or, for the string functions, a string) without
touching memory it does not own; the status strings; the mesh and point-cloud writers on host
arrays, with supported and refused file names."""
import ctypes as C
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import supereight2_gb300 as se  # noqa: E402

L = C.CDLL(sys.argv[1])
for name, (res, args) in se.SIGNATURES.items():
    fn = getattr(L, name)
    fn.restype = res
    fn.argtypes = args


def _zero(t):
    if t in (C.c_int, C.c_int64, C.c_longlong, C.c_uint, C.c_int8, C.c_uint64, C.c_size_t):
        return 0
    if t in (C.c_float, C.c_double):
        return 0.0
    return None  # pointers, structures by pointer, strings


# with null pointers: the destructors and the profiling switches accept them, every other entry
# point refuses them (SE_GPU_ERR_BAD_ARG = 1)
ACCEPT_NULL = {"se_gpu_map_destroy", "se_gpu_tracker_destroy", "se_gpu_frame_destroy", "se_gpu_occ_batch_destroy",
               "se_gpu_profiling_enable", "se_gpu_profiling_read"}
n_status = 0
for name, (res, args) in sorted(se.SIGNATURES.items()):
    out = getattr(L, name)(*[_zero(t) for t in args])
    if res is not C.c_int:
        assert out is not None, name
    elif name == "se_gpu_abi_version" or name == "se_gpu_profiling_count":
        assert out >= 1, (name, out)
    else:
        assert out == (0 if name in ACCEPT_NULL else 1), (name, out)
        n_status += 1
for s in range(7):
    assert L.se_gpu_status_string(s)
assert L.se_gpu_abi_version() >= 1
assert L.se_gpu_map_create(None, None) == 1 and L.se_gpu_last_error()

faces = np.random.default_rng(0).uniform(0, 4, (5, 3, 3)).astype(np.float32)
scales = np.arange(5, dtype=np.int8) % 3
T = np.eye(4, dtype=np.float32).reshape(16)
fp = faces.ctypes.data_as(C.POINTER(C.c_float))
Tp = T.ctypes.data_as(C.POINTER(C.c_float))
with tempfile.TemporaryDirectory() as d:
    for ext in ("ply", "vtk", "obj"):
        assert L.se_gpu_save_mesh(fp, scales.ctypes.data_as(C.POINTER(C.c_int8)), 5, Tp,
                                  os.path.join(d, "m." + ext).encode()) == 0
        assert L.se_gpu_save_mesh(fp, None, 0, Tp, os.path.join(d, "e." + ext).encode()) == 0
    assert L.se_gpu_save_mesh(fp, None, 5, Tp, os.path.join(d, "m.png").encode()) == 1
    pts = np.random.default_rng(1).uniform(-1, 1, (9, 3)).astype(np.float32)
    assert L.se_gpu_save_point_cloud_vtk(pts.ctypes.data_as(C.POINTER(C.c_float)), 9, Tp,
                                         os.path.join(d, "p.vtk").encode()) == 0
print("abi workload ok", n_status)
