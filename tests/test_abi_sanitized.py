"""The library's host code built with AddressSanitizer and UndefinedBehaviorSanitizer (nvcc's host
compiler with -fsanitize=address,undefined; the sm_103a device code unchanged) runs the calls
that need no GPU (tests/sanitize/abi_workload.py) without a report: every entry point with null
pointers and zero sizes (the destructors and profiling switches accept them, all others return
SE_GPU_ERR_BAD_ARG), the status strings, and the mesh and point-cloud writers on host arrays.
Host only; the sanitizer runtime is preloaded into a child Python process."""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SAN = ["-Xcompiler", "-fsanitize=address,-fsanitize=undefined,-fno-omit-frame-pointer"]


def test_abi_host_code_under_sanitizers(tmp_path):
    sys.path.insert(0, ROOT)
    from supereight2_gb300 import build
    try:
        nvcc = build.nvcc()
    except RuntimeError:
        pytest.skip("no nvcc")
    cxx = shutil.which("g++")
    asan = subprocess.run([cxx or "g++", "-print-file-name=libasan.so"], capture_output=True,
                          text=True).stdout.strip()
    if not os.path.isabs(asan) or not os.path.exists(asan):
        pytest.skip("no AddressSanitizer runtime")

    def compile_one(src):
        obj = str(tmp_path / (os.path.basename(src)[:-3] + ".o"))
        r = subprocess.run([nvcc, *build.common_flags(), *SAN, "-c", src, "-o", obj], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(compile_one, build.sources()))
    lib = str(tmp_path / "libse_gpu_san.so")
    subprocess.run([nvcc, *build.ARCH, "-shared", "-Xcompiler", "-fPIC", *SAN, *objs, "-o", lib], check=True)
    env = dict(os.environ, LD_PRELOAD=asan, ASAN_OPTIONS="detect_leaks=0:protect_shadow_gap=0",
               UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1")
    r = subprocess.run([sys.executable, os.path.join(HERE, "sanitize", "abi_workload.py"), lib], env=env,
                       capture_output=True, text=True, timeout=600)
    assert "runtime error" not in r.stderr and "AddressSanitizer" not in r.stderr, r.stderr[-4000:]
    assert r.returncode == 0 and "abi workload ok" in r.stdout, r.stderr[-4000:]
