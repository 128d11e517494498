"""The CPU oracle built with AddressSanitizer and UndefinedBehaviorSanitizer
(-fsanitize=address,undefined) runs its paths on small inputs (tests/sanitize/oracle_workload.py)
without a report: no out-of-bounds access, use after free or undefined operation in the
restatement the GPU path is checked against. Host only; the sanitizer runtime is preloaded
into a child Python process."""
import os
import shutil
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
FLAGS = ["-std=c++17", "-O1", "-g", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
         "-Wno-unknown-pragmas", "-Wno-unused-function", "-Wno-subobject-linkage",
         "-fsanitize=address,undefined", "-fno-omit-frame-pointer"]


def test_oracle_under_sanitizers(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    asan = subprocess.run([cxx, "-print-file-name=libasan.so"], capture_output=True, text=True).stdout.strip()
    if not os.path.isabs(asan) or not os.path.exists(asan):
        pytest.skip("no AddressSanitizer runtime")
    objs, procs = [], []
    for src in ("se_oracle.cpp", "se_oracle_occ.cpp"):
        obj = str(tmp_path / (src + ".o"))
        procs.append(subprocess.Popen([cxx, *FLAGS, "-c", os.path.join(ROOT, "oracle", src), "-o", obj]))
        objs.append(obj)
    assert all(p.wait() == 0 for p in procs)
    lib = str(tmp_path / "libse_oracle_san.so")
    subprocess.run([cxx, *FLAGS, "-shared", *objs, "-o", lib], check=True)
    env = dict(os.environ, SE_ORACLE_LIB=lib, LD_PRELOAD=asan, ASAN_OPTIONS="detect_leaks=0",
               UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1")
    r = subprocess.run([sys.executable, os.path.join(HERE, "sanitize", "oracle_workload.py")], env=env,
                       capture_output=True, text=True, timeout=600)
    assert "runtime error" not in r.stderr and "AddressSanitizer" not in r.stderr, r.stderr[-4000:]
    assert r.returncode == 0 and "workload ok" in r.stdout, r.stderr[-4000:]
