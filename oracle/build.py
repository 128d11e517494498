"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``se_oracle.cpp`` (TSDF maps, ICP) and ``se_oracle_occ.cpp`` (occupancy maps) into
``oracle/_build/libse_oracle.so`` with OpenMP and ``-ffp-contract=off`` (no fused multiply-add,
on x86-64 and aarch64 alike) so that its float arithmetic follows the operation order written in
the source; and ``se_oracle_f64.cpp`` (the same TSDF / ICP restatement with every float a
double) into ``oracle/_build/libse_oracle_f64.so``, linked with ``-Bsymbolic`` so that its calls
stay inside it although its exported names equal the FP32 library's.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libse_oracle.so")
LIB64_PATH = os.path.join(BUILD_DIR, "libse_oracle_f64.so")
SOURCES = [os.path.join(HERE, f) for f in ("se_oracle.cpp", "se_oracle_occ.cpp")]
SOURCES64 = [os.path.join(HERE, "se_oracle_f64.cpp")]
HEADERS = [os.path.join(HERE, f) for f in ("se_oracle.h", "oracle_common.hpp", "se_oracle.cpp")] + [
    os.path.join(os.path.dirname(HERE), "supereight2_gb300", "csrc", "mc_case_table.inc")]
FLAGS = ["-std=c++17", "-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-Wall",
         "-Wno-unknown-pragmas", "-Wno-unused-function", "-Wno-subobject-linkage"]


def _stale(lib, sources) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(p) > t for p in sources + HEADERS + [__file__])


def _compile(lib, sources, extra):
    tmp = lib + ".tmp"
    return subprocess.Popen(["g++", *FLAGS, *extra, *sources, "-o", tmp]), tmp, lib


def build(force: bool = False) -> str:
    """Compile both oracle libraries if missing or older than their sources (in parallel);
    return the FP32 library's path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    jobs = []
    if force or _stale(LIB_PATH, SOURCES):
        jobs.append(_compile(LIB_PATH, SOURCES, []))
    if force or _stale(LIB64_PATH, SOURCES64):
        jobs.append(_compile(LIB64_PATH, SOURCES64, ["-Wl,-Bsymbolic"]))
    for proc, tmp, lib in jobs:
        if proc.wait() != 0:
            raise subprocess.CalledProcessError(proc.returncode, "g++ " + lib)
        os.replace(tmp, lib)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
