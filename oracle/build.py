"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``se_oracle.cpp`` (TSDF maps, ICP) and ``se_oracle_occ.cpp`` (occupancy maps) into ``oracle/_build/libse_oracle.so`` with OpenMP and
``-ffp-contract=off`` (no fused multiply-add, on x86-64 and aarch64 alike) so that its float
arithmetic follows the operation order written in the source.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libse_oracle.so")
SOURCES = [os.path.join(HERE, f) for f in ("se_oracle.cpp", "se_oracle_occ.cpp")]
HEADERS = [os.path.join(HERE, f) for f in ("se_oracle.h", "oracle_common.hpp")]


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(p) > t for p in SOURCES + HEADERS + [__file__])


def build(force: bool = False) -> str:
    """Compile the oracle if it is missing or older than its sources; return the .so path."""
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + ".tmp"
    cmd = [
        "g++", "-std=c++17", "-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
        "-fPIC", "-shared", "-Wall", "-Wno-unknown-pragmas", "-Wno-unused-function",
        *SOURCES, "-o", tmp,
    ]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
