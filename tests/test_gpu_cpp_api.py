"""The C++ mirror of the reference API (include/se_gpu.hpp) builds against libse_gpu.so and
runs the reference's wall scenario through se::gpu::MapIntegrator / raycast_volume / Tracker."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build_cpp_test(tmp_path):
    from supereight2_gb300 import build
    lib = build.build()
    exe = str(tmp_path / "api_test")
    cmd = [build.nvcc(), "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "api_test.cpp"), "-o", exe,
           "-L", os.path.dirname(lib), "-lse_gpu", "-Xlinker", "-rpath=" + os.path.dirname(lib)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_cpp_header_compiles(tmp_path):
    """Host-only compile of the header (no GPU needed)."""
    src = tmp_path / "inc.cpp"
    src.write_text('#include "se_gpu.hpp"\nint main() { return se::gpu::identity()[0] == 1.0f ? 0 : 1; }\n')
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    "-fsyntax-only", str(src)], check=True)


@pytest.mark.gpu
def test_cpp_api_wall(tmp_path):
    exe = _build_cpp_test(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "cpp api ok" in r.stdout
