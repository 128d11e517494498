"""The C ABI library builds for sm_103a, loads, and exports exactly what include/se_gpu.h
declares. No GPU is needed: nothing here launches a kernel."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header):
    text = open(header).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(se_gpu_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_mapping_path():
    names = declared_functions(os.path.join(ROOT, "include", "se_gpu.h"))
    for required in ("se_gpu_map_create", "se_gpu_integrate_depth", "se_gpu_raycast",
                     "se_gpu_track", "se_gpu_map_download_blocks", "se_gpu_map_check"):
        assert required in names


def test_library_builds_loads_and_exports_every_declared_symbol():
    from supereight2_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    names = declared_functions(os.path.join(ROOT, "include", "se_gpu.h"))
    for n in names:
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    exported = sorted(l.split()[-1] for l in out.splitlines()
                      if " T " in l and l.split()[-1].startswith("se_gpu_"))
    assert exported == names


def test_python_mirror_binds_every_symbol():
    import supereight2_gb300 as se
    names = declared_functions(os.path.join(ROOT, "include", "se_gpu.h"))
    assert sorted(se.SIGNATURES) == names


def test_status_strings_without_device():
    import supereight2_gb300 as se
    L = se.library()
    assert L.se_gpu_abi_version() >= 1
    for s in range(7):
        assert L.se_gpu_status_string(s)


def test_library_targets_sm103a_only():
    from supereight2_gb300 import build
    flags = build.common_flags()
    assert "arch=compute_103a,code=sm_103a" in flags
    assert "--fmad=false" in flags


def test_no_device_is_reported_not_faulted():
    """Without a CUDA device map creation returns an error status (no CPU fallback)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    import supereight2_gb300 as se
    with pytest.raises(se.SeGpuError):
        se.Map(10.24, 0.02, max_blocks=1024)
