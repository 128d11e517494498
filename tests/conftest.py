"""Shared pytest configuration: the ``gpu`` marker and import paths.

Tests marked ``gpu`` need a GB300 (sm_103a) and the built ``libse_gpu.so``; everything else
runs on the CPU against the oracle, the scene generator and the library's exported symbols.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device of compute capability 10.3")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.set_num_threads(min(8, os.cpu_count() or 1))
    return pyoracle


@pytest.fixture(scope="session")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for gpu-marked tests")
    import supereight2_gb300 as se
    se.library()
    return se
