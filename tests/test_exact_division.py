"""The voxel-coordinate division x / res of the GPU path (div_res: a multiply by RN(1/res) and
one fused-multiply-add correction, Markstein's correction step) equals the IEEE quotient for
every float in [2^-20, 2^14) at three resolutions: the raycast and the field queries keep their
bit-exact voxel coordinates without a division instruction per sample."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path_factory.mktemp("div") / "exact_division_check")
    subprocess.run([cc, "-O2", "-ffp-contract=off", "-o", exe, os.path.join(HERE, "exact_division_check.c"), "-lm"],
                   check=True)
    return exe


@pytest.mark.parametrize("res", ["0.01", "0.02", "0.4"])
def test_division_by_resolution_is_exact(checker, res):
    out = subprocess.run([checker, res, "0x35800000", "0x46800000"], check=True, capture_output=True, text=True)
    bad, n = (int(v) for v in out.stdout.split())
    assert n == 0x46800000 - 0x35800000
    assert bad == 0
