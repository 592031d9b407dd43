"""The kernels' fast quotient (div_small_int, Markstein correction of the
hardware reciprocal estimate) equals IEEE division __fdiv_rn for every pair
of integers 0 <= a <= b <= 65536 (and sampled a up to 2^24)."""
import os
import subprocess

import pytest

from tests.conftest import REPO

pytestmark = pytest.mark.gpu


def test_division_exhaustive(tmp_path):
    from siml_gb300 import build
    exe = str(tmp_path / "divtest")
    subprocess.run([build._nvcc(), build.GENCODE, "-O3", "-std=c++17", "--fmad=false",
                    "-I", os.path.join(REPO, "siml_gb300", "csrc"), "-I", os.path.join(REPO, "include"),
                    os.path.join(REPO, "tests", "native", "division_test.cu"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches: 0" in r.stdout
