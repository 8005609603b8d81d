"""uint8 normals in float32 arithmetic equal numpy's float64 ones, for every
gradient triple a uint8 volume can produce (767^3 = 451 M triples, checked
exhaustively on the GPU by tests/cuda/u8_normals_check.cu, which includes the
library's own pyvr_gb300/csrc/normals.cuh)."""

import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "pyvr_gb300", "csrc")


def test_u8_normals_exhaustive(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "u8_normals_check")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-std=c++17",
                    f"-I{CSRC}", os.path.join(HERE, "cuda", "u8_normals_check.cu"), "-o", exe],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=300).stdout.split()
    triples, mismatches, fallbacks = (int(x) for x in out)
    assert triples == 767 ** 3
    assert mismatches == 0, f"{mismatches} of {triples} components differ from numpy's float64"
    # the float64 fallback is rare: the float pair decides almost every rounding
    assert fallbacks < 1e-4 * triples, fallbacks
