"""The march's per-sample normalisation uses the correctly rounded reciprocal
square root (__frsqrt_rn); the oracle computes it as (float)(1.0/sqrt((double)x)).
This checks, for every positive float (denormals and +inf included), that the
two agree bit for bit, with a small CUDA program built here."""

import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

SRC = r"""
#include <cstdio>
#include <cstdint>
__device__ unsigned long long g_mis;
__global__ void probe(uint32_t lo, uint32_t hi) {
    const uint64_t n = (uint64_t)hi - lo + 1, stride = (uint64_t)gridDim.x * blockDim.x;
    unsigned long long mis = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float x = __uint_as_float(lo + (uint32_t)i);
        const float a = __frsqrt_rn(x);
        const float d = (float)(1.0 / sqrt((double)x));
        mis += __float_as_uint(a) != __float_as_uint(d);
    }
    atomicAdd(&g_mis, mis);
}
int main() {
    probe<<<152 * 8, 256>>>(1u, 0x7f800000u);
    cudaError_t e = cudaDeviceSynchronize();
    unsigned long long mis = ~0ULL;
    cudaMemcpyFromSymbol(&mis, g_mis, sizeof(mis));
    printf("%s %llu\n", cudaGetErrorString(e), mis);
    return e == cudaSuccess ? 0 : 1;
}
"""


def test_rsqrt_rounding_matches_double_formula(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / "rsqrt.cu"
    src.write_text(SRC)
    exe = tmp_path / "rsqrt"
    subprocess.check_call([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", str(exe), str(src)])
    out = subprocess.check_output([str(exe)], text=True, timeout=300).split()
    assert out == ["no", "error", "0"], out
