// Exhaustive check of the float32 formulation of uint8 normals
// (pyvr_gb300/csrc/normals.cuh, GradientArith<uint8_t>) against numpy's
// float64 arithmetic: every gradient triple (g0, g1, g2) a uint8 volume can
// produce -- each component an integer in [-255, 255] (one-sided
// differences) or a multiple of 0.5 in [-127.5, 127.5] (central ones) -- and
// component 0 of the normal, which depends on g0 and S = g0^2 + g1^2 + g2^2
// only (so it covers every component).  Prints "triples mismatches fallbacks".
#include <cstdio>
#include <vector>

#include "normals.cuh"

__global__ void check(const float *g, int n, unsigned long long *mismatches, unsigned long long *fallbacks) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)n * n) return;
    const float g0 = g[t / n], g1 = g[t % n];
    unsigned long long bad = 0, slow = 0;
    for (int k = 0; k < n; ++k) {
        const float g2 = g[k];
        const pvr::U8Norm nn = pvr::u8_norm(g0, g1, g2);
        const float got = pvr::GradientArith<uint8_t>::finish(g0, g1, g2).x;
        const double d0 = g0, d1 = g1, d2 = g2;
        const double s = __dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2));
        const double nrm = __dadd_rn(__dsqrt_rn(s), 1e-8);
        const float want = __double2float_rn(__ddiv_rn(d0, nrm));
        bad += __float_as_uint(got) != __float_as_uint(want);
        // the fallback is taken where the float pair does not decide the rounding
        if (g0 != 0.0f) {
            const float qh = __fdiv_rn(g0, nn.nh);
            const float e2 = fmaf(-qh, nn.nl, fmaf(-qh, nn.nh, g0));
            const float corr = __fdiv_rn(e2, nn.nh);
            const float eb = fabsf(qh) * 3.637978807091713e-12f;
            slow += __fadd_rn(qh, __fsub_rn(corr, eb)) != __fadd_rn(qh, __fadd_rn(corr, eb));
        }
    }
    if (bad) atomicAdd(mismatches, bad);
    if (slow) atomicAdd(fallbacks, slow);
}

int main() {
    std::vector<float> g;
    for (int i = -255; i <= 255; ++i) g.push_back((float)i);
    for (int i = -255; i <= 255; i += 2) g.push_back(0.5f * (float)i);  // the odd halves
    const int n = (int)g.size();
    float *dg = nullptr;
    unsigned long long *dc = nullptr;
    if (cudaMalloc(&dg, n * sizeof(float)) != cudaSuccess || cudaMalloc(&dc, 2 * sizeof(unsigned long long)) != cudaSuccess) {
        std::printf("error: cudaMalloc\n");
        return 1;
    }
    cudaMemcpy(dg, g.data(), n * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemset(dc, 0, 2 * sizeof(unsigned long long));
    const long long threads = (long long)n * n;
    check<<<(unsigned)((threads + 255) / 256), 256>>>(dg, n, dc, dc + 1);
    unsigned long long c[2] = {0, 0};
    cudaError_t e = cudaMemcpy(c, dc, sizeof(c), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        std::printf("error: %s\n", cudaGetErrorString(e));
        return 1;
    }
    std::printf("%lld %llu %llu\n", threads * n, c[0], c[1]);
    cudaFree(dg);
    cudaFree(dc);
    return 0;
}
