// The RGBA LUT of set_transfer_functions, built on the device from the
// transfer functions' control points (pyvr/transferfunctions/color.py:185-197,
// opacity.py:185-193, pyvr/moderngl_renderer/manager.py:162-175): entry i is
// each channel's piecewise-linear interpolation at x_i = linspace(0, 1, size)[i],
// evaluated in double and rounded once to float32, with the "clear entry"
// prefix counts of the empty-space skip computed in the same launch.
//
// The interpolation restates numpy.interp: below the first control point the
// first value, above the last (or at it) the last value, otherwise the
// segment j = the last point with xp[j] <= x; at x == xp[j] the value fp[j];
// else slope = (fp[j+1] - fp[j]) / (xp[j+1] - xp[j]) and
// slope * (x - xp[j]) + fp[j] (if that is NaN, from the right end; if still
// NaN and both ends are equal, the end value).  linspace(0, 1, n) is
// i * (1 / (n - 1)) with the last entry exactly 1.
#include <cmath>
#include <cstring>

#include "pvr_internal.h"

namespace pvr {
namespace {

constexpr int kMaxPoints = 256;
constexpr int kBuildThreads = 1024;
constexpr int kMaxBuildSize = 1 << 16;

struct LutBuildParams {
    float4 *lut;
    int *prefix;
    int size;
    int n_ctf, n_otf;
    double cx[kMaxPoints];
    double crgb[kMaxPoints][3];
    double ox[kMaxPoints];
    double oa[kMaxPoints];
};

__device__ double interp(double x, const double *xp, const double *fp, int stride, int n) {
    if (n == 1) return fp[0];
    if (x != x) return x;
    if (x < xp[0]) return fp[0];
    if (x >= xp[n - 1]) return fp[(n - 1) * stride];
    int lo = 0, hi = n;  // last j with xp[j] <= x
    while (lo < hi) {
        const int mid = lo + ((hi - lo) >> 1);
        if (x >= xp[mid]) lo = mid + 1;
        else hi = mid;
    }
    const int j = lo - 1;
    const double y0 = fp[j * stride], y1 = fp[(j + 1) * stride];
    if (xp[j] == x) return y0;
    const double slope = (y1 - y0) / (xp[j + 1] - xp[j]);
    double r = slope * (x - xp[j]) + y0;
    if (r != r) {
        r = slope * (x - xp[j + 1]) + y1;
        if (r != r && y0 == y1) r = y0;
    }
    return r;
}

__global__ void __launch_bounds__(kBuildThreads) lut_build_kernel(const __grid_constant__ LutBuildParams p) {
    __shared__ int s_count[kBuildThreads];
    const int chunk = (p.size + kBuildThreads - 1) / kBuildThreads;
    const int i0 = threadIdx.x * chunk, i1 = min(p.size, i0 + chunk);
    const double step = p.size > 1 ? 1.0 / (double)(p.size - 1) : 0.0;
    int count = 0;
    for (int i = i0; i < i1; ++i) {
        const double x = (p.size > 1 && i == p.size - 1) ? 1.0 : (double)i * step;
        float4 e;
        e.x = __double2float_rn(interp(x, p.cx, &p.crgb[0][0], 3, p.n_ctf));
        e.y = __double2float_rn(interp(x, p.cx, &p.crgb[0][1], 3, p.n_ctf));
        e.z = __double2float_rn(interp(x, p.cx, &p.crgb[0][2], 3, p.n_ctf));
        e.w = __double2float_rn(interp(x, p.ox, p.oa, 1, p.n_otf));
        p.lut[i] = e;
        const bool clear = e.w == 0.0f && isfinite(e.x) && isfinite(e.y) && isfinite(e.z);
        count += clear ? 0 : 1;
    }
    // exclusive scan of the per-thread counts (Hillis-Steele over the block)
    s_count[threadIdx.x] = count;
    __syncthreads();
    for (int off = 1; off < kBuildThreads; off <<= 1) {
        const int v = threadIdx.x >= off ? s_count[threadIdx.x - off] : 0;
        __syncthreads();
        s_count[threadIdx.x] += v;
        __syncthreads();
    }
    int run = s_count[threadIdx.x] - count;  // entries before i0 that are not clear
    for (int i = i0; i < i1; ++i) {
        p.prefix[i] = run;
        const float4 e = p.lut[i];
        run += (e.w == 0.0f && isfinite(e.x) && isfinite(e.y) && isfinite(e.z)) ? 0 : 1;
    }
    if (threadIdx.x == kBuildThreads - 1) p.prefix[p.size] = s_count[kBuildThreads - 1];
}

bool sorted_finite(const double *x, int n) {
    for (int i = 0; i < n; ++i) {
        if (!std::isfinite(x[i])) return false;
        if (i && x[i] < x[i - 1]) return false;
    }
    return true;
}

}  // namespace
}  // namespace pvr

using pvr::fail;

extern "C" int pvr_lut_build(pvr_lut *l, const double *ctf_x, const double *ctf_rgb, int n_ctf,
                             const double *otf_x, const double *otf_a, int n_otf, int size, void *stream) {
    if (!l) return fail(PVR_ERR_VALUE, "null LUT handle");
    if (!ctf_x || !ctf_rgb || !otf_x || !otf_a) return fail(PVR_ERR_VALUE, "control points are NULL");
    if (n_ctf < 1 || n_ctf > pvr::kMaxPoints || n_otf < 1 || n_otf > pvr::kMaxPoints)
        return fail(PVR_ERR_VALUE, "1..%d control points per function", pvr::kMaxPoints);
    if (size < 1 || size > pvr::kMaxBuildSize)
        return fail(PVR_ERR_VALUE, "LUT size must be in 1..%d, got %d", pvr::kMaxBuildSize, size);
    if (!pvr::sorted_finite(ctf_x, n_ctf) || !pvr::sorted_finite(otf_x, n_otf))
        return fail(PVR_ERR_VALUE, "control point positions must be finite and sorted");
    if (size > l->cap) {
        if (l->d_lut || l->d_prefix) {
            cudaDeviceSynchronize();  // a queued batch may still read the old table
            cudaFree(l->d_lut);
            cudaFree(l->d_prefix);
            l->d_lut = nullptr;
            l->d_prefix = nullptr;
            l->cap = 0;
        }  // a new table waits for nothing
        PVR_CUDA(cudaMalloc(&l->d_lut, (size_t)size * sizeof(float4)));
        PVR_CUDA(cudaMalloc(&l->d_prefix, (size_t)(size + 1) * sizeof(int)));
        l->cap = size;
    }
    pvr::LutBuildParams p;
    std::memset(&p, 0, sizeof(p));
    p.lut = l->d_lut;
    p.prefix = l->d_prefix;
    p.size = size;
    p.n_ctf = n_ctf;
    p.n_otf = n_otf;
    for (int i = 0; i < n_ctf; ++i) {
        p.cx[i] = ctf_x[i];
        for (int c = 0; c < 3; ++c) p.crgb[i][c] = ctf_rgb[3 * i + c];
    }
    for (int i = 0; i < n_otf; ++i) {
        p.ox[i] = otf_x[i];
        p.oa[i] = otf_a[i];
    }
    void *args[] = {&p};
    PVR_CUDA(cudaLaunchKernel((const void *)pvr::lut_build_kernel, dim3(1), dim3(pvr::kBuildThreads), args, 0,
                              (cudaStream_t)stream));
    l->size = size;
    // the table is not on the host: the march keeps the exact per-brick skip
    // test, which finds no clear range when the table has no clear entry
    l->has_clear = true;
    return PVR_OK;
}

extern "C" int pvr_lut_read(const pvr_lut *l, float *rgba_out) {
    if (!l || !rgba_out) return fail(PVR_ERR_VALUE, "NULL argument");
    PVR_CUDA(cudaDeviceSynchronize());
    PVR_CUDA(cudaMemcpy(rgba_out, l->d_lut, (size_t)l->size * sizeof(float4), cudaMemcpyDeviceToHost));
    return PVR_OK;
}
