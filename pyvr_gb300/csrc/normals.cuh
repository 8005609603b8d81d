// Normals of the volume texels with the semantics of the reference's
// compute_normal_volume (pyvr/datasets/synthetic.py:109-122):
// g_axis = numpy.gradient along each array axis (central difference / 2
// inside, one-sided on the two faces, unit spacing), n = |g| + 1e-8 with the
// squares summed left to right, normal = g / n, cast to float32.  numpy
// evaluates this in float64 for integer input, in float16 (each operation
// rounded to half, sums accumulated in float) for float16 input, and in
// float32 for float32 input; GradientArith<T> gives the same float32 results
// for each storage type T.  axis() takes the values at i-1, i, i+1 along one
// axis (as floats, exact for every storage type; the ones outside [0, n) are
// not used), n >= 2; finish() turns the three gradients into the normal.
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

namespace pvr {

__device__ __forceinline__ float round_half(float x) { return __half2float(__float2half_rn(x)); }

template <typename T> struct GradientArith;

template <> struct GradientArith<float> {
    static __device__ __forceinline__ float axis(float vm, float v0, float vp, int i, int n) {
        if (i == 0) return __fsub_rn(vp, v0);
        if (i == n - 1) return __fsub_rn(v0, vm);
        return __fmul_rn(__fsub_rn(vp, vm), 0.5f);
    }
    static __device__ __forceinline__ float3 finish(float g0, float g1, float g2) {
        const float ss = __fadd_rn(__fadd_rn(__fmul_rn(g0, g0), __fmul_rn(g1, g1)), __fmul_rn(g2, g2));
        const float nrm = __fadd_rn(__fsqrt_rn(ss), 1e-8f);
        return make_float3(__fdiv_rn(g0, nrm), __fdiv_rn(g1, nrm), __fdiv_rn(g2, nrm));
    }
};

template <> struct GradientArith<__half> {
    static __device__ __forceinline__ float axis(float vm, float v0, float vp, int i, int n) {
        if (i == 0) return round_half(__fsub_rn(vp, v0));
        if (i == n - 1) return round_half(__fsub_rn(v0, vm));
        return round_half(__fdiv_rn(round_half(__fsub_rn(vp, vm)), 2.0f));
    }
    static __device__ __forceinline__ float3 finish(float g0, float g1, float g2) {
        // squares rounded to half; the sum accumulates in float, rounds once
        const float q0 = round_half(__fmul_rn(g0, g0));
        const float q1 = round_half(__fmul_rn(g1, g1));
        const float q2 = round_half(__fmul_rn(g2, g2));
        const float ss = round_half(__fadd_rn(__fadd_rn(q0, q1), q2));
        const float nrm = round_half(__fsqrt_rn(ss));  // + 1e-8 rounds to + 0 in half
        return make_float3(round_half(__fdiv_rn(g0, nrm)), round_half(__fdiv_rn(g1, nrm)),
                           round_half(__fdiv_rn(g2, nrm)));
    }
};

// uint8 input: numpy's float64 result, RN32(RN64(g / N)) with
// N = RN64(RN64(sqrt(S)) + 1e-8), S = g0^2 + g1^2 + g2^2, computed in float32
// arithmetic.  The gradients are exact in float32 (integers in [-255, 255]
// one-sided, multiples of 0.5 in [-127.5, 127.5] central) and so is S (a
// multiple of 0.25 below 2^18).  sqrt(S) + 1e-8 is carried as an unevaluated
// float pair Nh + Nl (Nh = RN(sqrt S), the exact remainder S - Nh^2 by FMA
// gives the low part), the quotient as qh = RN(g / Nh) plus a correction
// from the exact remainder g - qh*Nh (FMA).  The pair approximates g / N to
// about 2^-43 relative; when that interval around it does not decide the
// float32 rounding (the quotient lies within 2^-38 relative of a rounding
// boundary), the component is computed in float64 as numpy does.  Every
// (g0, g1, g2) a uint8 volume can produce -- the gradient set above cubed --
// is checked against the float64 formula on the GPU by the tests.
struct U8Norm {
    float nh, nl;  // N ~ nh + nl
    float s;       // S
};

__device__ __forceinline__ U8Norm u8_norm(float g0, float g1, float g2) {
    U8Norm r;
    r.s = __fadd_rn(__fadd_rn(__fmul_rn(g0, g0), __fmul_rn(g1, g1)), __fmul_rn(g2, g2));  // exact
    const float sh = __fsqrt_rn(r.s);
    const float rem = fmaf(-sh, sh, r.s);  // exact
    const float sl = sh > 0.0f ? __fdiv_rn(rem, __fmul_rn(2.0f, sh)) : 0.0f;
    r.nh = sh;
    r.nl = __fadd_rn(sl, 1e-8f);
    return r;
}

__device__ __noinline__ float u8_component_f64(float g, float s) {
    const double n = __dadd_rn(__dsqrt_rn((double)s), 1e-8);
    return __double2float_rn(__ddiv_rn((double)g, n));
}

__device__ __forceinline__ float u8_component(float g, const U8Norm &n) {
    if (g == 0.0f) return 0.0f;  // +0 / N (numpy's differences of equal values are +0)
    const float qh = __fdiv_rn(g, n.nh);
    const float e = fmaf(-qh, n.nh, g);   // g - qh*nh, exact
    const float e2 = fmaf(-qh, n.nl, e);  // g - qh*(nh + nl)
    const float corr = __fdiv_rn(e2, n.nh);
    const float eb = fabsf(qh) * 3.637978807091713e-12f;  // 2^-38 |q|
    const float lo = __fadd_rn(qh, __fsub_rn(corr, eb));
    const float hi = __fadd_rn(qh, __fadd_rn(corr, eb));
    if (lo == hi) return lo;
    return u8_component_f64(g, n.s);
}

template <> struct GradientArith<uint8_t> {
    static __device__ __forceinline__ float axis(float vm, float v0, float vp, int i, int n) {
        if (i == 0) return __fsub_rn(vp, v0);
        if (i == n - 1) return __fsub_rn(v0, vm);
        return __fmul_rn(__fsub_rn(vp, vm), 0.5f);  // exact
    }
    static __device__ __forceinline__ float3 finish(float g0, float g1, float g2) {
        const U8Norm n = u8_norm(g0, g1, g2);
        return make_float3(u8_component(g0, n), u8_component(g1, n), u8_component(g2, n));
    }
};

}  // namespace pvr
