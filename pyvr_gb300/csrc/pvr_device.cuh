// Device-side helpers shared by the march kernels.
//
// The arithmetic pins the rounding of every step of
// pyvr/shaders/volume.frag.glsl so that a frame is a deterministic function
// of its inputs: the .cu files are compiled with --fmad=false, so a*b+c is
// a rounded product and a rounded sum unless fmaf() is written; texture
// filtering uses lerp(a, b, t) = fmaf(t, b - a, a).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace pvr {

// Per-frame constants of one render: the reference's uniforms
// (volume.frag.glsl:3-19) after the host-side derivations.
struct MarchFrame {
    int width, height;
    float ip[8];        // rows 0-1 of inverse(projection) as GL reads it
    float iv[12];       // rows 0-2 of inverse(view)
    float cam[3];       // camera_pos
    float bmin[3];      // volume_min_bounds
    float bmax[3];      // volume_max_bounds
    float inv_ext[3];   // 1 / (volume_max_bounds - volume_min_bounds)
    float fext[3];      // texel count along world x, y, z (= W, H, D)
    int ext[3];
    int nb[3];          // bricks along world x, y, z
    float step;         // step_size
    float alpha_k;      // step_size / reference_step_size
    int max_steps;
    float light_dir[3]; // normalize(light_target - light_position), 0 if degenerate
    float ambient, diffuse;
    float value_scale;  // stored voxel value -> density
    int lut_size;
    float flut_size;
    float flut_max;     // lut_size - 1
    float alpha_k2;     // alpha_k * log2(e), for exp(-x) = 2^(-x log2 e) (fast arithmetic)
};

__device__ __forceinline__ float lerp_tex(float a, float b, float t) {
    return fmaf(t, b - a, a);
}

// Two lerps at once with the packed FP32x2 pipe (sm_100+): per lane the
// same two IEEE round-to-nearest operations as lerp_tex (b - a is formed
// exactly as fma(a, -1, b)).
__device__ __forceinline__ float2 lerp_tex2(float2 a, float2 b, float t) {
    return __ffma2_rn(make_float2(t, t), __ffma2_rn(a, make_float2(-1.0f, -1.0f), b), a);
}

// exp(x): k = rint(x/ln2), r = x - k*ln2 with ln2 split 0.693359375 +
// -2.12194440e-4 (Cody & Waite), exp(r) by its Taylor series to r^7
// (|r| <= ln2/2, truncation < 0.1 ulp), scaled by 2^k.  Flushes to 0 below
// -87.3 (where 1 - exp(x) is already 1.0f).
__device__ __forceinline__ float pvr_expf(float x) {
    if (x != x) return x;
    if (x > 88.72283f) return __int_as_float(0x7f800000);
    if (x < -87.33654f) return 0.0f;
    float kf = rintf(x * 1.44269504f);
    float r = fmaf(kf, -0.693359375f, x);
    r = fmaf(kf, 2.12194440e-4f, r);
    float p = 1.98412698e-4f;
    p = fmaf(p, r, 1.38888889e-3f);
    p = fmaf(p, r, 8.33333333e-3f);
    p = fmaf(p, r, 4.16666667e-2f);
    p = fmaf(p, r, 1.66666667e-1f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    const int k = (int)kf;  // -126 .. 128
    // one exact scaling by 2^k where 2^k is a float (k <= 127); k = 128 in
    // two halves.  Either way the only rounding is that of the final product.
    if (k <= 127) return p * __int_as_float((k + 127) << 23);
    return (p * __int_as_float((64 + 127) << 23)) * __int_as_float((k - 64 + 127) << 23);
}

// The fast arithmetic's two special functions, each one hardware
// instruction (PTX ISA: ex2.approx, rsqrt.approx; relative error about
// 2^-22).  ex2 flushes subnormal results to 0; rsqrt keeps subnormal inputs.
__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
    float y;
    asm("rsqrt.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Ray of pixel (px, py), py counted from the bottom row: vertex-stage uv at
// the pixel centre (volume.vert.glsl:8), ray_direction (frag:47-54) and the
// slab test (frag:56-68, 75-81).  Returns false for a miss.
__device__ __forceinline__ bool setup_ray(const MarchFrame &f, int px, int py, float pos[3],
                                          float dstep[3]) {
    float uvx = ((float)px + 0.5f) / (float)f.width;
    float uvy = ((float)py + 0.5f) / (float)f.height;
    float nx = uvx * 2.0f - 1.0f, ny = uvy * 2.0f - 1.0f;
    float ex = ((f.ip[0] * nx + f.ip[1] * ny) + f.ip[2] * -1.0f) + f.ip[3] * 1.0f;
    float ey = ((f.ip[4] * nx + f.ip[5] * ny) + f.ip[6] * -1.0f) + f.ip[7] * 1.0f;
    float w[3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
        w[r] = ((f.iv[r * 4 + 0] * ex + f.iv[r * 4 + 1] * ey) + f.iv[r * 4 + 2] * -1.0f) +
               f.iv[r * 4 + 3] * 0.0f;
    float wl = 1.0f / sqrtf((w[0] * w[0] + w[1] * w[1]) + w[2] * w[2]);
    float dir[3] = {w[0] * wl, w[1] * wl, w[2] * wl};
    float tn = 0.0f, tf = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float inv = 1.0f / dir[a];
        float t0 = (f.bmin[a] - f.cam[a]) * inv;
        float t1 = (f.bmax[a] - f.cam[a]) * inv;
        float lo = fminf(t0, t1), hi = fmaxf(t0, t1);
        tn = a == 0 ? lo : fmaxf(tn, lo);
        tf = a == 0 ? hi : fminf(tf, hi);
    }
    if (!(tn <= tf && tf > 0.0f)) return false;
    tn = fmaxf(tn, 0.0f);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        pos[a] = f.cam[a] + dir[a] * tn;
        dstep[a] = dir[a] * f.step;
    }
    return true;
}

}  // namespace pvr
