// Forward ray-march kernels: pyvr/shaders/volume.frag.glsl:main as CUDA.
//
// One thread marches one pixel's ray.  A 256-thread block covers a 16x16
// pixel tile made of eight 8x4 warp tiles, so the 32 rays of a warp are
// spatially close and their trilinear footprints share cache lines.  The
// RGBA LUT is staged in shared memory once per block.
//
// The march reproduces the reference loop (frag:87-119) exactly, with one
// shortcut that changes no output: the ray's texture coordinate is monotone
// in the step index along each axis (the position is advanced by repeated
// addition of the same float step), so the steps whose coordinate is valid
// (frag:92) form one contiguous run; once the ray has left that run, or can
// provably never enter it, every remaining iteration would be a no-op and
// the loop ends.
#include "pvr_device.cuh"
#include "pvr_internal.h"

namespace pvr {

constexpr int kTile = 16;
constexpr int kThreads = 256;

template <bool SMEM>
__device__ __forceinline__ float4 lut_entry(const float4 *lut, int i) {
    if (SMEM) return lut[i];
    return __ldg(lut + i);
}

// Shading + compositing of one in-box sample (frag:93-115), given the
// texture coordinate t (already known valid).
template <typename T, bool NORMALS, bool SMEM_LUT>
__device__ __forceinline__ void shade_sample(const MarchFrame &f, const T *__restrict__ vol,
                                             const float *__restrict__ nrm, const float4 *lut,
                                             const float t[3], float acc[4]) {
    long long o0[3], o1[3];
    float fr[3];
    const long long stride[3] = {f.stride_x, f.stride_y, 1};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float u = t[a] * f.fext[a] - 0.5f;
        float fl = floorf(u);
        fr[a] = u - fl;
        int k0 = (int)fl, k1 = k0 + 1;
        k0 = k0 < 0 ? 0 : k0;
        k1 = k1 > f.ext[a] - 1 ? f.ext[a] - 1 : k1;
        o0[a] = (long long)k0 * stride[a];
        o1[a] = (long long)k1 * stride[a];
    }
    const long long b00 = o0[0] + o0[1], b01 = o0[0] + o1[1];
    const long long b10 = o1[0] + o0[1], b11 = o1[0] + o1[1];
    // texture(volume_texture, tex.zyx): lerp along z, then y, then x
    float v00 = lerp_tex(load_voxel(vol, b00 + o0[2]), load_voxel(vol, b00 + o1[2]), fr[2]);
    float v01 = lerp_tex(load_voxel(vol, b01 + o0[2]), load_voxel(vol, b01 + o1[2]), fr[2]);
    float v10 = lerp_tex(load_voxel(vol, b10 + o0[2]), load_voxel(vol, b10 + o1[2]), fr[2]);
    float v11 = lerp_tex(load_voxel(vol, b11 + o0[2]), load_voxel(vol, b11 + o1[2]), fr[2]);
    float density = lerp_tex(lerp_tex(v00, v01, fr[1]), lerp_tex(v10, v11, fr[1]), fr[0]);
    density = density * f.value_scale;

    // texture(transfer_function_lut, vec2(density, 0.5)) (frag:96)
    float lu = density * f.flut_size - 0.5f;
    float lfl = floorf(lu);
    float la = lu - lfl;
    float lf1 = lfl + 1.0f;
    float lmax = (float)(f.lut_size - 1);
    int l0 = !(lfl >= 0.0f) ? 0 : (lfl > lmax ? f.lut_size - 1 : (int)lfl);
    int l1 = !(lf1 >= 0.0f) ? 0 : (lf1 > lmax ? f.lut_size - 1 : (int)lf1);
    float4 A = lut_entry<SMEM_LUT>(lut, l0), B = lut_entry<SMEM_LUT>(lut, l1);
    float cr = lerp_tex(A.x, B.x, la), cg = lerp_tex(A.y, B.y, la);
    float cb = lerp_tex(A.z, B.z, la), alpha_tf = lerp_tex(A.w, B.w, la);

    // Beer-Lambert opacity correction (frag:101)
    float alpha = 1.0f - pvr_expf(-(alpha_tf * f.alpha_k));

    // normal (frag:103-104)
    float n[3];
    if (NORMALS) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            float m00 = lerp_tex(__ldg(nrm + 3 * (b00 + o0[2]) + c), __ldg(nrm + 3 * (b00 + o1[2]) + c), fr[2]);
            float m01 = lerp_tex(__ldg(nrm + 3 * (b01 + o0[2]) + c), __ldg(nrm + 3 * (b01 + o1[2]) + c), fr[2]);
            float m10 = lerp_tex(__ldg(nrm + 3 * (b10 + o0[2]) + c), __ldg(nrm + 3 * (b10 + o1[2]) + c), fr[2]);
            float m11 = lerp_tex(__ldg(nrm + 3 * (b11 + o0[2]) + c), __ldg(nrm + 3 * (b11 + o1[2]) + c), fr[2]);
            n[c] = lerp_tex(lerp_tex(m00, m01, fr[1]), lerp_tex(m10, m11, fr[1]), fr[0]);
        }
    } else {
        n[0] = density;
        n[1] = 0.0f;
        n[2] = 0.0f;
    }
    // Lambert term (frag:107-110)
    float n2 = (n[0] * n[0] + n[1] * n[1]) + n[2] * n[2];
    float di = 0.0f;
    if (n2 > 0.0f) {
        float inv = 1.0f / sqrtf(n2);
        float d = ((n[0] * inv) * f.light_dir[0] + (n[1] * inv) * f.light_dir[1]) +
                  (n[2] * inv) * f.light_dir[2];
        di = fmaxf(d, 0.0f);
    }
    float light = f.ambient + f.diffuse * di;
    // front-to-back compositing (frag:112-115)
    float tr = 1.0f - acc[3];
    acc[0] = acc[0] + tr * ((cr * light) * alpha);
    acc[1] = acc[1] + tr * ((cg * light) * alpha);
    acc[2] = acc[2] + tr * ((cb * light) * alpha);
    acc[3] = acc[3] + tr * alpha;
}

__device__ __forceinline__ uint32_t blend_rgba8(const float acc[4]) {
    // SRC_ALPHA / ONE_MINUS_SRC_ALPHA over a cleared UNORM8 target.
    float a = fminf(fmaxf(acc[3], 0.0f), 1.0f);
    uint32_t r = (uint32_t)rintf((fminf(fmaxf(acc[0], 0.0f), 1.0f) * a) * 255.0f);
    uint32_t g = (uint32_t)rintf((fminf(fmaxf(acc[1], 0.0f), 1.0f) * a) * 255.0f);
    uint32_t b = (uint32_t)rintf((fminf(fmaxf(acc[2], 0.0f), 1.0f) * a) * 255.0f);
    uint32_t al = (uint32_t)rintf((a * a) * 255.0f);
    return r | (g << 8) | (b << 16) | (al << 24);
}

template <typename T, bool NORMALS, bool SMEM_LUT>
__global__ void __launch_bounds__(kThreads)
march_linear_kernel(const MarchFrame f, const T *__restrict__ vol, const float *__restrict__ nrm,
                    const float4 *__restrict__ lut_g, uint32_t *__restrict__ out8,
                    float4 *__restrict__ outf, unsigned long long *__restrict__ samples_out) {
    extern __shared__ float4 s_lut[];
    const float4 *lut = lut_g;
    if (SMEM_LUT) {
        for (int i = threadIdx.x; i < f.lut_size; i += kThreads) s_lut[i] = lut_g[i];
        __syncthreads();
        lut = s_lut;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int px = blockIdx.x * kTile + (warp & 1) * 8 + (lane & 7);
    const int py = blockIdx.y * kTile + (warp >> 1) * 4 + (lane >> 3);
    const bool in_image = px < f.width && py < f.height;
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    unsigned n_samples = 0;
    float pos[3], dstep[3];
    if (in_image && setup_ray(f, px, py, pos, dstep)) {
        bool entered = false;
        for (int i = 0; i < f.max_steps && acc[3] < 0.99f; ++i) {
            float t[3];
            bool valid = true;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                t[a] = (pos[a] - f.bmin[a]) * f.inv_ext[a];
                valid = valid && (t[a] >= 0.0f) && (t[a] <= 1.0f);
            }
            if (valid) {
                entered = true;
                ++n_samples;
                shade_sample<T, NORMALS, SMEM_LUT>(f, vol, nrm, lut, t, acc);
            } else {
                bool never = entered;
#pragma unroll
                for (int a = 0; a < 3; ++a)
                    never = never || (t[a] < 0.0f && dstep[a] <= 0.0f) ||
                            (t[a] > 1.0f && dstep[a] >= 0.0f);
                if (never) break;
            }
#pragma unroll
            for (int a = 0; a < 3; ++a) pos[a] = pos[a] + dstep[a];
        }
    }
    if (in_image) {
        const long long idx = (long long)py * f.width + px;
        if (out8) out8[idx] = blend_rgba8(acc);
        if (outf) outf[idx] = make_float4(acc[0], acc[1], acc[2], acc[3]);
    }
    if (samples_out) {
        unsigned long long s = n_samples;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0 && s) atomicAdd(samples_out, s);
    }
}

template <typename T, bool NORMALS>
static cudaError_t launch_typed(const MarchFrame &f, const void *vol, const float *nrm,
                                const float4 *lut, uint32_t *out8, float4 *outf,
                                unsigned long long *samples, cudaStream_t st) {
    dim3 grid((f.width + kTile - 1) / kTile, (f.height + kTile - 1) / kTile);
    if (f.lut_size <= kLutSmemMaxEntries) {
        size_t shm = (size_t)f.lut_size * sizeof(float4);
        march_linear_kernel<T, NORMALS, true><<<grid, kThreads, shm, st>>>(
            f, (const T *)vol, nrm, lut, out8, outf, samples);
    } else {
        march_linear_kernel<T, NORMALS, false><<<grid, kThreads, 0, st>>>(
            f, (const T *)vol, nrm, lut, out8, outf, samples);
    }
    return cudaGetLastError();
}

cudaError_t launch_march_linear(const MarchFrame &f, int dtype, const void *vol, const float *nrm,
                                const float4 *lut, uint32_t *out8, float4 *outf,
                                unsigned long long *samples, cudaStream_t st) {
    if (f.width <= 0 || f.height <= 0) return cudaSuccess;
    switch (dtype) {
    case PVR_U8:
        return nrm ? launch_typed<uint8_t, true>(f, vol, nrm, lut, out8, outf, samples, st)
                   : launch_typed<uint8_t, false>(f, vol, nrm, lut, out8, outf, samples, st);
    case PVR_F16:
        return nrm ? launch_typed<__half, true>(f, vol, nrm, lut, out8, outf, samples, st)
                   : launch_typed<__half, false>(f, vol, nrm, lut, out8, outf, samples, st);
    default:
        return nrm ? launch_typed<float, true>(f, vol, nrm, lut, out8, outf, samples, st)
                   : launch_typed<float, false>(f, vol, nrm, lut, out8, outf, samples, st);
    }
}

}  // namespace pvr
