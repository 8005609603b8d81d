// Forward ray-march kernel: pyvr/shaders/volume.frag.glsl:main as CUDA.
//
// One thread marches one pixel's ray.  A 256-thread block covers a 16x16
// pixel tile made of eight 8x4 warp tiles, so the 32 rays of a warp are
// spatially close and their trilinear footprints share cache lines.  The
// RGBA LUT is staged in shared memory once per block.  Voxels and normals
// are read from the bricked 16-byte texel records of layout.cu: each sample
// is 8 vector loads at fixed offsets from one record address.  Paired
// channels go through the packed FP32x2 pipe, which rounds each lane
// exactly like the scalar instruction; an add that consumes a packed
// product is always a scalar __fadd_rn, so no product/add pair can be
// fused into one rounding.
//
// The march reproduces the reference loop (frag:87-119) exactly, with two
// shortcuts that change no output bit:
//  - the ray's texture coordinate is monotone in the step index along each
//    axis (the position advances by repeated addition of one float step),
//    so the steps whose coordinate is valid (frag:92) form one contiguous
//    run; once the ray has left it, or provably cannot enter it, every
//    remaining iteration would be a no-op and the loop ends;
//  - a sample whose brick is flagged transparent for the current LUT adds
//    exactly +0 to every accumulator, so its fetches and shading are
//    skipped; the position still advances by the same float additions.
#include "pvr_device.cuh"
#include "pvr_internal.h"

namespace pvr {

constexpr int kTile = 16;
constexpr int kThreads = 256;
constexpr int kRowRecords = kApron;            // +1 texel along y
constexpr int kSliceRecords = kApron * kApron;  // +1 texel along x

template <bool SMEM>
__device__ __forceinline__ float4 lut_entry(const float4 *lut, int i) {
    if (SMEM) return lut[i];
    return __ldg(lut + i);
}

__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float2 dup2(float v) { return make_float2(v, v); }

// Shading + compositing of one in-box sample (frag:93-115).  p: the record
// of the footprint's lower corner; fr: the filter fractions (x, y, z).
template <bool NORMALS, bool SMEM_LUT>
__device__ __forceinline__ void shade_sample(const MarchFrame &f, const float4 *__restrict__ p,
                                             float fx, float fy, float fz, const float4 *lut,
                                             float2 &acc_rg, float2 &acc_ba) {
    float density;
    float n[3];
    if (NORMALS) {
        const float4 r000 = __ldg(p);
        const float4 r001 = __ldg(p + 1);
        const float4 r010 = __ldg(p + kRowRecords);
        const float4 r011 = __ldg(p + kRowRecords + 1);
        const float4 r100 = __ldg(p + kSliceRecords);
        const float4 r101 = __ldg(p + kSliceRecords + 1);
        const float4 r110 = __ldg(p + kSliceRecords + kRowRecords);
        const float4 r111 = __ldg(p + kSliceRecords + kRowRecords + 1);
        // texture(volume_texture, tex.zyx) and texture(normal_volume, ...):
        // lerp along z, then y, then x; lanes (value, nx) and (ny, nz)
        const float2 a = lerp_tex2(lerp_tex2(lerp_tex2(lo2(r000), lo2(r001), fz),
                                             lerp_tex2(lo2(r010), lo2(r011), fz), fy),
                                   lerp_tex2(lerp_tex2(lo2(r100), lo2(r101), fz),
                                             lerp_tex2(lo2(r110), lo2(r111), fz), fy), fx);
        const float2 b = lerp_tex2(lerp_tex2(lerp_tex2(hi2(r000), hi2(r001), fz),
                                             lerp_tex2(hi2(r010), hi2(r011), fz), fy),
                                   lerp_tex2(lerp_tex2(hi2(r100), hi2(r101), fz),
                                             lerp_tex2(hi2(r110), hi2(r111), fz), fy), fx);
        density = a.x * f.value_scale;
        n[0] = a.y;
        n[1] = b.x;
        n[2] = b.y;
    } else {
        const float *q = reinterpret_cast<const float *>(p);
        const float v000 = __ldg(q), v001 = __ldg(q + 4);
        const float v010 = __ldg(q + 4 * kRowRecords), v011 = __ldg(q + 4 * kRowRecords + 4);
        const float v100 = __ldg(q + 4 * kSliceRecords), v101 = __ldg(q + 4 * kSliceRecords + 4);
        const float v110 = __ldg(q + 4 * (kSliceRecords + kRowRecords));
        const float v111 = __ldg(q + 4 * (kSliceRecords + kRowRecords) + 4);
        const float2 zz0 = lerp_tex2(make_float2(v000, v010), make_float2(v001, v011), fz);
        const float2 zz1 = lerp_tex2(make_float2(v100, v110), make_float2(v101, v111), fz);
        const float2 yy = lerp_tex2(make_float2(zz0.x, zz1.x), make_float2(zz0.y, zz1.y), fy);
        density = lerp_tex(yy.x, yy.y, fx) * f.value_scale;
        // the reference's unbound normal sampler reads the R32F volume
        // texture: normal = (density, 0, 0)
        n[0] = density;
        n[1] = 0.0f;
        n[2] = 0.0f;
    }

    // texture(transfer_function_lut, vec2(density, 0.5)) (frag:96)
    const float lu = density * f.flut_size - 0.5f;
    const float lfl = floorf(lu);
    const float la = lu - lfl;
    const float lf1 = lfl + 1.0f;
    const float lmax = (float)(f.lut_size - 1);
    const int i0 = !(lfl >= 0.0f) ? 0 : (lfl > lmax ? f.lut_size - 1 : (int)lfl);
    const int i1 = !(lf1 >= 0.0f) ? 0 : (lf1 > lmax ? f.lut_size - 1 : (int)lf1);
    const float4 A = lut_entry<SMEM_LUT>(lut, i0), B = lut_entry<SMEM_LUT>(lut, i1);
    const float2 crg = lerp_tex2(lo2(A), lo2(B), la);
    const float2 cba = lerp_tex2(hi2(A), hi2(B), la);  // (blue, alpha_tf)

    // Beer-Lambert opacity correction (frag:101)
    const float alpha = 1.0f - pvr_expf(-(cba.y * f.alpha_k));

    // Lambert term (frag:107-110); a zero (or NaN) normal gives 0
    const float n2 = (n[0] * n[0] + n[1] * n[1]) + n[2] * n[2];
    float di = 0.0f;
    if (n2 > 0.0f) {
        const float inv = 1.0f / sqrtf(n2);
        const float d = ((n[0] * inv) * f.light_dir[0] + (n[1] * inv) * f.light_dir[1]) +
                        (n[2] * inv) * f.light_dir[2];
        di = fmaxf(d, 0.0f);
    }
    const float light = f.ambient + f.diffuse * di;
    // front-to-back compositing (frag:112-115):
    // acc.c += (1 - acc.a) * (c * light * alpha), acc.a += (1 - acc.a) * alpha
    // Products go through the packed pipe; every add that consumes a product
    // is a scalar __fadd_rn, which is never fused into an FMA.
    const float2 tr = dup2(1.0f - acc_ba.y);
    const float2 src_rg = __fmul2_rn(__fmul2_rn(crg, dup2(light)), dup2(alpha));
    const float src_b = __fmul_rn(__fmul_rn(cba.x, light), alpha);
    const float2 add_rg = __fmul2_rn(tr, src_rg);
    const float2 add_ba = __fmul2_rn(tr, make_float2(src_b, alpha));
    acc_rg = make_float2(__fadd_rn(acc_rg.x, add_rg.x), __fadd_rn(acc_rg.y, add_rg.y));
    acc_ba = make_float2(__fadd_rn(acc_ba.x, add_ba.x), __fadd_rn(acc_ba.y, add_ba.y));
}

__device__ __forceinline__ uint32_t blend_rgba8(float2 rg, float2 ba) {
    // SRC_ALPHA / ONE_MINUS_SRC_ALPHA over a cleared UNORM8 target.
    float a = fminf(fmaxf(ba.y, 0.0f), 1.0f);
    uint32_t r = (uint32_t)rintf((fminf(fmaxf(rg.x, 0.0f), 1.0f) * a) * 255.0f);
    uint32_t g = (uint32_t)rintf((fminf(fmaxf(rg.y, 0.0f), 1.0f) * a) * 255.0f);
    uint32_t b = (uint32_t)rintf((fminf(fmaxf(ba.x, 0.0f), 1.0f) * a) * 255.0f);
    uint32_t al = (uint32_t)rintf((a * a) * 255.0f);
    return r | (g << 8) | (b << 16) | (al << 24);
}

template <bool NORMALS, bool SMEM_LUT>
__global__ void __launch_bounds__(kThreads, 5)
march_kernel(const MarchFrame f, const float4 *__restrict__ records,
             const uint32_t *__restrict__ table, const float4 *__restrict__ lut_g,
             uint32_t *__restrict__ out8, float4 *__restrict__ outf,
             unsigned long long *__restrict__ counters) {
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
    float2 acc_rg = make_float2(0.0f, 0.0f), acc_ba = make_float2(0.0f, 0.0f);
    unsigned n_inbox = 0, n_shaded = 0;
    float pos[3], dstep[3];
    if (in_image && setup_ray(f, px, py, pos, dstep)) {
        // (x, y) lanes packed, z scalar; same per-lane operations as the
        // reference expressions
        float2 pxy = make_float2(pos[0], pos[1]);
        float pz = pos[2];
        const float2 dxy = make_float2(dstep[0], dstep[1]);
        const float dz = dstep[2];
        const float2 nbmin_xy = make_float2(-f.bmin[0], -f.bmin[1]);
        const float2 inv_xy = make_float2(f.inv_ext[0], f.inv_ext[1]);
        const float2 fext_xy = make_float2(f.fext[0], f.fext[1]);
        bool entered = false;
        int cur_brick = -1;
        bool transparent = false;
        const float4 *bp = records;
        for (int i = 0; i < f.max_steps && acc_ba.y < 0.99f; ++i) {
            // world_to_texture_coords (frag:25-27, 88)
            const float2 txy = __fmul2_rn(__fadd2_rn(pxy, nbmin_xy), inv_xy);
            const float tz = (pz - f.bmin[2]) * f.inv_ext[2];
            const bool valid = txy.x >= 0.0f && txy.x <= 1.0f && txy.y >= 0.0f &&
                               txy.y <= 1.0f && tz >= 0.0f && tz <= 1.0f;
            if (valid) {
                entered = true;
                ++n_inbox;
                // texel coordinate u = t*size - 0.5, lower texel k = floor(u)
                // (the subtraction consumes a product: scalar __fadd_rn)
                const float2 sxy = __fmul2_rn(txy, fext_xy);
                const float2 uxy = make_float2(__fadd_rn(sxy.x, -0.5f), __fadd_rn(sxy.y, -0.5f));
                const float uz = __fadd_rn(__fmul_rn(tz, f.fext[2]), -0.5f);
                const float2 flxy = make_float2(floorf(uxy.x), floorf(uxy.y));
                const float flz = floorf(uz);
                const float2 frxy = __fadd2_rn(uxy, make_float2(-flxy.x, -flxy.y));
                const float frz = uz - flz;
                const int kx = (int)flxy.x + 1, ky = (int)flxy.y + 1, kz = (int)flz + 1;
                const int id = ((kx >> kBrickLog2) * f.nb[1] + (ky >> kBrickLog2)) * f.nb[2] +
                               (kz >> kBrickLog2);
                if (id != cur_brick) {
                    cur_brick = id;
                    const uint32_t e = __ldg(table + id);
                    transparent = (e & kTransparentBit) != 0;
                    bp = records + (size_t)(e & kSlotMask) * kRecordsPerBrick;
                }
                if (!transparent) {
                    ++n_shaded;
                    const int j = (kx & (kBrick - 1)) * kSliceRecords +
                                  (ky & (kBrick - 1)) * kRowRecords + (kz & (kBrick - 1));
                    shade_sample<NORMALS, SMEM_LUT>(f, bp + j, frxy.x, frxy.y, frz, lut, acc_rg,
                                                    acc_ba);
                }
            } else {
                const bool never = entered || (txy.x < 0.0f && dxy.x <= 0.0f) ||
                                   (txy.x > 1.0f && dxy.x >= 0.0f) ||
                                   (txy.y < 0.0f && dxy.y <= 0.0f) ||
                                   (txy.y > 1.0f && dxy.y >= 0.0f) || (tz < 0.0f && dz <= 0.0f) ||
                                   (tz > 1.0f && dz >= 0.0f);
                if (never) break;
            }
            // current_world_pos += ray_dir * step_size (frag:118)
            pxy = __fadd2_rn(pxy, dxy);
            pz = pz + dz;
        }
    }
    if (in_image) {
        const long long idx = (long long)py * f.width + px;
        if (out8) out8[idx] = blend_rgba8(acc_rg, acc_ba);
        if (outf) outf[idx] = make_float4(acc_rg.x, acc_rg.y, acc_ba.x, acc_ba.y);
    }
    if (counters) {
        unsigned long long a = n_inbox, b = n_shaded;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
        }
        if (lane == 0 && a) {
            atomicAdd(counters, a);
            atomicAdd(counters + 1, b);
        }
    }
}

template <bool NORMALS>
static cudaError_t launch_n(const MarchFrame &f, const float4 *records, const uint32_t *table,
                            const float4 *lut, uint32_t *out8, float4 *outf,
                            unsigned long long *counters, cudaStream_t st) {
    dim3 grid((f.width + kTile - 1) / kTile, (f.height + kTile - 1) / kTile);
    if (f.lut_size <= kLutSmemMaxEntries) {
        size_t shm = (size_t)f.lut_size * sizeof(float4);
        march_kernel<NORMALS, true><<<grid, kThreads, shm, st>>>(f, records, table, lut, out8, outf,
                                                                 counters);
    } else {
        march_kernel<NORMALS, false><<<grid, kThreads, 0, st>>>(f, records, table, lut, out8, outf,
                                                                counters);
    }
    return cudaGetLastError();
}

cudaError_t launch_march(const MarchFrame &f, const float4 *records, const uint32_t *table,
                         bool normals, const float4 *lut, uint32_t *out8, float4 *outf,
                         unsigned long long *counters, cudaStream_t st) {
    if (f.width <= 0 || f.height <= 0) return cudaSuccess;
    return normals ? launch_n<true>(f, records, table, lut, out8, outf, counters, st)
                   : launch_n<false>(f, records, table, lut, out8, outf, counters, st);
}

}  // namespace pvr
