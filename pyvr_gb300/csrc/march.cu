// Forward ray-march kernel: pyvr/shaders/volume.frag.glsl:main as CUDA.
//
// One thread marches one pixel's ray.  A 256-thread block covers a 16x16
// pixel tile made of eight 8x4 warp tiles, so the 32 rays of a warp are
// spatially close and their trilinear footprints share cache lines.  The
// RGBA LUT is staged in shared memory once per block.  Voxels and normals
// are read from the bricked 16-byte texel records of layout.cu: each sample
// is 8 vector loads from one brick.
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

template <bool SMEM>
__device__ __forceinline__ float4 lut_entry(const float4 *lut, int i) {
    if (SMEM) return lut[i];
    return __ldg(lut + i);
}

template <bool NORMALS>
__device__ __forceinline__ float4 load_record(const float4 *p) {
    if (NORMALS) return __ldg(p);
    return make_float4(__ldg(reinterpret_cast<const float *>(p)), 0.0f, 0.0f, 0.0f);
}

// Shading + compositing of one in-box sample (frag:93-115).  bp: the brick's
// records; l0/l1: the footprint's local texel coordinates per axis;
// fr: the filter fractions.
template <bool NORMALS, bool SMEM_LUT>
__device__ __forceinline__ void shade_sample(const MarchFrame &f, const float4 *__restrict__ bp,
                                             const int l0[3], const int l1[3], const float fr[3],
                                             const float4 *lut, float acc[4]) {
    const int ox0 = l0[0] * (kApron * kApron), ox1 = l1[0] * (kApron * kApron);
    const int oy0 = l0[1] * kApron, oy1 = l1[1] * kApron;
    const int oz0 = l0[2], oz1 = l1[2];
    const float4 r000 = load_record<NORMALS>(bp + ox0 + oy0 + oz0);
    const float4 r001 = load_record<NORMALS>(bp + ox0 + oy0 + oz1);
    const float4 r010 = load_record<NORMALS>(bp + ox0 + oy1 + oz0);
    const float4 r011 = load_record<NORMALS>(bp + ox0 + oy1 + oz1);
    const float4 r100 = load_record<NORMALS>(bp + ox1 + oy0 + oz0);
    const float4 r101 = load_record<NORMALS>(bp + ox1 + oy0 + oz1);
    const float4 r110 = load_record<NORMALS>(bp + ox1 + oy1 + oz0);
    const float4 r111 = load_record<NORMALS>(bp + ox1 + oy1 + oz1);
    // texture(volume_texture, tex.zyx): lerp along z, then y, then x
#define PVR_TRI(c)                                                                        \
    lerp_tex(lerp_tex(lerp_tex(r000.c, r001.c, fr[2]), lerp_tex(r010.c, r011.c, fr[2]), fr[1]), \
             lerp_tex(lerp_tex(r100.c, r101.c, fr[2]), lerp_tex(r110.c, r111.c, fr[2]), fr[1]), fr[0])
    float density = PVR_TRI(x);
    density = density * f.value_scale;

    // texture(transfer_function_lut, vec2(density, 0.5)) (frag:96)
    float lu = density * f.flut_size - 0.5f;
    float lfl = floorf(lu);
    float la = lu - lfl;
    float lf1 = lfl + 1.0f;
    float lmax = (float)(f.lut_size - 1);
    int i0 = !(lfl >= 0.0f) ? 0 : (lfl > lmax ? f.lut_size - 1 : (int)lfl);
    int i1 = !(lf1 >= 0.0f) ? 0 : (lf1 > lmax ? f.lut_size - 1 : (int)lf1);
    float4 A = lut_entry<SMEM_LUT>(lut, i0), B = lut_entry<SMEM_LUT>(lut, i1);
    float cr = lerp_tex(A.x, B.x, la), cg = lerp_tex(A.y, B.y, la);
    float cb = lerp_tex(A.z, B.z, la), alpha_tf = lerp_tex(A.w, B.w, la);

    // Beer-Lambert opacity correction (frag:101)
    float alpha = 1.0f - pvr_expf(-(alpha_tf * f.alpha_k));

    // normal (frag:103-104); without a normal texture the reference's
    // sampler reads the R32F volume texture: (density, 0, 0)
    float n[3];
    if (NORMALS) {
        n[0] = PVR_TRI(y);
        n[1] = PVR_TRI(z);
        n[2] = PVR_TRI(w);
    } else {
        n[0] = density;
        n[1] = 0.0f;
        n[2] = 0.0f;
    }
#undef PVR_TRI
    // Lambert term (frag:107-110); a zero (or NaN) normal gives 0
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

template <bool NORMALS, bool SMEM_LUT>
__global__ void __launch_bounds__(kThreads)
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
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    unsigned n_inbox = 0, n_shaded = 0;
    float pos[3], dstep[3];
    if (in_image && setup_ray(f, px, py, pos, dstep)) {
        bool entered = false;
        int cur_brick = -1;
        bool transparent = false;
        const float4 *bp = records;
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
                ++n_inbox;
                // texel footprint (texel centres, clamp to edge) and its brick
                int l0[3], l1[3], bc[3];
                float fr[3];
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    float u = t[a] * f.fext[a] - 0.5f;
                    float fl = floorf(u);
                    fr[a] = u - fl;
                    int k = (int)fl;
                    int k0 = max(k, 0), k1 = min(k + 1, f.ext[a] - 1);
                    bc[a] = k0 >> kBrickLog2;
                    l0[a] = k0 - (bc[a] << kBrickLog2);
                    l1[a] = k1 - (bc[a] << kBrickLog2);
                }
                const int id = (bc[0] * f.nb[1] + bc[1]) * f.nb[2] + bc[2];
                if (id != cur_brick) {
                    cur_brick = id;
                    const uint32_t e = __ldg(table + id);
                    transparent = (e & kTransparentBit) != 0;
                    bp = records + (size_t)(e & kSlotMask) * kRecordsPerBrick;
                }
                if (!transparent) {
                    ++n_shaded;
                    shade_sample<NORMALS, SMEM_LUT>(f, bp, l0, l1, fr, lut, acc);
                }
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
