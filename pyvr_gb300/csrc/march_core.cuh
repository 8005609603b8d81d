// The ray-march kernel: pyvr/shaders/volume.frag.glsl:main as CUDA, run as
// a persistent kernel over a batch of renders.
//
// Work is a queue of pixel tiles over every job of the batch (one job =
// one render with its own volume, LUT, camera, light, config and size).
// The job table is the kernel's parameter block, so frame constants are
// read through the constant cache as in a single-render kernel.  Each
// 256-thread block pops a tile with one atomic, stages the tile's RGBA LUT
// (plus the LUT's "clear entry" prefix counts) in shared memory when the
// job changes, then marches one ray per thread.  Warps cover 8x4-pixel sub-tiles so the rays
// of a warp are spatially close and their trilinear footprints share cache
// lines.  Voxels and normals are read from the bricked 16-byte texel
// records of layout.cu: each sample is 8 vector loads at fixed offsets from
// one record address.  Paired channels go through the packed FP32x2 pipe,
// which rounds each lane exactly like the scalar instruction; an add that
// consumes a packed product is always a scalar __fadd_rn, so no
// product/add pair can be fused into one rounding.
//
// The march reproduces the reference loop (frag:87-119) exactly, with two
// shortcuts that change no output bit:
//  - the ray's texture coordinate is monotone in the step index along each
//    axis (the position advances by repeated addition of one float step),
//    so the steps whose coordinate is valid (frag:92) form one contiguous
//    run; once the ray has left it, or provably cannot enter it, every
//    remaining iteration would be a no-op and the loop ends;
//  - a sample in a brick whose value range maps only to LUT entries with
//    alpha exactly 0 (and a finite colour) adds exactly +0 to every
//    accumulator, so its fetches and shading are skipped; the position
//    still advances by the same float additions.  The LUT entry range is
//    exact: a lerp fmaf(t, b-a, a) with t in [0,1) stays within [a, b], so
//    a sample lies in the brick's value range, and the scale and the LUT
//    coordinate are monotone float operations evaluated as for a sample.
//
// A volume's records are 16-byte floats, or 8-byte halves (layout.cu); the
// half form decodes to floats, so the arithmetic is the same either way.
//
// Two arithmetics (pvr_set_arithmetic), chosen per launch:
//  - exact: every operation rounded as the CPU oracle rounds it (no FMA
//    contraction except the texture lerps, exp by pvr_expf, a correctly
//    rounded rsqrt), so a frame equals the oracle's bit for bit;
//  - fast (the default): the position recurrence, the validity test, the
//    texture addressing, the lerps and the LUT addressing are the exact
//    arithmetic's, so the same samples are taken from the same texels; the
//    shading tail fuses products into FMAs, takes exp(-x) as one hardware
//    ex2 of x*log2(e) and 1/|n| as one hardware rsqrt (relative errors
//    about 2^-22), and dots n with the light before scaling by 1/|n|.  The
//    images stay within 1 LSB per RGBA8 channel of the exact ones (tested
//    at the configurations' full sizes).
#pragma once

#include "pvr_device.cuh"
#include "pvr_internal.h"

namespace pvr {

__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float2 dup2(float v) { return make_float2(v, v); }

template <bool COMPACT> struct RecordOf { using T = float4; };
template <> struct RecordOf<true> { using T = uint2; };

// two halves (low, high) of a 32-bit word as floats, in one conversion
__device__ __forceinline__ float2 half_pair(uint32_t b) {
    __half2 h;
    memcpy(&h, &b, sizeof(h));
    return __half22float2(h);
}

// {value, nx, ny, nz} of one record
__device__ __forceinline__ float4 load_rec(const float4 *p) { return __ldg(p); }
__device__ __forceinline__ float4 load_rec(const uint2 *p) {
    const uint2 r = __ldg(p);
    const float2 a = half_pair(r.x), b = half_pair(r.y);
    return make_float4(a.x, a.y, b.x, b.y);
}
// the stored value of one record
__device__ __forceinline__ float load_value(const float4 *p) { return __ldg(reinterpret_cast<const float *>(p)); }
__device__ __forceinline__ float load_value(const uint2 *p) {
    return __half2float(__ldg(reinterpret_cast<const __half *>(p)));
}

template <bool SMEM>
__device__ __forceinline__ float4 lut_entry(const float4 *lut, int i) {
    if (SMEM) return lut[i];
    return __ldg(lut + i);
}
template <bool SMEM>
__device__ __forceinline__ int prefix_entry(const int *p, int i) {
    if (SMEM) return p[i];
    return __ldg(p + i);
}

// LUT entry index of density d: floor(d*size - 0.5) clamped to the table,
// as texture(transfer_function_lut, vec2(d, 0.5)) addresses it (frag:96).
// fl = floor(coordinate); NaN and negative coordinates give entry 0.
__device__ __forceinline__ int lut_index(float fl, float lmax) {
    return (int)fminf(fmaxf(fl, 0.0f), lmax);
}

// Shading + compositing of one in-box sample (frag:93-115).  p: the record
// of the footprint's lower corner; fx, fy, fz: the filter fractions.
template <int LOG2B, bool NORMALS, bool SMEM_LUT, bool FAST, typename Rec>
__device__ __forceinline__ void shade_sample(const MarchFrame &f, const Rec *__restrict__ p,
                                             float fx, float fy, float fz, const float4 *lut,
                                             float2 &acc_rg, float2 &acc_ba) {
    constexpr int ROW = brick_apron(LOG2B), SLICE = ROW * ROW;
    float density;
    float n[3];
    if (NORMALS) {
        const float4 r000 = load_rec(p);
        const float4 r001 = load_rec(p + 1);
        const float4 r010 = load_rec(p + ROW);
        const float4 r011 = load_rec(p + ROW + 1);
        const float4 r100 = load_rec(p + SLICE);
        const float4 r101 = load_rec(p + SLICE + 1);
        const float4 r110 = load_rec(p + SLICE + ROW);
        const float4 r111 = load_rec(p + SLICE + ROW + 1);
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
        density = __fmul_rn(a.x, f.value_scale);
        n[0] = a.y;
        n[1] = b.x;
        n[2] = b.y;
    } else {
        const float v000 = load_value(p), v001 = load_value(p + 1);
        const float v010 = load_value(p + ROW), v011 = load_value(p + ROW + 1);
        const float v100 = load_value(p + SLICE), v101 = load_value(p + SLICE + 1);
        const float v110 = load_value(p + SLICE + ROW), v111 = load_value(p + SLICE + ROW + 1);
        const float2 zz0 = lerp_tex2(make_float2(v000, v010), make_float2(v001, v011), fz);
        const float2 zz1 = lerp_tex2(make_float2(v100, v110), make_float2(v101, v111), fz);
        const float2 yy = lerp_tex2(make_float2(zz0.x, zz1.x), make_float2(zz0.y, zz1.y), fy);
        density = __fmul_rn(lerp_tex(yy.x, yy.y, fx), f.value_scale);
        // the reference's unbound normal sampler reads the R32F volume
        // texture: normal = (density, 0, 0)
        n[0] = density;
        n[1] = 0.0f;
        n[2] = 0.0f;
    }

    // texture(transfer_function_lut, vec2(density, 0.5)) (frag:96): entries
    // floor(lu) and floor(lu) + 1, each clamped to the table, and the lerp
    // weight lu - floor(lu)
    const float lu = FAST ? fmaf(density, f.flut_size, -0.5f) : __fadd_rn(__fmul_rn(density, f.flut_size), -0.5f);
    const float lfl = floorf(lu);
    const float la = __fadd_rn(lu, -lfl);
    const int i0 = lut_index(lfl, f.flut_max);
    const int i1 = lut_index(__fadd_rn(lfl, 1.0f), f.flut_max);
    const float4 A = lut_entry<SMEM_LUT>(lut, i0), B = lut_entry<SMEM_LUT>(lut, i1);
    const float2 crg = lerp_tex2(lo2(A), lo2(B), la);
    const float2 cba = lerp_tex2(hi2(A), hi2(B), la);  // (blue, alpha_tf)

    if (FAST) {
        // alpha = 1 - exp(-alpha_tf * step/ref) (frag:101)
        const float alpha = __fadd_rn(1.0f, -ex2_approx(-__fmul_rn(cba.y, f.alpha_k2)));
        // Lambert term (frag:107-110): dot(n, L) / |n|; a zero (or NaN)
        // normal gives 0
        const float n2 = fmaf(n[0], n[0], fmaf(n[1], n[1], __fmul_rn(n[2], n[2])));
        const float dl = fmaf(n[0], f.light_dir[0], fmaf(n[1], f.light_dir[1], __fmul_rn(n[2], f.light_dir[2])));
        const float di = n2 > 0.0f ? fmaxf(__fmul_rn(dl, rsqrt_approx(n2)), 0.0f) : 0.0f;
        const float la_ = __fmul_rn(fmaf(f.diffuse, di, f.ambient), alpha);
        // front-to-back compositing (frag:112-115)
        const float2 tr = dup2(__fadd_rn(1.0f, -acc_ba.y));
        acc_rg = __ffma2_rn(tr, __fmul2_rn(crg, dup2(la_)), acc_rg);
        acc_ba = __ffma2_rn(tr, make_float2(__fmul_rn(cba.x, la_), alpha), acc_ba);
        return;
    }

    // Beer-Lambert opacity correction (frag:101)
    const float alpha = __fadd_rn(1.0f, -pvr_expf(-__fmul_rn(cba.y, f.alpha_k)));

    // Lambert term (frag:107-110); a zero (or NaN) normal gives 0
    const float n2 = __fadd_rn(__fadd_rn(__fmul_rn(n[0], n[0]), __fmul_rn(n[1], n[1])), __fmul_rn(n[2], n[2]));
    float di = 0.0f;
    if (n2 > 0.0f) {
        // normalize(n) = n * rsqrt(n.n), the reciprocal square root rounded
        // once (correctly rounded: equal to RN(1/sqrt(x)) evaluated in double)
        const float inv = __frsqrt_rn(n2);
        const float d = __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(n[0], inv), f.light_dir[0]),
                                            __fmul_rn(__fmul_rn(n[1], inv), f.light_dir[1])),
                                  __fmul_rn(__fmul_rn(n[2], inv), f.light_dir[2]));
        di = fmaxf(d, 0.0f);
    }
    const float light = __fadd_rn(f.ambient, __fmul_rn(f.diffuse, di));
    // front-to-back compositing (frag:112-115):
    // acc.c += (1 - acc.a) * (c * light * alpha), acc.a += (1 - acc.a) * alpha
    const float2 tr = dup2(__fadd_rn(1.0f, -acc_ba.y));
    const float2 src_rg = __fmul2_rn(__fmul2_rn(crg, dup2(light)), dup2(alpha));
    const float src_b = __fmul_rn(__fmul_rn(cba.x, light), alpha);
    const float2 add_rg = __fmul2_rn(tr, src_rg);
    const float2 add_ba = __fmul2_rn(tr, make_float2(src_b, alpha));
    acc_rg = make_float2(__fadd_rn(acc_rg.x, add_rg.x), __fadd_rn(acc_rg.y, add_rg.y));
    acc_ba = make_float2(__fadd_rn(acc_ba.x, add_ba.x), __fadd_rn(acc_ba.y, add_ba.y));
}

__device__ __forceinline__ uint32_t blend_rgba8(float2 rg, float2 ba) {
    // SRC_ALPHA / ONE_MINUS_SRC_ALPHA over a cleared UNORM8 target.
    const float a = fminf(fmaxf(ba.y, 0.0f), 1.0f);
    const uint32_t r = (uint32_t)rintf(__fmul_rn(__fmul_rn(fminf(fmaxf(rg.x, 0.0f), 1.0f), a), 255.0f));
    const uint32_t g = (uint32_t)rintf(__fmul_rn(__fmul_rn(fminf(fmaxf(rg.y, 0.0f), 1.0f), a), 255.0f));
    const uint32_t b = (uint32_t)rintf(__fmul_rn(__fmul_rn(fminf(fmaxf(ba.x, 0.0f), 1.0f), a), 255.0f));
    const uint32_t al = (uint32_t)rintf(__fmul_rn(__fmul_rn(a, a), 255.0f));
    return r | (g << 8) | (b << 16) | (al << 24);
}

// Is a sample of this brick exactly transparent under the job's LUT?
// m = the brick's (min, max) stored values.
template <bool SMEM_LUT, bool FAST>
__device__ __forceinline__ bool brick_clear(const MarchFrame &f, float2 m, const int *prefix) {
    if (!(m.x == m.x)) return false;  // NaN in the brick
    const float d0 = __fmul_rn(m.x, f.value_scale), d1 = __fmul_rn(m.y, f.value_scale);
    const float dlo = fminf(d0, d1), dhi = fmaxf(d0, d1);
    if (!(dlo == dlo && dhi == dhi)) return false;
    // the LUT coordinates of the extreme densities, rounded as the march
    // rounds them (FAST: one FMA); both roundings are monotone in d
    const float clo = FAST ? fmaf(dlo, f.flut_size, -0.5f) : __fadd_rn(__fmul_rn(dlo, f.flut_size), -0.5f);
    const float chi = FAST ? fmaf(dhi, f.flut_size, -0.5f) : __fadd_rn(__fmul_rn(dhi, f.flut_size), -0.5f);
    const int ilo = lut_index(floorf(clo), f.flut_max);
    const int ihi = lut_index(__fadd_rn(floorf(chi), 1.0f), f.flut_max);
    return prefix_entry<SMEM_LUT>(prefix, ihi + 1) == prefix_entry<SMEM_LUT>(prefix, ilo);
}

// One pixel's ray of volume.frag.glsl:main (lines 70-122).
template <int LOG2B, int UNROLL, bool NORMALS, bool SMEM_LUT, bool COMPACT, bool FAST>
__device__ __forceinline__ void march_ray(const JobDesc &job, int px, int py, const float4 *lut,
                                          const int *prefix, float2 &acc_rg, float2 &acc_ba,
                                          unsigned &n_inbox, unsigned &n_shaded) {
    constexpr int B = 1 << LOG2B, ROW = brick_apron(LOG2B), SLICE = ROW * ROW;
    constexpr int RECS = brick_records(LOG2B);
    const MarchFrame &f = job.f;
    float pos[3], dstep[3];
    if (!setup_ray(f, px, py, pos, dstep)) return;
    // (x, y) lanes packed, z scalar; per lane the reference expressions
    float2 pxy = make_float2(pos[0], pos[1]);
    float pz = pos[2];
    const float2 dxy = make_float2(dstep[0], dstep[1]);
    const float dz = dstep[2];
    const float2 nbmin_xy = make_float2(-f.bmin[0], -f.bmin[1]);
    const float2 inv_xy = make_float2(f.inv_ext[0], f.inv_ext[1]);
    const float2 fext_xy = make_float2(f.fext[0], f.fext[1]);
    const float nbmin_z = -f.bmin[2], inv_z = f.inv_ext[2], fext_z = f.fext[2];
    const int nb1 = f.nb[1], nb2 = f.nb[2];
    bool entered = false;
    int cur_brick = -1;
    bool clear = false;
    using Rec = typename RecordOf<COMPACT>::T;
    const Rec *bp = static_cast<const Rec *>(job.records);
    int i = 0;
    for (;;) {
#pragma unroll
        for (int u = 0; u < UNROLL; ++u) {
            if (!(i < f.max_steps && acc_ba.y < 0.99f)) return;
            // world_to_texture_coords (frag:25-27, 88)
            const float2 txy = __fmul2_rn(__fadd2_rn(pxy, nbmin_xy), inv_xy);
            const float tz = __fmul_rn(__fadd_rn(pz, nbmin_z), inv_z);
            const bool valid = txy.x >= 0.0f && txy.x <= 1.0f && txy.y >= 0.0f &&
                               txy.y <= 1.0f && tz >= 0.0f && tz <= 1.0f;
            if (valid) {
                entered = true;
                ++n_inbox;
                // texel coordinate u = t*size - 0.5, lower texel k = floor(u)
                const float2 sxy = __fmul2_rn(txy, fext_xy);
                const float ux = __fadd_rn(sxy.x, -0.5f), uy = __fadd_rn(sxy.y, -0.5f);
                const float uz = __fadd_rn(__fmul_rn(tz, fext_z), -0.5f);
                const float flx = floorf(ux), fly = floorf(uy), flz = floorf(uz);
                const int kx = (int)flx + 1, ky = (int)fly + 1, kz = (int)flz + 1;
                const int id = ((kx >> LOG2B) * nb1 + (ky >> LOG2B)) * nb2 + (kz >> LOG2B);
                if (id != cur_brick) {
                    cur_brick = id;
                    const uint4 bi = __ldg(job.bricks + id);
                    bp = static_cast<const Rec *>(job.records) + (size_t)bi.x * RECS;
                    clear = job.skip &&
                            brick_clear<SMEM_LUT, FAST>(f, make_float2(__uint_as_float(bi.y),
                                                                       __uint_as_float(bi.z)),
                                                        prefix);
                }
                if (!clear) {
                    ++n_shaded;
                    const int j = (kx & (B - 1)) * SLICE + (ky & (B - 1)) * ROW + (kz & (B - 1));
                    shade_sample<LOG2B, NORMALS, SMEM_LUT, FAST>(f, bp + j, __fadd_rn(ux, -flx),
                                                                 __fadd_rn(uy, -fly), __fadd_rn(uz, -flz),
                                                                 lut, acc_rg, acc_ba);
                }
            } else {
                const bool never = entered || (txy.x < 0.0f && dxy.x <= 0.0f) ||
                                   (txy.x > 1.0f && dxy.x >= 0.0f) ||
                                   (txy.y < 0.0f && dxy.y <= 0.0f) ||
                                   (txy.y > 1.0f && dxy.y >= 0.0f) || (tz < 0.0f && dz <= 0.0f) ||
                                   (tz > 1.0f && dz >= 0.0f);
                if (never) return;
            }
            // current_world_pos += ray_dir * step_size (frag:118)
            pxy = __fadd2_rn(pxy, dxy);
            pz = __fadd_rn(pz, dz);
            ++i;
        }
    }
}

template <int LOG2B, int UNROLL, bool NORMALS, bool SMEM_LUT, bool COMPACT, bool FAST>
__device__ __forceinline__ void march_tile(const JobDesc &job, int px, int py, const float4 *lut,
                                           const int *prefix, int lane) {
    const bool in_image = px < job.f.width && py < job.f.height;
    float2 acc_rg = make_float2(0.0f, 0.0f), acc_ba = make_float2(0.0f, 0.0f);
    unsigned n_inbox = 0, n_shaded = 0;
    if (in_image)
        march_ray<LOG2B, UNROLL, NORMALS, SMEM_LUT, COMPACT, FAST>(job, px, py, lut, prefix, acc_rg, acc_ba,
                                                                   n_inbox, n_shaded);
    if (in_image) {
        const long long idx = (long long)py * job.f.width + px;
        if (job.out8) job.out8[idx] = blend_rgba8(acc_rg, acc_ba);
        if (job.outf) job.outf[idx] = make_float4(acc_rg.x, acc_rg.y, acc_ba.x, acc_ba.y);
    }
    if (job.counters) {
        unsigned long long a = n_inbox, b = n_shaded;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
        }
        if (lane == 0 && a) {
            atomicAdd(job.counters, a);
            atomicAdd(job.counters + 1, b);
        }
    }
}

// Persistent batch kernel of one variant: normals or not, LUT staged in
// shared memory or read from global memory, float or half records, exact or
// fast arithmetic (the launcher groups a batch's jobs by variant, so that
// each kernel carries one march and stays within its register budget).  The
// job table is the kernel's own parameter block (read through the constant
// cache).  Dynamic shared memory (SMEM_LUT): p.lut_smem_entries float4 LUT
// entries followed by as many + 1 prefix counts, at least every job's LUT.
template <int LOG2B, int UNROLL, bool NORMALS, bool SMEM_LUT, bool COMPACT, bool FAST>
__global__ void __launch_bounds__(kBatchThreads, COMPACT ? 5 : 4)
march_batch_kernel(const __grid_constant__ BatchParams p) {
    extern __shared__ float4 s_dyn[];
    float4 *s_lut = s_dyn;
    int *s_prefix = reinterpret_cast<int *>(s_dyn + p.lut_smem_entries);
    __shared__ int s_tile, s_job_idx;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int warps_x = p.tile_w >> 3;
    const int sub_x = (warp % warps_x) * 8 + (lane & 7);
    const int sub_y = (warp / warps_x) * 4 + (lane >> 3);
    int cur_job = -1;
    for (;;) {
        if (threadIdx.x == 0) {
            const int t = atomicAdd(p.work, 1);
            int lo = 0, hi = p.njobs - 1;  // last job whose first tile is <= t
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (p.tile_base[mid] <= t) lo = mid; else hi = mid - 1;
            }
            s_tile = t;
            s_job_idx = lo;
        }
        __syncthreads();
        const int t = s_tile, j = s_job_idx;
        if (t >= p.total_tiles) break;
        const JobDesc &job = p.jobs[j];
        if (SMEM_LUT && j != cur_job) {
            // stage the job's LUT (the previous tile's readers passed the
            // barrier at the end of the last round)
            for (int k = threadIdx.x; k < job.f.lut_size; k += kBatchThreads) s_lut[k] = job.lut[k];
            for (int k = threadIdx.x; k <= job.f.lut_size; k += kBatchThreads) s_prefix[k] = job.prefix[k];
            __syncthreads();
            cur_job = j;
        }
        const int local = t - job.tile_base;
        const int px = (local % job.tiles_x) * p.tile_w + sub_x;
        const int py = (local / job.tiles_x) * p.tile_h + sub_y;
        march_tile<LOG2B, UNROLL, NORMALS, SMEM_LUT, COMPACT, FAST>(job, px, py, SMEM_LUT ? s_lut : job.lut,
                                                                    SMEM_LUT ? s_prefix : job.prefix, lane);
        __syncthreads();  // s_tile / the staged LUT are rewritten next round
    }
}

// Single-job kernel: one block per tile of one render; the job descriptor
// is the parameter block itself (static offsets), as in a plain frame kernel.
// One instantiation per variant (normals, LUT in shared memory, half
// records, arithmetic), chosen on the host: each gets its own register
// allocation.  SMEM_LUT requires job.f.lut_size <= p.lut_smem_entries.  Half
// records need 16 fewer registers for a sample's 8 records: those variants
// run 6 blocks per SM (40 registers) instead of 5 (48).
template <int LOG2B, int UNROLL, bool NORMALS, bool SMEM_LUT, bool COMPACT, bool FAST>
__global__ void __launch_bounds__(kBatchThreads, COMPACT ? 6 : 5)
march_single_kernel(const __grid_constant__ SingleParams p) {
    extern __shared__ float4 s_dyn[];
    float4 *s_lut = s_dyn;
    int *s_prefix = reinterpret_cast<int *>(s_dyn + p.lut_smem_entries);
    const JobDesc &job = p.job;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int warps_x = p.tile_w >> 3;
    if (SMEM_LUT) {
        for (int k = threadIdx.x; k < job.f.lut_size; k += kBatchThreads) s_lut[k] = job.lut[k];
        for (int k = threadIdx.x; k <= job.f.lut_size; k += kBatchThreads) s_prefix[k] = job.prefix[k];
        __syncthreads();
    }
    const int t = blockIdx.x;
    const int px = (t % job.tiles_x) * p.tile_w + (warp % warps_x) * 8 + (lane & 7);
    const int py = (t / job.tiles_x) * p.tile_h + (warp / warps_x) * 4 + (lane >> 3);
    march_tile<LOG2B, UNROLL, NORMALS, SMEM_LUT, COMPACT, FAST>(job, px, py, SMEM_LUT ? s_lut : job.lut,
                                                                SMEM_LUT ? s_prefix : job.prefix, lane);
}

template <int LOG2B, int UNROLL, bool FAST>
const void *single_variant_of(int v) {
    switch (v & 7) {
    case 0: return (const void *)march_single_kernel<LOG2B, UNROLL, false, false, false, FAST>;
    case 1: return (const void *)march_single_kernel<LOG2B, UNROLL, true, false, false, FAST>;
    case 2: return (const void *)march_single_kernel<LOG2B, UNROLL, false, true, false, FAST>;
    case 3: return (const void *)march_single_kernel<LOG2B, UNROLL, true, true, false, FAST>;
    case 4: return (const void *)march_single_kernel<LOG2B, UNROLL, false, false, true, FAST>;
    case 5: return (const void *)march_single_kernel<LOG2B, UNROLL, true, false, true, FAST>;
    case 6: return (const void *)march_single_kernel<LOG2B, UNROLL, false, true, true, FAST>;
    default: return (const void *)march_single_kernel<LOG2B, UNROLL, true, true, true, FAST>;
    }
}

template <int LOG2B, int UNROLL>
const void *single_variant(int v) {
    return (v & kSingleFast) ? single_variant_of<LOG2B, UNROLL, true>(v) : single_variant_of<LOG2B, UNROLL, false>(v);
}

template <int LOG2B>
const void *single_kernel_log2(const Tuning &t, int variant) {
    if (t.steps_per_iter >= 4) return single_variant<LOG2B, 4>(variant);
    return single_variant<LOG2B, 1>(variant);
}

template <int LOG2B, int UNROLL, bool FAST>
const void *batch_variant_of(int v) {
    switch (v & 7) {
    case 0: return (const void *)march_batch_kernel<LOG2B, UNROLL, false, false, false, FAST>;
    case 1: return (const void *)march_batch_kernel<LOG2B, UNROLL, true, false, false, FAST>;
    case 2: return (const void *)march_batch_kernel<LOG2B, UNROLL, false, true, false, FAST>;
    case 3: return (const void *)march_batch_kernel<LOG2B, UNROLL, true, true, false, FAST>;
    case 4: return (const void *)march_batch_kernel<LOG2B, UNROLL, false, false, true, FAST>;
    case 5: return (const void *)march_batch_kernel<LOG2B, UNROLL, true, false, true, FAST>;
    case 6: return (const void *)march_batch_kernel<LOG2B, UNROLL, false, true, true, FAST>;
    default: return (const void *)march_batch_kernel<LOG2B, UNROLL, true, true, true, FAST>;
    }
}

template <int LOG2B, int UNROLL>
const void *batch_variant(int v) {
    return (v & kSingleFast) ? batch_variant_of<LOG2B, UNROLL, true>(v) : batch_variant_of<LOG2B, UNROLL, false>(v);
}

template <int LOG2B>
const void *batch_kernel_log2(const Tuning &t, int variant) {
    if (t.steps_per_iter >= 4) return batch_variant<LOG2B, 4>(variant);
    return batch_variant<LOG2B, 1>(variant);
}

template <int LOG2B>
int max_blocks_log2(const Tuning &t, int lut_smem_entries, int variant) {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel_log2<LOG2B>(t, variant), kBatchThreads,
                                                  batch_smem_bytes(lut_smem_entries));
    return n;
}

}  // namespace pvr
