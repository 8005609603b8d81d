// Device layout of a loaded volume for the march kernel.
//
// The reference keeps the voxels and the normals as two 3D textures
// (pyvr/moderngl_renderer/manager.py:77-135).  Here both are re-laid out
// once per volume into 16-byte texel records {stored value, nx, ny, nz}
// (the stored value converted exactly to float; uint8 and float16 keep
// their values, the scale to density is applied after interpolation),
// grouped in bricks of (kBrick+1)^3 records.  The brick grid is shifted by
// one texel: brick b holds, at local index l, the texel
// clamp(b*kBrick - 1 + l, 0, extent - 1) on each axis.  A sample with lower
// texel k = floor(u) in [-1, extent-1] uses brick (k+1)/kBrick and local
// indices j = (k+1) % kBrick and j+1, which hold exactly the clamp-to-edge
// texels k0 = clamp(k) and k1 = clamp(k+1) of the GL filter: the clamping
// is baked into the records, and the 8 texels of a sample sit at fixed
// offsets from one record address.  Bricks are
// stored in Morton order of their brick coordinates (a warp's rays walk
// neighbouring bricks, which then sit in neighbouring memory), located
// through a brick table whose top bit flags "transparent under the current
// LUT" for empty-space skipping.
#include <algorithm>
#include <vector>

#include "pvr_device.cuh"
#include "pvr_internal.h"

namespace pvr {

namespace {

template <typename T> __device__ __forceinline__ float raw_value(const T *p, long long i);
template <> __device__ __forceinline__ float raw_value<float>(const float *p, long long i) { return p[i]; }
template <> __device__ __forceinline__ float raw_value<uint8_t>(const uint8_t *p, long long i) {
    return (float)p[i];
}
template <> __device__ __forceinline__ float raw_value<__half>(const __half *p, long long i) {
    return __half2float(p[i]);
}

// One thread per record.  Voxel (x, y, z) along world axes lives at
// z + D*(y + H*x) of the (D,H,W) C-order buffer (the GL texture of size
// (D,H,W) read through the z/y/x swizzle, volume.frag.glsl:90).
template <typename T>
__global__ void build_records_kernel(BrickGeometry g, const T *__restrict__ vol,
                                     const float *__restrict__ nrm,
                                     const uint32_t *__restrict__ table,
                                     float4 *__restrict__ records) {
    const long long total = (long long)g.nbricks * kRecordsPerBrick;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < total;
         r += (long long)gridDim.x * blockDim.x) {
        const int brick = (int)(r / kRecordsPerBrick);
        const int rec = (int)(r - (long long)brick * kRecordsPerBrick);
        const int bz = brick % g.nb[2];
        const int by = (brick / g.nb[2]) % g.nb[1];
        const int bx = brick / (g.nb[2] * g.nb[1]);
        const int lz = rec % kApron, ly = (rec / kApron) % kApron, lx = rec / (kApron * kApron);
        const int x = min(max(bx * kBrick - 1 + lx, 0), g.ext[0] - 1);
        const int y = min(max(by * kBrick - 1 + ly, 0), g.ext[1] - 1);
        const int z = min(max(bz * kBrick - 1 + lz, 0), g.ext[2] - 1);
        const long long src = z + (long long)g.ext[2] * (y + (long long)g.ext[1] * x);
        float4 v;
        v.x = raw_value<T>(vol, src);
        if (nrm) {
            v.y = nrm[3 * src + 0];
            v.z = nrm[3 * src + 1];
            v.w = nrm[3 * src + 2];
        } else {
            v.y = v.z = v.w = 0.0f;
        }
        const uint32_t slot = table[brick] & kSlotMask;
        records[(size_t)slot * kRecordsPerBrick + rec] = v;
    }
}

// One warp per brick: min/max of the stored values over all its records
// (the footprints of every sample that maps to it).  A NaN marks the brick
// as never skippable.
__global__ void brick_minmax_kernel(BrickGeometry g, const uint32_t *__restrict__ table,
                                    const float4 *__restrict__ records, float2 *__restrict__ mm) {
    const int warps = blockDim.x >> 5;
    const int lane = threadIdx.x & 31;
    for (int b = blockIdx.x * warps + (threadIdx.x >> 5); b < g.nbricks; b += gridDim.x * warps) {
        const float4 *rp = records + (size_t)(table[b] & kSlotMask) * kRecordsPerBrick;
        float lo = __int_as_float(0x7f800000), hi = -lo;
        bool nan = false;
        for (int i = lane; i < kRecordsPerBrick; i += 32) {
            float v = rp[i].x;
            nan |= v != v;
            lo = fminf(lo, v);
            hi = fmaxf(hi, v);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        nan = __any_sync(0xffffffffu, nan);
        if (lane == 0) mm[b] = nan ? make_float2(__int_as_float(0x7fc00000), 0.0f) : make_float2(lo, hi);
    }
}

// Transparent flag of each brick for one LUT: every LUT entry that a sample
// of the brick can read has alpha exactly 0 and a finite colour.  Such a
// sample adds exactly +0 to every accumulator (volume.frag.glsl:101-115), so
// skipping it changes no bit of the result.  The entry range is exact, not
// padded: a lerp fmaf(t, b - a, a) with t in [0, 1) never leaves
// [min(a,b), max(a,b)], so a trilinear sample lies in the brick's value
// range, and the scale and the LUT coordinate d*size - 0.5 are monotone
// float operations evaluated here exactly as the march kernel does.
__global__ void brick_flags_kernel(BrickGeometry g, float value_scale, int lut_size,
                                   const int *__restrict__ opaque_prefix, int enable,
                                   const float2 *__restrict__ mm, uint32_t *__restrict__ table) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < g.nbricks; b += gridDim.x * blockDim.x) {
        float2 m = mm[b];
        bool transparent = false;
        if (enable && m.x == m.x) {
            float d0 = m.x * value_scale, d1 = m.y * value_scale;
            float dlo = fminf(d0, d1), dhi = fmaxf(d0, d1);
            float flo = floorf(dlo * (float)lut_size - 0.5f);
            float fhi = floorf(dhi * (float)lut_size - 0.5f) + 1.0f;
            float fmax_idx = (float)(lut_size - 1);
            int ilo = !(flo >= 0.0f) ? 0 : (flo > fmax_idx ? lut_size - 1 : (int)flo);
            int ihi = !(fhi >= 0.0f) ? 0 : (fhi > fmax_idx ? lut_size - 1 : (int)fhi);
            if (dlo == dlo && dhi == dhi)  // finite range (inf*0 etc. excluded)
                transparent = opaque_prefix[ihi + 1] - opaque_prefix[ilo] == 0;
        }
        uint32_t e = table[b] & kSlotMask;
        table[b] = transparent ? (e | kTransparentBit) : e;
    }
}

uint32_t spread3(uint32_t v) {  // 10 bits -> every third bit
    v &= 0x3ff;
    v = (v | (v << 16)) & 0x030000ff;
    v = (v | (v << 8)) & 0x0300f00f;
    v = (v | (v << 4)) & 0x030c30c3;
    v = (v | (v << 2)) & 0x09249249;
    return v;
}

}  // namespace

BrickGeometry make_brick_geometry(const int dims_dhw[3]) {
    BrickGeometry g;
    g.ext[0] = dims_dhw[2];  // world x <-> W
    g.ext[1] = dims_dhw[1];  // world y <-> H
    g.ext[2] = dims_dhw[0];  // world z <-> D
    // k + 1 ranges over [0, extent]
    for (int a = 0; a < 3; ++a) g.nb[a] = g.ext[a] / kBrick + 1;
    g.nbricks = g.nb[0] * g.nb[1] * g.nb[2];
    return g;
}

// Slot of every brick: rank of its Morton code (x, y, z interleaved).
std::vector<uint32_t> morton_slots(const BrickGeometry &g) {
    std::vector<std::pair<uint64_t, uint32_t>> key(g.nbricks);
    for (int bx = 0; bx < g.nb[0]; ++bx)
        for (int by = 0; by < g.nb[1]; ++by)
            for (int bz = 0; bz < g.nb[2]; ++bz) {
                uint32_t id = (uint32_t)((bx * g.nb[1] + by) * g.nb[2] + bz);
                uint64_t m = ((uint64_t)spread3(bx) << 2) | ((uint64_t)spread3(by) << 1) | spread3(bz);
                key[id] = {m, id};
            }
    std::sort(key.begin(), key.end());
    std::vector<uint32_t> table(g.nbricks);
    for (uint32_t s = 0; s < (uint32_t)g.nbricks; ++s) table[key[s].second] = s;
    return table;
}

cudaError_t launch_build_records(const BrickGeometry &g, int dtype, const void *vol, const float *nrm,
                                 const uint32_t *table, float4 *records, float2 *minmax,
                                 cudaStream_t st) {
    const long long total = (long long)g.nbricks * kRecordsPerBrick;
    int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 64);
    switch (dtype) {
    case PVR_U8:
        build_records_kernel<uint8_t><<<blocks, 256, 0, st>>>(g, (const uint8_t *)vol, nrm, table, records);
        break;
    case PVR_F16:
        build_records_kernel<__half><<<blocks, 256, 0, st>>>(g, (const __half *)vol, nrm, table, records);
        break;
    default:
        build_records_kernel<float><<<blocks, 256, 0, st>>>(g, (const float *)vol, nrm, table, records);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    int mblocks = std::max(1, std::min((g.nbricks + 7) / 8, 152 * 16));
    brick_minmax_kernel<<<mblocks, 256, 0, st>>>(g, table, records, minmax);
    return cudaGetLastError();
}

cudaError_t launch_brick_flags(const BrickGeometry &g, float value_scale, int lut_size,
                               const int *opaque_prefix, bool enable, const float2 *minmax,
                               uint32_t *table, cudaStream_t st) {
    int blocks = std::max(1, std::min((g.nbricks + 255) / 256, 152 * 8));
    brick_flags_kernel<<<blocks, 256, 0, st>>>(g, value_scale, lut_size, opaque_prefix, enable ? 1 : 0,
                                               minmax, table);
    return cudaGetLastError();
}

}  // namespace pvr
