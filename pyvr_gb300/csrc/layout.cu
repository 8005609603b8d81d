// Device layout of a loaded volume for the march kernel.
//
// The reference keeps the voxels and the normals as two 3D textures
// (pyvr/moderngl_renderer/manager.py:77-135).  Here both are re-laid out
// once per volume into 16-byte texel records {stored value, nx, ny, nz}
// (the stored value converted exactly to float; uint8 and float16 keep
// their values, the scale to density is applied after interpolation),
// grouped in bricks of (B+1)^3 records for bricks of B^3 texels.  The
// brick grid is shifted by one texel: brick b holds, at local index l, the
// texel clamp(b*B - 1 + l, 0, extent - 1) on each axis.  A sample with
// lower texel k = floor(u) in [-1, extent-1] uses brick (k+1)/B and local
// indices j = (k+1) % B and j+1, which hold exactly the clamp-to-edge texels
// clamp(k) and clamp(k+1) of the GL filter: the clamping is baked into the
// records, and the 8 texels of a sample sit at fixed offsets from one
// record address.  Bricks are stored in Morton order of their brick
// coordinates (a warp's rays walk neighbouring bricks, which then sit in
// neighbouring memory), located through a brick table.  A per-brick
// min/max of the stored values lets the march skip bricks that the current
// LUT makes exactly transparent.
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

__device__ __forceinline__ float round_half(float x) { return __half2float(__float2half_rn(x)); }

// Normal of array element (a, b, c) of the (D,H,W) volume, as
// pyvr/datasets/synthetic.py:109-122 computes it with numpy:
// g_axis = numpy.gradient along each array axis (central difference / 2
// inside, one-sided on the two faces, unit spacing), n = |g| + 1e-8 with
// the squares summed left to right, normal = g / n, cast to float32.
// numpy evaluates this in float64 for integer input, in float16 (each
// operation rounded to half, sums accumulated in float) for float16 input,
// and in float32 for float32 input; so does this function.
template <typename T> struct GradientArith;

template <> struct GradientArith<float> {
    static __device__ float3 normal(const float *v, const int dims[3], int a, int b, int c) {
        float g[3];
        const int idx[3] = {a, b, c};
        const long long stride[3] = {(long long)dims[1] * dims[2], dims[2], 1};
        const long long base = a * stride[0] + b * stride[1] + c;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const int i = idx[ax], n = dims[ax];
            const long long s = stride[ax];
            if (i == 0) g[ax] = __fsub_rn(v[base + s], v[base]);
            else if (i == n - 1) g[ax] = __fsub_rn(v[base], v[base - s]);
            else g[ax] = __fmul_rn(__fsub_rn(v[base + s], v[base - s]), 0.5f);
        }
        float ss = __fadd_rn(__fadd_rn(__fmul_rn(g[0], g[0]), __fmul_rn(g[1], g[1])), __fmul_rn(g[2], g[2]));
        float nrm = __fadd_rn(__fsqrt_rn(ss), 1e-8f);
        return make_float3(__fdiv_rn(g[0], nrm), __fdiv_rn(g[1], nrm), __fdiv_rn(g[2], nrm));
    }
};

template <> struct GradientArith<uint8_t> {
    static __device__ float3 normal(const uint8_t *v, const int dims[3], int a, int b, int c) {
        double g[3];
        const int idx[3] = {a, b, c};
        const long long stride[3] = {(long long)dims[1] * dims[2], dims[2], 1};
        const long long base = a * stride[0] + b * stride[1] + c;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const int i = idx[ax], n = dims[ax];
            const long long s = stride[ax];
            if (i == 0) g[ax] = (double)v[base + s] - (double)v[base];
            else if (i == n - 1) g[ax] = (double)v[base] - (double)v[base - s];
            else g[ax] = ((double)v[base + s] - (double)v[base - s]) / 2.0;  // exact
        }
        double ss = __dadd_rn(__dadd_rn(__dmul_rn(g[0], g[0]), __dmul_rn(g[1], g[1])), __dmul_rn(g[2], g[2]));
        double nrm = __dadd_rn(__dsqrt_rn(ss), 1e-8);
        return make_float3(__double2float_rn(__ddiv_rn(g[0], nrm)), __double2float_rn(__ddiv_rn(g[1], nrm)),
                           __double2float_rn(__ddiv_rn(g[2], nrm)));
    }
};

template <> struct GradientArith<__half> {
    static __device__ float3 normal(const __half *v, const int dims[3], int a, int b, int c) {
        float g[3];
        const int idx[3] = {a, b, c};
        const long long stride[3] = {(long long)dims[1] * dims[2], dims[2], 1};
        const long long base = a * stride[0] + b * stride[1] + c;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const int i = idx[ax], n = dims[ax];
            const long long s = stride[ax];
            if (i == 0) {
                g[ax] = round_half(__fsub_rn(__half2float(v[base + s]), __half2float(v[base])));
            } else if (i == n - 1) {
                g[ax] = round_half(__fsub_rn(__half2float(v[base]), __half2float(v[base - s])));
            } else {
                float d = round_half(__fsub_rn(__half2float(v[base + s]), __half2float(v[base - s])));
                g[ax] = round_half(__fdiv_rn(d, 2.0f));
            }
        }
        // squares rounded to half; the sum accumulates in float, rounds once
        float q0 = round_half(__fmul_rn(g[0], g[0]));
        float q1 = round_half(__fmul_rn(g[1], g[1]));
        float q2 = round_half(__fmul_rn(g[2], g[2]));
        float ss = round_half(__fadd_rn(__fadd_rn(q0, q1), q2));
        float nrm = round_half(__fsqrt_rn(ss));  // + 1e-8 rounds to + 0 in half
        return make_float3(round_half(__fdiv_rn(g[0], nrm)), round_half(__fdiv_rn(g[1], nrm)),
                           round_half(__fdiv_rn(g[2], nrm)));
    }
};

// One thread per record.  Voxel (x, y, z) along world axes lives at
// z + D*(y + H*x) of the (D,H,W) C-order buffer (the GL texture of size
// (D,H,W) read through the z/y/x swizzle, volume.frag.glsl:90); the normal
// texture is indexed the same way (manager.py:123-125).
template <typename T, int LOG2B>
__global__ void build_records_kernel(BrickGeometry g, const T *__restrict__ vol, int D, int H, int W,
                                     const float *__restrict__ nrm, int normals_mode,
                                     const uint32_t *__restrict__ table,
                                     float4 *__restrict__ records) {
    constexpr int B = 1 << LOG2B, A = B + 1, R = A * A * A;
    const int dims[3] = {D, H, W};
    const long long total = (long long)g.nbricks * R;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < total;
         r += (long long)gridDim.x * blockDim.x) {
        const int brick = (int)(r / R);
        const int rec = (int)(r - (long long)brick * R);
        const int bz = brick % g.nb[2];
        const int by = (brick / g.nb[2]) % g.nb[1];
        const int bx = brick / (g.nb[2] * g.nb[1]);
        const int lz = rec % A, ly = (rec / A) % A, lx = rec / (A * A);
        const int x = min(max(bx * B - 1 + lx, 0), g.ext[0] - 1);
        const int y = min(max(by * B - 1 + ly, 0), g.ext[1] - 1);
        const int z = min(max(bz * B - 1 + lz, 0), g.ext[2] - 1);
        const long long src = z + (long long)g.ext[2] * (y + (long long)g.ext[1] * x);
        float4 v;
        v.x = raw_value<T>(vol, src);
        if (normals_mode == PVR_NORMALS_GIVEN) {
            v.y = nrm[3 * src + 0];
            v.z = nrm[3 * src + 1];
            v.w = nrm[3 * src + 2];
        } else if (normals_mode == PVR_NORMALS_DEVICE) {
            // array position of flat element `src` in the (D,H,W) array
            const int c = (int)(src % W);
            const int b = (int)((src / W) % H);
            const int a = (int)(src / ((long long)W * H));
            const float3 n = GradientArith<T>::normal(vol, dims, a, b, c);
            v.y = n.x;
            v.z = n.y;
            v.w = n.z;
        } else {
            v.y = v.z = v.w = 0.0f;
        }
        const uint32_t slot = table[brick];
        records[(size_t)slot * R + rec] = v;
    }
}

// One warp per brick: min/max of the stored values over all its records
// (the footprints of every sample that maps to it), stored with the brick's
// record slot.  A NaN marks the brick as never skippable.
template <int LOG2B>
__global__ void brick_minmax_kernel(BrickGeometry g, const uint32_t *__restrict__ table,
                                    const float4 *__restrict__ records, uint4 *__restrict__ bricks) {
    constexpr int R = brick_records(LOG2B);
    const int warps = blockDim.x >> 5;
    const int lane = threadIdx.x & 31;
    for (int b = blockIdx.x * warps + (threadIdx.x >> 5); b < g.nbricks; b += gridDim.x * warps) {
        const uint32_t slot = table[b];
        const float4 *rp = records + (size_t)slot * R;
        float lo = __int_as_float(0x7f800000), hi = -lo;
        bool nan = false;
        for (int i = lane; i < R; i += 32) {
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
        if (lane == 0)
            bricks[b] = nan ? make_uint4(slot, 0x7fc00000u, 0u, 0u)
                            : make_uint4(slot, __float_as_uint(lo), __float_as_uint(hi), 0u);
    }
}

// A float survives float -> half -> float bit for bit (NaN: as some NaN).
__device__ __forceinline__ bool half_exact(float x, unsigned short &h) {
    const __half hv = __float2half_rn(x);
    h = __half_as_ushort(hv);
    const float back = __half2float(hv);
    if (x != x) return back != back;
    return __float_as_uint(back) == __float_as_uint(x);
}

// Compact records: {value, nx, ny, nz} as four halves in one 8-byte record.
// The march decodes them exactly, so a volume whose records all survive the
// round trip renders the same images from either form.
__global__ void compact_records_kernel(const float4 *__restrict__ in, uint2 *__restrict__ out, long long n,
                                       int *__restrict__ inexact) {
    bool ok = true;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float4 r = in[i];
        unsigned short h0, h1, h2, h3;
        ok &= half_exact(r.x, h0);
        ok &= half_exact(r.y, h1);
        ok &= half_exact(r.z, h2);
        ok &= half_exact(r.w, h3);
        out[i] = make_uint2((uint32_t)h0 | ((uint32_t)h1 << 16), (uint32_t)h2 | ((uint32_t)h3 << 16));
    }
    if (__any_sync(0xffffffffu, !ok) && (threadIdx.x & 31) == 0) atomicExch(inexact, 1);
}

__device__ __forceinline__ float4 record_at(const float4 *r, size_t i) { return r[i]; }
__device__ __forceinline__ float4 record_at(const uint2 *r, size_t i) {
    const uint2 q = r[i];
    return make_float4(__half2float(__ushort_as_half((unsigned short)(q.x & 0xffffu))),
                       __half2float(__ushort_as_half((unsigned short)(q.x >> 16))),
                       __half2float(__ushort_as_half((unsigned short)(q.y & 0xffffu))),
                       __half2float(__ushort_as_half((unsigned short)(q.y >> 16))));
}

// Scatter the normals held in the records back to (D,H,W,3): one thread per
// texel, reading the record of local index (k+1) % B in brick (k+1) / B.
template <int LOG2B, typename Rec>
__global__ void read_normals_kernel(BrickGeometry g, int D, int H, int W,
                                    const uint32_t *__restrict__ table,
                                    const Rec *__restrict__ records, float *__restrict__ out) {
    constexpr int B = 1 << LOG2B, A = B + 1, R = A * A * A;
    const long long total = (long long)D * H * W;
    for (long long src = blockIdx.x * (long long)blockDim.x + threadIdx.x; src < total;
         src += (long long)gridDim.x * blockDim.x) {
        // flat texel index src = z + D*(y + H*x) (world axes)
        const int z = (int)(src % D);
        const int y = (int)((src / D) % H);
        const int x = (int)(src / ((long long)D * H));
        const int kx = x + 1, ky = y + 1, kz = z + 1;
        const int id = ((kx >> LOG2B) * g.nb[1] + (ky >> LOG2B)) * g.nb[2] + (kz >> LOG2B);
        const int rec = ((kx & (B - 1)) * A + (ky & (B - 1))) * A + (kz & (B - 1));
        const float4 v = record_at(records, (size_t)table[id] * R + rec);
        out[3 * src + 0] = v.y;
        out[3 * src + 1] = v.z;
        out[3 * src + 2] = v.w;
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

template <typename T, int LOG2B>
cudaError_t build_typed(const BrickGeometry &g, const void *vol, const int dims[3], const float *nrm,
                        int normals_mode, const uint32_t *table, float4 *records, uint4 *bricks,
                        cudaStream_t st) {
    constexpr int R = brick_records(LOG2B);
    const long long total = (long long)g.nbricks * R;
    int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 64);
    build_records_kernel<T, LOG2B><<<blocks, 256, 0, st>>>(g, (const T *)vol, dims[0], dims[1], dims[2],
                                                          nrm, normals_mode, table, records);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    int mblocks = std::max(1, std::min((g.nbricks + 7) / 8, 152 * 16));
    brick_minmax_kernel<LOG2B><<<mblocks, 256, 0, st>>>(g, table, records, bricks);
    return cudaGetLastError();
}

template <int LOG2B>
cudaError_t build_log2(const BrickGeometry &g, int dtype, const void *vol, const int dims[3],
                       const float *nrm, int normals_mode, const uint32_t *table, float4 *records,
                       uint4 *bricks, cudaStream_t st) {
    switch (dtype) {
    case PVR_U8:
        return build_typed<uint8_t, LOG2B>(g, vol, dims, nrm, normals_mode, table, records, bricks, st);
    case PVR_F16:
        return build_typed<__half, LOG2B>(g, vol, dims, nrm, normals_mode, table, records, bricks, st);
    default:
        return build_typed<float, LOG2B>(g, vol, dims, nrm, normals_mode, table, records, bricks, st);
    }
}

}  // namespace

BrickGeometry make_brick_geometry(const int dims_dhw[3], int log2b) {
    BrickGeometry g;
    g.log2b = log2b;
    g.ext[0] = dims_dhw[2];  // world x <-> W
    g.ext[1] = dims_dhw[1];  // world y <-> H
    g.ext[2] = dims_dhw[0];  // world z <-> D
    // k + 1 ranges over [0, extent]
    for (int a = 0; a < 3; ++a) g.nb[a] = (g.ext[a] >> log2b) + 1;
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

cudaError_t launch_build_records(const BrickGeometry &g, int dtype, const void *vol, const int dims[3],
                                 const float *nrm, int normals_mode, const uint32_t *table,
                                 float4 *records, uint4 *bricks, cudaStream_t st) {
    switch (g.log2b) {
    case 2: return build_log2<2>(g, dtype, vol, dims, nrm, normals_mode, table, records, bricks, st);
    case 4: return build_log2<4>(g, dtype, vol, dims, nrm, normals_mode, table, records, bricks, st);
    default: return build_log2<3>(g, dtype, vol, dims, nrm, normals_mode, table, records, bricks, st);
    }
}

template <typename Rec>
void read_normals_typed(const BrickGeometry &g, const int dims[3], const uint32_t *table, const Rec *records,
                        float *out, int blocks, cudaStream_t st) {
    switch (g.log2b) {
    case 2: read_normals_kernel<2><<<blocks, 256, 0, st>>>(g, dims[0], dims[1], dims[2], table, records, out); break;
    case 4: read_normals_kernel<4><<<blocks, 256, 0, st>>>(g, dims[0], dims[1], dims[2], table, records, out); break;
    default: read_normals_kernel<3><<<blocks, 256, 0, st>>>(g, dims[0], dims[1], dims[2], table, records, out);
    }
}

cudaError_t launch_read_normals(const BrickGeometry &g, const int dims[3], const uint32_t *table,
                                const void *records, bool compact, float *out, cudaStream_t st) {
    const long long total = (long long)dims[0] * dims[1] * dims[2];
    int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 64);
    if (compact) read_normals_typed(g, dims, table, (const uint2 *)records, out, blocks, st);
    else read_normals_typed(g, dims, table, (const float4 *)records, out, blocks, st);
    return cudaGetLastError();
}

cudaError_t launch_compact_records(const float4 *records, uint2 *out, long long n, int *inexact,
                                   cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
    compact_records_kernel<<<blocks, 256, 0, st>>>(records, out, n, inexact);
    return cudaGetLastError();
}

}  // namespace pvr
