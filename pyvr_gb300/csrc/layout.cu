// Device layout of a loaded volume for the march kernel.
//
// The reference keeps the voxels and the normals as two 3D textures
// (pyvr/moderngl_renderer/manager.py:77-135).  Here both are re-laid out
// once per volume into texel records {stored value, nx, ny, nz}: 16-byte
// floats, or 8-byte halves for uint8 and float16 volumes (whose values are
// halves exactly; the normals are then rounded to half) -- the stored value
// keeps its value, the scale to density is applied after interpolation --
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

#include "normals.cuh"
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


// The normal of array element (a, b, c), its neighbours read from global
// memory.
template <typename T>
__device__ float3 normal_global(const T *v, const int dims[3], int a, int b, int c) {
    const int idx[3] = {a, b, c};
    const long long stride[3] = {(long long)dims[1] * dims[2], dims[2], 1};
    const long long base = a * stride[0] + b * stride[1] + c;
    float g[3];
    const float v0 = raw_value<T>(v, base);
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        const int i = idx[ax], n = dims[ax];
        const long long s = stride[ax];
        const float vm = i > 0 ? raw_value<T>(v, base - s) : 0.0f;
        const float vp = i < n - 1 ? raw_value<T>(v, base + s) : 0.0f;
        g[ax] = GradientArith<T>::axis(vm, v0, vp, i, n);
    }
    return GradientArith<T>::finish(g[0], g[1], g[2]);
}

template <typename Rec> __device__ __forceinline__ Rec make_record(float v, float3 n);
template <> __device__ __forceinline__ float4 make_record<float4>(float v, float3 n) {
    return make_float4(v, n.x, n.y, n.z);
}
// {value, nx, ny, nz} as halves, each rounded to nearest
template <> __device__ __forceinline__ uint2 make_record<uint2>(float v, float3 n) {
    const uint32_t h0 = __half_as_ushort(__float2half_rn(v)), h1 = __half_as_ushort(__float2half_rn(n.x));
    const uint32_t h2 = __half_as_ushort(__float2half_rn(n.y)), h3 = __half_as_ushort(__float2half_rn(n.z));
    return make_uint2(h0 | (h1 << 16), h2 | (h3 << 16));
}

constexpr int kLayoutThreads = 256;

// One block per brick (grid-stride over bricks; launched with one block per
// brick).  The block first stages
// the brick's texels plus a two-texel margin ((B+3)^3, clamped to the
// volume) in shared memory, then writes the brick's (B+1)^3 records: the
// stored value and the normal (given: read from `nrm`; computed on the
// device: numpy.gradient from the staged neighbours when the volume is
// cubic -- array axes are then the world axes -- else from global memory),
// and finally the brick's {slot, min, max} from a block reduction over the
// records' values (a NaN marks the brick as never skippable).  Voxel
// (x, y, z) along world axes lives at z + D*(y + H*x) of the (D,H,W) C-order
// buffer (the GL texture of size (D,H,W) read through the z/y/x swizzle,
// volume.frag.glsl:90); the normal texture is indexed the same way
// (manager.py:123-125).  Rec: float4 records, or uint2 half records (only
// for storage types whose values are halves exactly).
template <typename T, int LOG2B, typename Rec>
__global__ void __launch_bounds__(kLayoutThreads)
build_bricks_kernel(BrickGeometry g, const T *__restrict__ vol, int D, int H, int W,
                    const float *__restrict__ nrm, int normals_mode, const uint32_t *__restrict__ table,
                    Rec *__restrict__ records, uint4 *__restrict__ bricks) {
    constexpr int B = 1 << LOG2B, A = B + 1, R = A * A * A, S = B + 3, S3 = S * S * S;
    constexpr int WARPS = kLayoutThreads / 32;
    __shared__ float sv[S3];
    __shared__ float s_lo[WARPS], s_hi[WARPS];
    __shared__ int s_nan[WARPS];
    const int dims[3] = {D, H, W};
    const bool cubic = D == H && H == W;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int brick = blockIdx.x; brick < g.nbricks; brick += gridDim.x) {
        const int bz = brick % g.nb[2];
        const int by = (brick / g.nb[2]) % g.nb[1];
        const int bx = brick / (g.nb[2] * g.nb[1]);
        // staged region: world texels o + r, r in [0, S), o = b*B - 2
        const int ox = bx * B - 2, oy = by * B - 2, oz = bz * B - 2;
        for (int i = threadIdx.x; i < S3; i += kLayoutThreads) {
            const int rz = i % S, ry = (i / S) % S, rx = i / (S * S);
            const int x = min(max(ox + rx, 0), g.ext[0] - 1);
            const int y = min(max(oy + ry, 0), g.ext[1] - 1);
            const int z = min(max(oz + rz, 0), g.ext[2] - 1);
            sv[i] = raw_value<T>(vol, z + (long long)g.ext[2] * (y + (long long)g.ext[1] * x));
        }
        __syncthreads();
        const uint32_t slot = table[brick];
        float lo = __int_as_float(0x7f800000), hi = -lo;
        bool nan = false;
        for (int rec = threadIdx.x; rec < R; rec += kLayoutThreads) {
            const int lz = rec % A, ly = (rec / A) % A, lx = rec / (A * A);
            // record l of the brick holds texel clamp(b*B - 1 + l)
            const int x = min(max(bx * B - 1 + lx, 0), g.ext[0] - 1);
            const int y = min(max(by * B - 1 + ly, 0), g.ext[1] - 1);
            const int z = min(max(bz * B - 1 + lz, 0), g.ext[2] - 1);
            const int ri = ((x - ox) * S + (y - oy)) * S + (z - oz);  // in [1, S-2] per axis
            const float val = sv[ri];
            nan |= val != val;
            lo = fminf(lo, val);
            hi = fmaxf(hi, val);
            float3 n = make_float3(0.0f, 0.0f, 0.0f);
            const long long src = z + (long long)g.ext[2] * (y + (long long)g.ext[1] * x);
            if (normals_mode == PVR_NORMALS_GIVEN) {
                n = make_float3(nrm[3 * src + 0], nrm[3 * src + 1], nrm[3 * src + 2]);
            } else if (normals_mode == PVR_NORMALS_DEVICE) {
                if (cubic) {
                    // array position (a, b, c) = (x, y, z)
                    n = GradientArith<T>::finish(
                        GradientArith<T>::axis(sv[ri - S * S], val, sv[ri + S * S], x, g.ext[0]),
                        GradientArith<T>::axis(sv[ri - S], val, sv[ri + S], y, g.ext[1]),
                        GradientArith<T>::axis(sv[ri - 1], val, sv[ri + 1], z, g.ext[2]));
                } else {
                    // array position of flat element `src` in the (D,H,W) array
                    const int c = (int)(src % W);
                    const int b = (int)((src / W) % H);
                    const int a = (int)(src / ((long long)W * H));
                    n = normal_global<T>(vol, dims, a, b, c);
                }
            }
            records[(size_t)slot * R + rec] = make_record<Rec>(val, n);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        nan = __any_sync(0xffffffffu, nan);
        if (lane == 0) {
            s_lo[warp] = lo;
            s_hi[warp] = hi;
            s_nan[warp] = nan;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            bool any_nan = false;
            for (int w = 0; w < WARPS; ++w) {
                lo = fminf(lo, s_lo[w]);
                hi = fmaxf(hi, s_hi[w]);
                any_nan |= s_nan[w] != 0;
            }
            bricks[brick] = any_nan ? make_uint4(slot, 0x7fc00000u, 0u, 0u)
                                    : make_uint4(slot, __float_as_uint(lo), __float_as_uint(hi), 0u);
        }
        __syncthreads();  // sv and the partials are rewritten for the next brick
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

// Compact records: {value, nx, ny, nz} as four halves in one 8-byte record,
// each rounded to nearest.  The march decodes them exactly, so a volume
// whose records all survive the round trip renders the same images from
// either form.  *inexact gets bit 0 if some value does not survive it, bit 1
// if some normal component does not.
__global__ void compact_records_kernel(const float4 *__restrict__ in, uint2 *__restrict__ out, long long n,
                                       int *__restrict__ inexact) {
    unsigned bad = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float4 r = in[i];
        unsigned short h0, h1, h2, h3;
        const bool v_ok = half_exact(r.x, h0);
        const bool x_ok = half_exact(r.y, h1);
        const bool y_ok = half_exact(r.z, h2);
        const bool z_ok = half_exact(r.w, h3);
        bad |= (v_ok ? 0u : 1u) | ((x_ok && y_ok && z_ok) ? 0u : 2u);
        out[i] = make_uint2((uint32_t)h0 | ((uint32_t)h1 << 16), (uint32_t)h2 | ((uint32_t)h3 << 16));
    }
    bad = __reduce_or_sync(0xffffffffu, bad);
    if (bad && (threadIdx.x & 31) == 0) atomicOr(inexact, (int)bad);
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
                        int normals_mode, const uint32_t *table, void *records, bool half, uint4 *bricks,
                        cudaStream_t st) {
    // one block per brick: short blocks, so that render kernels on streams
    // of higher priority get SMs as soon as any layout block retires
    const int blocks = std::max(1, g.nbricks);
    if (half)
        build_bricks_kernel<T, LOG2B, uint2><<<blocks, kLayoutThreads, 0, st>>>(
            g, (const T *)vol, dims[0], dims[1], dims[2], nrm, normals_mode, table, (uint2 *)records, bricks);
    else
        build_bricks_kernel<T, LOG2B, float4><<<blocks, kLayoutThreads, 0, st>>>(
            g, (const T *)vol, dims[0], dims[1], dims[2], nrm, normals_mode, table, (float4 *)records, bricks);
    return cudaGetLastError();
}

template <int LOG2B>
cudaError_t build_log2(const BrickGeometry &g, int dtype, const void *vol, const int dims[3],
                       const float *nrm, int normals_mode, const uint32_t *table, void *records, bool half,
                       uint4 *bricks, cudaStream_t st) {
    switch (dtype) {
    case PVR_U8:
        return build_typed<uint8_t, LOG2B>(g, vol, dims, nrm, normals_mode, table, records, half, bricks, st);
    case PVR_F16:
        return build_typed<__half, LOG2B>(g, vol, dims, nrm, normals_mode, table, records, half, bricks, st);
    default:
        // float32 values are not halves: float records only
        return build_typed<float, LOG2B>(g, vol, dims, nrm, normals_mode, table, records, false, bricks, st);
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
                                 void *records, bool half, uint4 *bricks, cudaStream_t st) {
    if (half && dtype == PVR_F32) return cudaErrorInvalidValue;
    switch (g.log2b) {
    case 2: return build_log2<2>(g, dtype, vol, dims, nrm, normals_mode, table, records, half, bricks, st);
    case 4: return build_log2<4>(g, dtype, vol, dims, nrm, normals_mode, table, records, half, bricks, st);
    default: return build_log2<3>(g, dtype, vol, dims, nrm, normals_mode, table, records, half, bricks, st);
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
