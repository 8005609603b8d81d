// Host/device declarations shared between the C-ABI layer and the kernels.
#pragma once

#include <atomic>

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/pyvr_gb300.h"
#include "pvr_device.cuh"

namespace pvr {

// Brick of (2^log2)^3 texels, stored as (2^log2 + 1)^3 16-byte records
// (see layout.cu).  Supported sizes: 4, 8, 16.
constexpr int kMinBrickLog2 = 2;
constexpr int kMaxBrickLog2 = 4;
constexpr int kDefaultBrickLog2 = 3;

__host__ __device__ constexpr int brick_apron(int log2b) { return (1 << log2b) + 1; }
__host__ __device__ constexpr int brick_records(int log2b) {
    return brick_apron(log2b) * brick_apron(log2b) * brick_apron(log2b);
}

// Brick grid of one volume; axes are world x, y, z (= W, H, D of the
// (D,H,W) array).  nb = extent / brick + 1 (see layout.cu).
struct BrickGeometry {
    int ext[3];
    int nb[3];
    int nbricks;
    int log2b;
};

BrickGeometry make_brick_geometry(const int dims_dhw[3], int log2b);
std::vector<uint32_t> morton_slots(const BrickGeometry &g);

// normals_mode: 0 none, 1 from `nrm` (float32 (D,H,W,3)), 2 computed on the
// device from the stored values (numpy.gradient semantics).
// bricks[b] = {record slot, min, max (float bits), 0}: what the march needs
// when a ray enters brick b, in one 16-byte load.
// half: 8-byte half records (uint8 / float16 volumes only).
cudaError_t launch_build_records(const BrickGeometry &g, int dtype, const void *vol, const int dims[3],
                                 const float *nrm, int normals_mode, const uint32_t *table,
                                 void *records, bool half, uint4 *bricks, cudaStream_t st);
cudaError_t launch_read_normals(const BrickGeometry &g, const int dims[3], const uint32_t *table,
                                const void *records, bool compact, float *out, cudaStream_t st);
// Half-precision copy of n records ({value, nx, ny, nz} as four halves, 8
// bytes); *inexact is set to 1 if some float does not survive the round trip
// bit for bit (any NaN may stand for any other).
cudaError_t launch_compact_records(const float4 *records, uint2 *out, long long n, int *inexact,
                                   cudaStream_t st);

// One render of a batch, as the march kernel reads it.
struct JobDesc {
    MarchFrame f;
    const void *records;  // float4 records, or uint2 (four halves) when compact
    const uint4 *bricks;  // {slot, min bits, max bits, 0} per brick
    const float4 *lut;
    const int *prefix;  // prefix[i] = LUT entries before i that are not exactly clear
    uint32_t *out8;
    float4 *outf;
    unsigned long long *counters;  // [in-box samples, shaded samples] or null
    int tiles_x, tiles_y, tile_base;
    int normals;
    int skip;  // empty-space test on: the LUT has a clear entry and the light terms are finite
    int compact;  // 8-byte half records
    int fast;     // fast arithmetic (see pvr_set_arithmetic)
    int pad_[2];
};

// Kernel parameters of one persistent launch: up to kMaxLaunchJobs job
// descriptors passed by value (read through the constant cache).
constexpr int kMaxLaunchJobs = 96;
struct BatchParams {
    int njobs;
    int total_tiles;
    int tile_w, tile_h;
    int lut_smem_entries;
    int *work;
    int tile_base[kMaxLaunchJobs];
    JobDesc jobs[kMaxLaunchJobs];
};
static_assert(sizeof(BatchParams) <= 32000, "kernel parameter block too large");

// Kernel parameters of a launch with a single job (one block per tile).
struct SingleParams {
    JobDesc job;
    int tile_w, tile_h;
    int lut_smem_entries;
};

constexpr int kBatchThreads = 256;

// Launch tuning.  tile_w * tile_h == 256 with tile_w a multiple of 8 and
// tile_h a multiple of 4 (8x4-pixel warp tiles); steps_per_iter in {1, 4};
// blocks_per_sm: persistent blocks per SM.
struct Tuning {
    int tile_w = 16, tile_h = 16;
    int steps_per_iter = 1;
    int blocks_per_sm = 4;
};

// March kernels (march_core.cuh), one instantiation per brick size and
// variant.  Variant bits: normals, LUT staged in shared memory, half
// records, fast arithmetic.  The batch kernel function for a tuning and
// variant, the blocks of it that fit on an SM, and the single-job kernel.
constexpr int kSingleNormals = 1, kSingleSmemLut = 2, kSingleCompact = 4, kSingleFast = 8;
// LUTs up to this many entries are staged in shared memory
constexpr int kMaxSmemLut = 2048;
const void *batch_kernel(int log2b, const Tuning &t, int variant);
const void *single_kernel(int log2b, const Tuning &t, int variant);
size_t batch_smem_bytes(int lut_smem_entries);
int max_batch_blocks_per_sm(int log2b, const Tuning &t, int lut_smem_entries, int variant);
// the variant bits of a job before it is filled
int job_variant_of(const pvr_job &j, bool fast);
// the variant bits of a filled job
inline int job_variant(const JobDesc &j) {
    return (j.normals ? kSingleNormals : 0) | (j.f.lut_size <= kMaxSmemLut ? kSingleSmemLut : 0) |
           (j.compact ? kSingleCompact : 0) | (j.fast ? kSingleFast : 0);
}

}  // namespace pvr

// ---------------------------------------------------------------------------
// C-ABI resource objects (resources.cu)
// ---------------------------------------------------------------------------

struct pvr_volume {
    int device = 0;
    int dtype = PVR_F32;
    int dims[3] = {0, 0, 0};  // D, H, W
    float value_scale = 1.0f;
    float bmin[3] = {-0.5f, -0.5f, -0.5f}, bmax[3] = {0.5f, 0.5f, 0.5f};
    void *d_vol = nullptr;
    size_t vol_bytes = 0;
    float *d_nrm = nullptr;   // given normals, held until the records are built
    int normals_mode = 0;     // 0 none, 1 given, 2 computed on the device
    int log2b = pvr::kDefaultBrickLog2;
    pvr::BrickGeometry geo = {};
    void *d_records = nullptr;  // float4 records, or uint2 when compact
    size_t records_bytes = 0;
    bool compact = false;       // records stored as halves
    bool compact_exact = true;  // ... and every float of them survived exactly
    uint32_t *d_table = nullptr;  // brick -> record slot
    uint4 *d_bricks = nullptr;    // brick -> {slot, min, max}
    bool layout_ready = false;    // the layout is built or queued
    // recorded after the layout's work (volumes created by pvr_volume_create*):
    // device work on the volume waits for it; ready_done once it has completed
    cudaEvent_t ready = nullptr;
    mutable std::atomic<bool> ready_done{false};
};

struct pvr_lut {
    int device = 0;
    int size = 0, cap = 0;
    float4 *d_lut = nullptr;
    int *d_prefix = nullptr;
    bool has_clear = false;  // some entry has alpha exactly 0 and a finite colour
};

namespace pvr {
// helpers shared by the C-ABI translation units
int fail(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);
int ensure_volume_layout(pvr_volume *v, cudaStream_t st);
// Make `st` wait for the volume's layout if it may still be running.
void volume_stream_wait(const pvr_volume *v, cudaStream_t st);
int try_compact_records(pvr_volume *v, cudaStream_t st, bool round_normals);
cudaError_t vol_alloc(void **p, size_t bytes, cudaStream_t st);
void vol_free(void *p, cudaStream_t st);
void free_volume_buffers(pvr_volume *v, cudaStream_t st);
bool invert_gl(const float gl[16], double inv[16]);
void light_direction(const float pos[3], const float target[3], float out[3]);
int fill_job(const pvr_job &j, int tile_w, int tile_h, bool fast, JobDesc &out);
// the arithmetic renders use (pvr_set_arithmetic): true = fast (default)
bool arithmetic_fast();
}  // namespace pvr

#define PVR_CUDA(expr)                                                  \
    do {                                                                \
        cudaError_t e_ = (expr);                                        \
        if (e_ != cudaSuccess) return ::pvr::cuda_fail(e_, #expr);      \
    } while (0)
