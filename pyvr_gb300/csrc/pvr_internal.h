// Host/device declarations shared between the C-ABI layer and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "../../include/pyvr_gb300.h"

namespace pvr {

struct MarchFrame;

// A LUT of up to this many RGBA entries is staged in shared memory
// (48 KiB, the default dynamic shared-memory limit); larger ones are read
// through the read-only cache.
constexpr int kLutSmemMaxEntries = 3072;

// Bricks of kBrick^3 texels, stored with a one-texel apron on the high side
// of each axis: (kBrick+1)^3 16-byte records per brick.
constexpr int kBrickLog2 = 3;
constexpr int kBrick = 1 << kBrickLog2;
constexpr int kApron = kBrick + 1;
constexpr int kRecordsPerBrick = kApron * kApron * kApron;
constexpr uint32_t kSlotMask = 0x7fffffffu;
constexpr uint32_t kTransparentBit = 0x80000000u;

// Brick grid of one volume; axes are world x, y, z (= W, H, D of the
// (D,H,W) array).
struct BrickGeometry {
    int ext[3];
    int nb[3];
    int nbricks;
};

BrickGeometry make_brick_geometry(const int dims_dhw[3]);
std::vector<uint32_t> morton_slots(const BrickGeometry &g);

cudaError_t launch_build_records(const BrickGeometry &g, int dtype, const void *vol, const float *nrm,
                                 const uint32_t *table, float4 *records, float2 *minmax,
                                 cudaStream_t st);
cudaError_t launch_brick_flags(const BrickGeometry &g, float value_scale, int lut_size,
                               const int *opaque_prefix, bool enable, const float2 *minmax,
                               uint32_t *table, cudaStream_t st);

// counters[0] = in-box samples (reference loop iterations with a valid
// texture coordinate), counters[1] = samples actually shaded (not skipped).
cudaError_t launch_march(const MarchFrame &f, const float4 *records, const uint32_t *table,
                         bool normals, const float4 *lut, uint32_t *out8, float4 *outf,
                         unsigned long long *counters, cudaStream_t st);

}  // namespace pvr
