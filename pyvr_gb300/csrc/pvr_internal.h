// Host-side declarations shared between the C-ABI layer and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pyvr_gb300.h"

namespace pvr {

struct MarchFrame;

// A LUT of up to this many RGBA entries is staged in shared memory
// (48 KiB, the default dynamic shared-memory limit); larger ones are read
// through the read-only cache.
constexpr int kLutSmemMaxEntries = 3072;

cudaError_t launch_march_linear(const MarchFrame &f, int dtype, const void *vol,
                                const float *nrm, const float4 *lut, uint32_t *out8,
                                float4 *outf, unsigned long long *samples, cudaStream_t st);

}  // namespace pvr
