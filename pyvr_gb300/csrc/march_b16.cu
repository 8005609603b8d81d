// Batch march kernel instantiated for 16^3-texel bricks (see march_core.cuh).
#include "march_core.cuh"

namespace pvr {

cudaError_t launch_march_batch_b4(const Tuning &t, const BatchHeader *hdr, const int *tile_bases,
                                  const JobDesc *jobs, int *work, int grid, int lut_smem_entries,
                                  cudaStream_t st) {
    return launch_batch_log2<4>(t, hdr, tile_bases, jobs, work, grid, lut_smem_entries, st);
}

int max_batch_blocks_b4(const Tuning &t, int lut_smem_entries) {
    return max_blocks_log2<4>(t, lut_smem_entries);
}

}  // namespace pvr
