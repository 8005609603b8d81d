// Batch march kernel instantiated for 8^3-texel bricks (see march_core.cuh).
#include "march_core.cuh"

namespace pvr {

const void *batch_kernel_b3(const Tuning &t, int variant) { return batch_kernel_log2<3>(t, variant); }

const void *single_kernel_b3(const Tuning &t, int variant) { return single_kernel_log2<3>(t, variant); }

int max_batch_blocks_b3(const Tuning &t, int lut_smem_entries, int variant) {
    return max_blocks_log2<3>(t, lut_smem_entries, variant);
}

}  // namespace pvr
