// astc_encode_three.cu -- instantiates the quality-mode kernel
// (astc_search_kernel.cuh) for ASTC_QUALITY_THREE_PARTITIONS: PARTITIONS plus
// three-partition candidates, for RGB blocks only (three RGBA partitions
// would need 24 colour endpoint values, above the format's 18), in a unit of
// its own so the extra phase does not change the other modes' register
// allocation.
#include "astc_search_kernel.cuh"

namespace astc {

cudaError_t launch_encode_three(const EncodeJob& j, cudaStream_t stream) {
    if (j.has_alpha) return launch_encode_partitions(j, stream);
    return launch_search_kernels<3, true>(j, stream);
}

}  // namespace astc
