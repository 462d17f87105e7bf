// astc_encode_partitions.cu -- instantiates the search kernel
// (astc_search_kernel.cuh) for ASTC_QUALITY_PARTITIONS: THOROUGH plus the
// two-partition candidates of astc_pipeline_partition.cuh.  Compiled with
// --fmad=false.
#include "astc_search_kernel.cuh"

namespace astc {

cudaError_t launch_encode_partitions(const EncodeJob& j, cudaStream_t stream) {
    return launch_search_kernels<2>(j, stream);
}

}  // namespace astc
