// astc_encode_search.cu -- instantiates the search kernel
// (astc_search_kernel.cuh) for the fixed mode with the max-accumulation axis
// and for the search from one fit, and routes the other quality modes:
// ASTC_AXIS_BEST with the fixed mode to astc_encode_best.cu, the both-fits
// modes to astc_encode_thorough.cu, ASTC_QUALITY_PARTITIONS to
// astc_encode_partitions.cu, ASTC_QUALITY_THREE_PARTITIONS to
// astc_encode_three.cu.  Compiled with --fmad=false.
#include "astc_search_kernel.cuh"

namespace astc {

cudaError_t launch_encode_search(const EncodeJob& j, cudaStream_t stream) {
    // ASTC_AXIS_BEST with the fixed mode: its own register-resident kernel
    if (j.quality == ASTC_QUALITY_FAST && j.axis == ASTC_AXIS_BEST) return launch_encode_best(j, stream);
    // both fits: THOROUGH, and the search with ASTC_AXIS_BEST
    if (j.quality == ASTC_QUALITY_THOROUGH || (j.quality <= ASTC_QUALITY_SEARCH && j.axis == ASTC_AXIS_BEST))
        return launch_encode_thorough(j, stream);
    if (j.quality == ASTC_QUALITY_PARTITIONS) return launch_encode_partitions(j, stream);
    if (j.quality == ASTC_QUALITY_THREE_PARTITIONS) return launch_encode_three(j, stream);
    return launch_search_kernels<0>(j, stream);
}

}  // namespace astc
