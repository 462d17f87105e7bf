// astc_encode_thorough.cu -- instantiates the search kernel
// (astc_search_kernel.cuh) with both endpoint fits: ASTC_QUALITY_THOROUGH (the
// search from the fit whose fixed-mode block decodes with less error, plus
// dual-plane candidates) and ASTC_AXIS_BEST with ASTC_QUALITY_SEARCH (the
// search from that fit).  Compiled with --fmad=false.
#include "astc_search_kernel.cuh"

namespace astc {

cudaError_t launch_encode_thorough(const EncodeJob& j, cudaStream_t stream) {
    return launch_search_kernels<1>(j, stream);
}

}  // namespace astc
