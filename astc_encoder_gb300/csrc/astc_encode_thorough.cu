// astc_encode_thorough.cu -- instantiates the search kernel
// (astc_search_kernel.cuh) for ASTC_QUALITY_THOROUGH: both endpoint fits, the
// search from the one whose fixed-mode block decodes with less error.
// Compiled with --fmad=false.
#include "astc_search_kernel.cuh"

namespace astc {

cudaError_t launch_encode_thorough(const EncodeJob& j, cudaStream_t stream) {
    return launch_search_kernels<1>(j, stream);
}

}  // namespace astc
