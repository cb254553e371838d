// adaptive.cu -- placeholder entry points of the adaptive stages.
#include "apbf_internal.cuh"

namespace apbf {

apbf_status spread_kernel_width(apbf_ctx *, cudaStream_t) { set_error("spread_kernel_width: not built"); return APBF_ERR_NOT_BUILT; }
apbf_status update_transfers(apbf_ctx *, cudaStream_t) { set_error("update_transfers: not built"); return APBF_ERR_NOT_BUILT; }
apbf_status particle_transfer(apbf_ctx *, float, cudaStream_t) { set_error("particle_transfer: not built"); return APBF_ERR_NOT_BUILT; }

}  // namespace apbf
