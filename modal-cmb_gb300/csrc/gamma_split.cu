// gamma_split.cu -- split-precision tensor-core form of the mu-contraction.
#include "common.cuh"

namespace modal {

modal_status gamma_split_dev(modal_ctx *ctx)
{
    (void)ctx;
    set_error("modal_gamma: MODAL_PREC_SPLIT is not available in this build");
    return MODAL_ERR_STATE;
}

}  // namespace modal
