// Instantiates the batched stage kernel for STAGE_SSP_2 (batch_stage.cuh).
#include "batch_stage.cuh"

namespace fvgb {
StageFn batch_stage_ssp_2(int flux, bool linear, int grad, bool barth, bool ns) {
    return batch_detail::pick_kind<dev::STAGE_SSP_2>(flux, linear, grad, barth, ns);
}
}  // namespace fvgb
