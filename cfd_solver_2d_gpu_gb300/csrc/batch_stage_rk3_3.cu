// Instantiates the batched stage kernel for STAGE_RK3_3 (batch_stage.cuh).
#include "batch_stage.cuh"

namespace fvgb {
StageFn batch_stage_rk3_3(int flux, bool linear, int grad, bool barth, bool ns) {
    return batch_detail::pick_kind<dev::STAGE_RK3_3>(flux, linear, grad, barth, ns);
}
}  // namespace fvgb
