// Instantiates the batched stage kernel for STAGE_EULER (batch_stage.cuh).
#include "batch_stage.cuh"

namespace fvgb {
StageFn batch_stage_euler(int flux, bool linear, int grad, bool barth, bool ns) {
    return batch_detail::pick_kind<dev::STAGE_EULER>(flux, linear, grad, barth, ns);
}
}  // namespace fvgb
