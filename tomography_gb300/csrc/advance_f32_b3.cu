// FP32 breast-imaging advance kernels, three steps per launch.
#include "advance_inst.cuh"

namespace tomo {
AdvanceFn<float> advance_lookup_f32_b3(int T, int cols, int mode, int minb) {
    TOMO_ADV_CASE(float, kModeBreast, 3, 2, 2)
    TOMO_ADV_CASE(float, kModeBreast, 3, 1, 3)
    return nullptr;
}
}  // namespace tomo
