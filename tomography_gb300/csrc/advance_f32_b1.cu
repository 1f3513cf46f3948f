// FP32 breast-imaging advance kernels, two steps per launch.
#include "advance_inst.cuh"

namespace tomo {
AdvanceFn<float> advance_lookup_f32_b1(int T, int cols, int mode, int minb) {
    TOMO_ADV_CASE(float, kModeBreast, 2, 2, 2)
    TOMO_ADV_CASE(float, kModeBreast, 2, 2, 3)
    TOMO_ADV_CASE(float, kModeBreast, 2, 1, 2)
    TOMO_ADV_CASE(float, kModeBreast, 2, 1, 3)
    TOMO_ADV_CASE(float, kModeBreast, 2, 1, 4)
    return nullptr;
}
}  // namespace tomo
