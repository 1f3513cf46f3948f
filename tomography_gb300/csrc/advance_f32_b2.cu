// FP32 breast-imaging advance kernels, 1, 4, 6 and 8 steps per launch.
#include "advance_inst.cuh"

namespace tomo {
AdvanceFn<float> advance_lookup_f32_b2(int T, int cols, int mode, int minb) {
    TOMO_ADV_CASE(float, kModeBreast, 4, 1, 2)
    TOMO_ADV_CASE(float, kModeBreast, 4, 1, 3)
    TOMO_ADV_CASE(float, kModeBreast, 4, 2, 2)
    TOMO_ADV_CASE(float, kModeBreast, 1, 1, 2)
    TOMO_ADV_CASE(float, kModeBreast, 1, 1, 4)
    TOMO_ADV_CASE(float, kModeBreast, 6, 1, 2)
    TOMO_ADV_CASE(float, kModeBreast, 8, 1, 2)
    return nullptr;
}
}  // namespace tomo
