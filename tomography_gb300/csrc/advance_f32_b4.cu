// FP32 breast-imaging advance kernel with four columns per lane (16-byte row
// copies and field stores).
#include "advance_inst.cuh"

namespace tomo {
AdvanceFn<float> advance_lookup_f32_b4(int T, int cols, int mode, int minb) {
    TOMO_ADV_CASE(float, kModeBreast, 2, 4, 2)
    return nullptr;
}
}  // namespace tomo
