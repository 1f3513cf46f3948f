// FP64 advance kernels: the FP64 path of the breast and reference modes (also
// the on-GPU FP64 counterpart of the FP32 path in precision comparisons).
#include "advance_inst.cuh"

namespace tomo {
AdvanceFn<double> advance_lookup_f64(int T, int cols, int mode, int minb) {
    TOMO_ADV_CASE(double, kModeBreast, 1, 1, 2)
    TOMO_ADV_CASE(double, kModeBreast, 2, 1, 2)
    TOMO_ADV_CASE(double, kModeBreast, 2, 1, 3)
    TOMO_ADV_CASE(double, kModeBreast, 4, 1, 2)
    TOMO_ADV_CASE(double, kModeRef, 1, 1, 2)
    TOMO_ADV_CASE(double, kModeRef, 4, 1, 2)
    return nullptr;
}
}  // namespace tomo
