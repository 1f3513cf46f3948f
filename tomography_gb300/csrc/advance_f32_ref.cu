// FP32 advance kernels of the reference modes (plane wave, reference CPML
// semantics), the blockings the drop-in and the batch path of those modes use.
#include "advance_inst.cuh"

namespace tomo {
AdvanceFn<float> advance_lookup_f32_ref(int T, int cols, int mode, int minb) {
    TOMO_ADV_CASE(float, kModeRef, 1, 1, 2)
    TOMO_ADV_CASE(float, kModeRef, 2, 1, 2)
    TOMO_ADV_CASE(float, kModeRef, 2, 1, 3)
    TOMO_ADV_CASE(float, kModeRef, 4, 1, 2)
    TOMO_ADV_CASE(float, kModeRef, 4, 2, 2)
    return nullptr;
}
}  // namespace tomo
