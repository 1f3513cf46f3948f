// FP64 instantiations of the advance kernel: the FP64 path of the breast and
// reference modes (also used as the on-GPU FP64 oracle of the FP32 path).
#include "fdtd_advance.cuh"
#include "solve_desc.h"

namespace tomo {

template <typename Real>
using AdvanceFn = void (*)(const SolveDesc<Real>*, const WorkItem*, int, int*);

template <typename Real>
AdvanceFn<Real> advance_kernel_for(int T, int cols, int mode);
template <typename Real>
size_t advance_smem_bytes(int T, int cols);

#define TOMO_F64_CASE(MM, TT, CC) \
    if (mode == MM && T == TT && cols == CC) return &fdtd_advance_kernel<double, TT, CC, MM>;

template <>
AdvanceFn<double> advance_kernel_for<double>(int T, int cols, int mode) {
    TOMO_F64_CASE(kModeBreast, 1, 1)
    TOMO_F64_CASE(kModeBreast, 2, 1)
    TOMO_F64_CASE(kModeBreast, 4, 1)
    TOMO_F64_CASE(kModeRef, 1, 1)
    TOMO_F64_CASE(kModeRef, 4, 1)
    return nullptr;
}

template <>
size_t advance_smem_bytes<double>(int T, int cols) {
    if (T == 1 && cols == 1) return sizeof(AdvanceSmem<double, 1, 1>);
    if (T == 2 && cols == 1) return sizeof(AdvanceSmem<double, 2, 1>);
    if (T == 4 && cols == 1) return sizeof(AdvanceSmem<double, 4, 1>);
    return 0;
}

}  // namespace tomo
