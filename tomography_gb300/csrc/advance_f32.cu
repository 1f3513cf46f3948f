// FP32 instantiations of the advance kernel (field, CPML and Debye updates in
// FP32; DFT sums Kahan-compensated).  (T, COLS) pairs offered to the tuner;
// the reference modes get the pairs their drop-in uses.
#include "fdtd_advance.cuh"
#include "solve_desc.h"

namespace tomo {

template <typename Real>
using AdvanceFn = void (*)(const SolveDesc<Real>*, const WorkItem*, int, int*);

template <typename Real>
AdvanceFn<Real> advance_kernel_for(int T, int cols, int mode);
template <typename Real>
size_t advance_smem_bytes(int T, int cols);

#define TOMO_F32_CASE(MM, TT, CC) \
    if (mode == MM && T == TT && cols == CC) return &fdtd_advance_kernel<float, TT, CC, MM>;

template <>
AdvanceFn<float> advance_kernel_for<float>(int T, int cols, int mode) {
    TOMO_F32_CASE(kModeBreast, 1, 1)
    TOMO_F32_CASE(kModeBreast, 2, 1)
    TOMO_F32_CASE(kModeBreast, 2, 2)
    TOMO_F32_CASE(kModeBreast, 4, 1)
    TOMO_F32_CASE(kModeBreast, 4, 2)
    TOMO_F32_CASE(kModeBreast, 6, 1)
    TOMO_F32_CASE(kModeBreast, 8, 1)
    TOMO_F32_CASE(kModeRef, 1, 1)
    TOMO_F32_CASE(kModeRef, 2, 1)
    TOMO_F32_CASE(kModeRef, 4, 1)
    TOMO_F32_CASE(kModeRef, 4, 2)
    return nullptr;
}

template <>
size_t advance_smem_bytes<float>(int T, int cols) {
    if (T == 1 && cols == 1) return sizeof(AdvanceSmem<float, 1, 1>);
    if (T == 2 && cols == 1) return sizeof(AdvanceSmem<float, 2, 1>);
    if (T == 2 && cols == 2) return sizeof(AdvanceSmem<float, 2, 2>);
    if (T == 4 && cols == 1) return sizeof(AdvanceSmem<float, 4, 1>);
    if (T == 4 && cols == 2) return sizeof(AdvanceSmem<float, 4, 2>);
    if (T == 6 && cols == 1) return sizeof(AdvanceSmem<float, 6, 1>);
    if (T == 8 && cols == 1) return sizeof(AdvanceSmem<float, 8, 1>);
    return 0;
}

}  // namespace tomo
