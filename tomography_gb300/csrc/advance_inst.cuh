// Helpers for the translation units that instantiate the advance kernel.
// Each unit defines one lookup function over the (mode, T, COLS, MINB)
// variants it compiles; advance_registry.cu chains them.
#pragma once
#include "fdtd_advance.cuh"
#include "solve_desc.h"

namespace tomo {

template <typename Real>
using AdvanceFn = void (*)(const SolveDesc<Real>*, const WorkItem*, int, int*);

#define TOMO_ADV_CASE(REAL, MM, TT, CC, MB) \
    if (mode == MM && T == TT && cols == CC && minb == MB) return &fdtd_advance_kernel<REAL, TT, CC, MM, MB>;

}  // namespace tomo
