// Lookup of a compiled advance-kernel variant and its shared-memory size.
#include "advance_inst.cuh"
#include "engine_impl.cuh"

namespace tomo {

AdvanceFn<float> advance_lookup_f32_b1(int T, int cols, int mode, int minb);
AdvanceFn<float> advance_lookup_f32_b2(int T, int cols, int mode, int minb);
AdvanceFn<float> advance_lookup_f32_b3(int T, int cols, int mode, int minb);
AdvanceFn<float> advance_lookup_f32_b4(int T, int cols, int mode, int minb);
AdvanceFn<float> advance_lookup_f32_ref(int T, int cols, int mode, int minb);
AdvanceFn<double> advance_lookup_f64(int T, int cols, int mode, int minb);

template <>
AdvanceFn<float> advance_kernel_for<float>(const Blocking& b, int mode) {
    if (AdvanceFn<float> f = advance_lookup_f32_b1(b.T, b.cols, mode, b.minb)) return f;
    if (AdvanceFn<float> f = advance_lookup_f32_b2(b.T, b.cols, mode, b.minb)) return f;
    if (AdvanceFn<float> f = advance_lookup_f32_b3(b.T, b.cols, mode, b.minb)) return f;
    if (AdvanceFn<float> f = advance_lookup_f32_b4(b.T, b.cols, mode, b.minb)) return f;
    return advance_lookup_f32_ref(b.T, b.cols, mode, b.minb);
}

template <>
AdvanceFn<double> advance_kernel_for<double>(const Blocking& b, int mode) {
    return advance_lookup_f64(b.T, b.cols, mode, b.minb);
}

template <typename Real>
size_t advance_smem_bytes(int T, int cols) {
#define TOMO_SMEM(TT, CC) \
    if (T == TT && cols == CC) return advance_block_smem<Real, TT, CC>();
    TOMO_SMEM(1, 1)
    TOMO_SMEM(2, 1)
    TOMO_SMEM(2, 2)
    TOMO_SMEM(2, 4)
    TOMO_SMEM(3, 1)
    TOMO_SMEM(3, 2)
    TOMO_SMEM(4, 1)
    TOMO_SMEM(4, 2)
    TOMO_SMEM(6, 1)
    TOMO_SMEM(8, 1)
#undef TOMO_SMEM
    return 0;
}
template size_t advance_smem_bytes<float>(int, int);
template size_t advance_smem_bytes<double>(int, int);

}  // namespace tomo
