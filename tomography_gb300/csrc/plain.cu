// Launcher of the plain one-solve-per-launch path (plain_kernels.cuh).
#include "engine_impl.cuh"
#include "plain_kernels.cuh"

namespace tomo {

template <typename Real>
int launch_plain_step(int mode, const SolveDesc<Real>* d, int n, int nx, int ny, int n_contour, cudaStream_t st) {
    const dim3 blk(32, 8), grd((nx + 1 + 31) / 32, (ny + 1 + 7) / 8);
    if (mode == kModeRef) {
        plain_h_kernel<Real, kModeRef><<<grd, blk, 0, st>>>(d);
        plain_e_kernel<Real, kModeRef><<<grd, blk, 0, st>>>(d, n);
    } else {
        plain_h_kernel<Real, kModeBreast><<<grd, blk, 0, st>>>(d);
        plain_e_kernel<Real, kModeBreast><<<grd, blk, 0, st>>>(d, n);
    }
    if (n_contour <= 0) return 2;
    plain_dft_kernel<Real><<<(n_contour + 127) / 128, 128, 0, st>>>(d, n);
    return 3;
}

template int launch_plain_step<float>(int, const SolveDesc<float>*, int, int, int, int, cudaStream_t);
template int launch_plain_step<double>(int, const SolveDesc<double>*, int, int, int, int, cudaStream_t);

}  // namespace tomo
