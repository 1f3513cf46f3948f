// C++ drop-in for the reference's fitness entry point.
//
//   double FDTD_GPU(const std::vector<double>& arguments);   // FDTD_GPU.cuh:8
//
// Same signature, argument meaning (27 values: 3x3 patches of eps_inf, then
// del_eps, then sigma, FDTD_GPU.cu:657-693) and return value (fitness <= 0,
// higher is better) as the reference, so tao's ps.go(FDTD_GPU) /
// de.go(...) / anm.iterate(FDTD_GPU) (test.cxx:94-121) link against it
// unchanged.  The device state is created on the first call and reused.
//
// Differences by design:
//  * the far-field target vector is data, not a compiled literal
//    (FDTD_GPU.cu:996): it is read once from the file named by the
//    environment variable TOMO_MEASUREMENT_FILE, or set explicitly with
//    tomo_fdtd_gpu_set_target().  The file holds raw little-endian float32
//    values, or text: numbers separated by spaces, commas or newlines (a
//    UTF-8 byte order mark is skipped).  Both routes accept exactly 4000
//    values (E*F*A magnitudes) or 8000 (magnitudes then phases, the
//    reference's whole array) and use the first 4000, as the reference's
//    misfit does (FDTD_GPU.cu:1004-1008).  A NumPy .npy file, text with
//    anything else in it, or another length is an error;
//  * errors throw instead of exit(-1) (FDTD_GPU.cu:35-48): std::out_of_range
//    for a short argument vector (the reference's .at()), std::runtime_error
//    for everything else.
#ifndef TOMOGRAPHY_FDTD_HPP
#define TOMOGRAPHY_FDTD_HPP

#include <cstddef>
#include <vector>

double FDTD_GPU(const std::vector<double>& arguments);

extern "C" {
/* replace the target of the drop-in's global handle: n = 4000 magnitudes, or 8000
   (magnitudes then phases, of which the first 4000 are used); TOMO_EINVAL otherwise */
int tomo_fdtd_gpu_set_target(const float* target, size_t n);
/* release the drop-in's global handle (optional; also released at exit) */
void tomo_fdtd_gpu_release(void);
}

#endif
