// Allocation guard for running the reference's own GPU solver (checker only).
//
// Force-included (nvcc -include) into the reference translation units by
// oracle/build.py::build_reference_gpu; the sources themselves stay
// unchanged.  It routes the solver's device allocations, frees and
// synchronous copies through oracle/ref_gpu_driver.cpp:
//   * cudaMalloc / cudaFree: every allocation is padded by
//     TOMO_REF_GUARD_BYTES on both sides, so the out-of-range zero stores of
//     the reference's Field_reset kernel (FDTD_GPU.cu:436-503, launched on a
//     418 x 418 grid over arrays of 20 x 401 entries) land in padding;
//   * cudaMemcpy: device-to-host copies are recorded, which yields the
//     running-DFT surface currents the solver copies back after each
//     excitation (FDTD_GPU.cu:960-967).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

cudaError_t tomo_ref_guarded_malloc(void** ptr, size_t bytes);
cudaError_t tomo_ref_guarded_free(void* ptr);
cudaError_t tomo_ref_recorded_memcpy(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind);

template <typename T>
static inline cudaError_t tomo_ref_guarded_malloc_t(T** ptr, size_t bytes) {
    return tomo_ref_guarded_malloc(reinterpret_cast<void**>(ptr), bytes);
}

#define cudaMalloc(ptr, bytes) tomo_ref_guarded_malloc_t(ptr, bytes)
#define cudaFree(ptr) tomo_ref_guarded_free(ptr)
#define cudaMemcpy(dst, src, bytes, kind) tomo_ref_recorded_memcpy(dst, src, bytes, kind)
