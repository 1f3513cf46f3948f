// Trace-misfit reduction that allocates nothing (tomo_trace_misfit_static).
//
// Who needs it: callers that cannot call cudaMalloc -- a host framework whose
// caching allocator already owns (nearly) all device memory, a search driver
// that keeps its candidate traces in buffers it manages itself, or a serving
// loop that must not take the implicit device-wide synchronisation of
// cudaMalloc/cudaFree on its latency path.  They hand in device buffers for
// the inputs and the output; the per-solve partial sums this reduction needs
// live in a fixed file-scope device array instead of a buffer allocated per
// call.
//
// The array is part of the library image: every GPU that loads the library
// holds it (kMaxSolves * 2 doubles + one flag, about 1 MiB) until the process
// exits.  Host code cannot use the array's name as a device address, so the
// first call on each device (with that device current) looks its address up
// with cudaGetSymbolAddress and caches it for the life of the process; make
// that first call before any stream capture, and do not use the entry point
// across a cudaDeviceReset (the module may be loaded again at another
// address).  All calls share the one array: the partials are fully
// overwritten by every call, but two calls whose kernels overlap on the GPU
// (different streams, no ordering between them) race on the array and must
// not be issued.  The call stays asynchronous, so it reports no numeric
// status: the reduction kernel raises its non-finite flag (cleared at the
// start of every call) but nothing waits for it, and a non-finite trace
// shows up as a NaN or infinite fitness of its candidate.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "aux_kernels.cuh"
#include "engine.h"

namespace tomo {

constexpr size_t kNoAllocMaxSolves = 65536;   // solves (candidates x transmitters) per call
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_misfit_partials[2 * kNoAllocMaxSolves];
static __device__ __align__(256) int g_misfit_flag[4];

namespace {
std::mutex g_mu;
double* g_partials_addr[kMaxDevices] = {nullptr};
int* g_flag_addr[kMaxDevices] = {nullptr};
}  // namespace

}  // namespace tomo

using tomo::fail;

extern "C" int tomo_trace_misfit_static(const float* traces, const float* target, size_t n_cand, size_t n_tx,
                                        size_t n_per_solve, double* fitness, void* stream) {
    return tomo::guarded([&]() -> int {
        if (!traces || !target || !fitness) return fail(TOMO_EINVAL, "tomo_trace_misfit_static: NULL buffer");
        if (n_cand == 0 || n_tx == 0 || n_per_solve == 0)
            return fail(TOMO_EINVAL, "tomo_trace_misfit_static: empty problem");
        if (n_cand > tomo::kNoAllocMaxSolves || n_tx > tomo::kNoAllocMaxSolves ||
            n_cand * n_tx > tomo::kNoAllocMaxSolves)
            return fail(TOMO_EINVAL, "tomo_trace_misfit_static: " + std::to_string(n_cand) + " x " + std::to_string(n_tx) +
                                         " solves exceed the static scratch limit of " +
                                         std::to_string(tomo::kNoAllocMaxSolves) + " solves");
        if (n_per_solve > (size_t)0x7fffffff) return fail(TOMO_EINVAL, "tomo_trace_misfit_static: trace too long");
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return fail(TOMO_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
        if (dev < 0 || dev >= tomo::kMaxDevices) return fail(TOMO_ECUDA, "device index out of range");
        double* partials = nullptr;
        int* flag = nullptr;
        {
            std::lock_guard<std::mutex> lock(tomo::g_mu);
            if (!tomo::g_partials_addr[dev]) {
                // one-time set-up per device, with that device current
                void* p = nullptr;
                e = cudaGetSymbolAddress(&p, tomo::g_misfit_partials);
                if (e != cudaSuccess)
                    return fail(TOMO_ECUDA, std::string("cudaGetSymbolAddress(partials): ") + cudaGetErrorString(e));
                void* q = nullptr;
                e = cudaGetSymbolAddress(&q, tomo::g_misfit_flag);
                if (e != cudaSuccess)
                    return fail(TOMO_ECUDA, std::string("cudaGetSymbolAddress(flag): ") + cudaGetErrorString(e));
                tomo::g_partials_addr[dev] = static_cast<double*>(p);
                tomo::g_flag_addr[dev] = static_cast<int*>(q);
            }
            partials = tomo::g_partials_addr[dev];
            flag = tomo::g_flag_addr[dev];
        }
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        const int nsolves = (int)(n_cand * n_tx);
        e = cudaMemsetAsync(flag, 0, sizeof(int) * 4, st);   // the flag must start at zero every call
        if (e != cudaSuccess) return fail(TOMO_ECUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
        tomo::trace_partials_kernel<float><<<nsolves, 256, 0, st>>>(traces, n_per_solve, target, (int)n_per_solve,
                                                                    (int)n_tx, 0, partials, flag);
        tomo::trace_fitness_kernel<<<(int)((n_cand + 127) / 128), 128, 0, st>>>(partials, (int)n_tx, (int)n_cand, fitness);
        e = cudaGetLastError();
        if (e != cudaSuccess) return fail(TOMO_ECUDA, std::string("misfit launch: ") + cudaGetErrorString(e));
        return TOMO_OK;
    });
}
