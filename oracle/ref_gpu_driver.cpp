// Test-infrastructure driver around the reference's own GPU solver.
//
// Part of the oracle (checker) only: linked against the reference sources
// FDTD_GPU.cu and FDTD_common.cxx, compiled unchanged for sm_103a by
// oracle/build.py::build_reference_gpu, and used on the GPU host to produce
// the golden vectors tests/golden/ref_gpu_*.npz (tests/golden/make_golden_gpu.py)
// and to time the reference GPU path.  Nothing in the product links or runs it.
//
//   run <args.txt> <out.bin> <reps>
//       Calls the reference entry point  double FDTD_GPU(const vector<double>&)
//       (FDTD_GPU.cu:650-1110) reps times on the 27 arguments of args.txt and
//       records, from the last call, the running-DFT surface currents the
//       solver copies back after each excitation (FDTD_GPU.cu:960-967).  The
//       far field D and phase P are recomputed from them with the reference's
//       own N2FPostProcess (FDTD_GPU.cu:553-634), called exactly as
//       FDTD_GPU.cu:971-977 does.  Output records (float32): the eight
//       accumulator families [E][F][face length][2], D and P [E][F][A], the
//       fitness of every call and the wall time of every call in seconds.
//
// The allocation hooks declared in ref_gpu_guard.h are defined here: each
// device allocation is padded by TOMO_REF_GUARD_BYTES on both sides (see
// that header for why).
#include "ref_gpu_guard.h"
#undef cudaMalloc
#undef cudaFree
#undef cudaMemcpy

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <vector>

// The reference header defines short macros (dt, dx, nx, d, t0, tau, ...):
// no identifier below uses those spellings.
#include "FDTD_common.hxx"

#ifndef TOMO_REF_GUARD_BYTES
#define TOMO_REF_GUARD_BYTES 65536
#endif

// Same name and layout as the reference's complex type (two floats), so that
// N2FPostProcess links; only pointers to it cross the boundary.
struct cuComplex { float r; float i; };

double FDTD_GPU(const std::vector<double>& arguments);
void N2FPostProcess(float* D, float* P, float f, cuComplex* cjzxp, cuComplex* cjzyp, cuComplex* cjzxn,
                    cuComplex* cjzyn, cuComplex* cmxyp, cuComplex* cmyxp, cuComplex* cmxyn, cuComplex* cmyxn);

static std::map<char*, size_t> g_allocs;
static std::vector<std::vector<char>> g_d2h;   // device-to-host copies of the current call
static bool g_record = false;

cudaError_t tomo_ref_guarded_malloc(void** ptr, size_t bytes) {
    void* raw = nullptr;
    const size_t g = TOMO_REF_GUARD_BYTES;
    cudaError_t e = cudaMalloc(&raw, bytes + 2 * g);
    if (e != cudaSuccess) return e;
    e = cudaMemset(raw, 0, bytes + 2 * g);
    if (e != cudaSuccess) return e;
    char* user = static_cast<char*>(raw) + g;
    g_allocs[user] = bytes;
    *ptr = user;
    return cudaSuccess;
}

cudaError_t tomo_ref_guarded_free(void* ptr) {
    if (!ptr) return cudaSuccess;
    char* user = static_cast<char*>(ptr);
    auto it = g_allocs.find(user);
    if (it == g_allocs.end()) return cudaErrorInvalidDevicePointer;
    g_allocs.erase(it);
    return cudaFree(user - TOMO_REF_GUARD_BYTES);
}

cudaError_t tomo_ref_recorded_memcpy(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind) {
    cudaError_t e = cudaMemcpy(dst, src, bytes, kind);
    if (e == cudaSuccess && g_record && kind == cudaMemcpyDeviceToHost) {
        const char* p = static_cast<const char*>(dst);
        g_d2h.emplace_back(p, p + bytes);
    }
    return e;
}

static std::vector<double> read_args(const char* path) {
    std::vector<double> a;
    FILE* fp = std::fopen(path, "r");
    if (!fp) { std::perror(path); std::exit(2); }
    double v;
    while (std::fscanf(fp, "%lf", &v) == 1) a.push_back(v);
    std::fclose(fp);
    return a;
}

// Self-describing dump (as oracle/ref_driver.cpp): per record u32 name_len,
// name, u32 ndim, u32 shape[ndim], float32 data.
static void put_record(FILE* fp, const char* name, const std::vector<unsigned>& shape, const float* data) {
    unsigned nl = (unsigned)std::strlen(name), nd = (unsigned)shape.size();
    size_t count = 1;
    for (unsigned s : shape) count *= s;
    std::fwrite(&nl, 4, 1, fp);
    std::fwrite(name, 1, nl, fp);
    std::fwrite(&nd, 4, 1, fp);
    std::fwrite(shape.data(), 4, nd, fp);
    std::fwrite(data, 4, count, fp);
}

static int run(const char* args_path, const char* out_path, int reps) {
    const std::vector<double> args = read_args(args_path);
    const int E = numberofexcitationangles, F = numberoffrequencies, A = numberofobservationangles;
    const int ny_side = size_y_side, nx_side = size_x_side;
    std::vector<float> fits, secs;
    for (int r = 0; r < reps; ++r) {
        g_d2h.clear();
        g_record = (r == reps - 1);
        const auto tic = std::chrono::steady_clock::now();
        const double fit = FDTD_GPU(args);
        const auto toc = std::chrono::steady_clock::now();
        fits.push_back((float)fit);
        secs.push_back((float)std::chrono::duration<double>(toc - tic).count());
        std::fprintf(stderr, "call %d: fitness %.9g, %.3f s\n", r, fit, (double)secs.back());
    }
    // FDTD_GPU.cu:960-967: per excitation, the eight accumulator copies in this order
    const char* names[8] = {"cjzyn", "cjzxp", "cjzyp", "cjzxn", "cmxyn", "cmyxp", "cmxyp", "cmyxn"};
    const int lens[8] = {ny_side, nx_side, ny_side, nx_side, ny_side, nx_side, ny_side, nx_side};
    if ((int)g_d2h.size() != 8 * E) {
        std::fprintf(stderr, "expected %d device-to-host copies, recorded %zu\n", 8 * E, g_d2h.size());
        return 3;
    }
    for (int e = 0; e < E; ++e)
        for (int k = 0; k < 8; ++k)
            if (g_d2h[8 * e + k].size() != sizeof(cuComplex) * (size_t)lens[k] * F) {
                std::fprintf(stderr, "copy %d of excitation %d has %zu bytes\n", k, e, g_d2h[8 * e + k].size());
                return 3;
            }
    std::vector<float> D((size_t)E * F * A), P((size_t)E * F * A);
    for (int e = 0; e < E; ++e) {
        auto acc = [&](int k) { return reinterpret_cast<cuComplex*>(g_d2h[8 * e + k].data()); };
        for (int fi = 0; fi < F; ++fi) {
            const float freq = startfrequency + deltafreq * fi;   // FDTD_GPU.cu:973
            N2FPostProcess(D.data() + (size_t)e * A * F + (size_t)fi * A, P.data() + (size_t)e * A * F + (size_t)fi * A,
                           freq, acc(1) + nx_side * fi, acc(2) + ny_side * fi, acc(3) + nx_side * fi,
                           acc(0) + ny_side * fi, acc(6) + ny_side * fi, acc(5) + nx_side * fi, acc(4) + ny_side * fi,
                           acc(7) + nx_side * fi);
        }
    }
    FILE* fp = std::fopen(out_path, "wb");
    if (!fp) { std::perror(out_path); return 2; }
    for (int k = 0; k < 8; ++k) {
        std::vector<float> all;
        for (int e = 0; e < E; ++e) {
            const float* p = reinterpret_cast<const float*>(g_d2h[8 * e + k].data());
            all.insert(all.end(), p, p + 2 * (size_t)lens[k] * F);
        }
        put_record(fp, names[k], {(unsigned)E, (unsigned)F, (unsigned)lens[k], 2u}, all.data());
    }
    put_record(fp, "D", {(unsigned)E, (unsigned)F, (unsigned)A}, D.data());
    put_record(fp, "P", {(unsigned)E, (unsigned)F, (unsigned)A}, P.data());
    put_record(fp, "fitness", {(unsigned)fits.size()}, fits.data());
    put_record(fp, "seconds", {(unsigned)secs.size()}, secs.data());
    std::fclose(fp);
    return 0;
}

int main(int argc, char** argv) {
    if (argc >= 5 && std::strcmp(argv[1], "run") == 0) return run(argv[2], argv[3], std::max(1, std::atoi(argv[4])));
    std::fprintf(stderr, "usage: %s run <args.txt> <out.bin> <reps>\n", argv[0]);
    return 2;
}
