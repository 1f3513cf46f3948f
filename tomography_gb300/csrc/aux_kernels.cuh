// Set-up and post-process kernels of the forward path: material rasterisation,
// FP64 coefficient precompute, descriptor progress, far-field transform and
// misfit reductions.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "solve_desc.h"

namespace tomo {

constexpr double kPiD = 3.141592653589793238;
constexpr double kMu0D = kPiD * 4e-7;
constexpr double kEps0D = 8.85418e-12;

// ---------------------------------------------------------------------------
// Ellipse phantom raster (breast mode).  Per candidate: ell[k] = (cx, cy, a, b,
// cos, sin) in metres; material 0 background, 1 disc, 2+k ellipse k, later
// ellipses over earlier ones.  Explicit round-to-nearest intrinsics keep the
// arithmetic free of contraction so the map is bit-identical to a host
// evaluation of the same expression order.
static __global__ void raster_ellipse_kernel(uint8_t* __restrict__ mats, int mpitch, int nx, int ny, double dx,
                                      double disc_r, const double* __restrict__ ell, int nell, size_t mat_stride) {
    const int cand = blockIdx.z;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i > nx || j > ny) return;
    const double X = __dmul_rn(__dsub_rn((double)i, __dmul_rn(0.5, (double)nx)), dx);
    const double Y = __dmul_rn(__dsub_rn((double)j, __dmul_rn(0.5, (double)ny)), dx);
    uint8_t m = 0;
    if (disc_r > 0 && __dadd_rn(__dmul_rn(X, X), __dmul_rn(Y, Y)) <= __dmul_rn(disc_r, disc_r)) m = 1;
    const double* e = ell + (size_t)cand * nell * 6;
    for (int k = 0; k < nell; ++k, e += 6) {
        const double ex = __dsub_rn(X, e[0]), ey = __dsub_rn(Y, e[1]);
        const double u = __dadd_rn(__dmul_rn(ex, e[4]), __dmul_rn(ey, e[5]));
        const double v = __dsub_rn(__dmul_rn(ey, e[4]), __dmul_rn(ex, e[5]));
        const double q = __dadd_rn(__ddiv_rn(__dmul_rn(u, u), __dmul_rn(e[2], e[2])),
                                   __ddiv_rn(__dmul_rn(v, v), __dmul_rn(e[3], e[3])));
        if (q <= 1.0) m = (uint8_t)(2 + k);
    }
    mats[(size_t)cand * mat_stride + (size_t)j * mpitch + kMatPadLeft + i] = m;
}

// Receiver flags on the antenna cells of every candidate map.
static __global__ void mark_rx_kernel(uint8_t* mats, int mpitch, size_t mat_stride, const int* rx, int nrx, int ncand) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nrx * ncand) return;
    const int cand = t / nrx, r = t % nrx;
    mats[(size_t)cand * mat_stride + (size_t)rx[2 * r + 1] * mpitch + kMatPadLeft + rx[2 * r]] |= kMatRx;
}

// Per-material update coefficients in FP64 (FDTD_GPU.cu:739-741, 1118-1120;
// FDTD_CPU.cxx:979), rounded once to the field precision.  mp = [cand][32][3]
// (eps_inf, del_eps, sigma); tabs = [cand][32][kMatCoef].
template <typename Real>
__global__ void material_table_kernel(const double* __restrict__ mp, Real* __restrict__ tabs, int ncand, int nmat,
                                      double tau, double dt, double dx) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ncand * kMaxMat) return;
    const int m = t % kMaxMat;
    Real* out = tabs + (size_t)t * kMatCoef;
    for (int c = 0; c < kMatCoef; ++c) out[c] = Real(0);
    if (m >= nmat) return;
    const double einf = mp[3 * t], deps = mp[3 * t + 1], sig = mp[3 * t + 2];
    const double kp = (1 - dt / (2 * tau)) / (1 + dt / (2 * tau));
    const double beta = kEps0D * deps * dt / (tau * (1 + dt / (2 * tau)));
    const double den = 2 * einf * kEps0D + sig * dt + beta;
    out[kCa] = (Real)((2 * einf * kEps0D - sig * dt + beta) / den);
    out[kCb] = (Real)((2 * dt / dx) / den);
    out[kCj] = (Real)(((1 + kp) * dt) / den);
    out[kBp] = (Real)(beta / dt);
    out[kCi] = (Real)((-2 * kEps0D * einf + 2 * kEps0D - sig * dt - beta) / den);
    out[kCp] = (Real)((2 * kEps0D * einf - 2 * kEps0D - sig * dt + beta) / den);
    out[kCs] = (Real)((-2 * dt) / den);
}

// Progress every active solve by T steps after an advance launch.
template <typename Real>
__global__ void bump_kernel(SolveDesc<Real>* descs, int nsolves, int T, int* counter) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0) *counter = 0;   // work counter of the next advance launch
    if (s >= nsolves) return;
    SolveDesc<Real>& D = descs[s];
    if (D.active && D.step < D.steps_total) {
        D.step += T;
        D.parity ^= 1;
    }
}

// ---------------------------------------------------------------------------
// Far field (N2FPostProcess, FDTD_GPU.cu:553-634).  One block per (solve,
// frequency); warps loop over observation angles, lanes over contour points.
// geom[c] = (X, Y, face) with X, Y the contour point relative to the
// transform origin [m]; ang[a] = (cos phi, sin phi).
template <typename Real>
__device__ __forceinline__ void dev_sincos(Real a, Real* s, Real* c);
template <>
__device__ __forceinline__ void dev_sincos<float>(float a, float* s, float* c) { sincosf(a, s, c); }
template <>
__device__ __forceinline__ void dev_sincos<double>(double a, double* s, double* c) { sincos(a, s, c); }

template <typename Real>
__global__ void farfield_kernel(const Real* __restrict__ acc, size_t acc_stride, const Real* __restrict__ inc, int C,
                                int nfreq,
                                const double* __restrict__ freqs, const double* __restrict__ geom,
                                const double* __restrict__ ang, int nang, double dl, int norm, double tau,
                                double nbg, float* __restrict__ D, float* __restrict__ P) {
    // geom[c] = (X, Y, face) [m]; ang[a] = (cos phi, sin phi); sums in Real.
    // nbg: refractive index of the lossless background the contour lies in
    // (k = nbg k0, eta = eta0 / nbg); 1 for the reference's vacuum transform.
    // inc (total field, may be null): the incident grid's accumulators, added to
    // every solve's own (the legacy's single sum of both, by linearity).
    const int s = blockIdx.y, f = blockIdx.x;
    const Real* a = acc + (size_t)s * acc_stride + (size_t)f * C * 8;
    const Real* ia = inc ? inc + (size_t)f * C * 8 : nullptr;
    const double c0 = 1.0 / sqrt(kMu0D * kEps0D), eta0 = sqrt(kMu0D / kEps0D), eta = eta0 / nbg;
    const double fr = freqs[f], k = 2 * kPiD * fr * nbg / c0;
    double prad = 1.0;
    if (norm == 1) {
        double g = tau * sqrt(kPiD) * exp(-tau * tau * 2 * kPiD * fr * 2 * kPiD * fr / 4);
        prad = (0.5 / eta0) * g * g * 33.329;
    }
    const Real kr = (Real)k;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int ai = warp; ai < nang; ai += nw) {
        const Real cphi = (Real)ang[2 * ai], sphi = (Real)ang[2 * ai + 1];
        Real Nr = 0, Ni = 0, Lr = 0, Li = 0;
        for (int c = lane; c < C; c += 32) {
            const double* g = geom + 3 * c;
            Real sp, cp;
            dev_sincos<Real>(kr * ((Real)g[0] * cphi + (Real)g[1] * sphi), &sp, &cp);
            const Real* e = a + (size_t)c * 8;
            Real jr = e[0] - e[2], ji = e[1] - e[3];
            Real mr = e[4] - e[6], mi = e[5] - e[7];
            if (ia) {
                const Real* q = ia + (size_t)c * 8;
                jr += q[0] - q[2]; ji += q[1] - q[3];
                mr += q[4] - q[6]; mi += q[5] - q[7];
            }
            const int face = (int)g[2];
            const Real wt = (face == 0 || face == 2) ? -sphi : cphi;
            Nr -= jr * cp - ji * sp;
            Ni -= jr * sp + ji * cp;
            Lr += wt * (mr * cp - mi * sp);
            Li += wt * (mr * sp + mi * cp);
        }
        for (int o = 16; o > 0; o >>= 1) {
            Nr += __shfl_xor_sync(0xffffffffu, Nr, o);
            Ni += __shfl_xor_sync(0xffffffffu, Ni, o);
            Lr += __shfl_xor_sync(0xffffffffu, Lr, o);
            Li += __shfl_xor_sync(0xffffffffu, Li, o);
        }
        if (lane == 0) {
            const double Er = ((double)Lr + eta * (double)Nr) * dl, Ei = ((double)Li + eta * (double)Ni) * dl;
            const size_t o = ((size_t)s * nfreq + f) * nang + ai;
            D[o] = (float)(k * k * (Er * Er + Ei * Ei) / (8 * kPiD * eta * prad));
            P[o] = (float)atan2(Ei, Er);
        }
    }
}

// ---------------------------------------------------------------------------
// Trace misfit partials per solve: num = sum (s - t)^2, den = sum t^2 (FP64).
template <typename Real>
__global__ void trace_partials_kernel(const Real* __restrict__ traces, size_t tr_stride, const float* __restrict__ target,
                                      int n_per_solve, int n_tx, int tx_offset_mod, double* __restrict__ partials,
                                      int* __restrict__ nonfinite) {
    const int s = blockIdx.x;
    const int tx = s % n_tx;
    const Real* tr = traces + (size_t)s * tr_stride;
    const float* tg = target + (size_t)tx * n_per_solve;
    double num = 0, den = 0;
    int bad = 0;
    for (int i = threadIdx.x; i < n_per_solve; i += blockDim.x) {
        const double sv = (double)tr[i], tv = (double)tg[i];
        if (!isfinite(sv)) bad = 1;
        num += (sv - tv) * (sv - tv);
        den += tv * tv;
    }
    __shared__ double sn[32], sd[32];
    for (int o = 16; o > 0; o >>= 1) {
        num += __shfl_xor_sync(0xffffffffu, num, o);
        den += __shfl_xor_sync(0xffffffffu, den, o);
    }
    bad = __any_sync(0xffffffffu, bad);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { sn[w] = num; sd[w] = den; }
    if (bad && lane == 0) atomicOr(nonfinite, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) { a += sn[i]; b += sd[i]; }
        partials[2 * s] = a;
        partials[2 * s + 1] = b;
    }
    (void)tx_offset_mod;
}

// fitness[c] = -sum_tx num / sum_tx den, summed in transmitter order.
static __global__ void trace_fitness_kernel(const double* __restrict__ partials, int n_tx, int ncand, double* fitness) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncand) return;
    double a = 0, b = 0;
    for (int t = 0; t < n_tx; ++t) {
        a += partials[2 * (c * n_tx + t)];
        b += partials[2 * (c * n_tx + t) + 1];
    }
    fitness[c] = b > 0 ? -a / b : -a;
}

// Far-field misfit (FDTD_GPU.cu:1004-1022 absolute; FDTD_CPU.cxx:841-845 relative).
// D is [cand][n_exc][nfreq][nang] which matches the reference's index
// Phi_index*A*F + freq_index*A + angle.
static __global__ void ff_fitness_kernel(const float* __restrict__ D, const float* __restrict__ meas, int n_per_cand,
                                  double norm, int relative, double* fitness, int* nonfinite) {
    const int c = blockIdx.x;
    const float* d = D + (size_t)c * n_per_cand;
    double acc = 0;
    int bad = 0;
    for (int i = threadIdx.x; i < n_per_cand; i += blockDim.x) {
        const double diff = (double)d[i] - (double)meas[i];
        if (!isfinite((double)d[i])) bad = 1;
        double term = diff * diff / norm;
        if (relative) term /= (double)meas[i] * (double)meas[i];
        acc += term;
    }
    __shared__ double sa[32];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    bad = __any_sync(0xffffffffu, bad);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sa[w] = acc;
    if (bad && lane == 0) atomicOr(nonfinite, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) a += sa[i];
        fitness[c] = -a;
    }
}

// Traces of all solves to a packed host-layout buffer [solve][nrx][steps].
template <typename Real, typename Out>
__global__ void traces_pack_kernel(const Real* __restrict__ traces, size_t tr_stride, int n_per_solve, int nsolves,
                                   Out* __restrict__ out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)n_per_solve * nsolves) return;
    const size_t s = i / n_per_solve, r = i % n_per_solve;
    out[i] = (Out)traces[s * tr_stride + r];
}

}  // namespace tomo
