// Plain one-solve-per-launch FDTD path: one kernel launch per field update and
// time step, one solve per launch, no temporal blocking, no batching, no graph.
// This is the structure of the reference's GPU solver (FDTD_GPU.cu:940-990:
// H kernel, E kernel, DFT kernel per step), kept as the baseline that the
// batched wavefront path is measured against, and as an independent GPU
// implementation of the same arithmetic for parity tests.
//
// Step n advances the state of one solve from time n to n+1, in place in the
// first copy of each field (ez[0], hx[0], hy[0], jp[0], psi[0]):
//   plain_h_kernel    Hx, Hy + CPML psi_hyx / psi_hxy   (FDTD_GPU.cu:298-355)
//   plain_e_kernel    Ez, Debye Jp, CPML psi_ezx / psi_ezy, plane wave or point
//                     source, NaN clamp, receiver samples (FDTD_GPU.cu:358-434)
//   plain_dft_kernel  running DFT of J and M on the NTFF contour
//                     (FDTD_GPU.cu:231-280), one thread per contour point
// Every update uses the same explicitly rounded operations, in the same order,
// as the general path of the wavefront kernel, so both paths give the same
// bits for the same solve.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fdtd_advance.cuh"
#include "solve_desc.h"

namespace tomo {

template <typename Real, int MODE>
__global__ void __launch_bounds__(256) plain_h_kernel(const SolveDesc<Real>* __restrict__ Dp) {
    const SolveDesc<Real>& D = *Dp;
    using O = Op<Real>;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int m = blockIdx.y * blockDim.y + threadIdx.y;
    const int nx = D.nx, ny = D.ny, nc = D.ncpml, pitch = D.pitch;
    if (x >= nx || m >= ny) return;
    constexpr bool kRef = MODE == kModeRef;
    const Real chez = D.chez, dxr = D.dx;
    const Real* __restrict__ ez = D.ez[0];
    Real* __restrict__ hx = D.hx[0];
    Real* __restrict__ hy = D.hy[0];
    Real* __restrict__ psi = D.psi[0];
    const Real* __restrict__ cpml = D.cpml;
    const long long o = (long long)m * pitch + x;
    const Real ez0 = ez[o];
    const Real dEy = O::sub(ez[o + 1], ez0);
    const Real dEx = O::sub(ez[o + pitch], ez0);
    const Real hy0 = hy[o], hx0 = hx[o];
    Real hyv = O::fma(chez, dEy, hy0);
    Real hxv = O::fma(-chez, dEx, hx0);
    const int ixh = (x < nc) ? nc - 1 - x : ((x >= nx - nc) ? x - nx + nc : -1);
    const int iyh = (m < nc) ? nc - 1 - m : ((m >= ny - nc) ? m - ny + nc : -1);
    if (ixh >= 0) {
        const int xsx = (x < nc) ? x : x - (nx - nc) + nc;
        Real* p = psi + (size_t)m * 2 * nc + xsx;                        // psi_hyx, x strips
        const Real ps = O::fma(cpml[4 * nc + ixh], *p, O::mul(cpml[5 * nc + ixh], dEy));
        *p = ps;
        hyv = O::fma(O::mul(chez, dEy), cpml[3 * nc + ixh], hy0);
        hyv = O::fma(O::mul(chez, dxr), ps, hyv);
    }
    if (iyh >= 0) {
        const int ysx = (m < nc) ? m : m - (ny - nc) + nc;
        Real* p = psi + 2 * (size_t)(ny + 1) * 2 * nc + (size_t)ysx * (nx + 1) + x;   // psi_hxy, y strips
        const Real ps = O::fma(cpml[4 * nc + iyh], *p, O::mul(cpml[5 * nc + iyh], dEx));
        *p = ps;
        hxv = O::fma(-O::mul(chez, dEx), cpml[3 * nc + iyh], hx0);
        hxv = O::fma(-O::mul(chez, dxr), ps, hxv);
    }
    if (kRef && (D.flags & kNanClamp)) {
        if (dev_isnan(hxv)) hxv = Real(0);
        if (dev_isnan(hyv)) hyv = Real(0);
    }
    hx[o] = hxv;
    hy[o] = hyv;
}

template <typename Real, int MODE>
__global__ void __launch_bounds__(256) plain_e_kernel(const SolveDesc<Real>* __restrict__ Dp, int n) {
    const SolveDesc<Real>& D = *Dp;
    using O = Op<Real>;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int m = blockIdx.y * blockDim.y + threadIdx.y;
    const int nx = D.nx, ny = D.ny, nc = D.ncpml, pitch = D.pitch;
    if (x < 1 || x > nx - 1 || m < 1 || m > ny - 1) return;   // PEC boundary: Ez stays 0
    constexpr bool kRef = MODE == kModeRef;
    const Real Kp = D.Kp, dxr = D.dx;
    const Real* __restrict__ cpml = D.cpml;
    Real* __restrict__ ezp = D.ez[0];
    const Real* __restrict__ hx = D.hx[0];
    const Real* __restrict__ hy = D.hy[0];
    Real* __restrict__ jpp = D.jp[0];
    Real* __restrict__ psi = D.psi[0];
    const long long o = (long long)m * pitch + x;
    const uint32_t mb = D.mat[(long long)m * D.mpitch + x];
    const int mi = mb & kMatMask;
    const Real* cf = D.mtab + mi * kMatCoef;
    const Real Ca = cf[kCa], Cb = cf[kCb], Cj = cf[kCj], Bp = cf[kBp];
    const Real dHy = O::sub(hy[o], hy[o - 1]);
    const Real dHx = O::sub(hx[o], hx[o - pitch]);
    const Real ez = ezp[o];
    const bool jin = m >= D.jy0 && m <= D.jy1 && x >= D.jx0 && x <= D.jx1;   // dispersive box
    const Real jp = jin ? jpp[o] : Real(0);
    const int ixe = (x <= nc) ? nc - x : ((x >= nx - nc) ? x - nx + nc : -1);
    const int iye = (m <= nc) ? nc - m : ((m >= ny - nc) ? m - ny + nc : -1);
    const size_t psx_e = (size_t)(ny + 1) * 2 * nc;
    const size_t psy_e = 2 * (size_t)(ny + 1) * 2 * nc + 2 * (size_t)nc * (nx + 1);
    Real out, jpo;
    if (kRef) {
        Real gp = Real(0), gm = Real(0);
        const Real Ci = cf[kCi], Cp = cf[kCp];
        if (Ci != Real(0) || Cp != Real(0) || Bp != Real(0)) {
            // fwf() argument in FP64 (FDTD_GPU.cu:290)
            const double b = __dmul_rn(__dadd_rn(__dmul_rn(D.pw_ky, (double)m - D.pw_yoff),
                                                 __dmul_rn(D.pw_kx, (double)x - D.pw_xoff)),
                                       D.pw_dxc0);
            const double a0 = __dsub_rn(__dsub_rn(__dmul_rn((double)n + 0.5, D.dt), D.pw_t0l), b);
            const double a1 = __dsub_rn(__dsub_rn(__dmul_rn((double)n - 0.5, D.dt), D.pw_t0l), b);
            const Real u0 = (Real)__dmul_rn(a0, D.pw_inv_tau), u1 = (Real)__dmul_rn(a1, D.pw_inv_tau);
            gp = dev_exp<Real>(-O::mul(u0, u0));
            gm = dev_exp<Real>(-O::mul(u1, u1));
        }
        // FDTD_GPU.cu:378-385 (interior), then the strip overrides :389-416
        out = O::fma(Ca, ez, O::sub(O::mul(Cb, dHy), O::mul(Cb, dHx)));
        out = O::fma(Ci, gp, O::fma(Cp, gm, out));
        out = O::fma(-Cj, jp, out);
        // total-field incident grid: the legacy centre source (oldFDTD_GPU.cu:680-683)
        if ((D.flags & kPointSource) && m == D.src_y && x == D.src_x) out = O::fma(cf[kCs], D.src_wave[n], out);
        jpo = O::fma(Kp, jp, O::mul(Bp, O::add(O::sub(out, ez), O::sub(gp, gm))));
        if (ixe >= 0) {
            const int xsx = (x <= nc) ? x - 1 : x - (nx - nc) + nc;
            Real* p = psi + psx_e + (size_t)m * 2 * nc + xsx;
            const Real ps = O::fma(cpml[nc + ixe], *p, O::mul(cpml[2 * nc + ixe], dHy));
            *p = ps;
            out = O::fma(Ca, ez, O::mul(O::mul(Cb, O::sub(dHy, dHx)), cpml[ixe]));
            out = O::fma(O::mul(Cb, dxr), ps, out);
        }
        if (iye >= 0) {
            const int ysx = (m <= nc) ? m - 1 : m - (ny - nc) + nc;
            Real* p = psi + psy_e + (size_t)ysx * (nx + 1) + x;
            const Real ps = O::fma(cpml[nc + iye], *p, O::mul(cpml[2 * nc + iye], dHx));
            *p = ps;
            out = O::fma(Ca, ez, O::mul(O::mul(Cb, O::sub(dHy, dHx)), cpml[iye]));
            out = O::fma(-O::mul(Cb, dxr), ps, out);
        }
        if ((D.flags & kNanClamp) && dev_isnan(out)) out = Real(0);
    } else {
        Real cx = dHy, cy = dHx, qx = Real(0), qy = Real(0);
        if (ixe >= 0) {
            const int xsx = (x <= nc) ? x - 1 : x - (nx - nc) + nc;
            Real* p = psi + psx_e + (size_t)m * 2 * nc + xsx;
            qx = O::fma(cpml[nc + ixe], *p, O::mul(cpml[2 * nc + ixe], dHy));
            *p = qx;
            cx = O::mul(dHy, cpml[ixe]);
        }
        if (iye >= 0) {
            const int ysx = (m <= nc) ? m - 1 : m - (ny - nc) + nc;
            Real* p = psi + psy_e + (size_t)ysx * (nx + 1) + x;
            qy = O::fma(cpml[nc + iye], *p, O::mul(cpml[2 * nc + iye], dHx));
            *p = qy;
            cy = O::mul(dHx, cpml[iye]);
        }
        if (ixe >= 0 || iye >= 0)
            out = O::fma(Ca, ez, O::mul(Cb, O::fma(dxr, O::sub(qx, qy), O::sub(cx, cy))));
        else
            out = O::fma(Ca, ez, O::mul(Cb, O::sub(dHy, dHx)));
        out = O::fma(-Cj, jp, out);
        if ((D.flags & kPointSource) && m == D.src_y && x == D.src_x) out = O::fma(cf[kCs], D.src_wave[n], out);
        jpo = O::fma(Kp, jp, O::mul(Bp, O::sub(out, ez)));
    }
    ezp[o] = out;
    if (jin) jpp[o] = jpo;
    if (mb & kMatRx) {
        for (int rr = 0; rr < D.nrx; ++rr)
            if (D.rx[2 * rr] == x && D.rx[2 * rr + 1] == m) D.traces[(size_t)rr * D.steps_total + n] = out;
    }
}

// One thread per NTFF contour point (contour order of FDTD_common.cxx:4-46:
// bottom face left to right, right face upwards, top face right to left, left
// face downwards).  J from the tangential H, M from the face-averaged Ez.
template <typename Real>
__global__ void __launch_bounds__(128) plain_dft_kernel(const SolveDesc<Real>* __restrict__ Dp, int n) {
    const SolveDesc<Real>& D = *Dp;
    using O = Op<Real>;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int C = D.n_contour, nfreq = D.nfreq;
    if (c >= C || nfreq <= 0) return;
    const int nx = D.nx, ny = D.ny, d = D.nf_d, pitch = D.pitch;
    const int l1 = nx - 2 * d - 2, lv = ny - 2 * d;
    const Real* __restrict__ ez = D.ez[0];
    const Real half = Real(0.5);
    Real h, e;
    if (c < l1) {                       // bottom face, row d
        const int x = d + 1 + c;
        const long long o = (long long)d * pitch + x;
        h = D.hx[0][o];
        e = O::mul(O::add(ez[o], ez[o + pitch]), half);
    } else if (c < l1 + lv) {           // right face, column nx-d-1
        const int y = d + (c - l1);
        const long long o = (long long)y * pitch + (nx - d - 1);
        h = D.hy[0][o];
        e = O::mul(O::add(ez[o], ez[o + 1]), half);
    } else if (c < 2 * l1 + lv) {       // top face, row ny-d-1
        const int x = nx - d - 2 - (c - l1 - lv);
        const long long o = (long long)(ny - d - 1) * pitch + x;
        h = -D.hx[0][o];
        e = -O::mul(O::add(ez[o], ez[o + pitch]), half);
    } else {                            // left face, column d
        const int y = ny - d - 1 - (c - 2 * l1 - lv);
        const long long o = (long long)y * pitch + d;
        h = -D.hy[0][o];
        e = -O::mul(O::add(ez[o], ez[o + 1]), half);
    }
    dft_update(D.acc, D.phasor + (size_t)n * nfreq * 4, nfreq, C, c, h, e);
}

}  // namespace tomo
