// Wavefront temporal-blocking FDTD advance kernel (2D TMz Yee + CPML + Debye ADE).
//
// Work decomposition.  A work item is one vertical strip of one solve.  One
// warp owns the item: each lane holds COLS consecutive columns, so a warp
// spans P = 32*COLS columns; it writes back the item's owned columns (at most
// W = P - 2T of them) and recomputes the T columns on either side as halo.
// Strips near the left and right edges (PEC boundary, CPML, vertical NTFF
// faces) use the narrow COLS = 1 layout inside the same launch, so that the
// special handling below runs on as few lanes as possible.  The warp sweeps the
// strip bottom-to-top, one row per iteration, and carries T time levels in
// flight: level k receives row r-2k (from level k-1 one iteration earlier),
// advances row r-2k-1 from time n0+k to n0+k+1 and hands it to level k+1.
// Every row is therefore read from HBM once and written once per T time
// steps; x-neighbours come from warp shuffles, y-neighbours from registers.
// Levels are processed in descending order so that no level waits on another
// inside an iteration (independent instruction streams for the scheduler).
//
// Code paths, chosen warp-uniformly:
//  * interior block: every level of the iteration on an interior row of a
//    strip without special columns -- all T levels as one straight-line block,
//    so the scheduler interleaves their independent dependency chains;
//  * edge block (breast mode): the same for the narrow edge strips, with the
//    x-CPML terms computed on every lane and chosen per lane by select;
//  * otherwise per level: the fast path (interior rows, and in breast mode the
//    y-CPML rows), the edge path (other rows of the narrow strips, breast
//    mode) or the general path (boundary rows, NTFF face rows, source and
//    receiver rows, and in the reference modes the edge strips and the
//    plane-wave rows).
// All evaluate the same explicitly rounded formulas, so a cell gets the same
// bits whichever path computes it.  The running DFT of the NTFF contour is a
// separate kernel (dft_accumulate_kernel): the sweep only stores each level's
// contour samples.
//
// Physics per cell follows the reference kernels:
//   H update  FDTD_GPU.cu:298-355  (Hy += Chez dEz/dx, Hx -= Chez dEz/dy, CPML psi)
//   E update  FDTD_GPU.cu:358-434  (Ceze, Cezh, Debye polarisation current Jp,
//             scattered-field plane wave, CPML psi; PEC boundary)
//   DFT       FDTD_GPU.cu:231-280  (running DFT of J = n x H and M = -n x E on
//             the NTFF rectangle; contour order of FDTD_common.cxx:4-46)
// extended with a soft point current source (FDTD_CPU.cxx:324-327, 972-983)
// and receiver sampling (FDTD_CPU.cxx:808).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "solve_desc.h"

namespace tomo {

// One vertical strip of one solve: owned columns [x0, x1) of solve `solve`.
// Narrow items (COLS = 1 layout, 32 - 2T owned columns) cover the CPML,
// boundary and vertical NTFF-face columns near the left and right edges, where
// every row needs per-lane special handling; wide items (the kernel's COLS)
// cover the interior, whose halo stays clear of those columns.
//
// A strip may be cut into row segments (owned rows [y0, y1)) when a batch has
// too few strips to fill the GPU.  A segment's sweep starts 2T rows below y0
// and runs until every level has advanced row y1, recomputing those halo rows;
// only owned rows are written (fields, CPML psi, receiver samples, NTFF sums).
struct WorkItem {
    int solve;
    int x0, x1;
    int narrow;
    int y0, y1;
};

enum AdvanceMode : int {
    kModeBreast = 0,   // proper CPML, point current source, no plane wave
    kModeRef = 1       // reference CPML semantics, scattered-field plane wave, optional NaN clamp
};

constexpr int kMaxRowWords = 256;   // row-flag words per warp: grids up to 8192 rows

template <typename Real>
__device__ __forceinline__ Real dev_exp(Real v);
template <>
__device__ __forceinline__ float dev_exp<float>(float v) { return expf(v); }
template <>
__device__ __forceinline__ double dev_exp<double>(double v) { return exp(v); }

template <typename Real>
__device__ __forceinline__ bool dev_isnan(Real v) { return v != v; }

// Explicitly rounded arithmetic: the update formulas are written with these so
// that no instantiation (blocking depth, columns per lane, code path, register
// pressure) can contract them differently -- every configuration gives
// bit-identical fields.
template <typename Real>
struct Op;
template <>
struct Op<float> {
    static __device__ __forceinline__ float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
};
template <>
struct Op<double> {
    static __device__ __forceinline__ double fma(double a, double b, double c) { return __fma_rn(a, b, c); }
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
};

// Asynchronous global->shared copies (cp.async, completion per thread via
// commit/wait groups).  src_bytes = 0 zero-fills without reading global memory.
template <int BYTES>
__device__ __forceinline__ void cp_async(void* smem_dst, const void* gmem_src, bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    const int n = valid ? BYTES : 0;
    if constexpr (BYTES == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(gmem_src), "r"(n) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(d), "l"(gmem_src), "n"(BYTES), "r"(n)
                     : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Rows in flight ahead of the one being consumed.  A warp spends about a
// microsecond per row-iteration at full occupancy, so three rows ahead cover
// the HBM latency; the short ring keeps the shared memory of a 4-warp block
// small enough for three or more resident blocks per SM.
constexpr int kPrefetch = 3;
constexpr int kRowSlots = 4;       // ring slots per warp (kPrefetch + 1, a power of two)

// Kahan-compensated accumulation (FP32); plain accumulation in FP64.
template <typename Real>
__device__ __forceinline__ void acc_add(Real& sum, Real& comp, Real term) {
    using O = Op<Real>;
    Real y = O::sub(term, comp);
    Real t = O::add(sum, y);
    comp = O::sub(O::sub(t, sum), y);
    sum = t;
}
template <>
__device__ __forceinline__ void acc_add<double>(double& sum, double& comp, double term) {
    (void)comp;
    sum = __dadd_rn(sum, term);
}

// Contour index of a cell on a face (inverse of FDTD_common.cxx:4-46).
__device__ __forceinline__ int contour_index_yn(int nx, int ny, int d, int x) { return x - d - 1; }
__device__ __forceinline__ int contour_index_yp(int nx, int ny, int d, int x) {
    int l1 = nx - 2 * d - 2, l2 = l1 + (ny - 2 * d);
    return l2 + (nx - d - 2 - x);
}
__device__ __forceinline__ int contour_index_xp(int nx, int ny, int d, int y) { return (nx - 2 * d - 2) + (y - d); }
__device__ __forceinline__ int contour_index_xn(int nx, int ny, int d, int y) {
    int l1 = nx - 2 * d - 2, l3 = 2 * l1 + (ny - 2 * d);
    return l3 + (ny - d - 1 - y);
}

// One running-DFT update of one contour cell (J from h, M from the face-averaged e).
template <typename Real>
__device__ __forceinline__ void dft_update(Real* acc, const Real* ph, int nfreq, int C, int c, Real h, Real e) {
    for (int f = 0; f < nfreq; ++f) {
        const Real* p = ph + 4 * f;
        Real* a = acc + ((size_t)f * C + c) * 8;
        Real s0 = a[0], s1 = a[1], c0 = a[2], c1 = a[3], s2 = a[4], s3 = a[5], c2 = a[6], c3 = a[7];
        acc_add(s0, c0, Op<Real>::mul(h, p[0]));
        acc_add(s1, c1, Op<Real>::mul(h, p[1]));
        acc_add(s2, c2, Op<Real>::mul(e, p[2]));
        acc_add(s3, c3, Op<Real>::mul(e, p[3]));
        a[0] = s0; a[1] = s1; a[2] = c0; a[3] = c1; a[4] = s2; a[5] = s3; a[6] = c2; a[7] = c3;
    }
}

// Running DFT of the NTFF contour (FDTD_GPU.cu:231-280) for the time steps the
// last advance launch computed: one thread per (solve, contour point) adds the
// staged (h, e) samples of the launch's levels in time order, with the same
// compensated sums as one update per step.  Runs between the advance launch
// and the progress bump (which moves `step`).
// Accumulators of one (frequency, contour point) and a phasor as vectors
// (32 and 16 bytes, aligned: the accumulator and phasor arrays start on
// 128-byte boundaries and hold 8 and 4 values per entry).
template <typename Real>
struct Vec4;
template <>
struct Vec4<float> {
    using type = float4;
    static __device__ __forceinline__ void load(const float* p, float (&v)[4]) {
        const float4 x = *reinterpret_cast<const float4*>(p);
        v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
    }
    static __device__ __forceinline__ void store(float* p, const float (&v)[4]) {
        *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    }
};
template <>
struct Vec4<double> {
    static __device__ __forceinline__ void load(const double* p, double (&v)[4]) {
        const double2 x = reinterpret_cast<const double2*>(p)[0], y = reinterpret_cast<const double2*>(p)[1];
        v[0] = x.x; v[1] = x.y; v[2] = y.x; v[3] = y.y;
    }
    static __device__ __forceinline__ void store(double* p, const double (&v)[4]) {
        reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
        reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
    }
};

// The staging buffer holds kStageLevels levels: a launch of T steps writes its
// levels at slot ((step / T) % stage_group) * T, so stage_group launches fill
// it before one pass of this kernel sums them.  Called with n0 >= 0 (steps
// n0 .. n0 + nlev - 1 in slots 0 .. nlev - 1, the engine's fixed time loop) or
// with n0 < 0 (the levels of the launch that starts at the solve's current
// step, stage_group = 1: the serving loop, whose solves differ in progress).
constexpr int kStageLevels = 8;

template <typename Real>
__global__ void __launch_bounds__(128) dft_accumulate_kernel(const SolveDesc<Real>* __restrict__ descs, int T,
                                                             int n0_group, int nlev) {
    const SolveDesc<Real>& D = descs[blockIdx.x];
    const int c = blockIdx.y * blockDim.x + threadIdx.x;
    const int C = D.n_contour, nfreq = D.nfreq;
    if (!D.active || nfreq <= 0 || c >= C) return;
    const int n0 = n0_group >= 0 ? n0_group : D.step;
    const int nsteps = min(n0_group >= 0 ? nlev : T, D.steps_total - n0);
    for (int f = 0; f < nfreq; ++f) {
        Real* a = D.acc + ((size_t)f * C + c) * 8;
        Real j[4], mm[4];   // J: sum re, sum im, comp re, comp im; M likewise
        Vec4<Real>::load(a, j);
        Vec4<Real>::load(a + 4, mm);
        for (int k = 0; k < nsteps; ++k) {
            Real p[4];
            Vec4<Real>::load(D.phasor + ((size_t)(n0 + k) * nfreq + f) * 4, p);
            const Real* sp = D.stage + ((size_t)k * C + c) * 2;
            const Real h = sp[0], e = sp[1];
            acc_add(j[0], j[2], Op<Real>::mul(h, p[0]));
            acc_add(j[1], j[3], Op<Real>::mul(h, p[1]));
            acc_add(mm[0], mm[2], Op<Real>::mul(e, p[2]));
            acc_add(mm[1], mm[3], Op<Real>::mul(e, p[3]));
        }
        Vec4<Real>::store(a, j);
        Vec4<Real>::store(a + 4, mm);
    }
}

// Two adjacent values as one streaming store (aligned to twice the element size).
__device__ __forceinline__ void store_pair(float* p, const float (&v)[2]) {
    __stcg(reinterpret_cast<float2*>(p), make_float2(v[0], v[1]));
}
__device__ __forceinline__ void store_pair(double* p, const double (&v)[2]) {
    __stcg(reinterpret_cast<double2*>(p), make_double2(v[0], v[1]));
}
// Four adjacent floats as one streaming 16-byte store (aligned to 16 bytes).
__device__ __forceinline__ void store_quad(float* p, const float (&v)[4]) {
    __stcg(reinterpret_cast<float4*>(p), make_float4(v[0], v[1], v[2], v[3]));
}
__device__ __forceinline__ void store_quad(double* p, const double (&v)[4]) {
    __stcg(reinterpret_cast<double2*>(p), make_double2(v[0], v[1]));
    __stcg(reinterpret_cast<double2*>(p) + 1, make_double2(v[2], v[3]));
}

// Ca, Cb, Cj, Bp of one material from the per-warp table (one 16-byte load in FP32).
__device__ __forceinline__ void load_coefs(const float* t, float& a, float& b, float& c, float& d) {
    const float4 v = *reinterpret_cast<const float4*>(t);
    a = v.x; b = v.y; c = v.z; d = v.w;
}
__device__ __forceinline__ void load_coefs(const double* t, double& a, double& b, double& c, double& d) {
    const double2 v0 = reinterpret_cast<const double2*>(t)[0], v1 = reinterpret_cast<const double2*>(t)[1];
    a = v0.x; b = v0.y; c = v1.x; d = v1.y;
}

// Shared memory of one warp (a block holds four such regions, each sized for
// the larger of the narrow and the wide layout).
template <typename Real, int T, int COLS>
struct WarpSmem {
    // CPML psi sub-arrays held: hyx, ezx (x strips), hxy, ezy (y strips).  The
    // wide layout (COLS > 1) never holds an x-strip column, so it keeps the
    // y-strip pair only (see psi_slot).
    static constexpr int kPsiF = COLS == 1 ? 4 : 2;
    Real rows[kRowSlots][4][32 * COLS];   // prefetch ring: Ez, Hx, Hy, Jp of kRowSlots rows
    Real psring[kRowSlots][kPsiF][32 * COLS];   // prefetch ring: CPML psi at time n0
    Real pslev[T > 1 ? T - 1 : 1][kPsiF][4][32 * COLS];   // psi after level k, 4 rows in flight
    Real tab[kMaxMat][4];                 // Ca, Cb, Cj, Bp of every material
    Real cpml[6 * kMaxCpml];              // CPML profile (1/ke, be, ae, 1/km, bm, am)
    uint32_t rowbits[kMaxRowWords];       // "row needs the general path" flags
    uint32_t iterbits[kMaxRowWords + 1];  // "every level takes the straight-line block" flags, per iteration
    uint8_t mats[kRowSlots][32 * COLS + 16];   // prefetch ring: material bytes
};

// Slot of psi sub-array f (0 hyx, 1 ezx, 2 hxy, 3 ezy) in a layout's rings; the
// x-strip sub-arrays of the wide layout are never touched (slot 0 for them is
// only a placeholder in code that does not run).
template <int COLS>
__host__ __device__ constexpr int psi_slot(int f) {
    return COLS == 1 ? f : (f >= 2 ? f - 2 : 0);
}

template <typename Real, int T, int COLS>
constexpr size_t warp_smem_bytes() {
    constexpr size_t a = sizeof(WarpSmem<Real, T, COLS>), b = sizeof(WarpSmem<Real, T, 1>);
    return ((a > b ? a : b) + 15) / 16 * 16;
}

// Dynamic shared memory of a 4-warp block.
template <typename Real, int T, int COLS>
constexpr size_t advance_block_smem() { return 4 * warp_smem_bytes<Real, T, COLS>(); }

template <typename Real, int T, int COLS, int MODE>
__device__ void advance_item(const SolveDesc<Real>* __restrict__ Dp, const WorkItem& wi, WarpSmem<Real, T, COLS>& ws) {
    // The descriptor is read-only for the whole launch (restrict).
    const SolveDesc<Real>& D = *Dp;
    using O = Op<Real>;
    constexpr int P = 32 * COLS;
    static_assert(P > 2 * T, "a strip must own at least one column");
    constexpr bool kRef = MODE == kModeRef;
    constexpr bool kEdgePath = !kRef && COLS == 1;   // edge strips use the narrow layout
    const int lane = threadIdx.x & 31;
    const int nx = D.nx, ny = D.ny, nc = D.ncpml, S = D.steps_total, n0 = D.step;
    const int nsteps = min(T, S - n0);
    if (nsteps <= 0) return;
    const int pitch = D.pitch;
    // The warp's P columns end T columns right of the owned range [x0, x1)
    // (x1 - x0 <= P - 2T): a clipped strip carries extra halo on its left, so
    // its columns never reach further right than a full strip ending at x1.
    const int xs = wi.x1 + T - P;      // column of position 0
    const int ox0 = wi.x0, ox1 = wi.x1;
    const int y0 = wi.y0, y1 = wi.y1;   // owned rows
    const int src = D.parity, dst = 1 - src;
    const Real chez = D.chez, Kp = D.Kp, dxr = D.dx;
    const bool clampnan = kRef && (D.flags & kNanClamp) != 0;
    const bool psrc = (D.flags & kPointSource) != 0;
    const int C = D.n_contour, nfreq = D.nfreq, fd = D.nf_d;
    const int psx_h = 0, psx_e = (ny + 1) * 2 * nc;                 // x-strip psi sub-arrays
    const int psy0 = 2 * (ny + 1) * 2 * nc;
    const int psy_h = psy0, psy_e = psy0 + 2 * nc * (nx + 1);         // y-strip psi sub-arrays
    const uint8_t* __restrict__ matp = D.mat;
    Real* const cpml = ws.cpml;   // CPML profile, copied to shared memory below
    // [T][C][2] contour samples of this launch's levels, in its slots of the staging buffer
    Real* __restrict__ stage = D.stage + (size_t)((n0 / T) % D.stage_group) * T * C * 2;
    const int mpitch = D.mpitch, jx0 = D.jx0, jx1 = D.jx1, jy0 = D.jy0, jy1 = D.jy1;
    const int src_x = D.src_x, src_y = D.src_y;

    // hot material coefficients (of the solve's materials) and the CPML profile
    // -> shared memory (per warp)
    for (int i = lane; i < D.nmat * 4; i += 32) ws.tab[i >> 2][i & 3] = D.mtab[(i >> 2) * kMatCoef + (i & 3)];
    for (int i = lane; i < 6 * nc; i += 32) cpml[i] = D.cpml[i];

    // per-column constants
    int xcol[COLS];
    int ixh[COLS], ixe[COLS];
    bool owned[COLS];
    int face_slot[COLS];   // 0: xn face column, 1: xp face column, -1 none
    // The wide layout (COLS > 1) never holds a special column: the host puts
    // the PEC boundary, CPML and vertical NTFF-face columns, and the halo that
    // reaches them, into narrow items and checks every wide window before
    // launch (validate_items).  There the column state below is constant and
    // its code paths drop out of the wide instance.
    constexpr bool kWide = COLS > 1;
    bool wspecial = false, wdisp = false;
#pragma unroll
    for (int c = 0; c < COLS; ++c) {
        int x = xs + lane * COLS + c;
        xcol[c] = x;
        owned[c] = x >= ox0 && x < ox1;
        ixh[c] = ixe[c] = face_slot[c] = -1;
        if constexpr (!kWide) {
            ixh[c] = (x >= 0 && x < nc) ? nc - 1 - x : ((x >= nx - nc && x < nx) ? x - nx + nc : -1);
            ixe[c] = (x >= 1 && x <= nc) ? nc - x : ((x >= nx - nc && x <= nx - 1) ? x - nx + nc : -1);
            if (nfreq > 0 && owned[c]) {
                if (x == fd) face_slot[c] = 0;
                else if (x == nx - fd - 1) face_slot[c] = 1;
            }
            // CPML strips, PEC boundary and padding columns, vertical NTFF faces
            wspecial |= x <= nc || x >= nx - nc || (nfreq > 0 && (x == fd || x == nx - fd - 1));
        }
        wdisp |= x >= jx0 && x <= jx1;
    }
    bool has_face0 = false, has_face1 = false;
    if constexpr (!kWide) {
#pragma unroll
        for (int c = 0; c < COLS; ++c) {
            has_face0 |= face_slot[c] == 0;
            has_face1 |= face_slot[c] == 1;
        }
        has_face0 = __any_sync(0xffffffffu, has_face0);
        has_face1 = __any_sync(0xffffffffu, has_face1);
        wspecial = __any_sync(0xffffffffu, wspecial);
    }
    wdisp = __any_sync(0xffffffffu, wdisp);

    // rows that need the general path: CPML rows and boundaries, NTFF face rows,
    // plane-wave rows (reference modes), and -- only in the strips whose columns
    // (halo included) hold them -- the source row and receiver rows
    // Only the words the sweep reads are built: iterations [sweep_r0, sweep_r1]
    // advance rows down to 2T - 1 below the first (a short row segment needs a
    // few words, not the whole grid's).
    const int sweep_r0 = max(0, y0 - 2 * T);           // halo rows below the segment
    const int sweep_r1 = min(ny, y1) + 2 * T - 1;      // every level advances row y1 (or ny)
    const int iw_lo = sweep_r0 >> 5, iw_hi = sweep_r1 >> 5;
    uint32_t* rowbits = ws.rowbits;
    const int nwords = (ny + 1 + 31) >> 5;
    const int rw_lo = max(0, 32 * iw_lo - 2 * T - 1) >> 5, rw_hi = min(nwords - 1, iw_hi);
    const bool src_here = psrc && src_x >= xs && src_x < xs + P;
    for (int w = rw_lo + lane; w <= rw_hi; w += 32) {
        uint32_t bits = 0;
        for (int b = 0; b < 32; ++b) {
            const int m = 32 * w + b;
            // breast mode: y-CPML rows run on the fast path (uniform psi terms)
            bool sp = kRef ? (m <= nc || m >= ny - nc) : (m <= 0 || m >= ny);
            sp |= nfreq > 0 && (m == fd + 1 || m == ny - fd);
            sp |= src_here && m == src_y;
            sp |= kRef && wdisp && m >= jy0 && m <= jy1;
            if (sp) bits |= 1u << b;
        }
        rowbits[w] = bits;
    }
    __syncwarp();
    for (int rr = lane; rr < D.nrx; rr += 32) {
        const int x = D.rx[2 * rr], m = D.rx[2 * rr + 1];
        if (x >= xs && x < xs + P) atomicOr(&rowbits[m >> 5], 1u << (m & 31));
    }
    __syncwarp();

    // x-CPML profile of the lane's columns (the profile is in shared memory
    // by now).  The narrow layout, which holds the x-CPML columns, keeps the
    // six values per column in registers; the wide layout reads shared memory.
    // Columns outside the x strips get index 0; their values are never chosen.
    Real xpf[6][COLS];   // 1/ke, be, ae (E update), 1/km, bm, am (H update)
    if constexpr (COLS == 1) {
        const int ie = ixe[0] >= 0 ? ixe[0] : 0, ih = ixh[0] >= 0 ? ixh[0] : 0;
        xpf[0][0] = cpml[ie];
        xpf[1][0] = cpml[nc + ie];
        xpf[2][0] = cpml[2 * nc + ie];
        xpf[3][0] = cpml[3 * nc + ih];
        xpf[4][0] = cpml[4 * nc + ih];
        xpf[5][0] = cpml[5 * nc + ih];
    }
    // profile value `q` (0..5 as in the shared-memory table) of column c at index i
    auto xprof = [&](int q, int c, int i) -> Real {
        if constexpr (COLS == 1) return xpf[q][c];
        else return cpml[q * nc + i];
    };

    // Iterations r whose levels all take one straight-line block: every level's
    // row r - 2k - 1 in [row_lo, row_hi] and not flagged.  For strips without
    // special columns that is the interior block (rows off the y-CPML); for
    // the narrow edge strips (breast mode) the edge block, which also stays in
    // the row range of the strip's vertical NTFF faces.  One bit per
    // iteration, so that an iteration tests one flag instead of T rows.
    {
        int row_lo = nc + 1, row_hi = ny - nc - 1;
        if (wspecial && (has_face0 || has_face1)) {
            row_lo = max(row_lo, fd);
            row_hi = min(row_hi, ny - fd - 1);
        }
        const bool any = nsteps == T && (!wspecial || kEdgePath);
        for (int w = iw_lo + lane; w <= iw_hi; w += 32) {
            uint32_t bits = 0u;
            if (any)
                for (int b = 0; b < 32; ++b) {
                    const int r = 32 * w + b;
                    bool ok = true;
#pragma unroll
                    for (int k = 0; k < T; ++k) {
                        const int m = r - 2 * k - 1;
                        ok = ok && m >= row_lo && m <= row_hi && !((rowbits[m >> 5] >> (m & 31)) & 1u);
                    }
                    if (ok) bits |= 1u << b;
                }
            ws.iterbits[w] = bits;
        }
        __syncwarp();
    }

    // level registers
    Real pz[T][COLS], px_[T][COLS], py_[T][COLS], pj[T][COLS];   // row m input (prev)
    Real hz[T][COLS], hxr[T][COLS], hyr[T][COLS], hj[T][COLS];   // row m+1 input (handoff)
    Real hxn[T][COLS], ezn[T][COLS];                             // outputs of row m-1
    uint32_t pmat[T], hmat[T];                                   // material bytes of those rows, packed
#pragma unroll
    for (int k = 0; k < T; ++k) {
        pmat[k] = hmat[k] = 0u;
#pragma unroll
        for (int c = 0; c < COLS; ++c) {
            pz[k][c] = px_[k][c] = py_[k][c] = pj[k][c] = Real(0);
            hz[k][c] = hxr[k][c] = hyr[k][c] = hj[k][c] = Real(0);
            hxn[k][c] = ezn[k][c] = Real(0);
        }
    }

    const Real* __restrict__ ez_s = D.ez[src];
    const Real* __restrict__ hx_s = D.hx[src];
    const Real* __restrict__ hy_s = D.hy[src];
    const Real* __restrict__ jp_s = D.jp[src];
    Real* __restrict__ ez_d = D.ez[dst];
    Real* __restrict__ hx_d = D.hx[dst];
    Real* __restrict__ hy_d = D.hy[dst];
    Real* __restrict__ jp_d = D.jp[dst];
    // CPML psi, fields 0 hyx, 1 ezx (x strips), 2 hxy, 3 ezy (y strips).  Time
    // n0 comes from the global copy of the previous launch (prefetched with the
    // row), intermediate time levels live in warp-private shared memory, and
    // the last level writes the owned columns of the next global copy.
    const Real* __restrict__ psi_src = D.psi[src];
    Real* __restrict__ psi_dst = D.psi[dst];
    auto psi_in = [&](int k, int f, int m, int c) -> Real {
        if (k == 0) return ws.psring[m & (kRowSlots - 1)][psi_slot<COLS>(f)][lane * COLS + c];
        return ws.pslev[(k - 1) % (T > 1 ? T - 1 : 1)][psi_slot<COLS>(f)][m & 3][lane * COLS + c];
    };
    auto psi_out = [&](int k, int f, int m, int c, Real v, size_t goff) {
        if (k + 1 < T) ws.pslev[k % (T > 1 ? T - 1 : 1)][psi_slot<COLS>(f)][m & 3][lane * COLS + c] = v;
        else if (owned[c] && m >= y0 && m < y1) psi_dst[goff] = v;
    };
    // vertical NTFF faces: stage the (h, e) sample of an owned face cell of row m
    // at level k (outward normal -x on the left face, +x on the right face)
    // contour index of a face cell, linear in the row: ci = face_ci0 + face_dir * m
    // (contour_index_xn / contour_index_xp), and the outward-normal sign
    int face_ci0[COLS], face_dir[COLS];
    Real face_sg[COLS];
#pragma unroll
    for (int c = 0; c < COLS; ++c) {
        const bool xn = face_slot[c] == 0;
        face_ci0[c] = xn ? contour_index_xn(nx, ny, fd, 0) : contour_index_xp(nx, ny, fd, 0);
        face_dir[c] = xn ? -1 : 1;
        face_sg[c] = xn ? Real(-1) : Real(1);
    }
    auto stage_vertical = [&](int k, int m, int c, Real h, Real e) {
        if (face_slot[c] >= 0 && m >= y0 && m < y1) {
            Real* sp = stage + ((size_t)k * C + (face_ci0[c] + face_dir[c] * m)) * 2;
            sp[0] = face_sg[c] * h;
            sp[1] = face_sg[c] * e;
        }
    };
    bool wxs = false;   // warp holds an x-strip column (uniform; never in the wide layout)
    if constexpr (!kWide) {
#pragma unroll
        for (int c = 0; c < COLS; ++c) wxs |= ixh[c] >= 0 || ixe[c] >= 0;
        wxs = __any_sync(0xffffffffu, wxs);
    }

    // Rows stream through a per-warp shared-memory ring: row r + kPrefetch is
    // requested (cp.async) while row r is consumed, so kPrefetch rows of every
    // warp are in flight and HBM latency is hidden.  Each lane copies its own
    // columns of the four fields; lanes 0..P/4 copy the material bytes.
    constexpr int kBytes = COLS * (int)sizeof(Real);
    const int mstart = xs & ~3;        // 4-byte aligned start of the material window
    const int moff = xs - mstart;
    const int x0 = xs + lane * COLS;              // the lane's first column
    const Real* const ez_l = ez_s + x0;
    const Real* const hx_l = hx_s + x0;
    const Real* const hy_l = hy_s + x0;
    const Real* const jp_l = jp_s + x0;
    const uint8_t* const mat_l = matp + mstart + 4 * lane;
    const bool jcols = x0 + COLS - 1 >= jx0 && x0 <= jx1;   // the lane meets the dispersive columns
    auto issue_row = [&](int r) {
        const int slot = r & (kRowSlots - 1);
        const bool valid = r <= ny;
        const unsigned ro = (unsigned)(valid ? r : 0) * (unsigned)pitch;
        Real* d = &ws.rows[slot][0][lane * COLS];
        cp_async<kBytes>(d, ez_l + ro, valid);
        cp_async<kBytes>(d + P, hx_l + ro, valid);
        cp_async<kBytes>(d + 2 * P, hy_l + ro, valid);
        cp_async<kBytes>(d + 3 * P, jp_l + ro, valid && jcols && r >= jy0 && r <= jy1);
        if (lane <= P / 4)
            cp_async<4>(&ws.mats[slot][4 * lane], mat_l + (unsigned)(valid ? r : 0) * (unsigned)mpitch, valid);
        if (wxs) {
#pragma unroll
            for (int c = 0; c < COLS; ++c) {
                const int x = xcol[c];
                const bool hv = valid && ixh[c] >= 0 && r < ny;
                const bool ev = valid && ixe[c] >= 0 && r >= 1 && r <= ny - 1;
                const int xh = (x < nc) ? x : x - (nx - nc) + nc;
                const int xe = (x <= nc) ? x - 1 : x - (nx - nc) + nc;
                cp_async<sizeof(Real)>(&ws.psring[slot][psi_slot<COLS>(0)][lane * COLS + c],
                                       psi_src + (hv ? psx_h + (size_t)r * 2 * nc + xh : 0), hv);
                cp_async<sizeof(Real)>(&ws.psring[slot][psi_slot<COLS>(1)][lane * COLS + c],
                                       psi_src + (ev ? psx_e + (size_t)r * 2 * nc + xe : 0), ev);
            }
        }
        if (valid && (r <= nc || r >= ny - nc)) {
            const int yh = (r < nc) ? r : ((r >= ny - nc && r < ny) ? r - (ny - nc) + nc : -1);
            const int ye = (r >= 1 && r <= nc) ? r - 1 : ((r >= ny - nc && r <= ny - 1) ? r - (ny - nc) + nc : -1);
#pragma unroll
            for (int c = 0; c < COLS; ++c) {
                const int x = xcol[c];
                const bool hv = yh >= 0 && x >= 0 && x < nx;
                const bool ev = ye >= 0 && x >= 1 && x <= nx - 1;
                cp_async<sizeof(Real)>(&ws.psring[slot][psi_slot<COLS>(2)][lane * COLS + c],
                                       psi_src + (hv ? psy_h + (size_t)yh * (nx + 1) + x : 0), hv);
                cp_async<sizeof(Real)>(&ws.psring[slot][psi_slot<COLS>(3)][lane * COLS + c],
                                       psi_src + (ev ? psy_e + (size_t)ye * (nx + 1) + x : 0), ev);
            }
        }
        cp_async_commit();
    };
    const int rstart = sweep_r0, rmax = sweep_r1;
#pragma unroll 1
    for (int r = rstart; r < rstart + kPrefetch; ++r) issue_row(r);

    for (int r = rstart; r <= rmax; ++r) {
        // ---- level 0 input: row r from the ring; request row r + kPrefetch
        cp_async_wait<kPrefetch - 1>();
        __syncwarp();
        Real lz[COLS], lx[COLS], ly[COLS], lj[COLS];
        uint32_t lm = 0u;
        {
            const int slot = r & (kRowSlots - 1);
            const Real* sp = &ws.rows[slot][0][lane * COLS];
#pragma unroll
            for (int c = 0; c < COLS; ++c) {
                lz[c] = sp[c];
                lx[c] = sp[P + c];
                ly[c] = sp[2 * P + c];
                lj[c] = sp[3 * P + c];
                lm |= (uint32_t)ws.mats[slot][moff + lane * COLS + c] << (8 * c);
            }
        }

        // ---- every level on an interior row (the common case): one straight-line
        // block over all T levels, so the scheduler can interleave their
        // independent dependency chains; the formulas are the fast path's
        const bool straight = (ws.iterbits[r >> 5] >> (r & 31)) & 1u;
        const bool interior = !wspecial && straight;
        // the same for the narrow edge strips (breast mode): every level on the edge
        // path, off the y-CPML rows and inside the vertical NTFF faces' row range
        const bool edge_rows = kEdgePath && wspecial && straight;
        if (interior) {
#pragma unroll
            for (int k = T - 1; k >= 0; --k) {
                const int m = r - 2 * k - 1;
                Real iz[COLS], ix[COLS], iy[COLS], ij[COLS];
                const uint32_t im = (k == 0) ? lm : hmat[k];
#pragma unroll
                for (int c = 0; c < COLS; ++c) {
                    if (k == 0) { iz[c] = lz[c]; ix[c] = lx[c]; iy[c] = ly[c]; ij[c] = lj[c]; }
                    else { iz[c] = hz[k][c]; ix[c] = hxr[k][c]; iy[c] = hyr[k][c]; ij[c] = hj[k][c]; }
                }
                Real oz[COLS], ox[COLS], oy[COLS], oj[COLS];
                const Real ezR_last = __shfl_down_sync(0xffffffffu, pz[k][0], 1);
#pragma unroll
                for (int c = 0; c < COLS; ++c) {
                    const Real ez0 = pz[k][c];
                    const Real ezR = (c + 1 < COLS) ? pz[k][c + 1] : ezR_last;
                    oy[c] = O::fma(chez, O::sub(ezR, ez0), py_[k][c]);
                    ox[c] = O::fma(-chez, O::sub(iz[c], ez0), px_[k][c]);
                    if (clampnan) {
                        if (dev_isnan(ox[c])) ox[c] = Real(0);
                        if (dev_isnan(oy[c])) oy[c] = Real(0);
                    }
                }
                const Real hyL_first = __shfl_up_sync(0xffffffffu, oy[COLS - 1], 1);
#pragma unroll
                for (int c = 0; c < COLS; ++c) {
                    const int mi = (pmat[k] >> (8 * c)) & kMatMask;
                    Real Ca, Cb, Cj, Bp;
                    load_coefs(ws.tab[mi], Ca, Cb, Cj, Bp);
                    const Real hyL = (c > 0) ? oy[c - 1] : hyL_first;
                    const Real dHy = O::sub(oy[c], hyL);
                    const Real dHx = O::sub(ox[c], hxn[k][c]);
                    const Real ez = pz[k][c], jp = pj[k][c];
                    Real out;
                    if (kRef) out = O::fma(Ca, ez, O::sub(O::mul(Cb, dHy), O::mul(Cb, dHx)));
                    else out = O::fma(Ca, ez, O::mul(Cb, O::sub(dHy, dHx)));
                    out = O::fma(-Cj, jp, out);
                    oj[c] = O::fma(Kp, jp, O::mul(Bp, O::sub(out, ez)));
                    if (clampnan && dev_isnan(out)) out = Real(0);
                    oz[c] = out;
                }
#pragma unroll
                for (int c = 0; c < COLS; ++c) {
                    hxn[k][c] = ox[c];
                    ezn[k][c] = oz[c];
                }
                if (k + 1 < T) {
                    hmat[k + 1] = pmat[k];
#pragma unroll
                    for (int c = 0; c < COLS; ++c) {
                        hz[k + 1][c] = oz[c]; hxr[k + 1][c] = ox[c]; hyr[k + 1][c] = oy[c]; hj[k + 1][c] = oj[c];
                    }
                } else if (m >= y0 && m < y1) {   // owned rows only
                    const long long rowoff = (long long)m * pitch;
                    const bool jrow = m >= jy0 && m <= jy1;
                    if constexpr (COLS == 2 && T % 2 == 0) {
                        // both columns of a lane are owned or neither (the strip's
                        // window starts on an even column and T is even): one
                        // 2-element store per field, aligned since xs is even
                        if (owned[0]) {
                            store_pair(ez_d + rowoff + xcol[0], oz);
                            store_pair(hx_d + rowoff + xcol[0], ox);
                            store_pair(hy_d + rowoff + xcol[0], oy);
                            if (jrow && xcol[1] >= jx0 && xcol[0] <= jx1) {
                                if (xcol[0] >= jx0) __stcg(jp_d + rowoff + xcol[0], oj[0]);
                                if (xcol[1] <= jx1) __stcg(jp_d + rowoff + xcol[1], oj[1]);
                            }
                        }
                    } else if constexpr (COLS == 4) {
                        // a lane's four columns start on a multiple of 4 (16-byte aligned):
                        // one store per field where all four are owned, else per column
                        if (owned[0] && owned[3]) {
                            store_quad(ez_d + rowoff + xcol[0], oz);
                            store_quad(hx_d + rowoff + xcol[0], ox);
                            store_quad(hy_d + rowoff + xcol[0], oy);
                        } else {
#pragma unroll
                            for (int c = 0; c < COLS; ++c)
                                if (owned[c]) {
                                    __stcg(ez_d + rowoff + xcol[c], oz[c]);
                                    __stcg(hx_d + rowoff + xcol[c], ox[c]);
                                    __stcg(hy_d + rowoff + xcol[c], oy[c]);
                                }
                        }
                        if (jrow) {
#pragma unroll
                            for (int c = 0; c < COLS; ++c)
                                if (owned[c] && xcol[c] >= jx0 && xcol[c] <= jx1) __stcg(jp_d + rowoff + xcol[c], oj[c]);
                        }
                    } else {
#pragma unroll
                        for (int c = 0; c < COLS; ++c) {
                            if (owned[c]) {
                                const int x = xcol[c];
                                __stcg(ez_d + rowoff + x, oz[c]);
                                __stcg(hx_d + rowoff + x, ox[c]);
                                __stcg(hy_d + rowoff + x, oy[c]);
                                if (jrow && x >= jx0 && x <= jx1) __stcg(jp_d + rowoff + x, oj[c]);
                            }
                        }
                    }
                }
                pmat[k] = im;
#pragma unroll
                for (int c = 0; c < COLS; ++c) {
                    pz[k][c] = iz[c]; px_[k][c] = ix[c]; py_[k][c] = iy[c]; pj[k][c] = ij[c];
                }
            }
        } else if (edge_rows) {
#pragma unroll
            for (int k = T - 1; k >= 0; --k) {
                const int m = r - 2 * k - 1;
                Real iz[COLS], ix[COLS], iy[COLS], ij[COLS];
                const uint32_t im = (k == 0) ? lm : hmat[k];
#pragma unroll
                for (int c = 0; c < COLS; ++c) {
                    if (k == 0) { iz[c] = lz[c]; ix[c] = lx[c]; iy[c] = ly[c]; ij[c] = lj[c]; }
                    else { iz[c] = hz[k][c]; ix[c] = hxr[k][c]; iy[c] = hyr[k][c]; ij[c] = hj[k][c]; }
                }
                Real oz[COLS], ox[COLS], oy[COLS], oj[COLS];
                const Real ezR_last = __shfl_down_sync(0xffffffffu, pz[k][0], 1);
#pragma unroll
                for (int c = 0; c < COLS; ++c) {
                    const int x = xcol[c];
                    const bool hin = x >= 0 && x < nx;
                    const bool isx = ixh[c] >= 0;
                    const int i = isx ? ixh[c] : 0;
                    const Real ez0 = pz[k][c];
                    const Real ezR = (c + 1 < COLS) ? pz[k][c + 1] : ezR_last;
                    const Real hx0 = px_[k][c], hy0 = py_[k][c];
                    const Real dEy = O::sub(ezR, ez0);
                    const Real dEx = O::sub(iz[c], ez0);
                    const Real hy = O::fma(chez, dEy, hy0);
                    const Real hx = O::fma(-chez, dEx, hx0);
                    const Real psx = O::fma(xprof(4, c, i), psi_in(k, 0, m, c), O::mul(xprof(5, c, i), dEy));
                    Real hyc = O::fma(O::mul(chez, dEy), xprof(3, c, i), hy0);
                    hyc = O::fma(O::mul(chez, dxr), psx, hyc);
                    if (isx) {
                        const int xsx = (x < nc) ? x : x - (nx - nc) + nc;
                        psi_out(k, 0, m, c, psx, psx_h + (size_t)m * 2 * nc + xsx);
                    }
                    ox[c] = hin ? hx : hx0;
                    oy[c] = hin ? (isx ? hyc : hy) : hy0;
                }
                const Real hyL_first = __shfl_up_sync(0xffffffffu, oy[COLS - 1], 1);
#pragma unroll
                for (int c = 0; c < COLS; ++c) {
                    const int x = xcol[c];
                    const bool ein = x >= 1 && x <= nx - 1;
                    const bool isx = ixe[c] >= 0;
                    const int i = isx ? ixe[c] : 0;
                    const int mi = (pmat[k] >> (8 * c)) & kMatMask;
                    Real Ca, Cb, Cj, Bp;
                    load_coefs(ws.tab[mi], Ca, Cb, Cj, Bp);
                    const Real hyL = (c > 0) ? oy[c - 1] : hyL_first;
                    const Real dHy = O::sub(oy[c], hyL);
                    const Real dHx = O::sub(ox[c], hxn[k][c]);
                    const Real ez = pz[k][c], jp = pj[k][c];
                    const Real qxc = O::fma(xprof(1, c, i), psi_in(k, 1, m, c), O::mul(xprof(2, c, i), dHy));
                    if (isx) {
                        const int xsx = (x <= nc) ? x - 1 : x - (nx - nc) + nc;
                        psi_out(k, 1, m, c, qxc, psx_e + (size_t)m * 2 * nc + xsx);
                    }
                    const Real cxc = O::mul(dHy, xprof(0, c, i));
                    const Real outc = O::fma(Ca, ez, O::mul(Cb, O::fma(dxr, O::sub(qxc, Real(0)), O::sub(cxc, dHx))));
                    const Real outp = O::fma(Ca, ez, O::mul(Cb, O::sub(dHy, dHx)));
                    Real out = isx ? outc : outp;
                    out = O::fma(-Cj, jp, out);
                    const Real jpo = O::fma(Kp, jp, O::mul(Bp, O::sub(out, ez)));
                    oz[c] = ein ? out : Real(0);
                    oj[c] = ein ? jpo : jp;
                }
                if (has_face0 || has_face1) {
                    const Real ezR2_last = __shfl_down_sync(0xffffffffu, oz[0], 1);
#pragma unroll
                    for (int c = 0; c < COLS; ++c) {
                        const Real ezR2 = (c + 1 < COLS) ? oz[c + 1] : ezR2_last;
                        stage_vertical(k, m, c, oy[c], O::mul(O::add(oz[c], ezR2), Real(0.5)));
                    }
                }
#pragma unroll
                for (int c = 0; c < COLS; ++c) {
                    hxn[k][c] = ox[c];
                    ezn[k][c] = oz[c];
                }
                if (k + 1 < T) {
                    hmat[k + 1] = pmat[k];
#pragma unroll
                    for (int c = 0; c < COLS; ++c) {
                        hz[k + 1][c] = oz[c]; hxr[k + 1][c] = ox[c]; hyr[k + 1][c] = oy[c]; hj[k + 1][c] = oj[c];
                    }
                } else if (m >= y0 && m < y1) {   // owned rows only
                    const long long rowoff = (long long)m * pitch;
                    const bool jrow = m >= jy0 && m <= jy1;
#pragma unroll
                    for (int c = 0; c < COLS; ++c) {
                        if (owned[c]) {
                            const int x = xcol[c];
                            __stcg(ez_d + rowoff + x, oz[c]);
                            __stcg(hx_d + rowoff + x, ox[c]);
                            __stcg(hy_d + rowoff + x, oy[c]);
                            if (jrow && x >= jx0 && x <= jx1) __stcg(jp_d + rowoff + x, oj[c]);
                        }
                    }
                }
                pmat[k] = im;
#pragma unroll
                for (int c = 0; c < COLS; ++c) {
                    pz[k][c] = iz[c]; px_[k][c] = ix[c]; py_[k][c] = iy[c]; pj[k][c] = ij[c];
                }
            }
        } else {
#pragma unroll
            for (int k = T - 1; k >= 0; --k) {
                const int q = r - 2 * k;       // row received this iteration
                const int m = q - 1;           // row advanced this iteration
                Real iz[COLS], ix[COLS], iy[COLS], ij[COLS];
                const uint32_t im = (k == 0) ? lm : hmat[k];
#pragma unroll
                for (int c = 0; c < COLS; ++c) {
                    if (k == 0) { iz[c] = lz[c]; ix[c] = lx[c]; iy[c] = ly[c]; ij[c] = lj[c]; }
                    else { iz[c] = hz[k][c]; ix[c] = hxr[k][c]; iy[c] = hyr[k][c]; ij[c] = hj[k][c]; }
                }
                if (q < 0 || m > ny) continue;   // level idle (uniform)
                if (m >= 0) {
                    Real oz[COLS], ox[COLS], oy[COLS], oj[COLS];
                    const int n = n0 + k;        // time step index computed by this level
                    const bool rowbit = (rowbits[m >> 5] >> (m & 31)) & 1u;
                    const bool fast = !wspecial && !rowbit;
                    if (k < nsteps && fast) {
                        // ================= fast path: interior Yee + Debye; in breast mode
                        // also the rows of the y-CPML strips (row-uniform psi terms, the
                        // general path's formulas; rows 0 and ny stay on the general path)
                        const int iyh = kRef ? -1 : ((m < nc) ? nc - 1 - m : ((m >= ny - nc) ? m - ny + nc : -1));
                        const int iye = kRef ? -1 : ((m <= nc) ? nc - m : ((m >= ny - nc) ? m - ny + nc : -1));
                        const Real ezR_last = __shfl_down_sync(0xffffffffu, pz[k][0], 1);
#pragma unroll
                        for (int c = 0; c < COLS; ++c) {
                            const Real ez0 = pz[k][c];
                            const Real ezR = (c + 1 < COLS) ? pz[k][c + 1] : ezR_last;
                            oy[c] = O::fma(chez, O::sub(ezR, ez0), py_[k][c]);
                            const Real dEx = O::sub(iz[c], ez0);
                            ox[c] = O::fma(-chez, dEx, px_[k][c]);
                            if (iyh >= 0) {
                                const int ysx = (m < nc) ? m : m - (ny - nc) + nc;
                                const Real ps = O::fma(cpml[4 * nc + iyh], psi_in(k, 2, m, c), O::mul(cpml[5 * nc + iyh], dEx));
                                psi_out(k, 2, m, c, ps, psy_h + (size_t)ysx * (nx + 1) + xcol[c]);
                                ox[c] = O::fma(-O::mul(chez, dEx), cpml[3 * nc + iyh], px_[k][c]);
                                ox[c] = O::fma(-O::mul(chez, dxr), ps, ox[c]);
                            }
                            if (clampnan) {
                                if (dev_isnan(ox[c])) ox[c] = Real(0);
                                if (dev_isnan(oy[c])) oy[c] = Real(0);
                            }
                        }
                        const Real hyL_first = __shfl_up_sync(0xffffffffu, oy[COLS - 1], 1);
#pragma unroll
                        for (int c = 0; c < COLS; ++c) {
                            const int mi = (pmat[k] >> (8 * c)) & kMatMask;
                            Real Ca, Cb, Cj, Bp;
                            load_coefs(ws.tab[mi], Ca, Cb, Cj, Bp);
                            const Real hyL = (c > 0) ? oy[c - 1] : hyL_first;
                            const Real dHy = O::sub(oy[c], hyL);
                            const Real dHx = O::sub(ox[c], hxn[k][c]);
                            const Real ez = pz[k][c], jp = pj[k][c];
                            Real out;
                            if (kRef) {
                                out = O::fma(Ca, ez, O::sub(O::mul(Cb, dHy), O::mul(Cb, dHx)));
                            } else if (iye >= 0) {
                                const int ysx = (m <= nc) ? m - 1 : m - (ny - nc) + nc;
                                const Real qy = O::fma(cpml[nc + iye], psi_in(k, 3, m, c), O::mul(cpml[2 * nc + iye], dHx));
                                psi_out(k, 3, m, c, qy, psy_e + (size_t)ysx * (nx + 1) + xcol[c]);
                                const Real cy = O::mul(dHx, cpml[iye]);
                                out = O::fma(Ca, ez, O::mul(Cb, O::fma(dxr, O::sub(Real(0), qy), O::sub(dHy, cy))));
                            } else {
                                out = O::fma(Ca, ez, O::mul(Cb, O::sub(dHy, dHx)));
                            }
                            out = O::fma(-Cj, jp, out);
                            oj[c] = O::fma(Kp, jp, O::mul(Bp, O::sub(out, ez)));
                            if (clampnan && dev_isnan(out)) out = Real(0);
                            oz[c] = out;
                        }
                    } else if (kEdgePath && k < nsteps && !rowbit) {
                        // ================= edge path (breast mode, narrow strips at the left
                        // and right edges): the fast path's straight-line code with the
                        // x-CPML terms computed branch-free on every lane and chosen per lane
                        // by select, row-uniform y-CPML terms, and the PEC boundary and the
                        // padding columns held by select.  Each value is chosen from the same
                        // explicitly rounded formulas the general path evaluates, so every
                        // cell gets the same bits.  (Values computed for lanes that do not
                        // select them may come from stale shared memory; they are discarded.)
                        const int iyh = (m < nc) ? nc - 1 - m : ((m >= ny - nc) ? m - ny + nc : -1);
                        const int iye = (m <= nc) ? nc - m : ((m >= ny - nc) ? m - ny + nc : -1);
                        const Real ezR_last = __shfl_down_sync(0xffffffffu, pz[k][0], 1);
#pragma unroll
                        for (int c = 0; c < COLS; ++c) {
                            const int x = xcol[c];
                            const bool hin = x >= 0 && x < nx;
                            const bool isx = ixh[c] >= 0;
                            const int i = isx ? ixh[c] : 0;
                            const Real ez0 = pz[k][c];
                            const Real ezR = (c + 1 < COLS) ? pz[k][c + 1] : ezR_last;
                            const Real hx0 = px_[k][c], hy0 = py_[k][c];
                            const Real dEy = O::sub(ezR, ez0);
                            const Real dEx = O::sub(iz[c], ez0);
                            Real hy = O::fma(chez, dEy, hy0);
                            Real hx = O::fma(-chez, dEx, hx0);
                            const Real psx = O::fma(xprof(4, c, i), psi_in(k, 0, m, c), O::mul(xprof(5, c, i), dEy));
                            Real hyc = O::fma(O::mul(chez, dEy), xprof(3, c, i), hy0);
                            hyc = O::fma(O::mul(chez, dxr), psx, hyc);
                            if (isx) {
                                const int xsx = (x < nc) ? x : x - (nx - nc) + nc;
                                psi_out(k, 0, m, c, psx, psx_h + (size_t)m * 2 * nc + xsx);
                            }
                            hy = isx ? hyc : hy;
                            if (iyh >= 0) {
                                const int ysx = (m < nc) ? m : m - (ny - nc) + nc;
                                const Real ps = O::fma(cpml[4 * nc + iyh], psi_in(k, 2, m, c), O::mul(cpml[5 * nc + iyh], dEx));
                                if (hin) psi_out(k, 2, m, c, ps, psy_h + (size_t)ysx * (nx + 1) + x);
                                hx = O::fma(-O::mul(chez, dEx), cpml[3 * nc + iyh], hx0);
                                hx = O::fma(-O::mul(chez, dxr), ps, hx);
                            }
                            ox[c] = hin ? hx : hx0;
                            oy[c] = hin ? hy : hy0;
                        }
                        const Real hyL_first = __shfl_up_sync(0xffffffffu, oy[COLS - 1], 1);
#pragma unroll
                        for (int c = 0; c < COLS; ++c) {
                            const int x = xcol[c];
                            const bool ein = x >= 1 && x <= nx - 1;
                            const bool isx = ixe[c] >= 0;
                            const int i = isx ? ixe[c] : 0;
                            const int mi = (pmat[k] >> (8 * c)) & kMatMask;
                            Real Ca, Cb, Cj, Bp;
                            load_coefs(ws.tab[mi], Ca, Cb, Cj, Bp);
                            const Real hyL = (c > 0) ? oy[c - 1] : hyL_first;
                            const Real dHy = O::sub(oy[c], hyL);
                            const Real dHx = O::sub(ox[c], hxn[k][c]);
                            const Real ez = pz[k][c], jp = pj[k][c];
                            const Real qxc = O::fma(xprof(1, c, i), psi_in(k, 1, m, c), O::mul(xprof(2, c, i), dHy));
                            if (isx) {
                                const int xsx = (x <= nc) ? x - 1 : x - (nx - nc) + nc;
                                psi_out(k, 1, m, c, qxc, psx_e + (size_t)m * 2 * nc + xsx);
                            }
                            const Real cxc = O::mul(dHy, xprof(0, c, i));
                            const Real qx = isx ? qxc : Real(0);
                            const Real cx = isx ? cxc : dHy;
                            Real qy = Real(0), cy = dHx;
                            if (iye >= 0) {
                                const int ysx = (m <= nc) ? m - 1 : m - (ny - nc) + nc;
                                qy = O::fma(cpml[nc + iye], psi_in(k, 3, m, c), O::mul(cpml[2 * nc + iye], dHx));
                                if (ein) psi_out(k, 3, m, c, qy, psy_e + (size_t)ysx * (nx + 1) + x);
                                cy = O::mul(dHx, cpml[iye]);
                            }
                            const Real outc = O::fma(Ca, ez, O::mul(Cb, O::fma(dxr, O::sub(qx, qy), O::sub(cx, cy))));
                            const Real outp = O::fma(Ca, ez, O::mul(Cb, O::sub(dHy, dHx)));
                            Real out = (isx || iye >= 0) ? outc : outp;
                            out = O::fma(-Cj, jp, out);
                            const Real jpo = O::fma(Kp, jp, O::mul(Bp, O::sub(out, ez)));
                            oz[c] = ein ? out : Real(0);
                            oj[c] = ein ? jpo : jp;
                        }
                        // vertical NTFF faces: stage this level's (h, e) samples
                        if (nfreq > 0 && (has_face0 || has_face1) && m >= fd && m <= ny - fd - 1) {
                            const Real ezR2_last = __shfl_down_sync(0xffffffffu, oz[0], 1);
#pragma unroll
                            for (int c = 0; c < COLS; ++c) {
                                const Real ezR2 = (c + 1 < COLS) ? oz[c + 1] : ezR2_last;
                                stage_vertical(k, m, c, oy[c], O::mul(O::add(oz[c], ezR2), Real(0.5)));
                            }
                        }
                    } else if (k < nsteps) {
                        // ================= general path
                        const bool hrow = m < ny;
                        const int iyh = (m < nc) ? nc - 1 - m : ((m >= ny - nc && m < ny) ? m - ny + nc : -1);
                        Real ezR_last = __shfl_down_sync(0xffffffffu, pz[k][0], 1);
#pragma unroll
                        for (int c = 0; c < COLS; ++c) {
                            const int x = xcol[c];
                            Real ez0 = pz[k][c];
                            Real ezR = (c + 1 < COLS) ? pz[k][c + 1] : ezR_last;
                            Real hx0 = px_[k][c], hy0 = py_[k][c];
                            Real hx = hx0, hy = hy0;
                            if (hrow && x >= 0 && x < nx) {
                                Real dEy = O::sub(ezR, ez0);
                                Real dEx = O::sub(iz[c], ez0);
                                hy = O::fma(chez, dEy, hy0);
                                hx = O::fma(-chez, dEx, hx0);
                                if (ixh[c] >= 0) {
                                    const int i = ixh[c];
                                    const int xsx = (x < nc) ? x : x - (nx - nc) + nc;
                                    Real ps = O::fma(xprof(4, c, i), psi_in(k, 0, m, c), O::mul(xprof(5, c, i), dEy));
                                    psi_out(k, 0, m, c, ps, psx_h + (size_t)m * 2 * nc + xsx);
                                    hy = O::fma(O::mul(chez, dEy), xprof(3, c, i), hy0);
                                    hy = O::fma(O::mul(chez, dxr), ps, hy);
                                }
                                if (iyh >= 0) {
                                    const int ysx = (m < nc) ? m : m - (ny - nc) + nc;
                                    Real ps = O::fma(cpml[4 * nc + iyh], psi_in(k, 2, m, c), O::mul(cpml[5 * nc + iyh], dEx));
                                    psi_out(k, 2, m, c, ps, psy_h + (size_t)ysx * (nx + 1) + x);
                                    hx = O::fma(-O::mul(chez, dEx), cpml[3 * nc + iyh], hx0);
                                    hx = O::fma(-O::mul(chez, dxr), ps, hx);
                                }
                                if (clampnan) {
                                    if (dev_isnan(hx)) hx = Real(0);
                                    if (dev_isnan(hy)) hy = Real(0);
                                }
                            }
                            ox[c] = hx;
                            oy[c] = hy;
                        }
                        Real hyL_first = __shfl_up_sync(0xffffffffu, oy[COLS - 1], 1);
                        const bool erow = m >= 1 && m <= ny - 1;
                        const int iye = (m >= 1 && m <= nc) ? nc - m : ((m >= ny - nc && m <= ny - 1) ? m - ny + nc : -1);
#pragma unroll
                        for (int c = 0; c < COLS; ++c) {
                            const int x = xcol[c];
                            Real ez = pz[k][c];
                            Real jp = pj[k][c];
                            Real out = Real(0);
                            Real jpo = jp;
                            if (erow && x >= 1 && x <= nx - 1) {
                                const uint32_t mb = (pmat[k] >> (8 * c)) & 0xffu;
                                const int mi = mb & kMatMask;
                                const Real* cf = D.mtab + mi * kMatCoef;     // cold columns (global, cached)
                                Real Ca, Cb, Cj, Bp;
                                load_coefs(ws.tab[mi], Ca, Cb, Cj, Bp);
                                Real hyL = (c > 0) ? oy[c - 1] : hyL_first;
                                Real dHy = O::sub(oy[c], hyL);
                                Real dHx = O::sub(ox[c], hxn[k][c]);
                                Real gp = Real(0), gm = Real(0);
                                if (kRef) {
                                    const Real Ci = cf[kCi], Cp = cf[kCp];
                                    if (Ci != Real(0) || Cp != Real(0) || Bp != Real(0)) {
                                        // fwf() argument in FP64 (FDTD_GPU.cu:290): time minus the
                                        // projected travel time of the incident front to this cell
                                        const double b = __dmul_rn(__dadd_rn(__dmul_rn(D.pw_ky, (double)m - D.pw_yoff),
                                                                             __dmul_rn(D.pw_kx, (double)x - D.pw_xoff)),
                                                                   D.pw_dxc0);
                                        const double a0 = __dsub_rn(__dsub_rn(__dmul_rn((double)n + 0.5, D.dt), D.pw_t0l), b);
                                        const double a1 = __dsub_rn(__dsub_rn(__dmul_rn((double)n - 0.5, D.dt), D.pw_t0l), b);
                                        Real u0 = (Real)__dmul_rn(a0, D.pw_inv_tau), u1 = (Real)__dmul_rn(a1, D.pw_inv_tau);
                                        gp = dev_exp<Real>(-O::mul(u0, u0));
                                        gm = dev_exp<Real>(-O::mul(u1, u1));
                                    }
                                    // FDTD_GPU.cu:378-385 (interior), then the strip overrides :389-416
                                    out = O::fma(Ca, ez, O::sub(O::mul(Cb, dHy), O::mul(Cb, dHx)));
                                    out = O::fma(cf[kCi], gp, O::fma(cf[kCp], gm, out));
                                    out = O::fma(-Cj, jp, out);
                                    // total-field incident grid: the legacy centre source, added
                                    // before the strip overrides (oldFDTD_GPU.cu:680-683)
                                    if (psrc && m == src_y && x == src_x) out = O::fma(cf[kCs], D.src_wave[n], out);
                                    jpo = O::fma(Kp, jp, O::mul(Bp, O::add(O::sub(out, ez), O::sub(gp, gm))));
                                    if (ixe[c] >= 0) {
                                        const int i = ixe[c];
                                        const int xsx = (x <= nc) ? x - 1 : x - (nx - nc) + nc;
                                        Real ps = O::fma(xprof(1, c, i), psi_in(k, 1, m, c), O::mul(xprof(2, c, i), dHy));
                                        psi_out(k, 1, m, c, ps, psx_e + (size_t)m * 2 * nc + xsx);
                                        const Real rk = xprof(0, c, i);
                                        out = O::fma(Ca, ez, O::mul(O::mul(Cb, O::sub(dHy, dHx)), rk));
                                        out = O::fma(O::mul(Cb, dxr), ps, out);
                                    }
                                    if (iye >= 0) {
                                        const int ysx = (m <= nc) ? m - 1 : m - (ny - nc) + nc;
                                        Real ps = O::fma(cpml[nc + iye], psi_in(k, 3, m, c), O::mul(cpml[2 * nc + iye], dHx));
                                        psi_out(k, 3, m, c, ps, psy_e + (size_t)ysx * (nx + 1) + x);
                                        const Real rk = cpml[iye];
                                        out = O::fma(Ca, ez, O::mul(O::mul(Cb, O::sub(dHy, dHx)), rk));
                                        out = O::fma(-O::mul(Cb, dxr), ps, out);
                                    }
                                } else {
                                    Real cx = dHy, cy = dHx, qx = Real(0), qy = Real(0);
                                    if (ixe[c] >= 0) {
                                        const int i = ixe[c];
                                        const int xsx = (x <= nc) ? x - 1 : x - (nx - nc) + nc;
                                        qx = O::fma(xprof(1, c, i), psi_in(k, 1, m, c), O::mul(xprof(2, c, i), dHy));
                                        psi_out(k, 1, m, c, qx, psx_e + (size_t)m * 2 * nc + xsx);
                                        cx = O::mul(dHy, xprof(0, c, i));
                                    }
                                    if (iye >= 0) {
                                        const int ysx = (m <= nc) ? m - 1 : m - (ny - nc) + nc;
                                        qy = O::fma(cpml[nc + iye], psi_in(k, 3, m, c), O::mul(cpml[2 * nc + iye], dHx));
                                        psi_out(k, 3, m, c, qy, psy_e + (size_t)ysx * (nx + 1) + x);
                                        cy = O::mul(dHx, cpml[iye]);
                                    }
                                    // proper CPML: both stretched derivatives and both psi terms
                                    if (ixe[c] >= 0 || iye >= 0)
                                        out = O::fma(Ca, ez, O::mul(Cb, O::fma(dxr, O::sub(qx, qy), O::sub(cx, cy))));
                                    else
                                        out = O::fma(Ca, ez, O::mul(Cb, O::sub(dHy, dHx)));
                                    out = O::fma(-Cj, jp, out);
                                    if (psrc && m == src_y && x == src_x) out = O::fma(cf[kCs], D.src_wave[n], out);
                                    jpo = O::fma(Kp, jp, O::mul(Bp, O::sub(out, ez)));
                                }
                                if (clampnan && dev_isnan(out)) out = Real(0);
                                // receivers (owned cells only, so each sample is written once)
                                if ((mb & kMatRx) && owned[c] && m >= y0 && m < y1) {
                                    for (int rr = 0; rr < D.nrx; ++rr)
                                        if (D.rx[2 * rr] == x && D.rx[2 * rr + 1] == m)
                                            D.traces[(size_t)rr * S + n] = out;
                                }
                            }
                            oz[c] = out;
                            oj[c] = jpo;
                        }
                        // NTFF contour samples of this level, summed by the DFT kernel
                        if (nfreq > 0) {
                            // horizontal faces: face row m-1 is complete at this level
                            if ((m - 1 == fd || m - 1 == ny - fd - 1) && m - 1 >= y0 && m - 1 < y1) {
                                const bool yp = (m - 1 == ny - fd - 1);
#pragma unroll
                                for (int c = 0; c < COLS; ++c) {
                                    const int x = xcol[c];
                                    if (owned[c] && x >= fd + 1 && x <= nx - fd - 2) {
                                        Real e = O::mul(O::add(ezn[k][c], oz[c]), Real(0.5));
                                        Real h = hxn[k][c];
                                        int ci = yp ? contour_index_yp(nx, ny, fd, x) : contour_index_yn(nx, ny, fd, x);
                                        if (yp) { e = -e; h = -h; }
                                        Real* sp = stage + ((size_t)k * C + ci) * 2;
                                        sp[0] = h;
                                        sp[1] = e;
                                    }
                                }
                            }
                            // vertical faces
                            if ((has_face0 || has_face1) && m >= fd && m <= ny - fd - 1) {
                                const Real ezR2_last = __shfl_down_sync(0xffffffffu, oz[0], 1);
#pragma unroll
                                for (int c = 0; c < COLS; ++c) {
                                    const Real ezR2 = (c + 1 < COLS) ? oz[c + 1] : ezR2_last;
                                    stage_vertical(k, m, c, oy[c], O::mul(O::add(oz[c], ezR2), Real(0.5)));
                                }
                            }
                        }
                    } else {
                        // beyond the last time step: pass through unchanged (psi included)
#pragma unroll
                        for (int c = 0; c < COLS; ++c) {
                            oz[c] = pz[k][c]; ox[c] = px_[k][c]; oy[c] = py_[k][c]; oj[c] = pj[k][c];
                            const int x = xcol[c];
                            if (ixh[c] >= 0 && m < ny) {
                                const int xsx = (x < nc) ? x : x - (nx - nc) + nc;
                                psi_out(k, 0, m, c, psi_in(k, 0, m, c), psx_h + (size_t)m * 2 * nc + xsx);
                            }
                            if (ixe[c] >= 0 && m >= 1 && m <= ny - 1) {
                                const int xsx = (x <= nc) ? x - 1 : x - (nx - nc) + nc;
                                psi_out(k, 1, m, c, psi_in(k, 1, m, c), psx_e + (size_t)m * 2 * nc + xsx);
                            }
                            if (x >= 0 && x <= nx) {
                                const int iyh = (m < nc) ? m : ((m >= ny - nc && m < ny) ? m - (ny - nc) + nc : -1);
                                if (iyh >= 0 && x < nx)
                                    psi_out(k, 2, m, c, psi_in(k, 2, m, c), psy_h + (size_t)iyh * (nx + 1) + x);
                                const int iye = (m >= 1 && m <= nc) ? m - 1
                                                : ((m >= ny - nc && m <= ny - 1) ? m - (ny - nc) + nc : -1);
                                if (iye >= 0 && x >= 1 && x <= nx - 1)
                                    psi_out(k, 3, m, c, psi_in(k, 3, m, c), psy_e + (size_t)iye * (nx + 1) + x);
                            }
                        }
                    }
                    // ---- emit row m
#pragma unroll
                    for (int c = 0; c < COLS; ++c) {
                        hxn[k][c] = ox[c];
                        ezn[k][c] = oz[c];
                    }
                    if (k + 1 < T) {
                        hmat[k + 1] = pmat[k];
#pragma unroll
                        for (int c = 0; c < COLS; ++c) {
                            hz[k + 1][c] = oz[c]; hxr[k + 1][c] = ox[c]; hyr[k + 1][c] = oy[c]; hj[k + 1][c] = oj[c];
                        }
                    } else if (m >= y0 && m < y1) {   // owned rows only
                        const long long rowoff = (long long)m * pitch;
                        const bool jrow = m >= jy0 && m <= jy1;
#pragma unroll
                        for (int c = 0; c < COLS; ++c) {
                            if (owned[c]) {
                                const int x = xcol[c];
                                __stcg(ez_d + rowoff + x, oz[c]);
                                __stcg(hx_d + rowoff + x, ox[c]);
                                __stcg(hy_d + rowoff + x, oy[c]);
                                if (jrow && x >= jx0 && x <= jx1) __stcg(jp_d + rowoff + x, oj[c]);
                            }
                        }
                    }
                }
                // the received row becomes this level's previous row
                pmat[k] = im;
#pragma unroll
                for (int c = 0; c < COLS; ++c) {
                    pz[k][c] = iz[c]; px_[k][c] = ix[c]; py_[k][c] = iy[c]; pj[k][c] = ij[c];
                }
            }
        }

        // request row r + kPrefetch into the slot of row r - 1: every lane read that
        // slot's material bytes before the warp-wide sync at the top of this
        // iteration, and its own fields and psi earlier in program order
        issue_row(r + kPrefetch);
    }
    cp_async_wait<0>();   // the ring is reused by the warp's next item
    __syncwarp();
}

// Persistent kernel: warps take work items from a global counter (reset by the
// progress kernel after every launch), most expensive items first.  MINB is
// the minimum number of resident 128-thread blocks per SM requested from the
// register allocator (2: up to 255 registers per thread, 3: 168, 4: 128); the
// autotuner picks it with (T, COLS).
template <typename Real, int T, int COLS, int MODE, int MINB>
__global__ void __launch_bounds__(128, MINB) fdtd_advance_kernel(const SolveDesc<Real>* __restrict__ descs,
                                                                  const WorkItem* __restrict__ items, int nitems,
                                                                  int* __restrict__ counter) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char* const wbase = smem_raw + (threadIdx.x >> 5) * warp_smem_bytes<Real, T, COLS>();
    const int lane = threadIdx.x & 31;
    for (;;) {
        int it = 0;
        if (lane == 0) it = atomicAdd(counter, 1);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= nitems) break;
        const WorkItem wi = items[it];
        const SolveDesc<Real>* __restrict__ D = descs + wi.solve;
        if (!D->active) continue;
        if (COLS > 1 && wi.narrow)
            advance_item<Real, T, 1, MODE>(D, wi, *reinterpret_cast<WarpSmem<Real, T, 1>*>(wbase));
        else
            advance_item<Real, T, COLS, MODE>(D, wi, *reinterpret_cast<WarpSmem<Real, T, COLS>*>(wbase));
        __syncwarp();
    }
}

}  // namespace tomo
