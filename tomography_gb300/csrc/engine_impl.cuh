// Internal engine pieces shared by the batch path (engine.cu) and the
// serving loop (serve.cu): spec-derived class data, argument unpacking,
// per-range set-up / descriptor fill / post-process, and the advance launcher.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/tomography.h"
#include "aux_kernels.cuh"
#include "engine.h"
#include "fdtd_advance.cuh"
#include "solve_desc.h"

#define CUDA_TRY(expr)                                                                                      \
    do {                                                                                                    \
        cudaError_t e_ = (expr);                                                                            \
        if (e_ != cudaSuccess) return ::tomo::fail(TOMO_ECUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define TOMO_TRY(expr)            \
    do {                          \
        int rc_ = (expr);         \
        if (rc_) return rc_;      \
    } while (0)

namespace tomo {

extern const double kC0;
extern const double kEta0;

// --------------------------------------------------------------------- memory
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    int ensure(size_t n) {
        if (n <= bytes && p) return TOMO_OK;
        release();
        if (n == 0) n = 16;
        cudaError_t e = cudaMalloc(&p, n);
        if (e != cudaSuccess) {
            p = nullptr;
            cudaGetLastError();
            return fail(e == cudaErrorMemoryAllocation ? TOMO_ENOMEM_BUDGET : TOMO_ECUDA,
                        std::string("cudaMalloc(") + std::to_string(n) + "): " + cudaGetErrorString(e));
        }
        bytes = n;
        return TOMO_OK;
    }
    template <typename U>
    U* as() const { return reinterpret_cast<U*>(p); }
};

// ----------------------------------------------------------- spec-derived data
struct ProblemClass {
    tomo_spec spec;
    int nx, ny, nc, S, C, nfreq, nang, n_exc, nrx, nparam, nmat;
    int pitch, mpitch;
    double dt, chez, Kp, src_amp;
    std::vector<double> cpml;      // [6][nc]: 1/ke, be, ae, 1/km, bm, am
    std::vector<double> phasor;    // [S][nfreq][4]
    std::vector<double> wave;      // [S]
    std::vector<int> rx;           // [nrx][2]
    std::vector<uint8_t> patchmap; // reference modes, (ny+1) x mpitch
    std::vector<double> ffgeom;    // [C][3]: X, Y, face
    std::vector<double> ffang;     // [nang][2]: cos, sin
    // total-field variant: solves appended to each batch (0 or 1: the incident grid)
    int extra = 0;
    std::vector<double> inc_phasor; // [S][nfreq][4]: J at n dt, M folded over two levels
    std::vector<double> inc_wave;   // [S] incident source waveform
    std::vector<double> inc_tab;    // [kMaxMat][kMatCoef]: material 0 = vacuum + source coefficient
};

int validate_spec(const tomo_spec* s);
int build_class(const tomo_spec& s, ProblemClass& pc);
bool same_problem(const tomo_spec& a, const tomo_spec& b);

// Per-solve memory layout (elements of Real), identical for every solve of a class.
struct SolveLayout {
    size_t field_elems, psi_elems, tr_stride, acc_stride, stage_stride, per_solve, mat_stride;
};
SolveLayout solve_layout(const ProblemClass& pc, size_t real_bytes);

// Host-side unpacked arguments of a range of candidates.
struct Unpacked {
    std::vector<double> upload;   // [ncand][kMaxMat][3] then [ncand][K][6]
    std::vector<int> bbox;        // [ncand][4] dispersive box (x0, x1, y0, y1)
    size_t ncand = 0;
};
int unpack_args(const ProblemClass& pc, const double* args, size_t ncand, size_t nparam, Unpacked& u);

// Blocking of the advance kernel: time steps per launch, columns per lane, and
// the minimum resident blocks per SM its registers were allocated for.
struct Blocking {
    int T = 1, cols = 1, minb = 2;
    bool operator==(const Blocking& o) const { return T == o.T && cols == o.cols && minb == o.minb; }
    bool operator!=(const Blocking& o) const { return !(*this == o); }
};

template <typename Real>
using AdvanceFn = void (*)(const SolveDesc<Real>*, const WorkItem*, int, int*);
template <typename Real>
AdvanceFn<Real> advance_kernel_for(const Blocking& b, int mode);

inline int advance_mode(const tomo_spec& s) { return s.mode == TOMO_MODE_BREAST ? kModeBreast : kModeRef; }
template <typename Real>
size_t advance_smem_bytes(int T, int cols);

// Device copy of a ProblemClass.
template <typename Real>
struct ClassData {
    ProblemClass pc;
    SolveLayout lay{};
    DevBuf cpml, phasor, wave, rx, patch, freqs, ffgeom, ffang, target;
    DevBuf inc_phasor, inc_wave, inc_tab, inc_mat;   // total-field incident grid
    bool have_target = false;

    int init(const ProblemClass& p) {
        pc = p;
        lay = solve_layout(pc, sizeof(Real));
        std::vector<Real> t(pc.cpml.begin(), pc.cpml.end());
        TOMO_TRY(cpml.ensure(sizeof(Real) * std::max<size_t>(t.size(), 1)));
        if (!t.empty()) CUDA_TRY(cudaMemcpy(cpml.p, t.data(), sizeof(Real) * t.size(), cudaMemcpyHostToDevice));
        std::vector<Real> ph(pc.phasor.begin(), pc.phasor.end());
        TOMO_TRY(phasor.ensure(sizeof(Real) * std::max<size_t>(ph.size(), 4)));
        if (!ph.empty()) CUDA_TRY(cudaMemcpy(phasor.p, ph.data(), sizeof(Real) * ph.size(), cudaMemcpyHostToDevice));
        std::vector<Real> wv(pc.wave.begin(), pc.wave.end());
        TOMO_TRY(wave.ensure(sizeof(Real) * wv.size()));
        CUDA_TRY(cudaMemcpy(wave.p, wv.data(), sizeof(Real) * wv.size(), cudaMemcpyHostToDevice));
        TOMO_TRY(rx.ensure(sizeof(int) * std::max<size_t>(pc.rx.size(), 2)));
        if (!pc.rx.empty()) CUDA_TRY(cudaMemcpy(rx.p, pc.rx.data(), sizeof(int) * pc.rx.size(), cudaMemcpyHostToDevice));
        if (!pc.patchmap.empty()) {
            TOMO_TRY(patch.ensure(pc.patchmap.size()));
            CUDA_TRY(cudaMemcpy(patch.p, pc.patchmap.data(), pc.patchmap.size(), cudaMemcpyHostToDevice));
        }
        TOMO_TRY(freqs.ensure(sizeof(double) * TOMO_MAX_FREQS));
        CUDA_TRY(cudaMemcpy(freqs.p, pc.spec.freqs, sizeof(double) * TOMO_MAX_FREQS, cudaMemcpyHostToDevice));
        if (pc.C > 0) {
            TOMO_TRY(ffgeom.ensure(sizeof(double) * pc.ffgeom.size()));
            CUDA_TRY(cudaMemcpy(ffgeom.p, pc.ffgeom.data(), sizeof(double) * pc.ffgeom.size(), cudaMemcpyHostToDevice));
        }
        if (pc.nang > 0) {
            TOMO_TRY(ffang.ensure(sizeof(double) * pc.ffang.size()));
            CUDA_TRY(cudaMemcpy(ffang.p, pc.ffang.data(), sizeof(double) * pc.ffang.size(), cudaMemcpyHostToDevice));
        }
        if (pc.extra) {
            auto upload = [](DevBuf& b, const std::vector<double>& v) -> int {
                std::vector<Real> r(v.begin(), v.end());
                TOMO_TRY(b.ensure(sizeof(Real) * std::max<size_t>(r.size(), 4)));
                if (!r.empty()) CUDA_TRY(cudaMemcpy(b.p, r.data(), sizeof(Real) * r.size(), cudaMemcpyHostToDevice));
                return TOMO_OK;
            };
            TOMO_TRY(upload(inc_phasor, pc.inc_phasor));
            TOMO_TRY(upload(inc_wave, pc.inc_wave));
            TOMO_TRY(upload(inc_tab, pc.inc_tab));
            // all-vacuum material map with the patch map's layout
            TOMO_TRY(inc_mat.ensure(pc.patchmap.size()));
            CUDA_TRY(cudaMemset(inc_mat.p, 0, pc.patchmap.size()));
        }
        return TOMO_OK;
    }

    size_t target_size() const {
        return pc.spec.mode == TOMO_MODE_BREAST ? (size_t)pc.n_exc * pc.nrx * pc.S
                                                : (size_t)pc.n_exc * pc.nfreq * pc.nang;
    }

    int set_target(const float* t, size_t n) {
        if (!t || n != target_size())
            return fail(TOMO_EINVAL, "target has " + std::to_string(n) + " values, expected " + std::to_string(target_size()));
        TOMO_TRY(target.ensure(sizeof(float) * n));
        CUDA_TRY(cudaMemcpy(target.p, t, sizeof(float) * n, cudaMemcpyHostToDevice));
        have_target = true;
        return TOMO_OK;
    }
};

// Upload unpacked arguments and build material maps and FP64-derived
// coefficient tables for `ncand` candidates.  d_upload must hold
// u.upload.size() doubles.  Returns the number of kernels launched via *kernels.
template <typename Real>
int setup_materials(const ClassData<Real>& cd, const Unpacked& u, double* d_upload, uint8_t* d_mats, Real* d_tabs,
                    cudaStream_t st, int64_t* kernels, int64_t* h2d) {
    const tomo_spec& s = cd.pc.spec;
    const size_t ncand = u.ncand;
    if (h2d) {   // upload here unless the caller already did
        CUDA_TRY(cudaMemcpyAsync(d_upload, u.upload.data(), sizeof(double) * u.upload.size(), cudaMemcpyHostToDevice, st));
        *h2d += sizeof(double) * u.upload.size();
    }
    material_table_kernel<Real><<<(int)((ncand * kMaxMat + 127) / 128), 128, 0, st>>>(d_upload, d_tabs, (int)ncand,
                                                                                     cd.pc.nmat, s.tau, s.dt, s.dx);
    ++*kernels;
    if (s.mode == TOMO_MODE_BREAST) {
        dim3 blk(32, 8), grd((s.nx + 1 + 31) / 32, (s.ny + 1 + 7) / 8, (unsigned)ncand);
        raster_ellipse_kernel<<<grd, blk, 0, st>>>(d_mats, cd.pc.mpitch, s.nx, s.ny, s.dx, s.disc_radius,
                                                   d_upload + ncand * kMaxMat * 3, s.n_ellipses, cd.lay.mat_stride);
        mark_rx_kernel<<<(int)((cd.pc.nrx * ncand + 127) / 128), 128, 0, st>>>(d_mats, cd.pc.mpitch, cd.lay.mat_stride,
                                                                              cd.rx.template as<int>(), cd.pc.nrx,
                                                                              (int)ncand);
        *kernels += 2;
    }
    CUDA_TRY(cudaGetLastError());
    return TOMO_OK;
}

// Descriptors of the ncand*n_exc solves of a range whose state starts at
// state_base (per-solve stride cd.lay.per_solve elements).
template <typename Real>
void fill_descs(const ClassData<Real>& cd, const Unpacked& u, Real* state_base, const uint8_t* mats, const Real* tabs,
                SolveDesc<Real>* out) {
    const ProblemClass& pc = cd.pc;
    const tomo_spec& s = pc.spec;
    const SolveLayout& L = cd.lay;
    const int nsolves = (int)u.ncand * pc.n_exc;
    for (int sv = 0; sv < nsolves; ++sv) {
        const int cand = sv / pc.n_exc, exc = sv % pc.n_exc;
        SolveDesc<Real> D{};
        Real* sb = state_base + (size_t)sv * L.per_solve;
        D.nx = s.nx; D.ny = s.ny; D.pitch = pc.pitch; D.mpitch = pc.mpitch;
        D.ncpml = pc.nc; D.steps_total = pc.S; D.step = 0; D.parity = 0; D.active = 1; D.nmat = pc.nmat; D.stage_group = 1;
        D.nrx = pc.nrx; D.nf_d = s.nf2ff_d; D.nfreq = pc.nfreq; D.n_contour = pc.C;
        D.chez = (Real)pc.chez; D.Kp = (Real)pc.Kp; D.dx = (Real)s.dx;
        Real* f = sb + kPadLeft;
        D.ez[0] = f + 0 * L.field_elems; D.ez[1] = f + 1 * L.field_elems;
        D.hx[0] = f + 2 * L.field_elems; D.hx[1] = f + 3 * L.field_elems;
        D.hy[0] = f + 4 * L.field_elems; D.hy[1] = f + 5 * L.field_elems;
        D.jp[0] = f + 6 * L.field_elems; D.jp[1] = f + 7 * L.field_elems;
        Real* psib = sb + 8 * L.field_elems;
        D.psi[0] = psib;
        D.psi[1] = psib + L.psi_elems;
        D.psi_scratch = psib + 2 * L.psi_elems;
        D.psi_stride = (int)L.psi_elems;
        D.traces = psib + (size_t)9 * L.psi_elems;
        D.acc = D.traces + L.tr_stride;
        D.stage = D.acc + L.acc_stride;
        D.mtab = tabs + (size_t)cand * kMaxMat * kMatCoef;
        D.cpml = cd.cpml.template as<Real>();
        D.src_wave = cd.wave.template as<Real>();
        D.rx = cd.rx.template as<int>();
        D.phasor = cd.phasor.template as<Real>();
        const int* bb = &u.bbox[cand * 4];
        D.jx0 = bb[0]; D.jx1 = bb[1]; D.jy0 = bb[2]; D.jy1 = bb[3];
        D.dt = s.dt;
        if (s.mode == TOMO_MODE_BREAST) {
            D.flags = kPointSource;
            D.mat = mats + (size_t)cand * L.mat_stride + kMatPadLeft;
            D.src_x = pc.rx[2 * exc];
            D.src_y = pc.rx[2 * exc + 1];
        } else {
            D.flags = kRefCpml | kPlaneWave | (s.nan_clamp ? kNanClamp : 0);
            D.mat = cd.patch.template as<uint8_t>() + kMatPadLeft;
            D.src_x = D.src_y = -1;
            // fwf() (FDTD_GPU.cu:283-296): the excitation angle is a float in the reference
            const float phi = (float)(exc * 2 * kPiD / s.n_excitations);
            D.pw_kx = std::cos((double)phi);
            D.pw_ky = std::sin((double)phi);
            D.pw_xoff = s.pw_centred ? (double)(s.nx / 2) : 0.0;
            D.pw_yoff = s.pw_centred ? (double)(s.ny / 2) : 0.0;
            D.pw_t0l = s.pw_t0 - s.pw_l / kC0;
            D.pw_inv_tau = 1.0 / s.pw_tau;
            D.pw_dxc0 = s.dx / kC0;
        }
        out[sv] = D;
    }
}

// Descriptor of the total-field incident grid (oldFDTD_GPU.cu:425-482, 655-717):
// a reference-mode solve over an all-vacuum map with the legacy centre source,
// its running DFT against the folded incident phasors.  `state` is one
// solve's state block (per-solve stride of the class layout).
template <typename Real>
SolveDesc<Real> incident_desc(const ClassData<Real>& cd, Real* state) {
    const ProblemClass& pc = cd.pc;
    const tomo_spec& s = pc.spec;
    const SolveLayout& L = cd.lay;
    SolveDesc<Real> D{};
    D.nx = s.nx; D.ny = s.ny; D.pitch = pc.pitch; D.mpitch = pc.mpitch;
    D.ncpml = pc.nc; D.steps_total = pc.S; D.step = 0; D.parity = 0; D.active = 1; D.nmat = 1; D.stage_group = 1;
    D.nrx = 0; D.nf_d = s.nf2ff_d; D.nfreq = pc.nfreq; D.n_contour = pc.C;
    D.chez = (Real)pc.chez; D.Kp = (Real)pc.Kp; D.dx = (Real)s.dx;
    Real* f = state + kPadLeft;
    D.ez[0] = f + 0 * L.field_elems; D.ez[1] = f + 1 * L.field_elems;
    D.hx[0] = f + 2 * L.field_elems; D.hx[1] = f + 3 * L.field_elems;
    D.hy[0] = f + 4 * L.field_elems; D.hy[1] = f + 5 * L.field_elems;
    D.jp[0] = f + 6 * L.field_elems; D.jp[1] = f + 7 * L.field_elems;
    Real* psib = state + 8 * L.field_elems;
    D.psi[0] = psib;
    D.psi[1] = psib + L.psi_elems;
    D.psi_scratch = psib + 2 * L.psi_elems;
    D.psi_stride = (int)L.psi_elems;
    D.traces = psib + (size_t)9 * L.psi_elems;
    D.acc = D.traces + L.tr_stride;
    D.stage = D.acc + L.acc_stride;
    D.mtab = cd.inc_tab.template as<Real>();
    D.cpml = cd.cpml.template as<Real>();
    D.src_wave = cd.inc_wave.template as<Real>();
    D.rx = cd.rx.template as<int>();
    D.phasor = cd.inc_phasor.template as<Real>();
    D.jx0 = 1; D.jx1 = 0; D.jy0 = 1; D.jy1 = 0;   // no Debye current anywhere
    D.dt = s.dt;
    // the legacy's H_inc_update clamps NaN as the main H update does; the
    // vacuum grid's fields stay finite, so the flag only keeps the two alike
    D.flags = kRefCpml | kPointSource | (s.nan_clamp ? kNanClamp : 0);
    D.mat = cd.inc_mat.template as<uint8_t>() + kMatPadLeft;
    D.src_x = s.nx / 2;   // oldFDTD_GPU.cu:74-75
    D.src_y = s.ny / 2;
    return D;
}

// Far field + misfit (+ optional traces to float) of a contiguous range of
// solves whose first descriptor is `first` (host copy).  d_D/d_P hold
// nsolves*nfreq*nang floats; d_fit receives ncand values.
template <typename Real>
int post_range(const ClassData<Real>& cd, size_t ncand, const SolveDesc<Real>& first, bool want_fit, float* d_D,
               float* d_P, double* d_partials, double* d_fit, int* d_flag, float* d_trf, double* d_trd, cudaStream_t st,
               int64_t* kernels, const Real* inc_acc = nullptr) {
    const ProblemClass& pc = cd.pc;
    const tomo_spec& s = pc.spec;
    const int nsolves = (int)ncand * pc.n_exc;
    const size_t stride = cd.lay.per_solve;
    if (pc.nang > 0 && pc.C > 0 && d_D) {
        dim3 grd(pc.nfreq, nsolves);
        farfield_kernel<Real><<<grd, 256, 0, st>>>(first.acc, stride, inc_acc, pc.C, pc.nfreq, cd.freqs.template as<double>(),
                                                   cd.ffgeom.template as<double>(), cd.ffang.template as<double>(),
                                                   pc.nang, s.dx, s.ff_norm, s.pw_tau,
                                                   s.mode == TOMO_MODE_BREAST ? std::sqrt(s.bg_eps_inf) : 1.0, d_D, d_P);
        ++*kernels;
    }
    if (want_fit) {
        if (s.mode == TOMO_MODE_BREAST) {
            trace_partials_kernel<Real><<<nsolves, 256, 0, st>>>(first.traces, stride, cd.target.template as<float>(),
                                                                 pc.nrx * pc.S, pc.n_exc, 0, d_partials, d_flag);
            trace_fitness_kernel<<<(int)((ncand + 127) / 128), 128, 0, st>>>(d_partials, pc.n_exc, (int)ncand, d_fit);
            *kernels += 2;
        } else {
            const int nper = pc.n_exc * pc.nfreq * pc.nang;
            ff_fitness_kernel<<<(int)ncand, 256, 0, st>>>(d_D, cd.target.template as<float>(), nper,
                                                          (double)pc.n_exc * pc.nfreq, s.misfit == 1, d_fit, d_flag);
            ++*kernels;
        }
    }
    if ((d_trf || d_trd) && pc.nrx > 0) {
        const size_t n = (size_t)pc.nrx * pc.S * nsolves;
        if (d_trf)
            traces_pack_kernel<Real, float><<<(int)((n + 255) / 256), 256, 0, st>>>(first.traces, stride, pc.nrx * pc.S,
                                                                                    nsolves, d_trf);
        if (d_trd)
            traces_pack_kernel<Real, double><<<(int)((n + 255) / 256), 256, 0, st>>>(first.traces, stride, pc.nrx * pc.S,
                                                                                     nsolves, d_trd);
        *kernels += (d_trf ? 1 : 0) + (d_trd ? 1 : 0);
    }
    CUDA_TRY(cudaGetLastError());
    return TOMO_OK;
}

// Grid size of the persistent advance kernel.
template <typename Real>
int advance_grid(const Blocking& b, int mode, int nitems, int num_sms, int* blocks, size_t* smem) {
    AdvanceFn<Real> fn = advance_kernel_for<Real>(b, mode);
    if (!fn) return fail(TOMO_EINVAL, "unsupported (steps_per_launch, cols_per_lane) pair");
    *smem = advance_smem_bytes<Real>(b.T, b.cols);
    CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem));
    int per_sm = 0;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 128, *smem));
    per_sm = std::max(per_sm, 1);
    *blocks = std::max(1, std::min((nitems + 3) / 4, num_sms * per_sm));
    return TOMO_OK;
}

// Blockings the autotuner times, restricted to a fixed T or COLS when nonzero
// and to a fixed MINB when nonzero; the first entry is the default before the
// first batch is tuned.
template <typename Real>
std::vector<Blocking> tune_candidates(int mode, int fixT, int fixCols, int fixMinb) {
    static const int pref[][3] = {{2, 2, 3}, {2, 2, 2}, {2, 1, 3}, {2, 1, 2}, {2, 1, 4}, {3, 2, 2}, {3, 1, 3},
                                  {4, 1, 2}, {4, 1, 3}, {4, 2, 2}, {2, 4, 2}, {1, 1, 2}, {1, 1, 4}, {6, 1, 2},
                                  {8, 1, 2}};
    std::vector<Blocking> out;
    for (const auto& p : pref) {
        if ((fixT && p[0] != fixT) || (fixCols && p[1] != fixCols) || (fixMinb && p[2] != fixMinb)) continue;
        const Blocking b{p[0], p[1], p[2]};
        if (advance_kernel_for<Real>(b, mode)) out.push_back(b);
    }
    return out;
}

// One time step of one solve on the plain path (H, E and DFT kernels; the DFT
// kernel only when n_contour > 0).  Returns the number of kernels launched.
template <typename Real>
int launch_plain_step(int mode, const SolveDesc<Real>* d, int n, int nx, int ny, int n_contour, cudaStream_t st);

// Launches whose contour samples one DFT pass sums (the stage_group of the
// engine's descriptors at blocking T).
inline int stage_group_for(int T) { return std::max(1, kStageLevels / std::max(T, 1)); }

// One advance launch (T steps of every listed solve), then -- when cmax, the
// largest contour among the solves, is positive and dft_nlev is not 0 -- the
// running DFT of the staged contour samples (dft_n0 < 0: this launch's levels;
// else steps dft_n0 .. dft_n0 + dft_nlev - 1), then the progress bump.
// Returns the number of kernels.
template <typename Real>
int launch_advance(const Blocking& b, int mode, int blocks, size_t smem, const SolveDesc<Real>* descs,
                   const WorkItem* items, int nitems, int nsolves, int* counter, int cmax, cudaStream_t st,
                   int dft_n0 = -1, int dft_nlev = -1) {
    AdvanceFn<Real> fn = advance_kernel_for<Real>(b, mode);
    fn<<<blocks, 128, smem, st>>>(descs, items, nitems, counter);
    const bool dft = cmax > 0 && dft_nlev != 0;
    if (dft)
        dft_accumulate_kernel<Real><<<dim3(nsolves, (cmax + 127) / 128), 128, 0, st>>>(descs, b.T, dft_n0, dft_nlev);
    bump_kernel<Real><<<(nsolves + 127) / 128, 128, 0, st>>>(const_cast<SolveDesc<Real>*>(descs), nsolves, b.T,
                                                            counter);
    return dft ? 3 : 2;
}

// Largest NTFF contour of a class as launch_advance wants it (0: no NTFF).
inline int dft_contour(const ProblemClass& pc) { return pc.nfreq > 0 ? pc.C : 0; }

// Work items of nsolves solves of a grid with nx + 1 columns, starting at
// solve index `first`.  Columns x <= lo and x >= hi (PEC boundary, CPML,
// vertical NTFF faces: lo = max(ncpml, d), hi = min(nx - ncpml, nx - d - 1)
// with d the NTFF distance, or -1 without NTFF) need the general path on every
// row.  With COLS > 1 those columns, plus the T-column halo an interior strip
// would reach into them, go to narrow items (32 - 2T owned columns) and the
// rest to wide items (32*COLS - 2T), so the general path runs on as few lanes
// as possible.  The edge items of every solve come first: they cost the most.
inline void append_items(std::vector<WorkItem>& items, int first, int nsolves, int nx, int ny, int ncpml, int d, int T,
                         int cols, int nseg = 1) {
    const int W1 = 32 - 2 * T, W2 = 32 * cols - 2 * T;
    const int ncol = nx + 1;
    std::vector<WorkItem> edge, mid;   // one solve's items (solve index filled in below)
    const int lo = std::max(ncpml, d);
    const int hi = d >= 0 ? std::min(nx - ncpml, nx - d - 1) : nx - ncpml;
    // Wide items copy rows COLS elements at a time, so their column windows
    // start at multiples of COLS: every wide-item boundary is = T (mod COLS)
    // (the window of a full item starts at x0 - T, a clipped one at x1 + T - P).
    int a_min = lo + 1 + T;                                   // first interior column: a - T > lo
    a_min += (((T - a_min) % cols) + cols) % cols;
    int b_max = hi - T;                                       // interior end: b - 1 + T < hi
    b_max -= (((b_max - T) % cols) + cols) % cols;
    // Interior bounds: fewest items, then fewest narrow columns (the narrow
    // edge strips take the slack the wide strips would otherwise leave).
    int a = a_min, b = b_max;
    long best = -1;
    for (int aa = a_min; aa <= a_min + W1; aa += cols)
        for (int bb = b_max; bb >= b_max - W1 && bb - aa >= W2; bb -= cols) {
            const long n = (aa + W1 - 1) / W1 + (ncol - bb + W1 - 1) / W1 + (bb - aa + W2 - 1) / W2;
            const long key = n * 100000L + aa + (ncol - bb);
            if (best < 0 || key < best) {
                best = key;
                a = aa;
                b = bb;
            }
        }
    const bool aligned = cols == 1 || (2 * T) % cols == 0;   // then every wide boundary stays = T
    if (cols == 1 || !aligned || best < 0) {
        const int n = (ncol + W1 - 1) / W1;
        for (int q = 0; q < n; ++q) {
            const WorkItem w{0, q * W1, std::min((q + 1) * W1, ncol), cols > 1 ? 1 : 0, 0, ny + 1};
            (q == 0 || q == n - 1 ? edge : mid).push_back(w);
        }
    } else {
        for (int x = 0; x < a; x += W1) edge.push_back({0, x, std::min(x + W1, a), 1, 0, ny + 1});
        for (int x = b; x < ncol; x += W1) edge.push_back({0, x, std::min(x + W1, ncol), 1, 0, ny + 1});
        for (int x = a; x < b; x += W2) mid.push_back({0, x, std::min(x + W2, b), 0, 0, ny + 1});
    }
    // row segments: [0, ny] cut into nseg nearly equal ranges
    const int nrow = ny + 1;
    nseg = std::max(1, std::min(nseg, nrow));
    for (const std::vector<WorkItem>* list : {&edge, &mid})
        for (int sv = 0; sv < nsolves; ++sv)
            for (WorkItem w : *list)
                for (int g = 0; g < nseg; ++g) {
                    w.solve = first + sv;
                    w.y0 = (int)((long)nrow * g / nseg);
                    w.y1 = (int)((long)nrow * (g + 1) / nseg);
                    items.push_back(w);
                }
}

// Work items of one solve before row segmentation.
inline int items_per_solve(int nx, int ny, int ncpml, int d, int T, int cols) {
    std::vector<WorkItem> v;
    append_items(v, 0, 1, nx, ny, ncpml, d, T, cols, 1);
    return (int)v.size();
}

// Row segments per strip: 1 while a batch's strips fill the GPU, else enough
// to reach about min_items items, keeping segments at least 6T and 12 rows
// tall (each segment recomputes 2T halo rows; a sweep of one 4-solve call of
// 401 rows ran fastest at about 32 segments per strip, 12-13 rows each).
// TOMO_SEGMENTS fixes the count.
inline int choose_segments(long strips, int ny, int T, long min_items) {
    if (const char* e = std::getenv("TOMO_SEGMENTS")) return std::max(1, std::atoi(e));
    if (strips <= 0 || strips >= min_items) return 1;
    const int max_seg = std::max(1, (ny + 1) / std::max(12, 6 * T));
    return (int)std::max(1L, std::min<long>(max_seg, (min_items + strips - 1) / strips));
}

// Host check of work items before they reach the GPU: owned ranges inside the
// grid and no wider than the layout allows, column windows inside the zero
// padding of the field rows, and wide windows aligned for COLS-element copies.
// A violation is a geometry bug; it fails the call instead of launching.
inline int validate_items(const std::vector<WorkItem>& items, size_t first_item, int nx, int ny, int ncpml, int d,
                          int T, int cols) {
    for (size_t i = first_item; i < items.size(); ++i) {
        const WorkItem& w = items[i];
        const int c = (cols > 1 && !w.narrow) ? cols : 1;
        const int P = 32 * c;
        const int xs = w.x1 + T - P;
        bool bad = w.x0 < 0 || w.x1 > nx + 1 || w.x1 <= w.x0 || w.x1 - w.x0 > P - 2 * T || xs > w.x0 - T ||
                   xs < -kPadLeft || xs + P > nx + 1 + kPadRight || (xs % c) != 0 || w.y0 < 0 || w.y1 > ny + 1 ||
                   w.y1 <= w.y0;
        // the wide layout treats every column of its window as interior: no PEC
        // boundary, CPML or vertical NTFF-face column inside it
        if (c > 1) {
            bad = bad || xs <= ncpml || xs + P - 1 >= nx - ncpml;
            if (d >= 0) bad = bad || (d >= xs && d < xs + P) || (nx - d - 1 >= xs && nx - d - 1 < xs + P);
        }
        if (bad)
            return fail(TOMO_ECUDA, "internal error: work item (" + std::to_string(w.x0) + ", " + std::to_string(w.x1) +
                                        ") invalid for nx " + std::to_string(nx));
    }
    return TOMO_OK;
}

// NTFF distance of a class as append_items wants it (-1: no NTFF).
inline int item_face_distance(const ProblemClass& pc) { return pc.nfreq > 0 ? pc.spec.nf2ff_d : -1; }

// ------------------------------------------------------------------- engine
template <typename Real>
struct ServeStateT;

template <typename Real>
class EngineT : public EngineBase {
   public:
    EngineT() = default;
    ~EngineT() override;
    int init(const ProblemClass& pc);
    int set_stream(void* s) override;
    int set_budget(uint64_t b) override;
    int set_target(const float* t, size_t n) override { return cd_.set_target(t, n); }
    int stats(tomo_stats* st) override {
        if (!st) return fail(TOMO_EINVAL, "stats is NULL");
        *st = stats_;
        return TOMO_OK;
    }
    int forward(const double* args, size_t ncand, size_t nparam, const tomo_outputs* out) override;
    // serving (serve.cu)
    int submit(const double* args, size_t ncand, size_t nparam, uint64_t* ticket) override;
    int submit_spec(const tomo_spec* spec, const double* args, size_t ncand, size_t nparam, uint64_t* ticket) override;
    int set_target_spec(const tomo_spec* spec, const float* t, size_t n) override;
    int serve_step(int* n_active) override;
    int request_bytes(const tomo_spec* spec, size_t ncand, uint64_t* bytes) override;
    int poll(uint64_t ticket, double* fitness) override;
    int cancel(uint64_t ticket) override;
    int snapshot(size_t cand, int exc, int field, float* out, size_t n) override;

   private:
    int ensure_batch(int ncand);
    int build_graph(int nlaunch);
    int autotune(size_t ncand);
    void invalidate_graph() {
        if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
        graph_exec_ = nullptr;
    }
    void serve_release();
    ClassData<Real>* class_for(const tomo_spec* spec, int* rc);

    ClassData<Real> cd_;
    cudaStream_t stream_ = nullptr;
    bool own_stream_ = false;
    cudaEvent_t ev_[4] = {nullptr, nullptr, nullptr, nullptr};
    int num_sms_ = 0;
    Blocking blk_;                                 // blocking of the next batch
    bool have_batch_ = false;                      // a batch's final state is on the device
    int last_parity_ = 0;                          // ping-pong copy holding that state
    bool auto_T_ = false, auto_cols_ = false, auto_minb_ = false;   // tuned per batch size on first use
    int fix_T_ = 0, fix_cols_ = 0, fix_minb_ = 0;  // dimensions fixed by the spec or the environment
    std::map<int, Blocking> tuned_;                // solves per batch -> blocking
    Blocking items_blk_{-1, -1, -1};               // blocking the uploaded work items were cut for
    DevBuf d_tune_items_;
    uint64_t budget_ = (uint64_t)150 << 30;
    tomo_stats stats_{};
    // batch buffers
    int cap_cand_ = 0, cur_cand_ = 0, nsolves_ = 0, nitems_ = 0;
    DevBuf d_state_, d_mats_, d_tabs_, d_upload_, d_descs_, d_items_, d_partials_, d_fit_, d_D_, d_P_, d_flag_, d_trf_,
        d_trd_, d_counter_;
    Unpacked up_;
    std::vector<SolveDesc<Real>> h_descs_;
    cudaGraphExec_t graph_exec_ = nullptr;
    int graph_cand_ = -1, graph_launches_ = -1, graph_blocks_ = 0;
    Blocking graph_blk_{-1, -1, -1};
    // serving
    ServeStateT<Real>* serve_ = nullptr;
};

}  // namespace tomo
