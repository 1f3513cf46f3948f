// Host engine of the forward FDTD fitness path and its C ABI (include/tomography.h).
//
// Lifecycle of one batch (tomo_fitness_batch / tomo_forward):
//   host: unpack candidate arguments into per-material (eps_inf, del_eps, sigma)
//         triples and ellipse geometry (FDTD_GPU.cu:657-693 / FDTD_CPU.cxx:682-698)
//   H2D : one packed upload
//   GPU : material maps + FP64 coefficient tables, zero state, a CUDA graph of
//         ceil(steps/T) advance launches (each followed by the running DFT of
//         the NTFF contour and a progress bump), far field, misfit; the
//         blocking of the advance kernel is autotuned on the first batch of
//         each size
//   D2H : fitness (plus optional traces / far field)
// Device buffers persist across calls (the reference allocates and frees ~30
// buffers inside every call, FDTD_GPU.cu:858-1106).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "engine_impl.cuh"

namespace tomo {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

const double kC0 = 1.0 / std::sqrt(kMu0D * kEps0D);
const double kEta0 = std::sqrt(kMu0D / kEps0D);

// ---------------------------------------------------------------------------
// Presets
static void spec_zero(tomo_spec* s) { std::memset(s, 0, sizeof(*s)); }

int spec_reference(tomo_spec* s, int cpu_variant) {
    if (!s) return fail(TOMO_EINVAL, "spec is NULL");
    spec_zero(s);
    // FDTD_common.hxx:3-59
    const double br = 0.0315, dx = 0.001;
    s->mode = cpu_variant ? TOMO_MODE_REFERENCE_CPU : TOMO_MODE_REFERENCE_GPU;
    s->precision = TOMO_FP32;
    s->nx = s->ny = (int)std::ceil(12.7 * br / dx);
    s->dx = dx;
    s->dt = dx / kC0 / 2;
    s->steps = 2000;
    s->ncpml = 10;
    s->cpml_grading = 2;
    s->cpml_sigma_max = (2 + 1) / (150 * kPiD * dx);
    s->cpml_kappa_max = 10;
    s->cpml_alpha_max = 0.01;
    s->cpml_alpha_min = 0.0;
    s->tau = 7e-12;
    s->breast_radius = br;
    s->npatch = cpu_variant ? 9 : 3;
    s->n_excitations = 4;
    s->pw_tau = 3.3445267e-11;
    s->pw_t0 = std::sqrt(20.0) * s->pw_tau;
    s->pw_l = -br;
    s->pw_centred = cpu_variant ? 0 : 1;
    s->nan_clamp = cpu_variant ? 0 : 1;
    s->nf2ff_d = (int)std::floor(3.2 * br / dx);
    s->nfreq = 10;
    for (int f = 0; f < 10; ++f) s->freqs[f] = 1e9 + (1e10 - 1e9) / 9 * f;
    s->n_angles = 100;
    s->ff_norm = 1;
    s->misfit = cpu_variant ? 1 : 0;
    return TOMO_OK;
}

static void breast_derived(tomo_spec* s);

int spec_breast(tomo_spec* s, int config) {
    if (!s) return fail(TOMO_EINVAL, "spec is NULL");
    if (config < 0 || config > 4) return fail(TOMO_EINVAL, "breast config must be 0..4");
    spec_zero(s);
    s->mode = TOMO_MODE_BREAST;
    s->precision = TOMO_FP32;
    s->dx = 0.5e-3;
    s->nx = s->ny = 200;
    s->steps = 1000;
    s->ncpml = 10;
    s->n_ellipses = 3;
    s->n_antennas = 16;
    s->n_tx = 1;
    s->antenna_radius = 45e-3;
    s->nfreq = 3;
    s->freqs[0] = 3e9; s->freqs[1] = 6e9; s->freqs[2] = 9e9;
    s->n_angles = 72;
    s->disc_radius = 35e-3;
    s->disc_eps_inf = 3.1; s->disc_del_eps = 1.6; s->disc_sigma = 0.036;
    switch (config) {
        case 0: break;
        case 1:
            s->nx = s->ny = 400; s->ncpml = 12; s->steps = 3000; s->n_ellipses = 8; s->n_tx = 16;
            break;
        case 2:
            s->nx = s->ny = 600; s->dx = 0.25e-3; s->ncpml = 12; s->steps = 6000;
            s->n_antennas = 32; s->n_tx = 32; s->antenna_radius = 70e-3;
            s->nfreq = 8;
            for (int f = 0; f < 8; ++f) s->freqs[f] = 2e9 + 1e9 * f;
            s->n_angles = 360;
            break;
        case 3:
            // serving default request: 256^2, breast (35 mm disc) at 70% of the domain
            s->nx = s->ny = 256; s->dx = 0.1 / 256; s->ncpml = 10; s->steps = 4 * 256;
            s->n_ellipses = 8; s->n_tx = 16; s->antenna_radius = 42e-3;
            break;
        case 4:
            s->nx = s->ny = 2048; s->dx = 0.125e-3; s->ncpml = 16; s->steps = 20000;
            s->n_antennas = 32; s->n_tx = 32; s->n_ellipses = 16; s->antenna_radius = 70e-3;
            s->disc_eps_inf = 15.9; s->disc_del_eps = 23.8; s->disc_sigma = 0.83;   // skin layer
            s->nfreq = 16;
            for (int f = 0; f < 16; ++f) s->freqs[f] = 1e9 + 0.5e9 * f;
            s->n_angles = 720;
            break;
    }
    breast_derived(s);
    return TOMO_OK;
}

int spec_serving(tomo_spec* s, int edge, int n_antennas) {
    if (!s) return fail(TOMO_EINVAL, "spec is NULL");
    if (edge < 64 || edge > 8190) return fail(TOMO_EINVAL, "serving grid edge must be 64..8190");
    if (n_antennas < 1 || n_antennas > kMaxRx) return fail(TOMO_EINVAL, "n_antennas out of range");
    TOMO_TRY(spec_breast(s, 3));
    // the 35 mm disc stays at 70% of a 100 mm square domain whatever the edge
    s->nx = s->ny = edge;
    s->dx = 0.1 / edge;
    s->steps = 4 * edge;
    s->n_antennas = n_antennas;
    s->n_tx = n_antennas;
    breast_derived(s);
    return TOMO_OK;
}

// Parameters of the breast-imaging presets that follow from dx.
static void breast_derived(tomo_spec* s) {
    s->dt = 0.99 * s->dx / (kC0 * std::sqrt(2.0));
    s->cpml_grading = 3;
    s->cpml_sigma_max = 0.8 * (3 + 1) / (kEta0 * s->dx);
    s->cpml_kappa_max = 5;
    s->cpml_alpha_max = 0.05;
    s->cpml_alpha_min = 0;
    s->tau = 13e-12;
    s->bg_eps_inf = 9; s->bg_del_eps = 0; s->bg_sigma = 0;
    s->src_f0 = 6e9;
    const double fmax = kC0 / (20 * s->dx * std::sqrt(s->bg_eps_inf));
    const double band = std::max(fmax - s->src_f0, 1e9);
    s->src_tau = std::sqrt(std::log(10.0)) / (kPiD * band);
    s->src_t0 = 4 * s->src_tau;
    s->src_amp = 0;
    s->nf2ff_d = s->ncpml + 3;
    s->ff_norm = 0;
    s->misfit = 2;
}

int num_params(const tomo_spec* s) {
    if (!s) return -1;
    if (s->mode == TOMO_MODE_REFERENCE_GPU) return s->npatch * s->npatch * 3;
    if (s->mode == TOMO_MODE_REFERENCE_CPU) return s->npatch * s->npatch * 2;
    return 8 * s->n_ellipses;
}

int num_excitations(const tomo_spec* s) {
    if (!s) return -1;
    return s->mode == TOMO_MODE_BREAST ? s->n_tx : s->n_excitations;
}


int validate_spec(const tomo_spec* s) {
    if (!s) return fail(TOMO_EINVAL, "spec is NULL");
    if (s->mode < 0 || s->mode > 2) return fail(TOMO_EINVAL, "unknown mode");
    if (s->precision != TOMO_FP32 && s->precision != TOMO_FP64) return fail(TOMO_EINVAL, "unknown precision");
    if (s->nx < 16 || s->ny < 16 || s->nx > 8190 || s->ny > 8190) return fail(TOMO_EINVAL, "grid size out of range");
    if (s->steps < 1) return fail(TOMO_EINVAL, "steps must be positive");
    if (!(s->dx > 0) || !(s->dt > 0)) return fail(TOMO_EINVAL, "dx and dt must be positive");
    if (s->ncpml < 0 || s->ncpml > kMaxCpml || 2 * s->ncpml + 4 > std::min(s->nx, s->ny))
        return fail(TOMO_EINVAL, "ncpml out of range");
    if (s->nfreq < 0 || s->nfreq > TOMO_MAX_FREQS) return fail(TOMO_EINVAL, "nfreq out of range");
    if (s->nfreq > 0 && (s->nf2ff_d < 1 || 2 * s->nf2ff_d + 4 > std::min(s->nx, s->ny)))
        return fail(TOMO_EINVAL, "nf2ff_d out of range");
    if (s->nfreq > 0 && s->n_angles < 0) return fail(TOMO_EINVAL, "n_angles out of range");
    if (s->mode != TOMO_MODE_BREAST) {
        if (s->nx != s->ny) return fail(TOMO_EINVAL, "reference modes need a square grid");
        if (s->npatch < 1 || s->npatch * s->npatch + 1 > kMaxMat) return fail(TOMO_EINVAL, "npatch out of range");
        if (s->n_excitations < 1) return fail(TOMO_EINVAL, "n_excitations must be positive");
        if (!(s->pw_tau > 0)) return fail(TOMO_EINVAL, "pw_tau must be positive");
    } else {
        if (s->n_ellipses < 0 || s->n_ellipses + 2 > kMaxMat) return fail(TOMO_EINVAL, "n_ellipses out of range");
        if (s->n_antennas < 1 || s->n_antennas > kMaxRx) return fail(TOMO_EINVAL, "n_antennas out of range");
        if (s->n_tx < 1 || s->n_tx > s->n_antennas) return fail(TOMO_EINVAL, "n_tx out of range");
        if (!(s->src_tau > 0)) return fail(TOMO_EINVAL, "src_tau must be positive");
    }
    if (!(s->tau > 0)) return fail(TOMO_EINVAL, "tau must be positive");
    if (s->total_field != 0 && s->total_field != 1) return fail(TOMO_EINVAL, "total_field must be 0 or 1");
    if (s->total_field && s->mode != TOMO_MODE_REFERENCE_GPU)
        return fail(TOMO_EINVAL, "the total-field variant belongs to the reference GPU mode");
    return TOMO_OK;
}

bool same_problem(const tomo_spec& a, const tomo_spec& b) {
    tomo_spec x = a, y = b;
    x.steps_per_launch = y.steps_per_launch = 0;
    x.cols_per_lane = y.cols_per_lane = 0;
    return std::memcmp(&x, &y, sizeof(tomo_spec)) == 0;
}

static void cpml_profile(const tomo_spec& s, std::vector<double>& out) {
    // FDTD_GPU.cu:748-806; kappa stored as its reciprocal for the device.
    const int nc = s.ncpml;
    out.assign(6 * (size_t)nc, 0.0);
    for (int i = 0; i < nc; ++i) {
        double rho = (i + 0.25) / nc;
        double se = s.cpml_sigma_max * std::pow(rho, s.cpml_grading);
        double ke = std::pow(rho, s.cpml_grading) * (s.cpml_kappa_max - 1) + 1;
        double ale = s.cpml_alpha_min + (s.cpml_alpha_max - s.cpml_alpha_min) * rho;
        double be = std::exp(-(s.dt / kEps0D) * (se / ke + ale));
        double ae = ((be - 1) * se) / (s.dx * (se * ke + ale * ke * ke));
        rho = (i + 0.75) / nc;
        double sm = (kMu0D / kEps0D) * s.cpml_sigma_max * std::pow(rho, s.cpml_grading);
        double km = std::pow(rho, s.cpml_grading) * (s.cpml_kappa_max - 1) + 1;
        double alm = (kMu0D / kEps0D) * (s.cpml_alpha_min + (s.cpml_alpha_max - s.cpml_alpha_min) * rho);
        double bm = std::exp(-(s.dt / kMu0D) * (sm / km + alm));
        double am = (bm - 1) * sm / (s.dx * (sm * km + alm * km * km));
        out[0 * nc + i] = 1.0 / ke;
        out[1 * nc + i] = be;
        out[2 * nc + i] = ae;
        out[3 * nc + i] = 1.0 / km;
        out[4 * nc + i] = bm;
        out[5 * nc + i] = am;
    }
}

static void contour_point(int nx, int ny, int d, int index, int* x, int* y, int* face) {
    // FDTD_common.cxx:4-46
    int l1 = nx - 2 * d - 2, l2 = l1 + (ny - 2 * d), l3 = l2 + l1;
    if (index < l1) { *x = index + d + 1; *y = d; *face = 0; }
    else if (index < l2) { *x = nx - d - 1; *y = index - l1 + d; *face = 1; }
    else if (index < l3) { *x = nx - d - 2 - (index - l2); *y = ny - d - 1; *face = 2; }
    else { *x = d; *y = ny - d - 1 - (index - l3); *face = 3; }
}

int build_class(const tomo_spec& s, ProblemClass& pc) {
    TOMO_TRY(validate_spec(&s));
    pc.spec = s;
    pc.nx = s.nx; pc.ny = s.ny; pc.nc = s.ncpml; pc.S = s.steps;
    pc.nfreq = s.nfreq;
    pc.nang = s.nfreq > 0 ? s.n_angles : 0;
    pc.C = s.nfreq > 0 ? 2 * s.nx + 2 * s.ny - 8 * s.nf2ff_d - 4 : 0;
    pc.n_exc = num_excitations(&s);
    pc.nparam = num_params(&s);
    pc.dt = s.dt;
    pc.chez = (s.dt / s.dx) / kMu0D;
    pc.Kp = (1 - s.dt / (2 * s.tau)) / (1 + s.dt / (2 * s.tau));
    pc.pitch = ((kPadLeft + s.nx + 1 + kPadRight) + 31) / 32 * 32;
    pc.mpitch = (kMatPadLeft + s.nx + 1 + 160 + 31) / 32 * 32;
    cpml_profile(s, pc.cpml);
    // running-DFT phasors (FDTD_GPU.cu:251-276): J at n dt, M at (n + 1/2) dt, times dt;
    // the total-field variant takes M at (n - 1/2) dt (oldFDTD_GPU.cu:784,794,803,811)
    const double mshift = s.total_field ? -0.5 : 0.5;
    pc.phasor.assign((size_t)pc.S * std::max(pc.nfreq, 1) * 4, 0.0);
    for (int n = 0; n < pc.S; ++n)
        for (int f = 0; f < pc.nfreq; ++f) {
            double w = 2 * kPiD * s.freqs[f];
            double* p = &pc.phasor[((size_t)n * pc.nfreq + f) * 4];
            p[0] = s.dt * std::cos(w * n * s.dt);
            p[1] = -s.dt * std::sin(w * n * s.dt);
            p[2] = s.dt * std::cos(w * (n + mshift) * s.dt);
            p[3] = -s.dt * std::sin(w * (n + mshift) * s.dt);
        }
    // total field: the legacy sums (H + H_inc) and (Ez + (Ez_inc(n) + Ez_inc(n-1))/2)
    // in one accumulator.  By linearity that is this class's own sums plus one
    // incident solve's, whose M phasor absorbs the two-level average:
    // sum_n e_inc(n) (p(n) + p(n+1))/2 with p(S) = 0.  The incident grid is the
    // same for every candidate and excitation, so each batch carries one.
    pc.extra = s.total_field ? 1 : 0;
    pc.inc_phasor.clear();
    pc.inc_wave.clear();
    pc.inc_tab.clear();
    if (pc.extra) {
        pc.inc_phasor = pc.phasor;
        for (int n = 0; n < pc.S; ++n)
            for (int f = 0; f < pc.nfreq; ++f) {
                double* q = &pc.inc_phasor[((size_t)n * pc.nfreq + f) * 4];
                const double* p0 = &pc.phasor[((size_t)n * pc.nfreq + f) * 4];
                const double* p1 = n + 1 < pc.S ? &pc.phasor[((size_t)(n + 1) * pc.nfreq + f) * 4] : nullptr;
                q[2] = 0.5 * (p0[2] + (p1 ? p1[2] : 0.0));
                q[3] = 0.5 * (p0[3] + (p1 ? p1[3] : 0.0));
            }
        // E_inc_update (oldFDTD_GPU.cu:655-717): vacuum, Ceze = 1, Cezhy = dt/(dx eps0),
        // 100 Cezj fwf(n, 0, 0, 0, 0) at the centre, Cezj = -dt/eps0; fwf at the
        // origin with angle 0 and no offset is exp(-((n dt - t0)/tau)^2)
        pc.inc_tab.assign((size_t)kMaxMat * kMatCoef, 0.0);
        pc.inc_tab[kCa] = 1.0;
        pc.inc_tab[kCb] = s.dt / (s.dx * kEps0D);
        pc.inc_tab[kCs] = 100.0 * (-s.dt / kEps0D);
        pc.inc_wave.resize(pc.S);
        for (int n = 0; n < pc.S; ++n) {
            const double a = (n * s.dt - s.pw_t0) / s.pw_tau;
            pc.inc_wave[n] = std::exp(-a * a);
        }
    }
    pc.rx.clear();
    pc.patchmap.clear();
    if (s.mode == TOMO_MODE_BREAST) {
        pc.nmat = 2 + s.n_ellipses;
        pc.nrx = s.n_antennas;
        pc.rx.resize(2 * (size_t)pc.nrx);
        for (int a = 0; a < pc.nrx; ++a) {
            double th = 2 * kPiD * a / pc.nrx;
            pc.rx[2 * a] = (int)std::lround(s.nx / 2.0 + (s.antenna_radius / s.dx) * std::cos(th));
            pc.rx[2 * a + 1] = (int)std::lround(s.ny / 2.0 + (s.antenna_radius / s.dx) * std::sin(th));
            if (pc.rx[2 * a] < 1 || pc.rx[2 * a] > s.nx - 1 || pc.rx[2 * a + 1] < 1 || pc.rx[2 * a + 1] > s.ny - 1)
                return fail(TOMO_EINVAL, "antenna outside the grid");
        }
        // zero-mean Gaussian-modulated sine current source centred at src_f0
        pc.src_amp = s.src_amp > 0 ? s.src_amp : (2 * s.bg_eps_inf * kEps0D + s.bg_sigma * s.dt) / (2 * s.dt);
        pc.wave.resize(pc.S);
        for (int n = 0; n < pc.S; ++n) {
            double t = (n + 0.5) * s.dt - s.src_t0;
            pc.wave[n] = pc.src_amp * std::sin(2 * kPiD * s.src_f0 * t) * std::exp(-(t / s.src_tau) * (t / s.src_tau));
        }
    } else {
        pc.nmat = 1 + s.npatch * s.npatch;
        pc.nrx = 0;
        pc.src_amp = 0;
        pc.wave.assign(1, 0.0);
        // fixed patch map (FDTD_GPU.cu:718-731, 544-551; FDTD_CPU.cxx:530-537, 1078-1164)
        pc.patchmap.assign((size_t)(s.ny + 1) * pc.mpitch, 0);
        const double br = s.breast_radius, dx = s.dx, cell = 2 * br / (s.npatch * dx);
        for (int j = 0; j <= s.ny; ++j)
            for (int i = 0; i <= s.nx; ++i) {
                double rx = ((float)i - s.nx / 2) * dx, ry = ((float)j - s.ny / 2) * dx;
                float radius = (float)std::sqrt(rx * rx + ry * ry);
                uint8_t m = 0;
                if (radius <= br) {
                    int xc = (int)((double)(i - (s.nx / 2 - (int)(br / dx))) / cell);
                    int yc = (int)((j - (s.ny / 2 - br / dx)) / cell);
                    m = (uint8_t)(1 + xc + s.npatch * yc);
                }
                pc.patchmap[(size_t)j * pc.mpitch + kMatPadLeft + i] = m;
            }
    }
    // far-field geometry (FDTD_GPU.cu:579-625): contour point relative to the
    // transform origin (nx/2 - 1, ny/2 - 1) with nx/2 in float division, metres
    pc.ffgeom.resize(3 * (size_t)pc.C);
    for (int c = 0; c < pc.C; ++c) {
        int x, y, face;
        contour_point(s.nx, s.ny, s.nf2ff_d, c, &x, &y, &face);
        double flx = x, fly = y;
        if (face == 0 || face == 2) fly += 0.5; else flx += 0.5;
        pc.ffgeom[3 * c + 0] = s.dx * (flx - (s.nx / 2.0 - 1));
        pc.ffgeom[3 * c + 1] = s.dx * (fly - (s.ny / 2.0 - 1));
        pc.ffgeom[3 * c + 2] = face;
    }
    pc.ffang.resize(2 * (size_t)pc.nang);
    for (int a = 0; a < pc.nang; ++a) {
        double phi = 2 * kPiD / pc.nang * a;
        pc.ffang[2 * a] = std::cos(phi);
        pc.ffang[2 * a + 1] = std::sin(phi);
    }
    return TOMO_OK;
}

SolveLayout solve_layout(const ProblemClass& pc, size_t real_bytes) {
    SolveLayout L;
    const size_t rows = (size_t)pc.ny + 1;
    L.field_elems = rows * pc.pitch;
    L.psi_elems = (size_t)4 * pc.nc * (pc.ny + 1) + (size_t)4 * pc.nc * (pc.nx + 1) + 32;
    L.psi_elems = (L.psi_elems + 31) / 32 * 32;
    L.tr_stride = std::max<size_t>((size_t)pc.nrx * pc.S, 1);
    L.tr_stride = (L.tr_stride + 31) / 32 * 32;
    L.acc_stride = std::max<size_t>((size_t)pc.nfreq * pc.C * 8, 8);
    L.acc_stride = (L.acc_stride + 31) / 32 * 32;
    const int tmax = 8;
    L.stage_stride = pc.nfreq > 0 ? ((size_t)kStageLevels * pc.C * 2 + 31) / 32 * 32 : 32;
    L.per_solve = 8 * L.field_elems + (size_t)(tmax + 1) * L.psi_elems + L.tr_stride + L.acc_stride + L.stage_stride;
    L.per_solve = (L.per_solve + 63) / 64 * 64;
    L.mat_stride = rows * pc.mpitch;
    (void)real_bytes;
    return L;
}

int unpack_args(const ProblemClass& pc, const double* args, size_t ncand, size_t nparam, Unpacked& u) {
    // upload layout: [ncand][kMaxMat][3] material triples, then [ncand][K][6] ellipses
    const tomo_spec& s = pc.spec;
    if (!args || ncand == 0) return fail(TOMO_EINVAL, "no candidates");
    if ((int)nparam != pc.nparam)
        return fail(TOMO_EINVAL, "expected " + std::to_string(pc.nparam) + " parameters per candidate, got " +
                                     std::to_string(nparam));
    const int K = s.mode == TOMO_MODE_BREAST ? s.n_ellipses : 0;
    u.ncand = ncand;
    u.upload.assign(ncand * kMaxMat * 3 + ncand * (size_t)K * 6, 0.0);
    u.bbox.assign(ncand * 4, 0);
    for (size_t c = 0; c < ncand; ++c) {
        const double* a = args + c * nparam;
        double* mp = &u.upload[c * kMaxMat * 3];
        for (size_t i = 0; i < nparam; ++i)
            if (!std::isfinite(a[i])) return fail(TOMO_EINVAL, "non-finite candidate parameter");
        int* bb = &u.bbox[c * 4];
        if (s.mode != TOMO_MODE_BREAST) {
            // FDTD_GPU.cu:657-693, 718-738 (3x3: eps_inf, del_eps, sigma) and
            // FDTD_CPU.cxx:682-698, 1078-1164 (9x9: eps_r, sigma); the reference
            // stores the arguments as float.
            const int np2 = s.npatch * s.npatch;
            mp[0] = 1; mp[1] = 0; mp[2] = 0;
            for (int p = 0; p < np2; ++p) {
                if (s.mode == TOMO_MODE_REFERENCE_GPU) {
                    mp[3 * (1 + p) + 0] = (double)(float)a[p];
                    mp[3 * (1 + p) + 1] = (double)(float)a[np2 + p];
                    mp[3 * (1 + p) + 2] = (double)(float)a[2 * np2 + p];
                } else {
                    mp[3 * (1 + p) + 0] = (double)(float)a[p];
                    mp[3 * (1 + p) + 1] = 0;
                    mp[3 * (1 + p) + 2] = (double)(float)a[np2 + p];
                }
                if (!(mp[3 * (1 + p)] > 0)) return fail(TOMO_EINVAL, "permittivity must be positive");
            }
            const int r = (int)std::ceil(s.breast_radius / s.dx) + 2;
            bb[0] = std::max(1, s.nx / 2 - r); bb[1] = std::min(s.nx - 1, s.nx / 2 + r);
            bb[2] = std::max(1, s.ny / 2 - r); bb[3] = std::min(s.ny - 1, s.ny / 2 + r);
            continue;
        }
        mp[0] = s.bg_eps_inf; mp[1] = s.bg_del_eps; mp[2] = s.bg_sigma;
        mp[3] = s.disc_eps_inf; mp[4] = s.disc_del_eps; mp[5] = s.disc_sigma;
        double* el = &u.upload[ncand * kMaxMat * 3 + c * (size_t)K * 6];
        double xlo = 1e30, xhi = -1e30, ylo = 1e30, yhi = -1e30;
        auto grow = [&](double cx, double cy, double r) {
            xlo = std::min(xlo, cx - r); xhi = std::max(xhi, cx + r);
            ylo = std::min(ylo, cy - r); yhi = std::max(yhi, cy + r);
        };
        bool everywhere = s.bg_del_eps != 0;
        if (s.disc_radius > 0 && s.disc_del_eps != 0) grow(0, 0, s.disc_radius);
        for (int k = 0; k < K; ++k) {
            const double* e = a + 8 * k;
            if (!(e[2] > 0) || !(e[3] > 0)) return fail(TOMO_EINVAL, "ellipse semi-axes must be positive");
            if (!(e[5] > 0) || e[6] < 0 || e[7] < 0) return fail(TOMO_EINVAL, "ellipse material out of range");
            el[6 * k + 0] = e[0];
            el[6 * k + 1] = e[1];
            el[6 * k + 2] = e[2];
            el[6 * k + 3] = e[3];
            el[6 * k + 4] = std::cos(e[4]);
            el[6 * k + 5] = std::sin(e[4]);
            mp[3 * (2 + k) + 0] = e[5];
            mp[3 * (2 + k) + 1] = e[6];
            mp[3 * (2 + k) + 2] = e[7];
            if (e[6] != 0) grow(e[0], e[1], std::max(e[2], e[3]));
        }
        // Jp can be non-zero only where del_eps != 0: conservative cell box
        auto cell = [&](double v, int n, bool up) {
            double c = v / s.dx + 0.5 * n;
            double r = up ? std::ceil(c) + 1 : std::floor(c) - 1;
            r = std::max(1.0, std::min((double)(n - 1), r));
            return (int)r;
        };
        if (everywhere) { bb[0] = 1; bb[1] = s.nx - 1; bb[2] = 1; bb[3] = s.ny - 1; }
        else if (xhi < xlo) { bb[0] = 1; bb[1] = 0; bb[2] = 1; bb[3] = 0; }
        else {
            bb[0] = cell(xlo, s.nx, false); bb[1] = cell(xhi, s.nx, true);
            bb[2] = cell(ylo, s.ny, false); bb[3] = cell(yhi, s.ny, true);
        }
    }
    return TOMO_OK;
}

// ------------------------------------------------------------------- EngineT
template <typename Real>
EngineT<Real>::~EngineT() {
    serve_release();
    if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
    if (own_stream_ && stream_) cudaStreamDestroy(stream_);
    for (auto& e : ev_)
        if (e) cudaEventDestroy(e);
}

template <typename Real>
int EngineT<Real>::init(const ProblemClass& pc) {
    CUDA_TRY(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    own_stream_ = true;
    for (auto& e : ev_) CUDA_TRY(cudaEventCreate(&e));
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    CUDA_TRY(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev));
    TOMO_TRY(cd_.init(pc));
    TOMO_TRY(d_counter_.ensure(sizeof(int) * 4));
    CUDA_TRY(cudaMemset(d_counter_.p, 0, sizeof(int) * 4));
    // blocking: explicit spec values, else the environment, else autotuned per batch size
    auto env = [](const char* n) {
        const char* e = std::getenv(n);
        return e ? std::atoi(e) : 0;
    };
    fix_T_ = pc.spec.steps_per_launch > 0 ? pc.spec.steps_per_launch : env("TOMO_T");
    fix_cols_ = pc.spec.cols_per_lane > 0 ? pc.spec.cols_per_lane : env("TOMO_COLS");
    fix_minb_ = env("TOMO_MINB");
    auto_T_ = fix_T_ <= 0;
    auto_cols_ = fix_cols_ <= 0;
    auto_minb_ = fix_minb_ <= 0;
    const std::vector<Blocking> c = tune_candidates<Real>(advance_mode(pc.spec), std::max(fix_T_, 0),
                                                          std::max(fix_cols_, 0), std::max(fix_minb_, 0));
    if (c.empty())
        return fail(TOMO_EINVAL, "unsupported (steps_per_launch, cols_per_lane) pair for this mode and precision");
    blk_ = c.front();   // until the first batch is tuned
    return TOMO_OK;
}

// Autotuner: times every offered blocking (T, COLS, MINB) on the actual batch
// -- its materials, descriptors and state -- and keeps the fastest per batch
// size.  Every blocking computes the same bits, so the choice affects speed
// only.  Each blocking runs one warm-up launch and then about kTuneSteps time
// steps from step 0 (the descriptors are re-uploaded before each); the time
// per step (CUDA events around the timed launches) decides.  forward() then
// sets the state up again from scratch, so tuning leaves no trace in results.
template <typename Real>
int EngineT<Real>::autotune(size_t ncand) {
    constexpr int kTuneSteps = 16;
    const ProblemClass& pc = cd_.pc;
    const int mode = advance_mode(pc.spec);
    const std::vector<Blocking> cands =
        tune_candidates<Real>(mode, std::max(fix_T_, 0), std::max(fix_cols_, 0), std::max(fix_minb_, 0));
    if (cands.empty()) return fail(TOMO_EINVAL, "no blocking to tune");
    const int key = (int)ncand * pc.n_exc;
    stats_.tune_ms = 0;
    stats_.tuned_configs = 0;
    int maxT = 1;
    for (const Blocking& c : cands) maxT = std::max(maxT, c.T);
    // too few time steps to time every blocking inside the time loop: keep the default
    if (cands.size() <= 1 || pc.S < (1 + std::max(2, kTuneSteps / maxT)) * maxT + maxT) {
        tuned_[key] = blk_ = cands.front();
        return TOMO_OK;
    }
    blk_ = cands.front();
    TOMO_TRY(ensure_batch((int)ncand));
    const int nsolves = nsolves_;
    TOMO_TRY(d_upload_.ensure(sizeof(double) * up_.upload.size()));
    int64_t kernels = 0, h2d = 0;
    TOMO_TRY(setup_materials<Real>(cd_, up_, d_upload_.as<double>(), d_mats_.as<uint8_t>(), d_tabs_.as<Real>(), stream_,
                                   &kernels, &h2d));
    CUDA_TRY(cudaMemsetAsync(d_state_.p, 0, (size_t)nsolves * cd_.lay.per_solve * sizeof(Real), stream_));
    h_descs_.resize(nsolves);
    fill_descs<Real>(cd_, up_, d_state_.as<Real>(), d_mats_.as<uint8_t>(), d_tabs_.as<Real>(), h_descs_.data());
    if (pc.extra) h_descs_[nsolves - 1] = incident_desc<Real>(cd_, d_state_.as<Real>() + (size_t)(nsolves - 1) * cd_.lay.per_solve);
    double best = 1e300;
    Blocking bestb = cands.front();
    std::vector<WorkItem> items;
    for (const Blocking& c : cands) {
        items.clear();
        const int nseg = choose_segments(
            (long)nsolves * items_per_solve(pc.nx, pc.ny, pc.nc, item_face_distance(pc), c.T, c.cols), pc.ny, c.T,
            24L * num_sms_);
        append_items(items, 0, nsolves, pc.nx, pc.ny, pc.nc, item_face_distance(pc), c.T, c.cols, nseg);
        TOMO_TRY(validate_items(items, 0, pc.nx, pc.ny, pc.nc, item_face_distance(pc), c.T, c.cols));
        TOMO_TRY(d_tune_items_.ensure(sizeof(WorkItem) * items.size()));
        CUDA_TRY(cudaMemcpyAsync(d_tune_items_.p, items.data(), sizeof(WorkItem) * items.size(), cudaMemcpyHostToDevice,
                                 stream_));
        CUDA_TRY(cudaMemcpyAsync(d_descs_.p, h_descs_.data(), sizeof(SolveDesc<Real>) * nsolves,
                                 cudaMemcpyHostToDevice, stream_));
        int blocks = 0;
        size_t smem = 0;
        TOMO_TRY(advance_grid<Real>(c, mode, (int)items.size(), num_sms_, &blocks, &smem));
        const int L = std::max(2, kTuneSteps / c.T);
        launch_advance<Real>(c, mode, blocks, smem, d_descs_.as<SolveDesc<Real>>(), d_tune_items_.as<WorkItem>(),
                             (int)items.size(), nsolves, d_counter_.as<int>(), dft_contour(pc), stream_);
        CUDA_TRY(cudaEventRecord(ev_[1], stream_));
        for (int l = 0; l < L; ++l)
            launch_advance<Real>(c, mode, blocks, smem, d_descs_.as<SolveDesc<Real>>(), d_tune_items_.as<WorkItem>(),
                                 (int)items.size(), nsolves, d_counter_.as<int>(), dft_contour(pc), stream_);
        CUDA_TRY(cudaEventRecord(ev_[2], stream_));
        CUDA_TRY(cudaStreamSynchronize(stream_));
        CUDA_TRY(cudaGetLastError());
        float ms = 0;
        CUDA_TRY(cudaEventElapsedTime(&ms, ev_[1], ev_[2]));
        stats_.tune_ms += ms;
        ++stats_.tuned_configs;
        const double per_step = ms / (double)(L * c.T);
        if (per_step < best) {
            best = per_step;
            bestb = c;
        }
    }
    tuned_[key] = blk_ = bestb;
    return TOMO_OK;
}

template <typename Real>
int EngineT<Real>::set_stream(void* s) {
    CUDA_TRY(cudaStreamSynchronize(stream_));
    if (own_stream_) {
        cudaStreamDestroy(stream_);
        own_stream_ = false;
    }
    if (s) {
        stream_ = (cudaStream_t)s;
    } else {
        CUDA_TRY(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
        own_stream_ = true;
    }
    invalidate_graph();
    return TOMO_OK;
}

template <typename Real>
int EngineT<Real>::set_budget(uint64_t b) {
    budget_ = b ? b : (uint64_t)150 << 30;
    return TOMO_OK;
}

template <typename Real>
int EngineT<Real>::ensure_batch(int ncand) {
    const ProblemClass& pc = cd_.pc;
    const SolveLayout& L = cd_.lay;
    const int nsolves = ncand * pc.n_exc + pc.extra;   // + the total-field incident grid
    const size_t need = (size_t)nsolves * L.per_solve * sizeof(Real);
    if (need > budget_)
        return fail(TOMO_ENOMEM_BUDGET, "batch needs " + std::to_string(need >> 20) + " MiB, budget " +
                                            std::to_string(budget_ >> 20) + " MiB");
    if (ncand > cap_cand_) {
        invalidate_graph();
        cap_cand_ = 0;
        TOMO_TRY(d_state_.ensure(need));
        if (pc.spec.mode == TOMO_MODE_BREAST) TOMO_TRY(d_mats_.ensure(L.mat_stride * ncand));
        TOMO_TRY(d_tabs_.ensure(sizeof(Real) * kMaxMat * kMatCoef * ncand));
        TOMO_TRY(d_descs_.ensure(sizeof(SolveDesc<Real>) * nsolves));
        TOMO_TRY(d_partials_.ensure(sizeof(double) * 2 * nsolves));
        TOMO_TRY(d_fit_.ensure(sizeof(double) * ncand));
        TOMO_TRY(d_flag_.ensure(sizeof(int) * 4));
        if (pc.nang > 0) {
            TOMO_TRY(d_D_.ensure(sizeof(float) * (size_t)nsolves * pc.nfreq * pc.nang));
            TOMO_TRY(d_P_.ensure(sizeof(float) * (size_t)nsolves * pc.nfreq * pc.nang));
        }
        cap_cand_ = ncand;
    }
    std::vector<WorkItem> items;
    const int nseg = choose_segments(
        (long)nsolves * items_per_solve(pc.nx, pc.ny, pc.nc, item_face_distance(pc), blk_.T, blk_.cols), pc.ny,
        blk_.T, 24L * num_sms_);
    append_items(items, 0, nsolves, pc.nx, pc.ny, pc.nc, item_face_distance(pc), blk_.T, blk_.cols, nseg);
    TOMO_TRY(validate_items(items, 0, pc.nx, pc.ny, pc.nc, item_face_distance(pc), blk_.T, blk_.cols));
    if (nsolves != nsolves_ || (int)items.size() != nitems_ || ncand != cur_cand_ || blk_.T != items_blk_.T ||
        blk_.cols != items_blk_.cols) {
        invalidate_graph();
        TOMO_TRY(d_items_.ensure(sizeof(WorkItem) * items.size()));
        CUDA_TRY(cudaMemcpyAsync(d_items_.p, items.data(), sizeof(WorkItem) * items.size(), cudaMemcpyHostToDevice,
                                 stream_));
    }
    nsolves_ = nsolves;
    nitems_ = (int)items.size();
    cur_cand_ = ncand;
    items_blk_ = blk_;
    return TOMO_OK;
}

template <typename Real>
int EngineT<Real>::build_graph(int nlaunch) {
    if (graph_exec_ && graph_cand_ == cur_cand_ && graph_blk_ == blk_ && graph_launches_ == nlaunch)
        return TOMO_OK;
    invalidate_graph();
    int blocks = 0;
    size_t smem = 0;
    TOMO_TRY(advance_grid<Real>(blk_, advance_mode(cd_.pc.spec), nitems_, num_sms_, &blocks, &smem));
    cudaGraph_t graph;
    CUDA_TRY(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    // one DFT pass per group of stage_group launches (and after the last launch):
    // it sums the group's steps in time order, as one pass per launch would
    const int group = stage_group_for(blk_.T), S = cd_.pc.S, T = blk_.T;
    for (int l = 0; l < nlaunch; ++l) {
        const bool last_of_group = (l + 1) % group == 0 || l == nlaunch - 1;
        const int n0 = (l - l % group) * T;
        const int nlev = last_of_group ? std::min((l + 1) * T, S) - n0 : 0;
        launch_advance<Real>(blk_, advance_mode(cd_.pc.spec), blocks, smem, d_descs_.as<SolveDesc<Real>>(),
                             d_items_.as<WorkItem>(), nitems_, nsolves_, d_counter_.as<int>(), dft_contour(cd_.pc),
                             stream_, n0, nlev);
    }
    cudaError_t ce = cudaStreamEndCapture(stream_, &graph);
    if (ce != cudaSuccess) return fail(TOMO_ECUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
    ce = cudaGraphInstantiate(&graph_exec_, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) {
        graph_exec_ = nullptr;
        return fail(TOMO_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce));
    }
    graph_cand_ = cur_cand_; graph_blk_ = blk_; graph_launches_ = nlaunch; graph_blocks_ = blocks;
    return TOMO_OK;
}

template <typename Real>
int EngineT<Real>::forward(const double* args, size_t ncand, size_t nparam, const tomo_outputs* out) {
    const ProblemClass& pc = cd_.pc;
    const tomo_spec& s = pc.spec;
    const bool want_fit = out && out->fitness;
    if (want_fit && !cd_.have_target) return fail(TOMO_ENOTARGET, "fitness needs a target (tomo_set_target)");
    TOMO_TRY(unpack_args(pc, args, ncand, nparam, up_));
    stats_.tune_ms = 0;
    stats_.tuned_configs = 0;
    if ((auto_T_ || auto_cols_ || auto_minb_) && !s.plain) {
        auto it = tuned_.find((int)ncand * pc.n_exc);
        if (it != tuned_.end()) {
            blk_ = it->second;
        } else {
            TOMO_TRY(autotune(ncand));
        }
    }
    TOMO_TRY(ensure_batch((int)ncand));
    const int nsolves = nsolves_;
    int64_t kernels = 0, h2d = 0, d2h = 0;

    TOMO_TRY(d_upload_.ensure(sizeof(double) * up_.upload.size()));
    CUDA_TRY(cudaMemcpyAsync(d_upload_.p, up_.upload.data(), sizeof(double) * up_.upload.size(), cudaMemcpyHostToDevice,
                             stream_));
    h2d += sizeof(double) * up_.upload.size();
    CUDA_TRY(cudaEventRecord(ev_[0], stream_));
    TOMO_TRY(setup_materials<Real>(cd_, up_, d_upload_.as<double>(), d_mats_.as<uint8_t>(), d_tabs_.as<Real>(), stream_,
                                   &kernels, nullptr));
    CUDA_TRY(cudaMemsetAsync(d_state_.p, 0, (size_t)nsolves * cd_.lay.per_solve * sizeof(Real), stream_));
    h_descs_.resize(nsolves);
    fill_descs<Real>(cd_, up_, d_state_.as<Real>(), d_mats_.as<uint8_t>(), d_tabs_.as<Real>(), h_descs_.data());
    if (pc.extra) h_descs_[nsolves - 1] = incident_desc<Real>(cd_, d_state_.as<Real>() + (size_t)(nsolves - 1) * cd_.lay.per_solve);
    if (!s.plain)   // the time-loop graph runs one DFT pass per group of launches
        for (SolveDesc<Real>& D : h_descs_) D.stage_group = stage_group_for(blk_.T);
    CUDA_TRY(cudaMemcpyAsync(d_descs_.p, h_descs_.data(), sizeof(SolveDesc<Real>) * nsolves, cudaMemcpyHostToDevice,
                             stream_));
    h2d += sizeof(SolveDesc<Real>) * nsolves;

    // time loop: ceil(S/T) advance launches, each followed by the running DFT and
    // the progress bump, replayed as one CUDA graph
    const int nlaunch = (pc.S + blk_.T - 1) / blk_.T;
    if (s.plain) {
        // plain baseline path: one solve per launch, one launch per field update
        // and time step (H, E, DFT), no temporal blocking, no graph
        const int ncont = pc.nfreq > 0 ? pc.C : 0;
        CUDA_TRY(cudaEventRecord(ev_[1], stream_));
        for (int sv = 0; sv < nsolves; ++sv)
            for (int n = 0; n < pc.S; ++n)
                kernels += launch_plain_step<Real>(advance_mode(s), d_descs_.as<SolveDesc<Real>>() + sv, n, s.nx, s.ny,
                                                   ncont, stream_);
        CUDA_TRY(cudaEventRecord(ev_[2], stream_));
        CUDA_TRY(cudaGetLastError());
    } else {
        TOMO_TRY(build_graph(nlaunch));
        CUDA_TRY(cudaEventRecord(ev_[1], stream_));
        CUDA_TRY(cudaGraphLaunch(graph_exec_, stream_));
        CUDA_TRY(cudaEventRecord(ev_[2], stream_));
        const int group = stage_group_for(blk_.T);
        kernels += 2 * (int64_t)nlaunch + (dft_contour(pc) > 0 ? (nlaunch + group - 1) / group : 0);
    }

    CUDA_TRY(cudaMemsetAsync(d_flag_.p, 0, sizeof(int) * 4, stream_));
    float* d_trf = nullptr;
    double* d_trd = nullptr;
    const size_t ntr = (size_t)pc.nrx * pc.S * (nsolves - pc.extra);
    if (out && out->traces && pc.nrx > 0) {
        TOMO_TRY(d_trf_.ensure(sizeof(float) * ntr));
        d_trf = d_trf_.as<float>();
    }
    if (out && out->traces_f64 && pc.nrx > 0) {
        TOMO_TRY(d_trd_.ensure(sizeof(double) * ntr));
        d_trd = d_trd_.as<double>();
    }
    // the far field runs when it is returned or when the misfit needs it (the
    // reference modes); the breast mode's trace misfit does not
    const bool want_ff = out && (out->D || out->P || (want_fit && s.mode != TOMO_MODE_BREAST));
    TOMO_TRY(post_range<Real>(cd_, ncand, h_descs_[0], want_fit, want_ff ? d_D_.as<float>() : nullptr,
                              want_ff ? d_P_.as<float>() : nullptr,
                              d_partials_.as<double>(), d_fit_.as<double>(), d_flag_.as<int>(), d_trf, d_trd, stream_,
                              &kernels, pc.extra ? h_descs_[nsolves - 1].acc : nullptr));
    if (d_trf) {
        CUDA_TRY(cudaMemcpyAsync(out->traces, d_trf, sizeof(float) * ntr, cudaMemcpyDeviceToHost, stream_));
        d2h += sizeof(float) * ntr;
    }
    if (d_trd) {
        CUDA_TRY(cudaMemcpyAsync(out->traces_f64, d_trd, sizeof(double) * ntr, cudaMemcpyDeviceToHost, stream_));
        d2h += sizeof(double) * ntr;
    }
    if (out && pc.nang > 0) {
        const size_t n = (size_t)(nsolves - pc.extra) * pc.nfreq * pc.nang;
        if (out->D) {
            CUDA_TRY(cudaMemcpyAsync(out->D, d_D_.p, sizeof(float) * n, cudaMemcpyDeviceToHost, stream_));
            d2h += sizeof(float) * n;
        }
        if (out->P) {
            CUDA_TRY(cudaMemcpyAsync(out->P, d_P_.p, sizeof(float) * n, cudaMemcpyDeviceToHost, stream_));
            d2h += sizeof(float) * n;
        }
    }
    CUDA_TRY(cudaEventRecord(ev_[3], stream_));
    int flag = 0;
    if (want_fit) {
        CUDA_TRY(cudaMemcpyAsync(out->fitness, d_fit_.p, sizeof(double) * ncand, cudaMemcpyDeviceToHost, stream_));
        CUDA_TRY(cudaMemcpyAsync(&flag, d_flag_.p, sizeof(int), cudaMemcpyDeviceToHost, stream_));
        d2h += sizeof(double) * ncand + sizeof(int);
    }
    CUDA_TRY(cudaStreamSynchronize(stream_));
    CUDA_TRY(cudaGetLastError());
    float adv = 0, tot = 0;
    CUDA_TRY(cudaEventElapsedTime(&adv, ev_[1], ev_[2]));
    CUDA_TRY(cudaEventElapsedTime(&tot, ev_[0], ev_[3]));
    stats_.advance_ms = adv;
    stats_.total_ms = tot;
    stats_.cell_updates = (double)nsolves * (double)s.nx * (double)s.ny * (double)pc.S;
    stats_.launches = s.plain ? (int64_t)pc.S * nsolves : nlaunch;
    have_batch_ = true;
    last_parity_ = s.plain ? 0 : (nlaunch & 1);   // the plain path updates copy 0 in place
    stats_.kernels = kernels;
    stats_.steps_per_launch = blk_.T;
    stats_.cols_per_lane = blk_.cols;
    stats_.min_blocks_per_sm = blk_.minb;
    stats_.h2d_bytes = h2d;
    stats_.d2h_bytes = d2h;
    if (flag && s.mode != TOMO_MODE_REFERENCE_GPU) return fail(TOMO_ENUMERIC, "non-finite field or fitness detected");
    return TOMO_OK;
}

template <typename Real>
int EngineT<Real>::snapshot(size_t cand, int exc, int field, float* out, size_t n) {
    const ProblemClass& pc = cd_.pc;
    if (!have_batch_) return fail(TOMO_ENOTREADY, "no batch has run on this handle yet");
    if (field < TOMO_FIELD_EZ || field > TOMO_FIELD_HY) return fail(TOMO_EINVAL, "field must be 0 (Ez), 1 (Hx) or 2 (Hy)");
    if (exc < 0 || exc >= pc.n_exc || cand >= (size_t)cur_cand_)
        return fail(TOMO_EINVAL, "candidate or excitation out of range of the last batch");
    const size_t rows = field == TOMO_FIELD_EZ ? pc.ny + 1 : pc.ny, cols = field == TOMO_FIELD_EZ ? pc.nx + 1 : pc.nx;
    if (!out || n < rows * cols) return fail(TOMO_EINVAL, "snapshot needs " + std::to_string(rows * cols) + " values");
    const SolveDesc<Real>& D = h_descs_[cand * pc.n_exc + exc];
    const Real* src = (field == TOMO_FIELD_EZ ? D.ez : field == TOMO_FIELD_HX ? D.hx : D.hy)[last_parity_];
    std::vector<Real> host(rows * cols);
    CUDA_TRY(cudaMemcpy2DAsync(host.data(), cols * sizeof(Real), src, (size_t)pc.pitch * sizeof(Real),
                               cols * sizeof(Real), rows, cudaMemcpyDeviceToHost, stream_));
    CUDA_TRY(cudaStreamSynchronize(stream_));
    for (size_t i = 0; i < host.size(); ++i) out[i] = (float)host[i];
    return TOMO_OK;
}

template class EngineT<float>;
template class EngineT<double>;

// ---------------------------------------------------------------------------
int create_engine(const tomo_spec* spec, EngineBase** out) {
    if (!out) return fail(TOMO_EINVAL, "out is NULL");
    *out = nullptr;
    ProblemClass pc;
    TOMO_TRY(build_class(*spec, pc));
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(TOMO_ECUDA, "no CUDA device");
    }
    if (spec->precision == TOMO_FP64) {
        auto* e = new EngineT<double>();
        int rc = e->init(pc);
        if (rc) { delete e; return rc; }
        *out = e;
    } else {
        auto* e = new EngineT<float>();
        int rc = e->init(pc);
        if (rc) { delete e; return rc; }
        *out = e;
    }
    return TOMO_OK;
}

}  // namespace tomo

// Internal test hook (not part of the public ABI): the blockings the
// autotuner offers for a precision and mode, in preference order, as
// (T, cols, minb, dynamic shared memory per block in bytes) records.  Returns
// the count, or a negative status.
extern "C" int tomo_internal_blockings(int precision, int mode, int* out, int cap) {
    return tomo::guarded([&]() -> int {
        tomo_spec s{};
        s.mode = mode;
        const int am = tomo::advance_mode(s);
        std::vector<int> rec;
        auto put = [&](const std::vector<tomo::Blocking>& bs, bool f64) {
            for (const tomo::Blocking& b : bs) {
                const size_t smem = f64 ? tomo::advance_smem_bytes<double>(b.T, b.cols)
                                        : tomo::advance_smem_bytes<float>(b.T, b.cols);
                rec.insert(rec.end(), {b.T, b.cols, b.minb, (int)smem});
            }
        };
        if (precision == TOMO_FP64) put(tomo::tune_candidates<double>(am, 0, 0, 0), true);
        else put(tomo::tune_candidates<float>(am, 0, 0, 0), false);
        if (!out || (int)rec.size() > cap) return tomo::fail(TOMO_EINVAL, "blocking buffer too small");
        std::copy(rec.begin(), rec.end(), out);
        return (int)(rec.size() / 4);
    });
}

// Internal test hook (not part of the public ABI): the work items the engine
// launches for one solve of an nx x ny grid cut into nseg row segments, as
// (x0, x1, narrow, y0, y1) records, after the same host validation.  Returns
// the item count, or a negative status.
extern "C" int tomo_internal_work_items(int nx, int ny, int ncpml, int d, int T, int cols, int nseg, int* out,
                                        int cap) {
    return tomo::guarded([&]() -> int {
        std::vector<tomo::WorkItem> items;
        tomo::append_items(items, 0, 1, nx, ny, ncpml, d, T, cols, nseg);
        TOMO_TRY(tomo::validate_items(items, 0, nx, ny, ncpml, d, T, cols));
        if (!out || (int)items.size() > cap) return tomo::fail(TOMO_EINVAL, "item buffer too small");
        for (size_t i = 0; i < items.size(); ++i) {
            const tomo::WorkItem& w = items[i];
            const int rec[5] = {w.x0, w.x1, w.narrow, w.y0, w.y1};
            for (int j = 0; j < 5; ++j) out[5 * i + j] = rec[j];
        }
        return (int)items.size();
    });
}
