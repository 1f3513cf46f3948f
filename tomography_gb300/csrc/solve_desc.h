// Per-solve descriptor shared by the host engine and the device kernels.
//
// One "solve" is one forward FDTD run: one candidate material model driven by
// one excitation (a plane-wave angle in the reference modes, one transmitter
// antenna in the breast-imaging mode).  The advance kernel is descriptor
// driven: a launch advances every listed solve by up to T time steps, so
// solves of different grid sizes, candidates and progress can share a launch.
//
// Field layout in HBM (per solve, two ping-pong copies of each field):
//   rows y = 0..ny (ny+1 rows), row pitch `pitch` elements, element (x, y) at
//   base[x + y*pitch] with x = 0..nx; the base pointer is offset by kPadLeft
//   elements from the allocation so that the strip halo (x < 0) and the right
//   tail (x > nx) read zero padding.  Ez uses all (nx+1) x (ny+1) points, Hx and
//   Hy use x < nx, y < ny (the rest stays zero), exactly the reference's
//   (nx+1)^2 / nx^2 grids of FDTD_GPU.cu:880-884.
#pragma once
#include <stdint.h>

namespace tomo {

constexpr int kPadLeft = 32;     // elements of zero padding left of x = 0
constexpr int kPadRight = 160;   // elements of zero padding right of x = nx
constexpr int kMatPadLeft = 32;  // bytes of padding left of x = 0 in every material row
constexpr int kMaxMat = 128;     // material indices per solve (7 bits)
constexpr int kMatCoef = 8;      // coefficient columns, see MatCol
constexpr int kMaxRx = 64;
constexpr int kMaxCpml = 32;     // CPML cells per side (the profile lives in shared memory)

enum SolveFlags : int {
    kRefCpml = 1,     // reference E-update strip semantics (FDTD_GPU.cu:389-416)
    kNanClamp = 2,    // NaN -> 0 after each update (FDTD_GPU.cu:335-350, 425-430)
    kPlaneWave = 4,   // scattered-field plane-wave source (FDTD_GPU.cu:380-385)
    kPointSource = 8  // soft current source at (src_x, src_y)
};

enum MatCol : int { kCa = 0, kCb = 1, kCj = 2, kBp = 3, kCi = 4, kCp = 5, kCs = 6 };

enum MatBits : uint8_t { kMatMask = 0x7f, kMatRx = 0x80 };

template <typename Real>
struct SolveDesc {
    // geometry and progress
    int nx, ny, pitch, mpitch;   // field row pitch (elements), material row pitch (bytes)
    int ncpml, steps_total;
    int step;                    // index of the next time step to compute
    int parity;                  // which ping-pong copy holds the current state
    int flags;
    int nrx;
    int nf_d, nfreq, n_contour;  // NTFF contour distance, frequencies, contour points
    int src_x, src_y;
    int jx0, jx1, jy0, jy1;      // dispersive bounding box (Jp may be non-zero only inside)
    int psi_stride;              // elements per psi time copy
    int active;                  // 0: skip this solve
    int nmat;                    // materials in use: indices 0 .. nmat-1 of mtab
    int stage_group;             // launches that fill the contour staging buffer before one DFT pass
    Real chez;                   // dt/(mu0 dx)
    Real Kp;                     // Debye recursion coefficient
    Real dx;
    // state (ping-pong)
    Real* ez[2];
    Real* hx[2];
    Real* hy[2];
    Real* jp[2];
    Real* psi[2];                // persistent CPML psi copies (current / next)
    Real* psi_scratch;           // (T-1) intermediate copies for temporal blocking
    // inputs
    const uint8_t* mat;          // material index + receiver flag of (x, y) at mat[x + y*mpitch];
                                 // rows are padded (kMatPadLeft bytes left of x = 0)
    const Real* mtab;            // [kMaxMat][kMatCoef]
    const Real* cpml;            // [6][ncpml]: 1/ke, be, ae, 1/km, bm, am (index 0 innermost)
    const Real* src_wave;        // [steps_total] current-source waveform at (n+1/2) dt
    const int* rx;               // [nrx][2]
    Real* traces;                // [nrx][steps_total]
    const Real* phasor;          // [steps_total][nfreq][4]: dt*exp(-jwn dt), dt*exp(-jw(n+1/2)dt)
    Real* acc;                   // [nfreq][n_contour][8]: J sum re/im, J comp re/im, M sum, M comp
    Real* stage;                 // [8][n_contour][2]: (h, e) contour samples of the levels of the last
                                 // stage_group advance launches, summed into acc by the DFT kernel
    // plane wave (reference modes): g = exp(-(ar/tau)^2),
    // ar = (t dt - t0 + l/c0) - (ky (y - yoff) + kx (x - xoff)) dx/c0
    double pw_kx, pw_ky, pw_xoff, pw_yoff, pw_t0l, pw_inv_tau, pw_dxc0, dt;
};

}  // namespace tomo
