/*
 * CPU oracle for the 2D TMz FDTD forward solve: a plain-C restatement of the
 * reference algorithm, used ONLY as the checker by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  The product
 * never links, imports or executes anything in this directory.
 *
 * Compiled twice (oracle/build.py): ORACLE_REAL=double -> liboracle64.so (the
 * FP64 oracle) and ORACLE_REAL=float -> liboracle32.so (a port in the
 * reference's own precision, used for the reported CPU baseline).
 *
 * Reference files (travisdesell/tomography):
 *   FDTD_GPU.cu   H_field_update :298-355, E_field_update :358-434,
 *                 calculate_JandM :231-280, fwf :283-296, N2FPostProcess :553-634,
 *                 material/coefficients :718-743,1112-1122, CPML :748-806,
 *                 misfit :1004-1022
 *   FDTD_CPU.cxx  the same algorithm on the host (:146-373, :538-614, :893-1479),
 *                 relative misfit :841-845, point-current coefficient :972-983
 *   FDTD_common.cxx  contour index maps :4-46, incident power :48-51
 *   oldFDTD_GPU.cu   total-field variant: H_inc_update :425-482, E_inc_update
 *                 :655-717, calculate_JandM_total :762-824
 */
#ifndef TOMO_FDTD_ORACLE_H
#define TOMO_FDTD_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* per-material coefficient table columns */
enum {
    OR_CA = 0, /* Ceze   : Ez self coefficient                         */
    OR_CB = 1, /* Cezh   : curl-H coefficient (2dt/dx)/(2e0einf+sdt+b) */
    OR_CJ = 2, /* Cezjp  : polarisation-current coefficient            */
    OR_BP = 3, /* Beta_p/dt                                            */
    OR_CI = 4, /* Cezeic : incident-field coefficient at n+1/2         */
    OR_CP = 5, /* Cezeip : incident-field coefficient at n-1/2         */
    OR_CS = 6, /* Cezj   : point current-source coefficient            */
    ORACLE_NCOEF = 8
};

enum {
    ORACLE_REF_CPML = 1,   /* reference E-update strip semantics (FDTD_GPU.cu:389-416) */
    ORACLE_NAN_CLAMP = 2,  /* NaN -> 0 after each update (FDTD_GPU.cu:335-350,425-430) */
    ORACLE_PLANE_WAVE = 4, /* scattered-field plane-wave source (FDTD_GPU.cu:380-385)  */
    ORACLE_M_LAG = 8,      /* M phasor at (n - 1/2) dt (oldFDTD_GPU.cu:783,794,805,816)
                              instead of (n + 1/2) dt (FDTD_GPU.cu:253-276)           */
    ORACLE_TOTAL_FIELD = 16 /* legacy total-field NTFF (implies ORACLE_M_LAG): an
                              incident vacuum grid advanced after the main grid each
                              step, its fields added to the contour samples           */
};

typedef struct oracle_problem {
    int nx, ny;            /* H grid nx*ny, Ez grid (nx+1)*(ny+1), row-major x + y*stride */
    int steps, ncpml;
    int flags, nmat;
    double dx, dt;
    double chez;           /* dt/(mu0 dx)                                   */
    double Kp;             /* Debye recursion coefficient                   */
    const double *cpml;    /* [6][ncpml]: ke, be, ae (E), km, bm, am (H)    */
    const unsigned char *mat; /* (nx+1)*(ny+1); low 7 bits = material index */
    const double *mtab;    /* [nmat][ORACLE_NCOEF]                          */
    /* plane wave: g(t,x,y) = exp(-ar^2/tau^2),
       ar = t dt - t0 - (ky (y-yoff) dx + kx (x-xoff) dx - l)/c0            */
    double pw_kx, pw_ky, pw_xoff, pw_yoff, pw_t0, pw_tau, pw_l, pw_c0;
    /* point source: Ez += Cs(mat) * src_wave[n] at (src_x, src_y)         */
    int src_x, src_y;
    const double *src_wave;
    /* receivers: traces[r*steps + n] = Ez(rx[2r], rx[2r+1]) after step n  */
    int nrx;
    const int *rx;
    double *traces;
    /* running DFT on the contour at distance nf_d from the edge           */
    int nf_d, nfreq;
    const double *freqs;
    double *acc;           /* [nfreq][C][4]: J re, J im, M re, M im          */
    /* optional final state */
    double *ez_out, *hx_out, *hy_out, *jp_out;
    /* total field (ORACLE_TOTAL_FIELD; oldFDTD_GPU.cu:425-482,655-717,762-824):
       the incident grid has the main grid's size and CPML, Ceze = 1 and
       Cezhy = dt/(dx eps0), no Debye current, and inc_wave[n] added to its Ez at
       (inc_x, inc_y) in step n before the strip overrides (the legacy adds
       100 Cezj fwf(n) at the grid centre).  The contour samples become
       H + H_inc and face-avg(Ez) + (face-avg(Ez_inc(n)) + face-avg(Ez_inc(n-1)))/2,
       summed with J at n dt and M at (n - 1/2) dt.                              */
    int inc_x, inc_y;
    const double *inc_wave;   /* [steps] */
    /* optional: the incident grid's share of acc on its own, with its two-level
       time average folded into the M phasor: q(n) = (p(n) + p(n+1))/2, p(S) = 0.
       acc(total) = acc(main grid alone, ORACLE_M_LAG) + inc_acc.               */
    double *inc_acc;          /* [nfreq][C][4] */
} oracle_problem;

/* one forward solve; returns 0 on success, -1 on bad input */
int oracle_solve(const oracle_problem *p);
/* many independent solves on up to nthreads host threads; returns 0 or the first error */
int oracle_solve_many(const oracle_problem *probs, int n, int nthreads);

/* NTFF contour: size and index -> (x, y, face) with face 0=yn 1=xp 2=yp 3=xn */
int oracle_contour_size(int nx, int ny, int d);
void oracle_contour_point(int nx, int ny, int d, int index, int *x, int *y, int *face);

/* Far field from the DFT accumulators, D/P laid out [nfreq][nangle], in a
   background of refractive index nbg (k = nbg k0, eta = eta0 / nbg; 1 for the
   reference's vacuum):
   norm = 0: D = k^2 |L + eta N|^2 / (8 pi eta)
   norm = 1: reference normalisation, additionally / (Prad(f) * 33.329)   */
void oracle_far_field(int nx, int ny, int d, double dx, int nfreq, const double *freqs, const double *acc,
                      int nangle, int norm, double tau, double nbg, double *D, double *P);

/* CPML profile (FDTD_GPU.cu:748-806), out = [6][ncpml] as in oracle_problem */
void oracle_cpml_profile(int ncpml, double grading, double sigma_max, double kappa_max, double alpha_max,
                         double alpha_min, double dx, double dt, double *out);

/* per-material coefficients (FDTD_GPU.cu:739-741, 1112-1122; FDTD_CPU.cxx:972-983) */
void oracle_material_coefs(double eps_inf, double del_eps, double sigma, double tau, double dt, double dx,
                           double *out /* ORACLE_NCOEF */, double *Kp);

/* reference patch map: circle of radius br about the grid centre split in
   npatch x npatch patches (FDTD_GPU.cu:544-551,718-743; FDTD_CPU.cxx:530-537,
   1078-1164).  mat = 0 outside, 1 + patch inside. */
void oracle_patch_map(int nx, int ny, double dx, double br, int npatch, unsigned char *mat);

/* ellipse phantom: background 0, optional disc (radius > 0) = 1, ellipse k = 2+k
   drawn in order; ell = [k][6] (cx, cy, a, b, cos, sin) in metres. */
void oracle_ellipse_map(int nx, int ny, double dx, double disc_radius, int nell, const double *ell,
                        unsigned char *mat);

#ifdef __cplusplus
}
#endif
#endif
