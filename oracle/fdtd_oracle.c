/*
 * CPU oracle (checker only) -- see fdtd_oracle.h for the scope statement and
 * the reference line map.  ORACLE_REAL selects the field precision.
 */
#include "fdtd_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#ifndef ORACLE_REAL
#define ORACLE_REAL double
#endif
typedef ORACLE_REAL real;

#define PI_D 3.141592653589793238
#define MU0_D (PI_D * 4e-7)
#define EPS0_D 8.85418e-12

/* ---------------------------------------------------------------- contour */
/* FDTD_common.cxx:4-46 (CPUgetx/yfromthreadIdNF2FF) and the face predicates
   FDTD_GPU.cu:182-228: faces in index order yn, xp, yp, xn. */
int oracle_contour_size(int nx, int ny, int d) { return 2 * nx + 2 * ny - 8 * d - 4; }

void oracle_contour_point(int nx, int ny, int d, int index, int *x, int *y, int *face) {
    int l1 = nx - 2 * d - 2;           /* yn count            */
    int l2 = l1 + (ny - 2 * d);        /* + xp count          */
    int l3 = l2 + l1;                  /* + yp count          */
    if (index < l1) { *x = index + d + 1; *y = d; *face = 0; }
    else if (index < l2) { *x = nx - d - 1; *y = index - l1 + d; *face = 1; }
    else if (index < l3) { *x = nx - d - 2 - (index - l2); *y = ny - d - 1; *face = 2; }
    else { *x = d; *y = ny - d - 1 - (index - l3); *face = 3; }
}

/* ------------------------------------------------------------ precompute */
void oracle_cpml_profile(int nc, double m, double sigma_max, double kappa_max, double alpha_max, double alpha_min,
                         double dx, double dt, double *out) {
    /* FDTD_GPU.cu:752-794: E-profile at rho=(i+0.25)/nc, H-profile at (i+0.75)/nc,
       index 0 innermost. */
    double *ke = out, *be = out + nc, *ae = out + 2 * nc, *km = out + 3 * nc, *bm = out + 4 * nc,
           *am = out + 5 * nc;
    for (int i = 0; i < nc; ++i) {
        double rho = (i + 0.25) / nc;
        double se = sigma_max * pow(rho, m);
        ke[i] = pow(rho, m) * (kappa_max - 1) + 1;
        double ale = alpha_min + (alpha_max - alpha_min) * rho;
        be[i] = exp(-(dt / EPS0_D) * (se / ke[i] + ale));
        ae[i] = ((be[i] - 1) * se) / (dx * (se * ke[i] + ale * ke[i] * ke[i]));
        rho = (i + 0.75) / nc;
        double sm = (MU0_D / EPS0_D) * sigma_max * pow(rho, m);
        km[i] = pow(rho, m) * (kappa_max - 1) + 1;
        double alm = (MU0_D / EPS0_D) * (alpha_min + (alpha_max - alpha_min) * rho);
        bm[i] = exp(-(dt / MU0_D) * (sm / km[i] + alm));
        am[i] = (bm[i] - 1) * sm / (dx * (sm * km[i] + alm * km[i] * km[i]));
    }
}

void oracle_material_coefs(double eps_inf, double del_eps, double sigma, double tau, double dt, double dx,
                           double *out, double *Kp) {
    /* FDTD_common.hxx:59 (Kp), FDTD_GPU.cu:739-741 (Beta_p, Cezhy, Ceze),
       FDTD_GPU.cu:1118-1120 (Cezeic, Cezeip, Cezjp), FDTD_CPU.cxx:979 (Cezj). */
    double kp = (1 - dt / (2 * tau)) / (1 + dt / (2 * tau));
    double beta = EPS0_D * del_eps * dt / (tau * (1 + dt / (2 * tau)));
    double den = 2 * eps_inf * EPS0_D + sigma * dt + beta;
    for (int c = 0; c < ORACLE_NCOEF; ++c) out[c] = 0.0;
    out[OR_CA] = (2 * eps_inf * EPS0_D - sigma * dt + beta) / den;
    out[OR_CB] = (2 * dt / dx) / den;
    out[OR_CJ] = ((1 + kp) * dt) / den;
    out[OR_BP] = beta / dt;
    out[OR_CI] = (-2 * EPS0_D * eps_inf + 2 * EPS0_D - sigma * dt - beta) / den;
    out[OR_CP] = (2 * EPS0_D * eps_inf - 2 * EPS0_D - sigma * dt + beta) / den;
    out[OR_CS] = (-2 * dt) / den;
    if (Kp) *Kp = kp;
}

void oracle_patch_map(int nx, int ny, double dx, double br, int npatch, unsigned char *mat) {
    /* circle test FDTD_GPU.cu:724-727 (radius kept as float as in the
       reference), patch index FDTD_GPU.cu:544-551 / FDTD_CPU.cxx:530-537. */
    double cell = 2 * br / (npatch * dx);
    for (int j = 0; j <= ny; ++j)
        for (int i = 0; i <= nx; ++i) {
            double rx = ((float)i - nx / 2) * dx, ry = ((float)j - ny / 2) * dx;
            float radius = (float)sqrt(rx * rx + ry * ry);
            unsigned char m = 0;
            if (radius <= br) {
                int xc = (int)((double)(i - (nx / 2 - (int)(br / dx))) / cell);
                int yc = (int)((j - (ny / 2 - br / dx)) / cell);
                m = (unsigned char)(1 + xc + npatch * yc);
            }
            mat[i + j * (nx + 1)] = m;
        }
}

void oracle_ellipse_map(int nx, int ny, double dx, double disc_radius, int nell, const double *ell,
                        unsigned char *mat) {
    /* Phantom rasterisation of the ellipse parameterisation.  The operation
       order is fixed and compiled without contraction so that the device
       rasteriser (explicit _rn intrinsics) produces the identical map. */
    double r2 = disc_radius * disc_radius;
    for (int j = 0; j <= ny; ++j)
        for (int i = 0; i <= nx; ++i) {
            double X = ((double)i - 0.5 * (double)nx) * dx;
            double Y = ((double)j - 0.5 * (double)ny) * dx;
            unsigned char m = 0;
            if (disc_radius > 0 && X * X + Y * Y <= r2) m = 1;
            for (int k = 0; k < nell; ++k) {
                const double *e = ell + 6 * k;
                double ex = X - e[0], ey = Y - e[1];
                double u = ex * e[4] + ey * e[5];
                double v = ey * e[4] - ex * e[5];
                double q = (u * u) / (e[2] * e[2]) + (v * v) / (e[3] * e[3]);
                if (q <= 1.0) m = (unsigned char)(2 + k);
            }
            mat[i + j * (nx + 1)] = m;
        }
}

/* ------------------------------------------------------------------ solve */
static double pw_g(const oracle_problem *p, double t, int x, int y) {
    /* fwf, FDTD_GPU.cu:283-296 */
    double xx = x - p->pw_xoff, yy = y - p->pw_yoff;
    double ar = t * p->dt - p->pw_t0 - (p->pw_ky * yy * p->dx + p->pw_kx * xx * p->dx - p->pw_l) / p->pw_c0;
    return exp(-ar * ar / (p->pw_tau * p->pw_tau));
}

static real nan_clamp(real v) { return isnan(v) ? (real)0 : v; }

/* H update of one grid (FDTD_GPU.cu:298-355; oldFDTD_GPU.cu:425-482 runs the
   same update on the incident grid) */
static void h_update(int nx, int ny, int nc, real chez, real dxr, const real *km, const real *bm, const real *am,
                     int clampnan, const real *Ez, real *Hx, real *Hy, real *phyx, real *phxy) {
    const int se = nx + 1, sh = nx;
    for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
            const size_t h = (size_t)x + (size_t)y * sh, e = (size_t)x + (size_t)y * se;
            real dEy = Ez[e + 1] - Ez[e];
            real dEx = Ez[e + se] - Ez[e];
            real hy = Hy[h] + chez * dEy;
            real hx = Hx[h] - chez * dEx;
            int ix = x < nc ? nc - 1 - x : (x >= nx - nc ? x - nx + nc : -1);
            if (ix >= 0) {
                hy = Hy[h] + chez * dEy / km[ix];
                phyx[h] = bm[ix] * phyx[h] + am[ix] * dEy;
                hy += chez * dxr * phyx[h];
            }
            int iy = y < nc ? nc - 1 - y : (y >= ny - nc ? y - ny + nc : -1);
            if (iy >= 0) {
                hx = Hx[h] - chez * dEx / km[iy];
                phxy[h] = bm[iy] * phxy[h] + am[iy] * dEx;
                hx -= chez * dxr * phxy[h];
            }
            if (clampnan) { hx = nan_clamp(hx); hy = nan_clamp(hy); }
            Hx[h] = hx;
            Hy[h] = hy;
        }
}

/* E update of the incident vacuum grid (oldFDTD_GPU.cu:655-717): Ceze = 1,
   Cezhy = cb, the source added at (sx, sy) before the CPML strip branches,
   which overwrite the interior value as written; Ezp keeps the previous level. */
static void e_update_incident(int nx, int ny, int nc, real cb, real dxr, const real *ke, const real *be,
                              const real *ae, int sx, int sy, real src, const real *Hx, const real *Hy, real *Ez,
                              real *Ezp, real *pezx, real *pezy) {
    const int se = nx + 1, sh = nx;
    for (int y = 0; y <= ny; ++y)
        for (int x = 0; x <= nx; ++x) {
            const size_t e = (size_t)x + (size_t)y * se;
            real out = 0;
            if (!(x == 0 || y == 0 || x == nx || y == ny)) {
                const size_t h = (size_t)x + (size_t)y * sh;
                real dHy = Hy[h] - Hy[h - 1];
                real dHx = Hx[h] - Hx[h - sh];
                real ez = Ez[e];
                out = ez + cb * dHy - cb * dHx;
                if (x == sx && y == sy) out = out + src;
                if (x <= nc) {
                    int i = nc - x;
                    out = ez + cb * dHy / ke[i] - cb * dHx / ke[i];
                    pezx[e] = be[i] * pezx[e] + ae[i] * dHy;
                    out += cb * dxr * pezx[e];
                }
                if (x >= nx - nc) {
                    int i = x - nx + nc;
                    out = ez + cb * dHy / ke[i] - cb * dHx / ke[i];
                    pezx[e] = be[i] * pezx[e] + ae[i] * dHy;
                    out += cb * dxr * pezx[e];
                }
                if (y <= nc) {
                    int i = nc - y;
                    out = ez + cb * dHy / ke[i] - cb * dHx / ke[i];
                    pezy[e] = be[i] * pezy[e] + ae[i] * dHx;
                    out -= cb * dxr * pezy[e];
                }
                if (y >= ny - nc) {
                    int i = y - ny + nc;
                    out = ez + cb * dHy / ke[i] - cb * dHx / ke[i];
                    pezy[e] = be[i] * pezy[e] + ae[i] * dHx;
                    out -= cb * dxr * pezy[e];
                }
            }
            Ezp[e] = Ez[e];
            Ez[e] = out;
        }
}

int oracle_solve(const oracle_problem *p) {
    const int nx = p->nx, ny = p->ny, nc = p->ncpml, S = p->steps;
    if (nx < 4 || ny < 4 || S < 0 || nc < 0 || 2 * nc >= nx || 2 * nc >= ny || p->nmat < 1 || p->nmat > 128)
        return -1;
    const int se = nx + 1, sh = nx; /* row strides of Ez and H arrays */
    const size_t nE = (size_t)(nx + 1) * (ny + 1), nH = (size_t)nx * ny;
    real *Ez = calloc(nE, sizeof(real)), *Jp = calloc(nE, sizeof(real));
    real *Hx = calloc(nH, sizeof(real)), *Hy = calloc(nH, sizeof(real));
    real *pezx = calloc(nE, sizeof(real)), *pezy = calloc(nE, sizeof(real));
    real *phyx = calloc(nH, sizeof(real)), *phxy = calloc(nH, sizeof(real));
    real tab[128][ORACLE_NCOEF];
    real prof[6][64];
    const int total = (p->flags & ORACLE_TOTAL_FIELD) != 0;
    const int mlag = total || (p->flags & ORACLE_M_LAG) != 0;
    /* incident grid (total field): Ez now / previous level, H, psi */
    real *Ezi = NULL, *Ezip = NULL, *Hxi = NULL, *Hyi = NULL, *pezxi = NULL, *pezyi = NULL, *phyxi = NULL,
         *phxyi = NULL;
    if (total) {
        Ezi = calloc(nE, sizeof(real)); Ezip = calloc(nE, sizeof(real));
        pezxi = calloc(nE, sizeof(real)); pezyi = calloc(nE, sizeof(real));
        Hxi = calloc(nH, sizeof(real)); Hyi = calloc(nH, sizeof(real));
        phyxi = calloc(nH, sizeof(real)); phxyi = calloc(nH, sizeof(real));
    }
    if (!Ez || !Jp || !Hx || !Hy || !pezx || !pezy || !phyx || !phxy || nc > 64 ||
        (total && (!Ezi || !Ezip || !Hxi || !Hyi || !pezxi || !pezyi || !phyxi || !phxyi || !p->inc_wave))) {
        free(Ez); free(Jp); free(Hx); free(Hy); free(pezx); free(pezy); free(phyx); free(phxy);
        free(Ezi); free(Ezip); free(Hxi); free(Hyi); free(pezxi); free(pezyi); free(phyxi); free(phxyi);
        return -1;
    }
    for (int m = 0; m < p->nmat; ++m)
        for (int c = 0; c < ORACLE_NCOEF; ++c) tab[m][c] = (real)p->mtab[m * ORACLE_NCOEF + c];
    for (int a = 0; a < 6; ++a)
        for (int i = 0; i < nc; ++i) prof[a][i] = (real)p->cpml[a * nc + i];
    const real *ke = prof[0], *be = prof[1], *ae = prof[2], *km = prof[3], *bm = prof[4], *am = prof[5];
    const real chez = (real)p->chez, Kp = (real)p->Kp, dxr = (real)p->dx;
    const int ref = (p->flags & ORACLE_REF_CPML) != 0, clampnan = (p->flags & ORACLE_NAN_CLAMP) != 0;
    const int pw = (p->flags & ORACLE_PLANE_WAVE) != 0;
    const int C = p->nfreq > 0 ? oracle_contour_size(nx, ny, p->nf_d) : 0;
    if (p->nfreq > 0) memset(p->acc, 0, sizeof(double) * 4 * (size_t)C * p->nfreq);
    if (total && p->nfreq > 0 && p->inc_acc) memset(p->inc_acc, 0, sizeof(double) * 4 * (size_t)C * p->nfreq);
    const real cbi = (real)(p->dt / (p->dx * EPS0_D));   /* Cezhy of vacuum */

    for (int n = 0; n < S; ++n) {
        /* ---- H update (FDTD_GPU.cu:298-355) */
        h_update(nx, ny, nc, chez, dxr, km, bm, am, clampnan, Ez, Hx, Hy, phyx, phxy);
        /* ---- E update (FDTD_GPU.cu:358-434) */
        for (int y = 0; y <= ny; ++y)
            for (int x = 0; x <= nx; ++x) {
                const size_t e = (size_t)x + (size_t)y * se;
                if (x == 0 || y == 0 || x == nx || y == ny) { Ez[e] = 0; continue; }
                const size_t h = (size_t)x + (size_t)y * sh;
                const real *cf = tab[p->mat[e] & 127];
                real dHy = Hy[h] - Hy[h - 1];
                real dHx = Hx[h] - Hx[h - sh];
                real gp = 0, gm = 0;
                if (pw && (cf[OR_CI] != 0 || cf[OR_CP] != 0 || cf[OR_BP] != 0)) {
                    gp = (real)pw_g(p, n + 0.5, x, y);
                    gm = (real)pw_g(p, n - 0.5, x, y);
                }
                int ix = (x >= 1 && x <= nc) ? nc - x : ((x >= nx - nc && x <= nx - 1) ? x - nx + nc : -1);
                int iy = (y >= 1 && y <= nc) ? nc - y : ((y >= ny - nc && y <= ny - 1) ? y - ny + nc : -1);
                real ez = Ez[e], out;
                if (ref) {
                    out = cf[OR_CA] * ez + cf[OR_CB] * dHy - cf[OR_CB] * dHx + cf[OR_CI] * gp + cf[OR_CP] * gm -
                          cf[OR_CJ] * Jp[e];
                    Jp[e] = Kp * Jp[e] + cf[OR_BP] * (out - ez + gp - gm);
                    if (ix >= 0) {
                        out = cf[OR_CA] * ez + cf[OR_CB] * dHy / ke[ix] - cf[OR_CB] * dHx / ke[ix];
                        pezx[e] = be[ix] * pezx[e] + ae[ix] * dHy;
                        out += cf[OR_CB] * dxr * pezx[e];
                    }
                    if (iy >= 0) {
                        out = cf[OR_CA] * ez + cf[OR_CB] * dHy / ke[iy] - cf[OR_CB] * dHx / ke[iy];
                        pezy[e] = be[iy] * pezy[e] + ae[iy] * dHx;
                        out -= cf[OR_CB] * dxr * pezy[e];
                    }
                } else {
                    real cx = dHy, cy = dHx, px = 0, py = 0;
                    if (ix >= 0) {
                        cx = dHy / ke[ix];
                        pezx[e] = be[ix] * pezx[e] + ae[ix] * dHy;
                        px = pezx[e];
                    }
                    if (iy >= 0) {
                        cy = dHx / ke[iy];
                        pezy[e] = be[iy] * pezy[e] + ae[iy] * dHx;
                        py = pezy[e];
                    }
                    out = cf[OR_CA] * ez + cf[OR_CB] * ((cx - cy) + dxr * (px - py)) + cf[OR_CI] * gp +
                          cf[OR_CP] * gm - cf[OR_CJ] * Jp[e];
                    if (x == p->src_x && y == p->src_y && p->src_wave) out += cf[OR_CS] * (real)p->src_wave[n];
                    Jp[e] = Kp * Jp[e] + cf[OR_BP] * (out - ez + gp - gm);
                }
                if (clampnan) out = nan_clamp(out);
                Ez[e] = out;
            }
        /* ---- receivers */
        for (int r = 0; r < p->nrx; ++r)
            p->traces[(size_t)r * S + n] = (double)Ez[p->rx[2 * r] + (size_t)p->rx[2 * r + 1] * se];
        /* ---- incident grid (total field): H then E, after the main grid
           (oldFDTD_GPU.cu:425-482, 655-717) */
        if (total) {
            h_update(nx, ny, nc, chez, dxr, km, bm, am, clampnan, Ezi, Hxi, Hyi, phyxi, phxyi);
            e_update_incident(nx, ny, nc, cbi, dxr, ke, be, ae, p->inc_x, p->inc_y, (real)p->inc_wave[n], Hxi, Hyi,
                              Ezi, Ezip, pezxi, pezyi);
        }
        /* ---- running DFT on the contour (FDTD_GPU.cu:231-280; total field
           oldFDTD_GPU.cu:762-824 with the M phasor at (n - 1/2) dt) */
        for (int f = 0; f < p->nfreq; ++f) {
            double w = 2 * PI_D * p->freqs[f];
            double tm = mlag ? n - 0.5 : n + 0.5;
            double pjr = cos(w * n * p->dt), pji = -sin(w * n * p->dt);
            double pmr = cos(w * tm * p->dt), pmi = -sin(w * tm * p->dt);
            double *a = p->acc + (size_t)f * C * 4;
            /* the incident share alone: M phasor folded over the two levels */
            double qmr = 0.5 * pmr, qmi = 0.5 * pmi;
            if (n + 1 < S) {
                qmr += 0.5 * cos(w * (tm + 1) * p->dt);
                qmi += -0.5 * sin(w * (tm + 1) * p->dt);
            }
            double *ia = (total && p->inc_acc) ? p->inc_acc + (size_t)f * C * 4 : NULL;
            for (int c = 0; c < C; ++c) {
                int x, y, face;
                oracle_contour_point(nx, ny, p->nf_d, c, &x, &y, &face);
                const size_t e = (size_t)x + (size_t)y * se, h = (size_t)x + (size_t)y * sh;
                real ez, hv;
                double s;
                if (face == 0) { ez = (Ez[e] + Ez[e + se]) / 2; hv = Hx[h]; s = 1; }
                else if (face == 1) { ez = (Ez[e] + Ez[e + 1]) / 2; hv = Hy[h]; s = 1; }
                else if (face == 2) { ez = (Ez[e + se] + Ez[e]) / 2; hv = Hx[h]; s = -1; }
                else { ez = (Ez[e] + Ez[e + 1]) / 2; hv = Hy[h]; s = -1; }
                if (total) {
                    /* oldFDTD_GPU.cu:781-782, 789-790, 799-800, 808-809 */
                    const size_t e2 = (face == 0 || face == 2) ? e + se : e + 1;
                    real hi = (face == 0 || face == 2) ? Hxi[h] : Hyi[h];
                    real eia = (Ezi[e2] + Ezi[e] + Ezip[e2] + Ezip[e]) / 4;
                    if (ia) {
                        double ji = s * (double)hi * p->dt, mi = s * (double)((Ezi[e] + Ezi[e2]) / 2) * p->dt;
                        ia[4 * c + 0] += ji * pjr;
                        ia[4 * c + 1] += ji * pji;
                        ia[4 * c + 2] += mi * qmr;
                        ia[4 * c + 3] += mi * qmi;
                    }
                    ez = ez + eia;
                    hv = hv + hi;
                }
                double jv = s * (double)hv * p->dt, mv = s * (double)ez * p->dt;
                a[4 * c + 0] += jv * pjr;
                a[4 * c + 1] += jv * pji;
                a[4 * c + 2] += mv * pmr;
                a[4 * c + 3] += mv * pmi;
            }
        }
    }
    if (p->ez_out) for (size_t i = 0; i < nE; ++i) p->ez_out[i] = Ez[i];
    if (p->jp_out) for (size_t i = 0; i < nE; ++i) p->jp_out[i] = Jp[i];
    if (p->hx_out) for (size_t i = 0; i < nH; ++i) p->hx_out[i] = Hx[i];
    if (p->hy_out) for (size_t i = 0; i < nH; ++i) p->hy_out[i] = Hy[i];
    free(Ez); free(Jp); free(Hx); free(Hy); free(pezx); free(pezy); free(phyx); free(phxy);
    free(Ezi); free(Ezip); free(Hxi); free(Hyi); free(pezxi); free(pezyi); free(phyxi); free(phxyi);
    return 0;
}

typedef struct {
    const oracle_problem *probs;
    int n, next, err;
    pthread_mutex_t lock;
} pool_t;

static void *pool_worker(void *arg) {
    pool_t *pool = (pool_t *)arg;
    for (;;) {
        pthread_mutex_lock(&pool->lock);
        int i = pool->next++;
        pthread_mutex_unlock(&pool->lock);
        if (i >= pool->n) return NULL;
        int rc = oracle_solve(&pool->probs[i]);
        if (rc) {
            pthread_mutex_lock(&pool->lock);
            if (!pool->err) pool->err = rc;
            pthread_mutex_unlock(&pool->lock);
        }
    }
}

int oracle_solve_many(const oracle_problem *probs, int n, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > n) nthreads = n;
    if (nthreads > 256) nthreads = 256;
    pool_t pool = {probs, n, 0, 0, PTHREAD_MUTEX_INITIALIZER};
    pthread_t th[256];
    for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, pool_worker, &pool);
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    return pool.err;
}

/* ------------------------------------------------------------- far field */
void oracle_far_field(int nx, int ny, int d, double dx, int nfreq, const double *freqs, const double *acc,
                      int nangle, int norm, double tau, double nbg, double *D, double *P) {
    /* N2FPostProcess, FDTD_GPU.cu:553-634; calc_incident_power FDTD_common.cxx:48-51.
       The reference transforms in vacuum (nbg = 1); the breast mode's contour
       lies in its lossless background, whose wavenumber and impedance are
       nbg k0 and eta0 / nbg. */
    const double c0 = 1.0 / sqrt(MU0_D * EPS0_D), eta0 = sqrt(MU0_D / EPS0_D), eta = eta0 / nbg;
    const int C = oracle_contour_size(nx, ny, d);
    const double cxo = nx / 2.0 - 1, cyo = ny / 2.0 - 1;
    for (int f = 0; f < nfreq; ++f) {
        const double fr = freqs[f], k = 2 * PI_D * fr * nbg / c0;
        const double *a = acc + (size_t)f * C * 4;
        double prad = 1.0;
        if (norm == 1) {
            double g = tau * sqrt(PI_D) * exp(-tau * tau * 2 * PI_D * fr * 2 * PI_D * fr / 4);
            prad = (0.5 / eta0) * g * g * 33.329;
        }
        for (int ai = 0; ai < nangle; ++ai) {
            double phi = 2 * PI_D / nangle * ai, sphi = sin(phi), cphi = cos(phi);
            double Nr = 0, Ni = 0, Lr = 0, Li = 0;
            for (int c = 0; c < C; ++c) {
                int x, y, face;
                oracle_contour_point(nx, ny, d, c, &x, &y, &face);
                double flx = x, fly = y;
                if (face == 0 || face == 2) fly += 0.5; else flx += 0.5;
                double rx = flx - cxo, ry = fly - cyo;
                double rho = sqrt((dx * rx) * (dx * rx) + (dx * ry) * (dx * ry));
                double psi = atan2(ry, rx) - phi;
                double ph = k * rho * cos(psi), er = cos(ph), ei = sin(ph);
                double jr = a[4 * c], ji = a[4 * c + 1], mr = a[4 * c + 2], mi = a[4 * c + 3];
                /* N += -J e dl ; L += w M e dl, w = -sin(phi) (y faces) or cos(phi) (x faces) */
                double wt = (face == 0 || face == 2) ? -sphi : cphi;
                Nr += -(jr * er - ji * ei) * dx;
                Ni += -(jr * ei + ji * er) * dx;
                Lr += wt * (mr * er - mi * ei) * dx;
                Li += wt * (mr * ei + mi * er) * dx;
            }
            double Er = Lr + eta * Nr, Ei = Li + eta * Ni;
            D[(size_t)f * nangle + ai] = k * k * (Er * Er + Ei * Ei) / (8 * PI_D * eta * prad);
            P[(size_t)f * nangle + ai] = atan2(Ei, Er);
        }
    }
}
