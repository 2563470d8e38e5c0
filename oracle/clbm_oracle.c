/*
 * clbm_oracle.c -- CPU restatement of the reference D3Q19 cascaded-LBM + IBM time step.
 *
 * TEST INFRASTRUCTURE. This file is the correctness oracle and the timed CPU baseline
 * ("port"). Only the tests, the smoke check and the benchmark's CPU leg load it; the
 * CUDA library never links or calls it.
 *
 * It restates, kernel by kernel and in the same operation order, the reference's
 * unfused 12-kernel sequence on the reference's own array-of-structures layout
 * f[(i*Ny + j)*Nz + k][q] (Taichi field shape (Nx, Ny, Nz, 19), z fastest):
 *
 *   clbm_moving.py:75-91    _init_feq          -> or_init_feq
 *   clbm_moving.py:96-115   _macro_with_force  -> or_macro_with_force
 *   clbm_moving.py:120-249  _collide           -> or_collide
 *   clbm_moving.py:254-261  _stream            -> or_stream
 *   clbm_moving.py:266-294  _bc_inlet          -> or_bc_inlet
 *   clbm_moving.py:296-300  _bc_outlet         -> or_bc_outlet
 *   clbm_moving.py:305-321  _macro_post        -> or_macro_post
 *   clbm_moving.py:326-343  step               -> oracle_lbm_step
 *   airfoil_moving.py:27-38   _phi1d           -> or_phi1d
 *   airfoil_moving.py:100-127 _update_markers  -> or_update_markers
 *   airfoil_moving.py:132-137 _zero_forces     -> or_zero_forces
 *   airfoil_moving.py:142-170 _interpolate     -> or_interpolate
 *   airfoil_moving.py:175-183 _marker_forces   -> or_marker_forces
 *   airfoil_moving.py:188-214 _spread          -> or_spread (serial, marker order)
 *   airfoil_moving.py:219-225 _clip_forces     -> or_clip_forces
 *   airfoil_moving.py:230-255 compute_force    -> oracle_compute_force
 *   main_moving.py:62-74      _motion_state    -> oracle_motion_state (double)
 *
 * Arithmetic: REAL is float (liboracle_f32) or double (liboracle_f64, the FP64 oracle).
 * Constants that the reference writes as Python float expressions (for example
 * 1.0 - s_v, 2.0/3.0, W[q] * coeff) are evaluated in double and rounded once to REAL,
 * which is how the float32 kernels see them; float32 operands are combined in source
 * order. Build with -ffp-contract=off so no FMA contraction changes the rounding.
 *
 * Lift/drag is not part of the reference. oracle_body_force restates this project's
 * definition: the force on the body is minus the sum of the clipped Eulerian force
 * density over all cells, reduced in double (also the marker-side sum of F_k).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef ORACLE_REAL
#define ORACLE_REAL float
#endif
typedef ORACLE_REAL REAL;

/* D3Q19 velocity set and weights, clbm_moving.py:21-30 (order fixes the Zou-He lists) */
static const int EX[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
static const int EY[19] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
static const int EZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
static const double WD[19] = {1.0 / 3,
                              1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18,
                              1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36,
                              1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36,
                              1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36};

/* Raw-moment exponents (p,q,r) in the reference order, config_moving.py:62-68 */
static const int PQR[19][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0},
                               {1, 0, 1}, {0, 1, 1}, {2, 0, 0}, {0, 2, 0}, {0, 0, 2},
                               {2, 1, 0}, {1, 2, 0}, {2, 0, 1}, {0, 2, 1}, {1, 0, 2},
                               {0, 1, 2}, {2, 2, 0}, {2, 0, 2}, {0, 2, 2}};

/* closure_oracle.c: the learned closure for one cell (higher-order post-collision
   moments, or the shear rate of the eddy-viscosity form) */
double oracle_closure_post(const float *params, const double *f, double nu, double *post9);

typedef struct {
    int nx, ny, nz, n;
    double s_v, s_e, ux_in, uy_in;
    float *closure;  /* learned-closure parameters (NULL: the reference's s_q = s_pi = 1) */
    REAL minv[19][19];
    REAL *f, *f_post, *rho, *ux, *uy, *uz, *fx, *fy, *fz;
    REAL *X0, *Y0, *Z0, *X, *Y, *Z, *VX, *VY, *Uk, *Vk, *FXk, *FYk;
} oracle_t;

static inline size_t c3(const oracle_t *o, int i, int j, int k) {
    return ((size_t)i * o->ny + j) * o->nz + k;
}
static inline int pmod(int a, int m) { int r = a % m; return r < 0 ? r + m : r; }

/* M_raw^-1 (config_moving.py:69-73): Gauss-Jordan in double, then rounded to REAL. */
static void build_minv(REAL out[19][19]) {
    double a[19][38];
    for (int r = 0; r < 19; ++r) {
        for (int c = 0; c < 19; ++c) {
            double v = 1.0;
            for (int t = 0; t < PQR[r][0]; ++t) v *= EX[c];
            for (int t = 0; t < PQR[r][1]; ++t) v *= EY[c];
            for (int t = 0; t < PQR[r][2]; ++t) v *= EZ[c];
            a[r][c] = v;
            a[r][19 + c] = (r == c) ? 1.0 : 0.0;
        }
    }
    for (int c = 0; c < 19; ++c) {
        int piv = c;
        for (int r = c + 1; r < 19; ++r)
            if (fabs(a[r][c]) > fabs(a[piv][c])) piv = r;
        if (piv != c)
            for (int t = 0; t < 38; ++t) { double s = a[c][t]; a[c][t] = a[piv][t]; a[piv][t] = s; }
        double d = a[c][c];
        for (int t = 0; t < 38; ++t) a[c][t] /= d;
        for (int r = 0; r < 19; ++r) {
            if (r == c) continue;
            double m = a[r][c];
            if (m != 0.0)
                for (int t = 0; t < 38; ++t) a[r][t] -= m * a[c][t];
        }
    }
    for (int r = 0; r < 19; ++r)
        for (int c = 0; c < 19; ++c) out[r][c] = (REAL)a[r][19 + c];
}

/* ------------------------------------------------------------------ LBM kernels */

static void or_init_feq(oracle_t *o) {
    const REAL ux0 = (REAL)o->ux_in, uy0 = (REAL)o->uy_in;
    const REAL cs2 = (REAL)(1.0 / 3.0), cs4 = (REAL)((1.0 / 3.0) * (1.0 / 3.0));
    const REAL u2 = ux0 * ux0 + uy0 * uy0;
    REAL feq[19];
    for (int q = 0; q < 19; ++q) {
        REAL eu = (REAL)EX[q] * ux0 + (REAL)EY[q] * uy0;
        feq[q] = (REAL)WD[q] * ((REAL)1.0 + eu / cs2 + (REAL)0.5 * eu * eu / cs4
                                - (REAL)0.5 * u2 / cs2);
    }
    size_t ncell = (size_t)o->nx * o->ny * o->nz;
    for (size_t c = 0; c < ncell; ++c) {
        for (int q = 0; q < 19; ++q) o->f[c * 19 + q] = feq[q];
        o->rho[c] = (REAL)1.0;
        o->ux[c] = ux0;
        o->uy[c] = uy0;
        o->uz[c] = (REAL)0.0;
    }
}

static void or_macro_with_force(oracle_t *o) {
    size_t ncell = (size_t)o->nx * o->ny * o->nz;
#pragma omp parallel for schedule(static)
    for (long long cl = 0; cl < (long long)ncell; ++cl) {
        size_t c = (size_t)cl;
        const REAL *fc = o->f + c * 19;
        REAL r = 0, mx = 0, my = 0, mz = 0;
        for (int q = 0; q < 19; ++q) {
            REAL fq = fc[q];
            r += fq;
            mx += (REAL)EX[q] * fq;
            my += (REAL)EY[q] * fq;
            mz += (REAL)EZ[q] * fq;
        }
        o->rho[c] = r;
        o->ux[c] = mx / r + (REAL)0.5 * o->fx[c] / r;
        o->uy[c] = my / r + (REAL)0.5 * o->fy[c] / r;
        o->uz[c] = mz / r + (REAL)0.5 * o->fz[c] / r;
    }
}

static void or_collide(oracle_t *o) {
    const REAL one_m_sv = (REAL)(1.0 - o->s_v);
    const REAL s_e = (REAL)o->s_e;
    const REAL cs2 = (REAL)(1.0 / 3.0), cs4 = (REAL)((1.0 / 3.0) * (1.0 / 3.0));
    const double coeff = 1.0 - o->s_v * 0.5;
    REAL wc[19];
    for (int q = 0; q < 19; ++q) wc[q] = (REAL)(WD[q] * coeff);
    size_t ncell = (size_t)o->nx * o->ny * o->nz;
#pragma omp parallel for schedule(static)
    for (long long cl = 0; cl < (long long)ncell; ++cl) {
        size_t c = (size_t)cl;
        const REAL *fc = o->f + c * 19;
        REAL *fp = o->f_post + c * 19;
        const REAL u = o->ux[c], v = o->uy[c], w = o->uz[c], r = o->rho[c];
        const REAL Fx = o->fx[c], Fy = o->fy[c], Fz = o->fz[c];
        REAL k110 = 0, k101 = 0, k011 = 0, k200 = 0, k020 = 0, k002 = 0;
        REAL k210 = 0, k120 = 0, k201 = 0, k021 = 0, k102 = 0, k012 = 0;
        REAL k220 = 0, k202 = 0, k022 = 0;
        for (int q = 0; q < 19; ++q) {
            REAL fq = fc[q];
            REAL xix = (REAL)EX[q] - u, xiy = (REAL)EY[q] - v, xiz = (REAL)EZ[q] - w;
            REAL xix2 = xix * xix, xiy2 = xiy * xiy, xiz2 = xiz * xiz;
            k110 += fq * xix * xiy;
            k101 += fq * xix * xiz;
            k011 += fq * xiy * xiz;
            k200 += fq * xix2;
            k020 += fq * xiy2;
            k002 += fq * xiz2;
            k210 += fq * xix2 * xiy;
            k120 += fq * xix * xiy2;
            k201 += fq * xix2 * xiz;
            k021 += fq * xiy2 * xiz;
            k102 += fq * xix * xiz2;
            k012 += fq * xiy * xiz2;
            k220 += fq * xix2 * xiy2;
            k202 += fq * xix2 * xiz2;
            k022 += fq * xiy2 * xiz2;
        }
        (void)k210; (void)k120; (void)k201; (void)k021; (void)k102; (void)k012;
        (void)k220; (void)k202; (void)k022;
        REAL k210s = 0, k120s = 0, k201s = 0, k021s = 0, k102s = 0, k012s = 0;
        REAL osv = one_m_sv;  /* 1 - shear rate of this cell */
        REAL k220s = r / (REAL)9.0, k202s = r / (REAL)9.0, k022s = r / (REAL)9.0;
        if (o->closure && (size_t)cl / ((size_t)o->ny * o->nz) > 0 &&
            (size_t)cl / ((size_t)o->ny * o->nz) < (size_t)o->nx - 1) {
            /* learned closure (not part of the reference): the third/fourth-order central
               moments relax with the network's rate instead of 1 (mode 0), or the shear
               moments with the network's eddy-viscosity rate instead of s_v (mode 1); the
               inlet and outlet columns keep the plain rates */
            double fd[19], post[9];
            for (int q = 0; q < 19; ++q) fd[q] = (double)fc[q];
            const double nu = (1.0 / o->s_v - 0.5) / 3.0;
            const double se = oracle_closure_post(o->closure, fd, nu, post);
            if (se > 0.0) {
                osv = (REAL)(1.0 - se);
            } else {
                k210s = (REAL)post[0]; k120s = (REAL)post[1]; k201s = (REAL)post[2];
                k021s = (REAL)post[3]; k102s = (REAL)post[4]; k012s = (REAL)post[5];
                k220s += (REAL)post[6]; k202s += (REAL)post[7]; k022s += (REAL)post[8];
            }
        }
        /* cascade relaxation, clbm_moving.py:170-196 */
        REAL k110s = k110 * osv, k101s = k101 * osv, k011s = k011 * osv;
        REAL kA = k200 + k020 + k002;
        REAL kA_eq = r;
        REAL kD = k200 - k020, kE = k200 - k002;
        REAL kAs = kA - s_e * (kA - kA_eq);
        REAL kDs = kD * osv, kEs = kE * osv;
        REAL k200s = (kAs + kDs + kEs) / (REAL)3.0;
        REAL k020s = (kAs - (REAL)2.0 * kDs + kEs) / (REAL)3.0;
        REAL k002s = (kAs + kDs - (REAL)2.0 * kEs) / (REAL)3.0;
        /* central -> raw, clbm_moving.py:198-231 */
        REAL T[19];
        T[0] = r;
        T[1] = u * r;
        T[2] = v * r;
        T[3] = w * r;
        T[4] = k110s + u * v * r;
        T[5] = k101s + u * w * r;
        T[6] = k011s + v * w * r;
        T[7] = k200s + u * u * r;
        T[8] = k020s + v * v * r;
        T[9] = k002s + w * w * r;
        T[10] = k210s + (REAL)2.0 * u * k110s + v * k200s + u * u * v * r;
        T[11] = k120s + (REAL)2.0 * v * k110s + u * k020s + u * v * v * r;
        T[12] = k201s + (REAL)2.0 * u * k101s + w * k200s + u * u * w * r;
        T[13] = k021s + (REAL)2.0 * v * k011s + w * k020s + v * v * w * r;
        T[14] = k102s + (REAL)2.0 * w * k101s + u * k002s + u * w * w * r;
        T[15] = k012s + (REAL)2.0 * w * k011s + v * k002s + v * w * w * r;
        T[16] = (k220s + (REAL)2.0 * u * k120s + (REAL)2.0 * v * k210s
                 + (REAL)4.0 * u * v * k110s + v * v * k200s + u * u * k020s
                 + u * u * v * v * r);
        T[17] = (k202s + (REAL)2.0 * u * k102s + (REAL)2.0 * w * k201s
                 + (REAL)4.0 * u * w * k101s + w * w * k200s + u * u * k002s
                 + u * u * w * w * r);
        T[18] = (k022s + (REAL)2.0 * v * k012s + (REAL)2.0 * w * k021s
                 + (REAL)4.0 * v * w * k011s + w * w * k020s + v * v * k002s
                 + v * v * w * w * r);
        /* f* = M_inv T (dense, zeros included), clbm_moving.py:233-238 */
        for (int q = 0; q < 19; ++q) {
            REAL val = 0;
            for (int t = 0; t < 19; ++t) val += o->minv[q][t] * T[t];
            fp[q] = val;
        }
        /* Guo forcing, clbm_moving.py:240-249 */
        for (int q = 0; q < 19; ++q) {
            REAL ex = (REAL)EX[q], ey = (REAL)EY[q], ez = (REAL)EZ[q];
            REAL eu = ex * u + ey * v + ez * w;
            REAL cx = (ex - u) / cs2 + eu * ex / cs4;
            REAL cy = (ey - v) / cs2 + eu * ey / cs4;
            REAL cz = (ez - w) / cs2 + eu * ez / cs4;
            fp[q] += wc[q] * (cx * Fx + cy * Fy + cz * Fz);
        }
    }
}

static void or_stream(oracle_t *o) {
    const int nx = o->nx, ny = o->ny, nz = o->nz;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k)
                for (int q = 0; q < 19; ++q) {
                    int is = (i - EX[q] + nx) % nx, js = (j - EY[q] + ny) % ny,
                        ks = (k - EZ[q] + nz) % nz;
                    o->f[c3(o, i, j, k) * 19 + q] = o->f_post[c3(o, is, js, ks) * 19 + q];
                }
}

static void or_bc_inlet(oracle_t *o) {
    const REAL ux_in = (REAL)o->ux_in, uy_in = (REAL)o->uy_in;
    const REAL c23 = (REAL)(2.0 / 3.0), c16 = (REAL)(1.0 / 6.0);
    for (int j = 0; j < o->ny; ++j)
        for (int k = 0; k < o->nz; ++k) {
            REAL *f = o->f + c3(o, 0, j, k) * 19;
            REAL S_known = f[0] + f[3] + f[4] + f[5] + f[6] + f[15] + f[16] + f[17] + f[18];
            REAL S_out = f[2] + f[8] + f[10] + f[12] + f[14];
            REAL rho_in = (S_known + (REAL)2.0 * S_out) / ((REAL)1.0 - ux_in);
            REAL diff_y = f[3] - f[4];
            REAL diff_z = f[5] - f[6];
            f[1] = f[2] + c23 * rho_in * ux_in;
            f[7] = f[10] + c16 * rho_in * ux_in + (REAL)0.5 * rho_in * uy_in - (REAL)0.5 * diff_y;
            f[9] = f[8] + c16 * rho_in * ux_in - (REAL)0.5 * rho_in * uy_in + (REAL)0.5 * diff_y;
            f[11] = f[14] + c16 * rho_in * ux_in - (REAL)0.5 * diff_z;
            f[13] = f[12] + c16 * rho_in * ux_in + (REAL)0.5 * diff_z;
        }
}

static void or_bc_outlet(oracle_t *o) {
    for (int j = 0; j < o->ny; ++j)
        for (int k = 0; k < o->nz; ++k)
            memcpy(o->f + c3(o, o->nx - 1, j, k) * 19, o->f + c3(o, o->nx - 2, j, k) * 19,
                   19 * sizeof(REAL));
}

static void or_macro_post(oracle_t *o) {
    size_t ncell = (size_t)o->nx * o->ny * o->nz;
#pragma omp parallel for schedule(static)
    for (long long cl = 0; cl < (long long)ncell; ++cl) {
        size_t c = (size_t)cl;
        const REAL *fc = o->f + c * 19;
        REAL r = 0, mx = 0, my = 0, mz = 0;
        for (int q = 0; q < 19; ++q) {
            REAL fq = fc[q];
            r += fq;
            mx += (REAL)EX[q] * fq;
            my += (REAL)EY[q] * fq;
            mz += (REAL)EZ[q] * fq;
        }
        o->rho[c] = r;
        o->ux[c] = mx / r;
        o->uy[c] = my / r;
        o->uz[c] = mz / r;
    }
}

/* ------------------------------------------------------------------ IBM kernels */

static inline REAL or_phi1d(REAL rr) {
    REAL s = rr < 0 ? -rr : rr;
    REAL result = 0;
    if (s < (REAL)1.0) {
        REAL a = (REAL)1.0 + (REAL)4.0 * s - (REAL)4.0 * s * s;
        if (a < 0) a = 0;
        result = ((REAL)3.0 - (REAL)2.0 * s + (REAL)sqrt(a)) / (REAL)8.0;
    } else if (s < (REAL)2.0) {
        REAL a = (REAL)-7.0 + (REAL)12.0 * s - (REAL)4.0 * s * s;
        if (a < 0) a = 0;
        result = ((REAL)5.0 - (REAL)2.0 * s - (REAL)sqrt(a)) / (REAL)8.0;
    }
    return result;
}

static void or_update_markers(oracle_t *o, REAL xc, REAL yc, REAL theta, REAL vx, REAL vy,
                              REAL omega) {
    const REAL cos_t = (REAL)cos(theta), sin_t = (REAL)sin(theta);
    for (int m = 0; m < o->n; ++m) {
        REAL x0m = o->X0[m], y0m = o->Y0[m];
        REAL xk = xc + x0m * cos_t - y0m * sin_t;
        REAL yk = yc + x0m * sin_t + y0m * cos_t;
        o->X[m] = xk;
        o->Y[m] = yk;
        o->Z[m] = o->Z0[m];
        REAL rx = xk - xc, ry = yk - yc;
        o->VX[m] = vx - omega * ry;
        o->VY[m] = vy + omega * rx;
    }
}

static void or_zero_forces(oracle_t *o) {
    size_t ncell = (size_t)o->nx * o->ny * o->nz;
    memset(o->fx, 0, ncell * sizeof(REAL));
    memset(o->fy, 0, ncell * sizeof(REAL));
    memset(o->fz, 0, ncell * sizeof(REAL));
}

static void or_interpolate(oracle_t *o) {
    const int nx = o->nx, ny = o->ny, nz = o->nz;
#pragma omp parallel for schedule(static)
    for (int m = 0; m < o->n; ++m) {
        REAL xk = o->X[m], yk = o->Y[m], zk = o->Z[m];
        int ib = (int)floor(xk) - 1, jb = (int)floor(yk) - 1, kb = (int)floor(zk) - 1;
        REAL us = 0, vs = 0;
        for (int di = 0; di < 4; ++di) {
            int ii = ib + di;
            ii = ii < 0 ? 0 : (ii > nx - 1 ? nx - 1 : ii);
            REAL phx = or_phi1d((REAL)ii - xk);
            for (int dj = 0; dj < 4; ++dj) {
                int jj = pmod(jb + dj + ny, ny);
                REAL phy = or_phi1d((REAL)jj - yk);
                for (int dk = 0; dk < 4; ++dk) {
                    int kk = pmod(kb + dk + nz, nz);
                    REAL phz = or_phi1d((REAL)kk - zk);
                    REAL wijk = phx * phy * phz;
                    size_t c = c3(o, ii, jj, kk);
                    us += o->ux[c] * wijk;
                    vs += o->uy[c] * wijk;
                }
            }
        }
        o->Uk[m] = us;
        o->Vk[m] = vs;
    }
}

static void or_marker_forces(oracle_t *o) {
    const REAL fmax = (REAL)0.05;
    for (int m = 0; m < o->n; ++m) {
        REAL ex = -(o->Uk[m] - o->VX[m]);
        REAL ey = -(o->Vk[m] - o->VY[m]);
        REAL a = ex < fmax ? ex : fmax;
        o->FXk[m] = -fmax > a ? -fmax : a;
        REAL b = ey < fmax ? ey : fmax;
        o->FYk[m] = -fmax > b ? -fmax : b;
    }
}

static void or_spread(oracle_t *o) {
    const int nx = o->nx, ny = o->ny, nz = o->nz;
    for (int m = 0; m < o->n; ++m) {
        REAL xk = o->X[m], yk = o->Y[m], zk = o->Z[m];
        REAL fxk = o->FXk[m], fyk = o->FYk[m];
        int ib = (int)floor(xk) - 1, jb = (int)floor(yk) - 1, kb = (int)floor(zk) - 1;
        for (int di = 0; di < 4; ++di) {
            int ii = ib + di;
            ii = ii < 0 ? 0 : (ii > nx - 1 ? nx - 1 : ii);
            REAL phx = or_phi1d((REAL)ii - xk);
            for (int dj = 0; dj < 4; ++dj) {
                int jj = pmod(jb + dj + ny, ny);
                REAL phy = or_phi1d((REAL)jj - yk);
                for (int dk = 0; dk < 4; ++dk) {
                    int kk = pmod(kb + dk + nz, nz);
                    REAL phz = or_phi1d((REAL)kk - zk);
                    REAL wijk = phx * phy * phz;
                    size_t c = c3(o, ii, jj, kk);
                    o->fx[c] += fxk * wijk;
                    o->fy[c] += fyk * wijk;
                }
            }
        }
    }
}

static void or_clip_forces(oracle_t *o) {
    const REAL fmax = (REAL)0.05;
    size_t ncell = (size_t)o->nx * o->ny * o->nz;
#pragma omp parallel for schedule(static)
    for (long long cl = 0; cl < (long long)ncell; ++cl) {
        size_t c = (size_t)cl;
        REAL a = o->fx[c] < fmax ? o->fx[c] : fmax;
        o->fx[c] = -fmax > a ? -fmax : a;
        REAL b = o->fy[c] < fmax ? o->fy[c] : fmax;
        o->fy[c] = -fmax > b ? -fmax : b;
        o->fz[c] = 0;
    }
}

/* ------------------------------------------------------------------ exported API */

void *oracle_create(int nx, int ny, int nz, double s_v, double s_e, double ux_in,
                    double uy_in, int n, const float *X0, const float *Y0, const float *Z0) {
    if (nx < 3 || ny < 1 || nz < 1 || n < 0) return NULL;
    oracle_t *o = (oracle_t *)calloc(1, sizeof(oracle_t));
    o->nx = nx; o->ny = ny; o->nz = nz; o->n = n;
    o->s_v = s_v; o->s_e = s_e; o->ux_in = ux_in; o->uy_in = uy_in;
    build_minv(o->minv);
    size_t nc = (size_t)nx * ny * nz;
    o->f = (REAL *)calloc(nc * 19, sizeof(REAL));
    o->f_post = (REAL *)calloc(nc * 19, sizeof(REAL));
    REAL **g[] = {&o->rho, &o->ux, &o->uy, &o->uz, &o->fx, &o->fy, &o->fz};
    for (size_t t = 0; t < sizeof(g) / sizeof(g[0]); ++t) *g[t] = (REAL *)calloc(nc, sizeof(REAL));
    size_t nm = n > 0 ? (size_t)n : 1;
    REAL **mk[] = {&o->X0, &o->Y0, &o->Z0, &o->X, &o->Y, &o->Z, &o->VX, &o->VY,
                   &o->Uk, &o->Vk, &o->FXk, &o->FYk};
    for (size_t t = 0; t < sizeof(mk) / sizeof(mk[0]); ++t) *mk[t] = (REAL *)calloc(nm, sizeof(REAL));
    for (int m = 0; m < n; ++m) {
        o->X0[m] = (REAL)X0[m];
        o->Y0[m] = (REAL)Y0[m];
        o->Z0[m] = (REAL)Z0[m];
    }
    or_init_feq(o);
    return o;
}

void oracle_destroy(void *h) {
    oracle_t *o = (oracle_t *)h;
    if (!o) return;
    void *p[] = {o->f, o->f_post, o->rho, o->ux, o->uy, o->uz, o->fx, o->fy, o->fz,
                 o->X0, o->Y0, o->Z0, o->X, o->Y, o->Z, o->VX, o->VY, o->Uk, o->Vk,
                 o->FXk, o->FYk, o->closure};
    for (size_t t = 0; t < sizeof(p) / sizeof(p[0]); ++t) free(p[t]);
    free(o);
}

/* Learned closure for later collisions (params: 2188 floats, copied; NULL: off). */
void oracle_set_closure(void *h, const float *params) {
    oracle_t *o = (oracle_t *)h;
    free(o->closure);
    o->closure = NULL;
    if (!params) return;
    o->closure = (float *)malloc(sizeof(float) * 2188);
    memcpy(o->closure, params, sizeof(float) * 2188);
}

int oracle_real_size(void) { return (int)sizeof(REAL); }

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_minv(void *h, REAL *out) { memcpy(out, ((oracle_t *)h)->minv, sizeof(REAL) * 361); }

/* ibm.compute_force(ux, uy, xc, yc, theta, vx, vy, omega), airfoil_moving.py:230-255.
 * The six motion values arrive in double and are truncated to REAL at the kernel boundary,
 * as Taichi truncates the f32-annotated arguments (airfoil_moving.py:101-103). */
void oracle_compute_force(void *h, double xc, double yc, double theta, double vx, double vy,
                          double omega) {
    oracle_t *o = (oracle_t *)h;
    or_update_markers(o, (REAL)xc, (REAL)yc, (REAL)theta, (REAL)vx, (REAL)vy, (REAL)omega);
    or_zero_forces(o);
    or_interpolate(o);
    or_marker_forces(o);
    or_spread(o);
    or_clip_forces(o);
}

/* lbm.step(fx, fy, fz) with the oracle's own force arrays, clbm_moving.py:326-343 */
void oracle_lbm_step(void *h) {
    oracle_t *o = (oracle_t *)h;
    or_macro_with_force(o);
    or_collide(o);
    or_stream(o);
    or_bc_inlet(o);
    or_bc_outlet(o);
    or_macro_post(o);
}

/* _motion_state(step), main_moving.py:62-74, in double. out = xc, yc, theta, vx, vy, omega */
void oracle_motion_state(long long step, double x0, double y0, double a_heave,
                         double a_pitch, double phi_pitch, double aoa0, double w,
                         double *out) {
    double t = (double)step;
    out[0] = x0;
    out[1] = y0 + a_heave * sin(w * t);
    out[2] = aoa0 + a_pitch * sin(w * t + phi_pitch);
    out[3] = 0.0;
    out[4] = a_heave * w * cos(w * t);
    out[5] = a_pitch * w * cos(w * t + phi_pitch);
}

/* Sums of the force the IBM injects, in double: out[0..1] = sum over cells of the clipped
 * Eulerian fx, fy; out[2..3] = sum over markers of FX_k, FY_k. The force on the body is
 * the negative of either pair. */
void oracle_body_force(void *h, double *out) {
    oracle_t *o = (oracle_t *)h;
    size_t ncell = (size_t)o->nx * o->ny * o->nz;
    double sx = 0, sy = 0, mx = 0, my = 0;
    for (size_t c = 0; c < ncell; ++c) { sx += (double)o->fx[c]; sy += (double)o->fy[c]; }
    for (int m = 0; m < o->n; ++m) { mx += (double)o->FXk[m]; my += (double)o->FYk[m]; }
    out[0] = sx; out[1] = sy; out[2] = mx; out[3] = my;
}

/* Full time loop: steps step0+1 .. step0+nsteps of the driver loop (main_moving.py:116-122)
 * with the motion law evaluated per step; body-force sums per step go to hist[4*s]. */
void oracle_run(void *h, long long step0, int nsteps, double x0, double y0, double a_heave,
                double a_pitch, double phi_pitch, double aoa0, double w, double *hist) {
    double ms[6];
    for (int s = 0; s < nsteps; ++s) {
        oracle_motion_state(step0 + 1 + s, x0, y0, a_heave, a_pitch, phi_pitch, aoa0, w, ms);
        oracle_compute_force(h, ms[0], ms[1], ms[2], ms[3], ms[4], ms[5]);
        if (hist) oracle_body_force(h, hist + 4 * (size_t)s);
        oracle_lbm_step(h);
    }
}

/* ---- state access (copies) ---- */
void oracle_get_f(void *h, REAL *out) {
    oracle_t *o = (oracle_t *)h;
    memcpy(out, o->f, sizeof(REAL) * 19 * (size_t)o->nx * o->ny * o->nz);
}
void oracle_set_f(void *h, const REAL *in) {
    oracle_t *o = (oracle_t *)h;
    memcpy(o->f, in, sizeof(REAL) * 19 * (size_t)o->nx * o->ny * o->nz);
    or_macro_post(o);
}
void oracle_get_macro(void *h, REAL *rho, REAL *ux, REAL *uy, REAL *uz) {
    oracle_t *o = (oracle_t *)h;
    size_t b = sizeof(REAL) * (size_t)o->nx * o->ny * o->nz;
    memcpy(rho, o->rho, b); memcpy(ux, o->ux, b); memcpy(uy, o->uy, b); memcpy(uz, o->uz, b);
}
void oracle_get_forces(void *h, REAL *fx, REAL *fy, REAL *fz) {
    oracle_t *o = (oracle_t *)h;
    size_t b = sizeof(REAL) * (size_t)o->nx * o->ny * o->nz;
    memcpy(fx, o->fx, b); memcpy(fy, o->fy, b); memcpy(fz, o->fz, b);
}
void oracle_set_forces(void *h, const REAL *fx, const REAL *fy, const REAL *fz) {
    oracle_t *o = (oracle_t *)h;
    size_t b = sizeof(REAL) * (size_t)o->nx * o->ny * o->nz;
    memcpy(o->fx, fx, b); memcpy(o->fy, fy, b); memcpy(o->fz, fz, b);
}
/* out: 9 arrays of n: X, Y, Z, VX, VY, U_k, V_k, FX_k, FY_k */
void oracle_get_markers(void *h, REAL *out) {
    oracle_t *o = (oracle_t *)h;
    REAL *src[9] = {o->X, o->Y, o->Z, o->VX, o->VY, o->Uk, o->Vk, o->FXk, o->FYk};
    for (int t = 0; t < 9; ++t) memcpy(out + (size_t)t * o->n, src[t], sizeof(REAL) * o->n);
}
