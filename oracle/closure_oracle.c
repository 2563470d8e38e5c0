/*
 * closure_oracle.c -- CPU restatement of the learned sub-grid closure (test
 * infrastructure: only the tests and the smoke check load it; the CUDA library never
 * links or calls it).
 *
 * The closure is this project's own addition, not part of the reference. Two forms
 * (parameter mode): 0, the rate s_h = 1 + span tanh(z3) of the third/fourth-order central
 * moments; 1, an eddy viscosity: the deviatoric second-order moments relax with
 * s = 1 / (1/2 + 3 nu 2^(span g)), g = tanh(z3) where positive and tanh(z3) / 20 below.
 * What the CUDA kernels compute, restated here in double precision:
 *   - features: the 19 non-equilibrium central moments of a cell about u = m / rho, in
 *     the M_raw moment order (config_moving.py:62-68), divided by rho; computed directly
 *     as sum_q f_q (e_x - u)^p (e_y - v)^q (e_z - w)^r, the way _collide forms its
 *     central moments (clbm_moving.py:139-168), not by the binomial expansion the kernels
 *     use, so the two formulations check each other;
 *   - the network 19 -> 32 -> 32 -> 1, GELU (tanh form), s_h = 1 + span tanh(z3);
 *     round = 1 rounds the tensor-core operands to BF16 (standardised inputs, W1, h1,
 *     W2, W3) as the kernels do, round = 0 stays in double (for finite differences);
 *   - the loss, mode 0 sum_j (t_j - (1 - s_h) p_j)^2 over the nine third/fourth-order
 *     moments, mode 1 sum_j (tau_j + 2 nu_t S_j)^2 over the five deviatoric sub-grid
 *     stress components, times wscale, and its gradient by back-propagation (round = 1
 *     also rounds the operands of the backward products as the kernels do);
 *   - the box filter of a fine lattice (populations, velocity, velocity products) and the
 *     training samples of a coarse cell from two filtered states.
 *
 * Parameter layout (floats): mu[19] @0, sinv[19] @19, W1[32][32] @40 (out, in), b1 @1064,
 * W2[32][32] @1096, b2 @2120, W3[32] @2152, b3 @2184, span @2185, mode @2186, nu @2187
 * (2188 in all). The gradient array follows the parameter array from W1 on (2145 entries).
 * A sample is 19 features, 9 higher-order targets, then tau and S (xy, xz, yz, xx - yy,
 * xx - zz each).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#define CL_IN 19
#define CL_H 32
#define CL_MU 0
#define CL_SINV 19
#define CL_W1 40
#define CL_B1 (CL_W1 + CL_H * CL_H)
#define CL_W2 (CL_B1 + CL_H)
#define CL_B2 (CL_W2 + CL_H * CL_H)
#define CL_W3 (CL_B2 + CL_H)
#define CL_B3 (CL_W3 + CL_H)
#define CL_SPAN (CL_B3 + 1)
#define CL_MODE (CL_SPAN + 1)
#define CL_NU (CL_MODE + 1)
#define CL_NPARAM (CL_NU + 1)
#define CL_NTRAIN (CL_SPAN - CL_W1)
#define CL_NT 9
#define CL_NSGS 10
#define CL_SAMPLE (CL_IN + CL_NT + CL_NSGS)

static const int CEX[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
static const int CEY[19] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
static const int CEZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
static const int CPQR[19][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0},
                                {1, 0, 1}, {0, 1, 1}, {2, 0, 0}, {0, 2, 0}, {0, 0, 2},
                                {2, 1, 0}, {1, 2, 0}, {2, 0, 1}, {0, 2, 1}, {1, 0, 2},
                                {0, 1, 2}, {2, 2, 0}, {2, 0, 2}, {0, 2, 2}};

int oracle_closure_nparams(void) { return CL_NPARAM; }

/* Round to the nearest bfloat16 (ties to even), through float. */
static double bf16r(double x) {
    float f = (float)x;
    uint32_t u;
    memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    u &= 0xFFFF0000u;
    memcpy(&f, &u, 4);
    return (double)f;
}

static double rnd(double x, int round) { return round ? bf16r(x) : x; }

static double gelu(double z) {
    const double k = 0.7978845608028654;
    return 0.5 * z * (1.0 + tanh(k * (z + 0.044715 * z * z * z)));
}

static double gelu_grad(double z) {
    const double k = 0.7978845608028654;
    const double t = tanh(k * (z + 0.044715 * z * z * z));
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * k * (1.0 + 3.0 * 0.044715 * z * z);
}

static double ipow(double b, int e) { return e == 0 ? 1.0 : (e == 1 ? b : b * b); }

/* Non-equilibrium central moments / rho_n of f about (u, v, w): equilibrium rho/3 removed
 * from the second diagonal and rho/9 from the fourth, rho = sum f. */
static void central_about(const double *f, double u, double v, double w, double rho_n, double *x) {
    double r = 0.0;
    for (int q = 0; q < 19; ++q) r += f[q];
    for (int i = 0; i < CL_IN; ++i) {
        double s = 0.0;
        for (int q = 0; q < 19; ++q)
            s += f[q] * ipow(CEX[q] - u, CPQR[i][0]) * ipow(CEY[q] - v, CPQR[i][1]) *
                 ipow(CEZ[q] - w, CPQR[i][2]);
        x[i] = s;
    }
    x[0] = 0.0;  /* k000 - rho */
    for (int i = 7; i < 10; ++i) x[i] -= r / 3.0;
    for (int i = 16; i < 19; ++i) x[i] -= r / 9.0;
    for (int i = 0; i < CL_IN; ++i) x[i] /= rho_n;
}

/* Features of n cells: f is [n][19] full populations, x gets [n][19]. */
void oracle_closure_features(const double *f, int n, double *x) {
    for (int c = 0; c < n; ++c) {
        const double *fc = f + (size_t)c * 19;
        double r = 0, mx = 0, my = 0, mz = 0;
        for (int q = 0; q < 19; ++q) {
            r += fc[q];
            mx += CEX[q] * fc[q];
            my += CEY[q] * fc[q];
            mz += CEZ[q] * fc[q];
        }
        central_about(fc, mx / r, my / r, mz / r, r, x + (size_t)c * CL_IN);
    }
}

/* Effective viscosity of the eddy-viscosity form for th = tanh(z3), nu 2^(span g) with
 * g = th (th >= 0) or th / 20 (th < 0), and d nu_eff / d th. */
static double cl_nu_eff(const float *p, double th, double *dnudth) {
    const double slope = th >= 0.0 ? 1.0 : 0.05;
    const double nue = (double)p[CL_NU] * exp2((double)p[CL_SPAN] * slope * th);
    *dnudth = nue * log(2.0) * p[CL_SPAN] * slope;
    return nue;
}

/* Rate of the closure's form for the network output th = tanh(z3). */
static double cl_rate(const float *p, double th) {
    if ((int)p[CL_MODE] == 1) {
        double d;
        return 1.0 / (0.5 + 3.0 * cl_nu_eff(p, th, &d));
    }
    return 1.0 + p[CL_SPAN] * th;
}

/* Box filter of a fine lattice (nx, ny, nz, 19 post-stream populations, reference layout)
 * onto the coarse lattice (nx/2, ny/2, nz/2, 28): mean populations, mean velocity and
 * mean velocity products (xx, yy, zz, xy, xz, yz). */
void oracle_closure_filter(const double *ff, int nx, int ny, int nz, double *out) {
    const int cx = nx / 2, cy = ny / 2, cz = nz / 2;
    for (int X = 0; X < cx; ++X)
        for (int Y = 0; Y < cy; ++Y)
            for (int Z = 0; Z < cz; ++Z) {
                double acc[28] = {0};
                for (int s = 0; s < 8; ++s) {
                    const int x = 2 * X + (s & 1), y = 2 * Y + ((s >> 1) & 1), z = 2 * Z + (s >> 2);
                    const double *f = ff + (((size_t)x * ny + y) * nz + z) * 19;
                    double r = 0, mx = 0, my = 0, mz = 0;
                    for (int q = 0; q < 19; ++q) {
                        acc[q] += f[q];
                        r += f[q];
                        mx += CEX[q] * f[q];
                        my += CEY[q] * f[q];
                        mz += CEZ[q] * f[q];
                    }
                    const double u = mx / r, v = my / r, w = mz / r;
                    acc[19] += u; acc[20] += v; acc[21] += w;
                    acc[22] += u * u; acc[23] += v * v; acc[24] += w * w;
                    acc[25] += u * v; acc[26] += u * w; acc[27] += v * w;
                }
                double *o = out + (((size_t)X * cy + Y) * cz + Z) * 28;
                for (int i = 0; i < 28; ++i) o[i] = acc[i] / 8.0;
            }
}

/* Samples of coarse cells from the filtered states f0, f1 in the reference layout
 * (nx, ny, nz, 19), z fastest: features of f0 at the cell, targets from
 * f*_q = f1_q(x + e_q) (y, z periodic) about the velocity and density of f0. */
void oracle_closure_samples(const double *f0, const double *f1, int nx, int ny, int nz,
                            const long long *cells, int n, double *out) {
#define C28(a, x, y, z) ((a) + (((size_t)(x) * ny + (y)) * nz + (z)) * 28)
    for (int j = 0; j < n; ++j) {
        const long long id = cells[j];
        const int x = (int)(id % nx);
        const long long row = id / nx;
        const int y = (int)(row % ny), z = (int)(row / ny);
        const double *fc = C28(f0, x, y, z);
        double fs[19];
        for (int q = 0; q < 19; ++q) {
            int yy = (y + CEY[q] + ny) % ny, zz = (z + CEZ[q] + nz) % nz;
            fs[q] = C28(f1, x + CEX[q], yy, zz)[q];
        }
        double r = 0, mx = 0, my = 0, mz = 0;
        for (int q = 0; q < 19; ++q) {
            r += fc[q];
            mx += CEX[q] * fc[q];
            my += CEY[q] * fc[q];
            mz += CEZ[q] * fc[q];
        }
        double *o = out + (size_t)j * CL_SAMPLE;
        central_about(fc, mx / r, my / r, mz / r, r, o);
        double t[CL_IN];
        central_about(fs, mx / r, my / r, mz / r, r, t);
        for (int i = 0; i < CL_NT; ++i) o[CL_IN + i] = t[10 + i];
        /* sub-grid stress and filtered strain rate (central differences, y/z periodic) */
        const double *a = fc + 19;
        const double txx = a[3] - a[0] * a[0], tyy = a[4] - a[1] * a[1], tzz = a[5] - a[2] * a[2];
        const double txy = a[6] - a[0] * a[1], txz = a[7] - a[0] * a[2], tyz = a[8] - a[1] * a[2];
        const int yp = (y + 1) % ny, ym = (y + ny - 1) % ny, zp = (z + 1) % nz, zm = (z + nz - 1) % nz;
        double du[3][3];  /* du[i][c] = d <u_c> / d x_i */
        for (int c = 0; c < 3; ++c) {
            du[0][c] = 0.5 * (C28(f0, x + 1, y, z)[19 + c] - C28(f0, x - 1, y, z)[19 + c]);
            du[1][c] = 0.5 * (C28(f0, x, yp, z)[19 + c] - C28(f0, x, ym, z)[19 + c]);
            du[2][c] = 0.5 * (C28(f0, x, y, zp)[19 + c] - C28(f0, x, y, zm)[19 + c]);
        }
        const double sxy = 0.5 * (du[1][0] + du[0][1]), sxz = 0.5 * (du[2][0] + du[0][2]);
        const double syz = 0.5 * (du[2][1] + du[1][2]);
        const double sg[CL_NSGS] = {txy, txz, tyz, txx - tyy, txx - tzz,
                                    sxy, sxz, syz, du[0][0] - du[1][1], du[0][0] - du[2][2]};
        for (int i = 0; i < CL_NSGS; ++i) o[CL_IN + CL_NT + i] = sg[i];
    }
#undef C28
}

typedef struct {
    double xs[CL_H], z1[CL_H], h1[CL_H], z2[CL_H], h2[CL_H], z3, th, s;
} cl_fwd_t;

static void cl_forward1(const float *p, const double *x, int round, cl_fwd_t *o) {
    for (int i = 0; i < CL_H; ++i)
        o->xs[i] = i < CL_IN ? rnd(((double)x[i] - p[CL_MU + i]) * p[CL_SINV + i], round) : 0.0;
    for (int n = 0; n < CL_H; ++n) {
        double a = 0.0;
        for (int k = 0; k < CL_H; ++k) a += rnd(p[CL_W1 + n * CL_H + k], round) * o->xs[k];
        o->z1[n] = a + p[CL_B1 + n];
        o->h1[n] = rnd(gelu(o->z1[n]), round);
    }
    for (int n = 0; n < CL_H; ++n) {
        double a = 0.0;
        for (int k = 0; k < CL_H; ++k) a += rnd(p[CL_W2 + n * CL_H + k], round) * o->h1[k];
        o->z2[n] = a + p[CL_B2 + n];
        o->h2[n] = gelu(o->z2[n]);
    }
    double z3 = p[CL_B3];
    for (int n = 0; n < CL_H; ++n) z3 += rnd(p[CL_W3 + n], round) * o->h2[n];
    o->z3 = z3;
    o->th = tanh(z3);
    o->s = cl_rate(p, o->th);
}

/* s_h of n feature rows x [n][19]. */
void oracle_closure_forward(const float *params, const double *x, int n, int round, double *s) {
    cl_fwd_t o;
    for (int c = 0; c < n; ++c) {
        cl_forward1(params, x + (size_t)c * CL_IN, round, &o);
        s[c] = o.s;
    }
}

/* Loss sum over n samples [n][28] and the gradient of the mean loss (CL_NTRAIN). */
void oracle_closure_loss_grad(const float *params, const double *samples, int n, double wscale,
                              int round, double *loss, double *grad) {
    const float *p = params;
    cl_fwd_t o;
    double L = 0.0;
    if (grad) memset(grad, 0, sizeof(double) * CL_NTRAIN);
    for (int c = 0; c < n; ++c) {
        const double *sm = samples + (size_t)c * CL_SAMPLE;
        cl_forward1(p, sm, round, &o);
        double dldth = 0.0;
        if ((int)p[CL_MODE] == 1) {
            double dnudth;
            const double nut = cl_nu_eff(p, o.th, &dnudth) - p[CL_NU];
            double dldnu = 0.0;
            for (int j = 0; j < CL_NSGS / 2; ++j) {
                const double S = sm[CL_IN + CL_NT + CL_NSGS / 2 + j];
                const double rj = sm[CL_IN + CL_NT + j] + 2.0 * nut * S;
                L += wscale * rj * rj;
                dldnu += 4.0 * wscale * rj * S;
            }
            dldth = dldnu * dnudth;
        } else {
            const double oms = -p[CL_SPAN] * o.th;
            double dlds = 0.0;
            for (int j = 0; j < CL_NT; ++j) {
                const double pj = sm[10 + j], rj = sm[CL_IN + j] - oms * pj;
                L += wscale * rj * rj;
                dlds += 2.0 * wscale * rj * pj;
            }
            dldth = dlds * p[CL_SPAN];
        }
        if (!grad) continue;
        const double d3 = dldth * (1.0 - o.th * o.th);
        const double d3r = rnd(d3, round);  /* operand of the weight-gradient product */
        double d2[CL_H], d1[CL_H];
        for (int j = 0; j < CL_H; ++j)
            d2[j] = rnd(d3 * rnd(p[CL_W3 + j], round) * gelu_grad(o.z2[j]), round);
        for (int k = 0; k < CL_H; ++k) {
            double a = 0.0;
            for (int j = 0; j < CL_H; ++j) a += d2[j] * rnd(p[CL_W2 + j * CL_H + k], round);
            d1[k] = rnd(a * gelu_grad(o.z1[k]), round);
        }
        double *g = grad;
        for (int j = 0; j < CL_H; ++j) {
            for (int k = 0; k < CL_H; ++k) g[(CL_W1 - CL_W1) + j * CL_H + k] += d1[j] * o.xs[k];
            g[(CL_B1 - CL_W1) + j] += d1[j];
            for (int k = 0; k < CL_H; ++k) g[(CL_W2 - CL_W1) + j * CL_H + k] += d2[j] * o.h1[k];
            g[(CL_B2 - CL_W1) + j] += d2[j];
            g[(CL_W3 - CL_W1) + j] += d3r * rnd(o.h2[j], round);
        }
        g[CL_B3 - CL_W1] += d3r;
    }
    *loss = L;
    if (grad)
        for (int i = 0; i < CL_NTRAIN; ++i) grad[i] /= n;
}

/* The closure for one cell (used by the oracle's collision). Mode 0: post-collision
 * third-order central moments and fourth-order deviations from rho/9, k* = (1 - s_h) k,
 * into post9, returns 0. Mode 1: returns the cell's shear rate s (nu from the solver). */
double oracle_closure_post(const float *params, const double *f, double nu, double *post9) {
    double r = 0, mx = 0, my = 0, mz = 0;
    for (int q = 0; q < 19; ++q) {
        r += f[q];
        mx += CEX[q] * f[q];
        my += CEY[q] * f[q];
        mz += CEZ[q] * f[q];
    }
    double x[CL_IN];
    central_about(f, mx / r, my / r, mz / r, r, x);
    cl_fwd_t o;
    cl_forward1(params, x, 1, &o);
    if ((int)params[CL_MODE] == 1) {
        const double g = o.th >= 0.0 ? o.th : 0.05 * o.th;
        const double nue = nu * exp2((double)params[CL_SPAN] * g);
        for (int i = 0; i < 9; ++i) post9[i] = 0.0;
        return 1.0 / (0.5 + 3.0 * nue);
    }
    for (int i = 0; i < 9; ++i) post9[i] = (1.0 - o.s) * x[10 + i] * r;
    return 0.0;
}
