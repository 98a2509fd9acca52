/*
 * cs3d_oracle.c -- CPU restatement, in plain C with OpenMP, of the
 * per-Runge-Kutta-stage path of 3DCompactSolver.  TEST INFRASTRUCTURE: the
 * parity tests, the smoke check and the CPU-baseline leg of the benchmark use
 * it as the checker.  The GPU product never links, loads or calls it.
 *
 * It follows the reference's algorithm operation by operation so that,
 * compiled with -O2 -fno-fast-math -ffp-contract=off, it agrees bit for bit
 * with the reference's own sources compiled with the same flags (the pinning
 * test in tests/test_oracle_pin.py checks that).  The layout transposes of the
 * reference (Utils.cpp:95-240) are pure copies; here each line is gathered
 * into a contiguous buffer instead, which gives the same numbers.
 *
 * Citations are file:line in the reference project.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "../include/cs3d.h"

/* ------------------------------------------------------------------ */
/* Ideal gas constants, IdealGas.hpp:36-46                             */
/* ------------------------------------------------------------------ */
typedef struct {
    double gamma, Pr, p_ref, rho_ref, T_ref, mu_ref, R_gas, cp;
} gas_t;

static void gas_init(gas_t *g, double mu_ref) {
    g->gamma = 1.4;
    g->Pr = 0.7;
    g->p_ref = 1.0 / g->gamma;
    g->rho_ref = 1.0;
    g->T_ref = 1.0;
    g->mu_ref = mu_ref;
    g->R_gas = g->p_ref / g->rho_ref / g->T_ref;
    g->cp = g->R_gas * g->gamma / (g->gamma - 1.0);
}
/* IdealGas.hpp:49-80 */
static inline double g_mu(const gas_t *g, double T) { return g->mu_ref * pow(T / g->T_ref, 0.76); }
static inline double g_amu(const gas_t *g, double T) {
    return 0.76 * (g->mu_ref / pow(g->T_ref, 0.76)) * pow(T, 0.76 - 1.0);
}
static inline double g_p(const gas_t *g, double rho, double rhoE, double U, double V, double W) {
    return (g->gamma - 1) * (rhoE - 0.5 * rho * (U * U + V * V + W * W));
}
static inline double g_p_ideal(const gas_t *g, double rho, double T) { return rho * g->R_gas * T; }
static inline double g_T(const gas_t *g, double rho, double p) { return p / (rho * g->R_gas); }
static inline double g_sos(const gas_t *g, double rho, double p) { return sqrt(g->gamma * p / rho); }
static inline double g_rhoE(const gas_t *g, double rho, double p, double U, double V, double W) {
    return p / (g->gamma - 1.0) + 0.5 * rho * (U * U + V * V + W * W);
}
/* Utils.hpp:52-54 */
static inline double neumann6(double f1, double f2, double f3, double f4, double f5, double f6) {
    return (f1 * 360.0 - f2 * 450.0 + f3 * 400.0 - f4 * 225.0 + f5 * 72.0 - f6 * 10.0) / 147.0;
}

/* ------------------------------------------------------------------ */
/* Line solvers, Utils.cpp:4-46                                         */
/* ------------------------------------------------------------------ */
/* Thomas algorithm: forward elimination with multipliers a[i]/w[i-1], then
 * back substitution with division by the modified diagonal (Utils.cpp:4-20). */
static void thomas(const double *a, const double *b, const double *c, const double *d, double *x,
                   double *w, int n) {
    memcpy(w, b, (size_t)n * sizeof(double));
    memcpy(x, d, (size_t)n * sizeof(double));
    for (int i = 1; i < n; i++) {
        double m = a[i] / w[i - 1];
        w[i] = w[i] - m * c[i - 1];
        x[i] = x[i] - m * x[i - 1];
    }
    x[n - 1] /= w[n - 1];
    for (int i = n - 2; i >= 0; i--) x[i] = (x[i] - c[i] * x[i + 1]) / w[i];
}

/* Cyclic tridiagonal system by Sherman-Morrison (Utils.cpp:22-46): corner
 * entries alpha (top right) and beta (bottom left); gamma = -b[0]. */
static void cyclic(const double *a, const double *b, const double *c, double alpha, double beta,
                   const double *r, int n, double *x, double *scratch) {
    double *bb = scratch, *u = scratch + n, *z = scratch + 2 * n, *w = scratch + 3 * n;
    double gamma = -b[0];
    for (int i = 0; i < n; i++) bb[i] = b[i];
    bb[0] = b[0] - gamma;
    bb[n - 1] = b[n - 1] - alpha * beta / gamma;
    thomas(a, bb, c, r, x, w, n);
    for (int i = 0; i < n; i++) u[i] = 0.0;
    u[0] = gamma;
    u[n - 1] = alpha;
    thomas(a, bb, c, u, z, w, n);
    double fact = (x[0] + beta * x[n - 1] / gamma) / (1.0 + z[0] + beta * z[n - 1] / gamma);
    for (int i = 0; i < n; i++) x[i] -= fact * z[i];
}

/* ------------------------------------------------------------------ */
/* Compact operators along one line, Derivatives.hpp:79-161,            */
/* Derivatives.cpp:119-284, Filter.hpp:54-104, Filter.cpp:5-117          */
/* ------------------------------------------------------------------ */
typedef struct {
    int N, bc;            /* length, CS3D_PERIODIC_SOLVE / CS3D_DIRICHLET_SOLVE */
    double dh, alphaF;
    double *lo1, *di1, *up1; /* 1st-derivative matrix diagonals */
    double *lo2, *di2, *up2; /* 2nd-derivative matrix diagonals */
    double *loF, *diF, *upF; /* filter matrix diagonals */
} lineop_t;

/* coefficients, Derivatives.hpp:79-120 */
#define D1_ALPHA (1.0 / 3.0)
#define D1_A (14.0 / 9.0)
#define D1_B (1.0 / 9.0)
#define D1_ALPHA11 5.0
#define D1_A1 (-197.0 / 60.0)
#define D1_B1 (-5.0 / 12.0)
#define D1_C1 5.0
#define D1_D1 (-5.0 / 3.0)
#define D1_E1 (5.0 / 12.0)
#define D1_F1 (-1.0 / 20.0)
#define D1_ALPHA21 (1.0 / 8.0)
#define D1_ALPHA22 (3.0 / 4.0)
#define D1_A2 (-43.0 / 96.0)
#define D1_B2 (-5.0 / 6.0)
#define D1_C2 (9.0 / 8.0)
#define D1_D2 (1.0 / 6.0)
#define D1_E2 (-1.0 / 96.0)
#define D2_ALPHA (2.0 / 11.0)
#define D2_A (12.0 / 11.0)
#define D2_B (3.0 / 11.0)
#define D2_ALPHA11 10.0
#define D2_A1 (145.0 / 12.0)
#define D2_B1 (-76.0 / 3.0)
#define D2_C1 (29.0 / 2.0)
#define D2_D1 (-4.0 / 3.0)
#define D2_E1 (1.0 / 12.0)
#define D2_ALPHA21 (2.0 / 11.0)
#define D2_ALPHA22 (-131.0 / 22.0)
#define D2_A2 (177.0 / 88.0)
#define D2_B2 (-507.0 / 44.0)
#define D2_C2 (783.0 / 44.0)
#define D2_D2 (-201.0 / 22.0)
#define D2_E2 (81.0 / 88.0)
#define D2_F2 (-3.0 / 44.0)

static void lineop_init(lineop_t *op, int N, int bc, double dh, double alphaF) {
    op->N = N;
    op->bc = bc;
    op->dh = dh;
    op->alphaF = alphaF;
    double *m = (double *)malloc(sizeof(double) * 9 * (size_t)N);
    op->lo1 = m; op->di1 = m + N; op->up1 = m + 2 * N;
    op->lo2 = m + 3 * N; op->di2 = m + 4 * N; op->up2 = m + 5 * N;
    op->loF = m + 6 * N; op->diF = m + 7 * N; op->upF = m + 8 * N;
    for (int i = 0; i < N; i++) {
        op->di1[i] = 1.0; op->lo1[i] = D1_ALPHA; op->up1[i] = D1_ALPHA;
        op->di2[i] = 1.0; op->lo2[i] = D2_ALPHA; op->up2[i] = D2_ALPHA;
        op->diF[i] = 1.0; op->loF[i] = alphaF; op->upF[i] = alphaF;
    }
    if (bc == CS3D_DIRICHLET_SOLVE) {
        /* Derivatives.hpp:145-160 */
        op->up1[0] = D1_ALPHA11; op->up1[1] = D1_ALPHA22; op->lo1[1] = D1_ALPHA21;
        op->lo1[N - 1] = D1_ALPHA11; op->lo1[N - 2] = D1_ALPHA22; op->up1[N - 2] = D1_ALPHA21;
        op->up2[0] = D2_ALPHA11; op->up2[1] = D2_ALPHA22; op->lo2[1] = D2_ALPHA21;
        op->lo2[N - 1] = D2_ALPHA11; op->lo2[N - 2] = D2_ALPHA22; op->up2[N - 2] = D2_ALPHA21;
        /* Filter.hpp:89-104: rows 0-2 and N-3..N-1 are explicit */
        for (int r = 0; r < 3; r++) {
            op->loF[r] = 0.0; op->upF[r] = 0.0;
            op->loF[N - 1 - r] = 0.0; op->upF[N - 1 - r] = 0.0;
        }
    }
}

static void lineop_free(lineop_t *op) { free(op->lo1); }

/* Derivatives.cpp:119-150 */
static void rhs_d1_periodic(double dh, const double *f, int N, double *r) {
    double cc2 = -D1_B / 4.0, cc3 = -D1_A / 2.0, cc4 = D1_A / 2.0, cc5 = D1_B / 4.0;
    for (int i = 0; i < N; i++) {
        int im2 = (i - 2 + N) % N, im1 = (i - 1 + N) % N, ip1 = (i + 1) % N, ip2 = (i + 2) % N;
        r[i] = cc2 * f[im2] + cc3 * f[im1] + cc4 * f[ip1] + cc5 * f[ip2];
    }
    for (int i = 0; i < N; i++) r[i] /= dh;
}
/* Derivatives.cpp:153-181 */
static void rhs_d2_periodic(double dh, const double *f, int N, double *r) {
    double cc1 = D2_B / 4.0, cc2 = D2_A, cc3 = -(D2_B / 2.0 + 2.0 * D2_A), cc4 = D2_A, cc5 = D2_B / 4.0;
    for (int i = 0; i < N; i++) {
        int im2 = (i - 2 + N) % N, im1 = (i - 1 + N) % N, ip1 = (i + 1) % N, ip2 = (i + 2) % N;
        r[i] = cc1 * f[im2] + cc2 * f[im1] + cc3 * f[i] + cc4 * f[ip1] + cc5 * f[ip2];
    }
    for (int i = 0; i < N; i++) r[i] /= dh * dh;
}
/* Derivatives.cpp:183-212 */
static void rhs_d1_dirichlet(double dh, const double *f, int N, double *r) {
    double cc2 = -D1_B / 4.0, cc3 = -D1_A / 2.0, cc4 = D1_A / 2.0, cc5 = D1_B / 4.0;
    r[0] = D1_A1 * f[0] + D1_B1 * f[1] + D1_C1 * f[2] + D1_D1 * f[3] + D1_E1 * f[4] + D1_F1 * f[5];
    r[1] = D1_A2 * f[0] + D1_B2 * f[1] + D1_C2 * f[2] + D1_D2 * f[3] + D1_E2 * f[4];
    for (int i = 2; i < N - 2; i++)
        r[i] = cc2 * f[i - 2] + cc3 * f[i - 1] + cc4 * f[i + 1] + cc5 * f[i + 2];
    r[N - 2] = -D1_E2 * f[N - 5] - D1_D2 * f[N - 4] - D1_C2 * f[N - 3] - D1_B2 * f[N - 2] - D1_A2 * f[N - 1];
    r[N - 1] = -D1_F1 * f[N - 6] - D1_E1 * f[N - 5] - D1_D1 * f[N - 4] - D1_C1 * f[N - 3] -
               D1_B1 * f[N - 2] - D1_A1 * f[N - 1];
    for (int i = 0; i < N; i++) r[i] /= dh;
}
/* Derivatives.cpp:214-247 */
static void rhs_d2_dirichlet(double dh, const double *f, int N, double *r) {
    double cc1 = D2_B / 4.0, cc2 = D2_A, cc3 = -(D2_B / 2.0 + 2.0 * D2_A), cc4 = D2_A, cc5 = D2_B / 4.0;
    r[0] = D2_A1 * f[0] + D2_B1 * f[1] + D2_C1 * f[2] + D2_D1 * f[3] + D2_E1 * f[4];
    r[1] = D2_A2 * f[0] + D2_B2 * f[1] + D2_C2 * f[2] + D2_D2 * f[3] + D2_E2 * f[4] + D2_F2 * f[5];
    for (int i = 2; i < N - 2; i++)
        r[i] = cc1 * f[i - 2] + cc2 * f[i - 1] + cc3 * f[i] + cc4 * f[i + 1] + cc5 * f[i + 2];
    r[N - 2] = D2_F2 * f[N - 6] + D2_E2 * f[N - 5] + D2_D2 * f[N - 4] + D2_C2 * f[N - 3] +
               D2_B2 * f[N - 2] + D2_A2 * f[N - 1];
    r[N - 1] = D2_E1 * f[N - 5] + D2_D1 * f[N - 4] + D2_C1 * f[N - 3] + D2_B1 * f[N - 2] + D2_A1 * f[N - 1];
    for (int i = 0; i < N; i++) r[i] /= dh * dh;
}

/* filter RHS coefficients, Filter.hpp:54-81 */
typedef struct { double a0_8, a1_8, a2_8, a3_8, a4_8, a0_6, a1_6, a2_6, a3_6; } fcoef_t;
static fcoef_t fcoef(double aF) {
    fcoef_t c;
    c.a0_8 = (93.0 + 70.0 * aF) / 128.0;
    c.a1_8 = (7.0 + 18.0 * aF) / 16.0;
    c.a2_8 = (-7.0 + 14.0 * aF) / 32.0;
    c.a3_8 = (1.0 - 2.0 * aF) / 16.0;
    c.a4_8 = (-1.0 + 2.0 * aF) / 128.0;
    c.a0_6 = (11.0 + 10.0 * aF) / 16.0;
    c.a1_6 = (15.0 + 34.0 * aF) / 32.0;
    c.a2_6 = (-3.0 + 6.0 * aF) / 16.0;
    c.a3_6 = (1.0 - 2.0 * aF) / 32.0;
    return c;
}
#define FA00 (15.0 / 16.0)
#define FA01 (4.0 / 16.0)
#define FA02 (-6.0 / 16.0)
#define FA03 (4.0 / 16.0)
#define FA04 (-1.0 / 16.0)
#define FB00 (1.0 / 16.0)
#define FB01 (3.0 / 4.0)
#define FB02 (6.0 / 16.0)
#define FB03 (-4.0 / 16.0)
#define FB04 (1.0 / 16.0)
#define FC00 (-1.0 / 16.0)
#define FC01 (4.0 / 16.0)
#define FC02 (5.0 / 8.0)
#define FC03 (4.0 / 16.0)
#define FC04 (-1.0 / 16.0)

/* Filter.cpp:5-62: 9-point symmetric stencil with periodic wrap; the sum
 * runs from the -4 neighbour to the +4 neighbour. */
static void rhs_filter_periodic(double aF, const double *f, int N, double *r) {
    fcoef_t c = fcoef(aF);
    double cc0 = c.a0_8, cc1 = c.a1_8 / 2.0, cc2 = c.a2_8 / 2.0, cc3 = c.a3_8 / 2.0, cc4 = c.a4_8 / 2.0;
    for (int i = 0; i < N; i++) {
#define W(o) f[((i + (o)) % N + N) % N]
        r[i] = cc4 * W(-4) + cc3 * W(-3) + cc2 * W(-2) + cc1 * W(-1) + cc0 * W(0) + cc1 * W(1) +
               cc2 * W(2) + cc3 * W(3) + cc4 * W(4);
#undef W
    }
}
/* Filter.cpp:64-96 */
static void rhs_filter_dirichlet(double aF, const double *f, int N, double *r) {
    fcoef_t c = fcoef(aF);
    double aa0 = c.a0_6, aa1 = c.a1_6 / 2.0, aa2 = c.a2_6 / 2.0, aa3 = c.a3_6 / 2.0;
    double cc0 = c.a0_8, cc1 = c.a1_8 / 2.0, cc2 = c.a2_8 / 2.0, cc3 = c.a3_8 / 2.0, cc4 = c.a4_8 / 2.0;
    r[0] = FA00 * f[0] + FA01 * f[1] + FA02 * f[2] + FA03 * f[3] + FA04 * f[4];
    r[1] = FB00 * f[0] + FB01 * f[1] + FB02 * f[2] + FB03 * f[3] + FB04 * f[4];
    r[2] = FC00 * f[0] + FC01 * f[1] + FC02 * f[2] + FC03 * f[3] + FC04 * f[4];
    r[3] = aa3 * f[0] + aa2 * f[1] + aa1 * f[2] + aa0 * f[3] + aa1 * f[4] + aa2 * f[5] + aa3 * f[6];
    r[N - 1] = FA00 * f[N - 1] + FA01 * f[N - 2] + FA02 * f[N - 3] + FA03 * f[N - 4] + FA04 * f[N - 5];
    r[N - 2] = FB00 * f[N - 1] + FB01 * f[N - 2] + FB02 * f[N - 3] + FB03 * f[N - 4] + FB04 * f[N - 5];
    r[N - 3] = FC00 * f[N - 1] + FC01 * f[N - 2] + FC02 * f[N - 3] + FC03 * f[N - 4] + FC04 * f[N - 5];
    r[N - 4] = aa3 * f[N - 1] + aa2 * f[N - 2] + aa1 * f[N - 3] + aa0 * f[N - 4] + aa1 * f[N - 5] +
               aa2 * f[N - 6] + aa3 * f[N - 7];
    for (int i = 4; i < N - 4; i++)
        r[i] = cc4 * f[i - 4] + cc3 * f[i - 3] + cc2 * f[i - 2] + cc1 * f[i - 1] + cc0 * f[i] +
               cc1 * f[i + 1] + cc2 * f[i + 2] + cc3 * f[i + 3] + cc4 * f[i + 4];
}

/* One operator on one contiguous line: kind 1 = 1st derivative
 * (Compact1stPeriodic/Dirichlet, Derivatives.cpp:250-275), 2 = 2nd
 * derivative (:258-284), 3 = filter (FilterPeriodic/Dirichlet,
 * Filter.cpp:98-117).  work holds 6*N doubles. */
static void line_apply(const lineop_t *op, int kind, const double *f, double *out, double *work) {
    int N = op->N;
    double *r = work, *scr = work + N;
    if (op->bc == CS3D_PERIODIC_SOLVE) {
        if (kind == 1) {
            rhs_d1_periodic(op->dh, f, N, r);
            cyclic(op->lo1, op->di1, op->up1, D1_ALPHA, D1_ALPHA, r, N, out, scr);
        } else if (kind == 2) {
            rhs_d2_periodic(op->dh, f, N, r);
            cyclic(op->lo2, op->di2, op->up2, D2_ALPHA, D2_ALPHA, r, N, out, scr);
        } else {
            rhs_filter_periodic(op->alphaF, f, N, r);
            cyclic(op->loF, op->diF, op->upF, op->alphaF, op->alphaF, r, N, out, scr);
        }
    } else {
        if (kind == 1) {
            rhs_d1_dirichlet(op->dh, f, N, r);
            thomas(op->lo1, op->di1, op->up1, r, out, scr, N);
        } else if (kind == 2) {
            rhs_d2_dirichlet(op->dh, f, N, r);
            thomas(op->lo2, op->di2, op->up2, r, out, scr, N);
        } else {
            rhs_filter_dirichlet(op->alphaF, f, N, r);
            thomas(op->loF, op->diF, op->upF, r, out, scr, N);
        }
    }
}

/* ------------------------------------------------------------------ */
/* Solver state                                                         */
/* ------------------------------------------------------------------ */
enum {
    /* conserved */
    A_RHO1, A_RHOU1, A_RHOV1, A_RHOW1, A_RHOE1,
    A_RHOK, A_RHOUK, A_RHOVK, A_RHOWK, A_RHOEK,
    A_RHO2, A_RHOU2, A_RHOV2, A_RHOW2, A_RHOE2,
    A_RHOK2, A_RHOUK2, A_RHOVK2, A_RHOWK2, A_RHOEK2,
    /* primitives */
    A_U, A_V, A_W, A_P, A_T, A_MU, A_SOS, A_AMU,
    /* sponge */
    A_SRHO, A_SRHOU, A_SRHOV, A_SRHOW, A_SRHOE, A_SIGMA,
    /* derivatives, CSolver_AWS.hpp:51-72 */
    A_UX, A_UY, A_UZ, A_VX, A_VY, A_VZ, A_WX, A_WY, A_WZ,
    A_UXX, A_UYY, A_UZZ, A_VXX, A_VYY, A_VZZ, A_WXX, A_WYY, A_WZZ,
    A_UXY, A_UXZ, A_UYZ, A_VXY, A_VXZ, A_VYZ, A_WXY, A_WXZ, A_WYZ,
    A_TX, A_TY, A_TZ, A_TXX, A_TYY, A_TZZ,
    A_CEX, A_CEY, A_CEZ, A_MXX, A_MXY, A_MXZ, A_MYX, A_MYY, A_MYZ,
    A_MZX, A_MZY, A_MZZ, A_EX, A_EY, A_EZ,
    /* scratch */
    A_T1, A_T2, A_T3, A_T4, A_F1, A_F2,
    A_COUNT
};

static const char *A_NAMES[A_COUNT] = {
    "rho1", "rhoU1", "rhoV1", "rhoW1", "rhoE1", "rhok", "rhoUk", "rhoVk", "rhoWk", "rhoEk",
    "rho2", "rhoU2", "rhoV2", "rhoW2", "rhoE2", "rhok2", "rhoUk2", "rhoVk2", "rhoWk2", "rhoEk2",
    "U", "V", "W", "p", "T", "mu", "sos", "Amu",
    "spongeRhoAvg", "spongeRhoUAvg", "spongeRhoVAvg", "spongeRhoWAvg", "spongeRhoEAvg", "sigma",
    "Ux", "Uy", "Uz", "Vx", "Vy", "Vz", "Wx", "Wy", "Wz",
    "Uxx", "Uyy", "Uzz", "Vxx", "Vyy", "Vzz", "Wxx", "Wyy", "Wzz",
    "Uxy", "Uxz", "Uyz", "Vxy", "Vxz", "Vyz", "Wxy", "Wxz", "Wyz",
    "Tx", "Ty", "Tz", "Txx", "Tyy", "Tzz",
    "contEulerX", "contEulerY", "contEulerZ", "momXEulerX", "momXEulerY", "momXEulerZ",
    "momYEulerX", "momYEulerY", "momYEulerZ", "momZEulerX", "momZEulerY", "momZEulerZ",
    "engyEulerX", "engyEulerY", "engyEulerZ",
    "temp", "temp2", "temp3", "temp4", "ftmp1", "ftmp2"};

typedef struct or_solver {
    cs3d_config cfg;
    int Nx, Ny, Nz;
    size_t N;
    double dx, dy, dz;
    double *x, *y, *z;
    gas_t g;
    lineop_t op[3];
    double *a[A_COUNT];
    int sponge_flag;
    int nstages;
    int rkStep, rkLast;
    int timeStep, filterTimeStep;
    double time, dt;
    double avgT, epsP, spongeP, spongeStrength;
} or_solver;

#define IDX(i, j, k) ((size_t)(k) * (size_t)s->Nx * (size_t)s->Ny + (size_t)(j) * (size_t)s->Nx + (size_t)(i))

/* Apply a line operator along direction dir to every line of field in,
 * writing field out (both XYZ).  Lines are gathered into a contiguous buffer,
 * which is what the reference's transposes achieve. */
static void field_apply(or_solver *s, int dir, int kind, const double *in, double *out) {
    int Nd = dir == 0 ? s->Nx : dir == 1 ? s->Ny : s->Nz;
    int n1 = dir == 0 ? s->Ny : s->Nx;          /* first other index */
    int n2 = dir == 2 ? s->Ny : s->Nz;          /* second other index */
    size_t stride = dir == 0 ? 1 : dir == 1 ? (size_t)s->Nx : (size_t)s->Nx * s->Ny;
    const lineop_t *op = &s->op[dir];
    long nl = (long)n1 * n2;
#pragma omp parallel
    {
        double *buf = (double *)malloc(sizeof(double) * 8 * (size_t)Nd);
        double *fin = buf, *fout = buf + Nd, *work = buf + 2 * Nd;
#pragma omp for schedule(static)
        for (long l = 0; l < nl; l++) {
            int a1 = (int)(l % n1), a2 = (int)(l / n1);
            size_t base;
            if (dir == 0) base = IDX(0, a1, a2);
            else if (dir == 1) base = IDX(a1, 0, a2);
            else base = IDX(a1, a2, 0);
            for (int t = 0; t < Nd; t++) fin[t] = in[base + t * stride];
            line_apply(op, kind, fin, fout, work);
            for (int t = 0; t < Nd; t++) out[base + t * stride] = fout[t];
        }
        free(buf);
    }
}

/* ------------------------------------------------------------------ */
/* create / destroy                                                     */
/* ------------------------------------------------------------------ */
or_solver *or_create(const cs3d_config *c) {
    if (!c || c->Nx < 3 || c->Ny < 3 || c->Nz < 3) return NULL;
    or_solver *s = (or_solver *)calloc(1, sizeof(or_solver));
    s->cfg = *c;
    s->Nx = c->Nx; s->Ny = c->Ny; s->Nz = c->Nz;
    s->N = (size_t)c->Nx * c->Ny * c->Nz;
    /* Domain.hpp:28-45 */
    s->x = (double *)malloc(sizeof(double) * c->Nx);
    s->y = (double *)malloc(sizeof(double) * c->Ny);
    s->z = (double *)malloc(sizeof(double) * c->Nz);
    for (int i = 0; i < c->Nx; i++) s->x[i] = (((double)i) / ((double)c->Nx - 1.0)) * c->Lx;
    for (int j = 0; j < c->Ny; j++) s->y[j] = (((double)j) / ((double)c->Ny - 1.0)) * c->Ly;
    for (int k = 0; k < c->Nz; k++) s->z[k] = (((double)k) / ((double)c->Nz - 1.0)) * c->Lz;
    s->dx = s->x[1] - s->x[0];
    s->dy = s->y[1] - s->y[0];
    s->dz = s->z[1] - s->z[0];
    gas_init(&s->g, c->mu_ref);
    lineop_init(&s->op[0], c->Nx, c->bc_type[0], s->dx, c->alphaF);
    lineop_init(&s->op[1], c->Ny, c->bc_type[1], s->dy, c->alphaF);
    lineop_init(&s->op[2], c->Nz, c->bc_type[2], s->dz, c->alphaF);
    for (int f = 0; f < A_COUNT; f++) {
        s->a[f] = (double *)calloc(s->N, sizeof(double));
        if (!s->a[f]) return NULL;
    }
    s->nstages = c->rk == CS3D_TVDRK3 ? 3 : 4;
    /* SpongeBC.hpp:56-62 */
    s->avgT = 15.0;
    s->epsP = 0.005;
    s->spongeP = 1.0 / s->g.gamma;
    s->spongeStrength = 6.0;
    /* sponge strength (SpongeBC.hpp:64-150) with sigma starting at zero */
    const double L[3] = {c->Lx, c->Ly, c->Lz};
    const double dflt[3] = {0.25, 0.125, 0.25};
    double *coord[3] = {s->x, s->y, s->z};
    int Nd[3] = {s->Nx, s->Ny, s->Nz};
    s->sponge_flag = 0;
    for (int f = 0; f < 6; f++) {
        int dir = f / 2, hi = f % 2;
        double band;
        if (c->sponge_mode == CS3D_SPONGE_REFERENCE)
            band = (c->bc_kind[f] == CS3D_SPONGE) ? dflt[dir] * L[dir] : 0.0;
        else
            band = c->sponge_frac[f] * L[dir];
        if (band <= 0.0) continue;
        s->sponge_flag = 1;
        for (int a = 0; a < Nd[dir]; a++) {
            double xc = coord[dir][a], sx;
            if (!hi) { if (!(xc < band)) continue; sx = (band - xc) / band; }
            else { if (!(xc > L[dir] - band)) continue; sx = (xc - (L[dir] - band)) / band; }
            double val = s->spongeStrength * (0.068 * pow(sx, 2.0) + 0.845 * pow(sx, 8.0));
            for (int k = 0; k < s->Nz; k++)
                for (int j = 0; j < s->Ny; j++)
                    for (int i = 0; i < s->Nx; i++) {
                        int idx3[3] = {i, j, k};
                        if (idx3[dir] != a) continue;
                        size_t ii = IDX(i, j, k);
                        s->a[A_SIGMA][ii] = fmax(val, s->a[A_SIGMA][ii]);
                    }
        }
    }
    return s;
}

void or_destroy(or_solver *s) {
    if (!s) return;
    for (int f = 0; f < A_COUNT; f++) free(s->a[f]);
    for (int d = 0; d < 3; d++) lineop_free(&s->op[d]);
    free(s->x); free(s->y); free(s->z);
    free(s);
}

/* ------------------------------------------------------------------ */
/* Boundary handling                                                    */
/* ------------------------------------------------------------------ */
/* Visit every point of face f (0..5 = X0,X1,Y0,Y1,Z0,Z1) in the order of
 * the FOR_X0..FOR_Z1 loops (Macros.hpp:60-65); for each, `nb[m]` is the
 * index m+1 points into the domain (the GET3DINDEX_XYZ_?p? / ?m? macros). */
typedef void (*face_fn)(or_solver *s, size_t ip, const size_t nb[6], void *ctx);
static void for_face(or_solver *s, int f, face_fn fn, void *ctx) {
    int dir = f / 2, hi = f % 2;
    int Nd = dir == 0 ? s->Nx : dir == 1 ? s->Ny : s->Nz;
    int fix = hi ? Nd - 1 : 0;
    int sgn = hi ? -1 : 1;
    int n1 = dir == 0 ? s->Ny : s->Nx, n2 = dir == 2 ? s->Ny : s->Nz;
#pragma omp parallel for schedule(static)
    for (long l = 0; l < (long)n1 * n2; l++) {
        int a1 = (int)(l % n1), a2 = (int)(l / n1);
        int i, j, k;
        if (dir == 0) { i = fix; j = a1; k = a2; }
        else if (dir == 1) { i = a1; j = fix; k = a2; }
        else { i = a1; j = a2; k = fix; }
        size_t ip = IDX(i, j, k), nb[6];
        for (int m = 0; m < 6; m++) {
            int o = sgn * (m + 1);
            nb[m] = dir == 0 ? IDX(i + o, j, k) : dir == 1 ? IDX(i, j + o, k) : IDX(i, j, k + o);
        }
        fn(s, ip, nb, ctx);
    }
}

typedef struct { double *rho, *rhoU, *rhoV, *rhoW, *rhoE; double uw[3]; int dir; } wall_ctx;

/* preStepBCHandling body for one wall point, CSolver_AWS.cpp:576-593 */
static void wall_pre(or_solver *s, size_t ip, const size_t nb[6], void *vc) {
    wall_ctx *c = (wall_ctx *)vc;
    double *U = s->a[A_U], *V = s->a[A_V], *W = s->a[A_W], *T = s->a[A_T], *p = s->a[A_P];
    U[ip] = c->uw[0];
    V[ip] = c->uw[1];
    W[ip] = c->uw[2];
    c->rhoU[ip] = c->dir == 0 ? 0.0 : c->rho[ip] * c->uw[0];
    c->rhoV[ip] = c->dir == 1 ? 0.0 : c->rho[ip] * c->uw[1];
    c->rhoW[ip] = c->dir == 2 ? 0.0 : c->rho[ip] * c->uw[2];
    T[ip] = neumann6(T[nb[0]], T[nb[1]], T[nb[2]], T[nb[3]], T[nb[4]], T[nb[5]]);
    p[ip] = g_p_ideal(&s->g, c->rho[ip], T[ip]);
    c->rhoE[ip] = g_rhoE(&s->g, c->rho[ip], p[ip], U[ip], V[ip], W[ip]);
}

/* Wall velocity (U,V,W) of face f for kind: zero for ADIABATIC_WALL; the
 * tangential moving-wall speeds for MOVING_ADIABATIC_WALL. */
static void wall_velocity(const or_solver *s, int f, int kind, double uw[3]) {
    uw[0] = uw[1] = uw[2] = 0.0;
    if (kind != CS3D_MOVING_ADIABATIC_WALL) return;
    const double *v = s->cfg.wall_vel;
    switch (f) {
    case 0: uw[1] = v[0]; uw[2] = v[1]; break;
    case 1: uw[1] = v[2]; uw[2] = v[3]; break;
    case 2: uw[0] = v[4]; uw[2] = v[5]; break;
    case 3: uw[0] = v[6]; uw[2] = v[7]; break;
    case 4: uw[0] = v[8]; uw[1] = v[9]; break;
    case 5: uw[0] = v[10]; uw[1] = v[11]; break;
    }
}

static void stage_input(or_solver *s, double **q) {
    int base = s->rkStep == 1 ? A_RHO1 : A_RHOK;
    for (int f = 0; f < 5; f++) q[f] = s->a[base + f];
}

/* CSolver_AWS.cpp:553-826: all ADIABATIC_WALL faces in the order
 * X0,X1,Y0,Y1,Z0,Z1, then all MOVING_ADIABATIC_WALL faces in that order. */
static void pre_bc(or_solver *s) {
    double *q[5];
    stage_input(s, q);
    for (int pass = 0; pass < 2; pass++) {
        int kind = pass == 0 ? CS3D_ADIABATIC_WALL : CS3D_MOVING_ADIABATIC_WALL;
        for (int f = 0; f < 6; f++) {
            if (s->cfg.bc_kind[f] != kind) continue;
            wall_ctx c = {q[0], q[1], q[2], q[3], q[4], {0, 0, 0}, f / 2};
            wall_velocity(s, f, kind, c.uw);
            for_face(s, f, wall_pre, &c);
        }
    }
}

/* ------------------------------------------------------------------ */
/* preStepDerivatives, CSolver_AWS.cpp:829-1243                          */
/* ------------------------------------------------------------------ */
static void primitives_from(or_solver *s, double **q) {
    double *U = s->a[A_U], *V = s->a[A_V], *W = s->a[A_W], *p = s->a[A_P], *T = s->a[A_T];
#pragma omp parallel for schedule(static)
    for (long ip = 0; ip < (long)s->N; ip++) {
        U[ip] = q[1][ip] / q[0][ip];
        V[ip] = q[2][ip] / q[0][ip];
        W[ip] = q[3][ip] / q[0][ip];
        p[ip] = g_p(&s->g, q[0][ip], q[4][ip], U[ip], V[ip], W[ip]);
        T[ip] = g_T(&s->g, q[0][ip], p[ip]);
    }
}

static void pre_derivatives(or_solver *s) {
    double *q[5];
    stage_input(s, q);
    double **A = s->a;
    double *U = A[A_U], *V = A[A_V], *W = A[A_W], *p = A[A_P], *T = A[A_T];
    double *t1 = A[A_T1], *t2 = A[A_T2], *t3 = A[A_T3], *t4 = A[A_T4];

    /* X phase: Euler x-fluxes from the stage-start primitives (:862-867) */
#pragma omp parallel for schedule(static)
    for (long ip = 0; ip < (long)s->N; ip++) {
        t1[ip] = q[1][ip] * U[ip] + p[ip];
        t2[ip] = q[2][ip] * U[ip];
        t3[ip] = q[3][ip] * U[ip];
        t4[ip] = q[4][ip] * U[ip] + U[ip] * p[ip];
    }
    field_apply(s, 0, 1, U, A[A_UX]);
    field_apply(s, 0, 1, q[1], A[A_CEX]);
    field_apply(s, 0, 1, V, A[A_VX]);
    field_apply(s, 0, 1, W, A[A_WX]);
    field_apply(s, 0, 2, U, A[A_UXX]);
    field_apply(s, 0, 2, V, A[A_VXX]);
    field_apply(s, 0, 2, W, A[A_WXX]);
    field_apply(s, 0, 1, T, A[A_TX]);
    field_apply(s, 0, 2, T, A[A_TXX]);
    field_apply(s, 0, 1, t1, A[A_MXX]);
    field_apply(s, 0, 1, t2, A[A_MYX]);
    field_apply(s, 0, 1, t3, A[A_MZX]);
    field_apply(s, 0, 1, t4, A[A_EX]);

    /* Y phase: primitives recomputed from the conserved variables (:950-963) */
    primitives_from(s, q);
#pragma omp parallel for schedule(static)
    for (long ip = 0; ip < (long)s->N; ip++) {
        t1[ip] = q[1][ip] * V[ip];
        t2[ip] = q[2][ip] * V[ip] + p[ip];
        t3[ip] = q[3][ip] * V[ip];
        t4[ip] = q[4][ip] * V[ip] + V[ip] * p[ip];
    }
    field_apply(s, 1, 1, U, A[A_UY]);
    field_apply(s, 1, 1, V, A[A_VY]);
    field_apply(s, 1, 1, W, A[A_WY]);
    field_apply(s, 1, 1, A[A_UX], A[A_UXY]);
    field_apply(s, 1, 1, A[A_VX], A[A_VXY]);
    field_apply(s, 1, 1, A[A_WX], A[A_WXY]);
    field_apply(s, 1, 1, q[2], A[A_CEY]);
    field_apply(s, 1, 2, U, A[A_UYY]);
    field_apply(s, 1, 2, V, A[A_VYY]);
    field_apply(s, 1, 2, W, A[A_WYY]);
    field_apply(s, 1, 1, T, A[A_TY]);
    field_apply(s, 1, 2, T, A[A_TYY]);
    field_apply(s, 1, 1, t1, A[A_MXY]);
    field_apply(s, 1, 1, t2, A[A_MYY]);
    field_apply(s, 1, 1, t3, A[A_MZY]);
    field_apply(s, 1, 1, t4, A[A_EY]);

    /* Z phase (:1095-1223) */
    primitives_from(s, q);
#pragma omp parallel for schedule(static)
    for (long ip = 0; ip < (long)s->N; ip++) {
        t1[ip] = q[1][ip] * W[ip];
        t2[ip] = q[2][ip] * W[ip];
        t3[ip] = q[3][ip] * W[ip] + p[ip];
        t4[ip] = q[4][ip] * W[ip] + W[ip] * p[ip];
    }
    field_apply(s, 2, 1, U, A[A_UZ]);
    field_apply(s, 2, 2, U, A[A_UZZ]);
    field_apply(s, 2, 1, V, A[A_VZ]);
    field_apply(s, 2, 2, V, A[A_VZZ]);
    field_apply(s, 2, 1, W, A[A_WZ]);
    field_apply(s, 2, 2, W, A[A_WZZ]);
    field_apply(s, 2, 1, T, A[A_TZ]);
    field_apply(s, 2, 2, T, A[A_TZZ]);
    field_apply(s, 2, 1, A[A_UX], A[A_UXZ]);
    field_apply(s, 2, 1, A[A_VX], A[A_VXZ]);
    field_apply(s, 2, 1, A[A_WX], A[A_WXZ]);
    field_apply(s, 2, 1, A[A_UY], A[A_UYZ]);
    field_apply(s, 2, 1, A[A_VY], A[A_VYZ]);
    field_apply(s, 2, 1, A[A_WY], A[A_WYZ]);
    field_apply(s, 2, 1, q[3], A[A_CEZ]);
    field_apply(s, 2, 1, t1, A[A_MXZ]);
    field_apply(s, 2, 1, t2, A[A_MYZ]);
    field_apply(s, 2, 1, t3, A[A_MZZ]);
    field_apply(s, 2, 1, t4, A[A_EZ]);

    /* back to the stage input's primitives (:1226-1233) */
    primitives_from(s, q);
}

/* ------------------------------------------------------------------ */
/* Right-hand sides, CSolver_AWS.cpp:1246-1504                            */
/* ------------------------------------------------------------------ */
static void solve_eqn_set(or_solver *s) {
    double *q[5];
    stage_input(s, q);
    double **A = s->a;
    const double dt = s->dt;
    const gas_t *g = &s->g;
    const int spg = s->sponge_flag;
    double *U = A[A_U], *V = A[A_V], *W = A[A_W], *mu = A[A_MU], *Amu = A[A_AMU];
    double *Ux = A[A_UX], *Uy = A[A_UY], *Uz = A[A_UZ], *Vx = A[A_VX], *Vy = A[A_VY], *Vz = A[A_VZ];
    double *Wx = A[A_WX], *Wy = A[A_WY], *Wz = A[A_WZ];
    double *Uxx = A[A_UXX], *Uyy = A[A_UYY], *Uzz = A[A_UZZ], *Vxx = A[A_VXX], *Vyy = A[A_VYY];
    double *Vzz = A[A_VZZ], *Wxx = A[A_WXX], *Wyy = A[A_WYY], *Wzz = A[A_WZZ];
    double *Uxy = A[A_UXY], *Uxz = A[A_UXZ], *Vxy = A[A_VXY], *Vyz = A[A_VYZ], *Wxz = A[A_WXZ];
    double *Wyz = A[A_WYZ];
    double *Tx = A[A_TX], *Ty = A[A_TY], *Tz = A[A_TZ], *Txx = A[A_TXX], *Tyy = A[A_TYY], *Tzz = A[A_TZZ];
    double *sig = A[A_SIGMA];

#pragma omp parallel for schedule(static)
    for (long ip = 0; ip < (long)s->N; ip++) {
        double src;
        /* continuity, :1261-1270 */
        src = spg ? sig[ip] * (A[A_SRHO][ip] - q[0][ip]) : 0.0;
        A[A_RHOK2][ip] = dt * (-A[A_CEX][ip] - A[A_CEY][ip] - A[A_CEZ][ip] + src);

        double MuX = Amu[ip] * Tx[ip], MuY = Amu[ip] * Ty[ip], MuZ = Amu[ip] * Tz[ip];
        double r;
        /* x-momentum, :1297-1316 */
        src = spg ? sig[ip] * (A[A_SRHOU][ip] - q[1][ip]) : 0.0;
        r = mu[ip] * ((4.0 / 3.0) * Uxx[ip] + Uyy[ip] + Uzz[ip] + (1.0 / 3.0) * Vxy[ip] + (1.0 / 3.0) * Wxz[ip]);
        r += (4.0 / 3.0) * MuX * (Ux[ip] - 0.5 * Vy[ip] - 0.5 * Wz[ip]) + MuY * (Uy[ip] + Vx[ip]) +
             MuZ * (Wx[ip] + Uz[ip]);
        r += -A[A_MXX][ip] - A[A_MXY][ip] - A[A_MXZ][ip] + src;
        r *= dt;
        A[A_RHOUK2][ip] = r;
        /* y-momentum, :1345-1365 */
        src = spg ? sig[ip] * (A[A_SRHOV][ip] - q[2][ip]) : 0.0;
        r = mu[ip] * ((4.0 / 3.0) * Vyy[ip] + Vxx[ip] + Vzz[ip] + (1.0 / 3.0) * Uxy[ip] + (1.0 / 3.0) * Wyz[ip]);
        r += (4.0 / 3.0) * MuY * (Vy[ip] - 0.5 * Ux[ip] - 0.5 * Wz[ip]) + MuX * (Uy[ip] + Vx[ip]) +
             MuZ * (Wy[ip] + Vz[ip]);
        r += -A[A_MYX][ip] - A[A_MYY][ip] - A[A_MYZ][ip] + src;
        r *= dt;
        A[A_RHOVK2][ip] = r;
        /* z-momentum, :1393-1414 */
        src = spg ? sig[ip] * (A[A_SRHOW][ip] - q[3][ip]) : 0.0;
        r = mu[ip] * ((4.0 / 3.0) * Wzz[ip] + Wyy[ip] + Wxx[ip] + (1.0 / 3.0) * Uxz[ip] + (1.0 / 3.0) * Vyz[ip]);
        r += (4.0 / 3.0) * MuZ * (Wz[ip] - 0.5 * Ux[ip] - 0.5 * Vy[ip]) + MuX * (Wx[ip] + Uz[ip]) +
             MuY * (Wy[ip] + Vz[ip]);
        r += -A[A_MZX][ip] - A[A_MZY][ip] - A[A_MZZ][ip] + src;
        r *= dt;
        A[A_RHOWK2][ip] = r;
        /* energy, :1446-1495 (sponge source entered twice, :1491,1495) */
        src = spg ? sig[ip] * (A[A_SRHOE][ip] - q[4][ip]) : 0.0;
        double qtemp = g->cp / g->Pr *
                       (MuX * Tx[ip] + MuY * Ty[ip] + MuZ * Tz[ip] + mu[ip] * Txx[ip] + mu[ip] * Tyy[ip] +
                        mu[ip] * Tzz[ip]);
        double vtemp1 =
            mu[ip] * (U[ip] * ((4.0 / 3.0) * Uxx[ip] + Uyy[ip] + Uzz[ip]) +
                      V[ip] * (Vxx[ip] + (4.0 / 3.0) * Vyy[ip] + Vzz[ip]) +
                      W[ip] * (Wxx[ip] + Wyy[ip] + (4.0 / 3.0) * Wzz[ip]) +
                      (4.0 / 3.0) * (Ux[ip] * Ux[ip] + Vy[ip] * Vy[ip] + Wz[ip] * Wz[ip]) + Uy[ip] * Uy[ip] +
                      Uz[ip] * Uz[ip] + Vx[ip] * Vx[ip] + Vz[ip] * Vz[ip] + Wx[ip] * Wx[ip] +
                      Wy[ip] * Wy[ip] - (4.0 / 3.0) * (Ux[ip] * Vy[ip] + Ux[ip] * Wz[ip] + Vy[ip] * Wz[ip]) +
                      2.0 * (Uy[ip] * Vx[ip] + Uz[ip] * Wx[ip] + Vz[ip] * Wy[ip]) +
                      (1.0 / 3.0) * (U[ip] * Vxy[ip] + U[ip] * Wxz[ip] + V[ip] * Uxy[ip]) +
                      (1.0 / 3.0) * (V[ip] * Wyz[ip] + W[ip] * Uxz[ip] + W[ip] * Vyz[ip]));
        double vtemp2 = (4.0 / 3.0) * (U[ip] * MuX * Ux[ip] + V[ip] * MuY * Vy[ip] + W[ip] * MuZ * Wz[ip]) -
                        (2.0 / 3.0) * U[ip] * MuX * (Vy[ip] + Wz[ip]) -
                        (2.0 / 3.0) * V[ip] * MuY * (Ux[ip] + Wz[ip]) -
                        (2.0 / 3.0) * W[ip] * MuZ * (Ux[ip] + Vy[ip]) + U[ip] * MuY * (Uy[ip] + Vx[ip]) +
                        U[ip] * MuZ * (Uz[ip] + Wx[ip]) + V[ip] * MuX * (Uy[ip] + Vx[ip]) +
                        V[ip] * MuZ * (Vz[ip] + Wy[ip]) + W[ip] * MuX * (Uz[ip] + Wx[ip]) +
                        W[ip] * MuY * (Vz[ip] + Wy[ip]);
        double engyEuler = -A[A_EX][ip] - A[A_EY][ip] - A[A_EZ][ip] + src;
        A[A_RHOEK2][ip] = dt * (qtemp + vtemp1 + vtemp2 + engyEuler + src);
    }
}

/* postStepBCHandling, CSolver_AWS.cpp:1506-1679 */
typedef struct { int dir; } post_ctx;
static void wall_post(or_solver *s, size_t ip, const size_t nb[6], void *vc) {
    (void)nb;
    int dir = ((post_ctx *)vc)->dir;
    double *ce = s->a[dir == 0 ? A_CEX : dir == 1 ? A_CEY : A_CEZ];
    s->a[A_RHOK2][ip] = -s->dt * ce[ip];
    s->a[A_RHOUK2][ip] = 0.0;
    s->a[A_RHOVK2][ip] = 0.0;
    s->a[A_RHOWK2][ip] = 0.0;
    s->a[A_RHOEK2][ip] = 0.0;
}
static void sponge_post(or_solver *s, size_t ip, const size_t nb[6], void *vc) {
    (void)nb; (void)vc;
    for (int f = 0; f < 5; f++) s->a[A_RHOK2 + f][ip] = 0.0;
}
static void post_bc(or_solver *s) {
    for (int f = 0; f < 6; f++) {
        int k = s->cfg.bc_kind[f];
        if (k == CS3D_ADIABATIC_WALL || k == CS3D_MOVING_ADIABATIC_WALL) {
            post_ctx c = {f / 2};
            for_face(s, f, wall_post, &c);
        }
    }
    for (int f = 0; f < 6; f++)
        if (s->cfg.bc_kind[f] == CS3D_SPONGE) for_face(s, f, sponge_post, NULL);
}

/* ------------------------------------------------------------------ */
/* RK updates, RK4.hpp:35-118, TVDRK3.hpp:38-96                          */
/* ------------------------------------------------------------------ */
static void rk_update(or_solver *s) {
    double **A = s->a;
    long N = (long)s->N;
    int st = s->rkStep;
    if (s->cfg.rk == CS3D_TVDRK3) {
        const double a2 = 3.0 / 4.0, a3 = 1.0 / 3.0, b2 = 1.0 / 4.0, b3 = 2.0 / 3.0;
        const double c1 = 1.0, c2 = 1.0 / 4.0, c3 = 2.0 / 3.0;
#pragma omp parallel for schedule(static)
        for (long ip = 0; ip < N; ip++)
            for (int f = 0; f < 5; f++) {
                double q1 = A[A_RHO1 + f][ip], dq = A[A_RHOK2 + f][ip];
                if (st == 1) A[A_RHOK + f][ip] = q1 + c1 * dq;
                else if (st == 2) A[A_RHOK + f][ip] = a2 * q1 + b2 * A[A_RHOK + f][ip] + c2 * dq;
                else A[A_RHO2 + f][ip] = a3 * q1 + b3 * A[A_RHOK + f][ip] + c3 * dq;
            }
    } else {
        const double a[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
        const double b[3] = {1.0 / 2.0, 1.0 / 2.0, 1.0};
#pragma omp parallel for schedule(static)
        for (long ip = 0; ip < N; ip++)
            for (int f = 0; f < 5; f++) {
                double q1 = A[A_RHO1 + f][ip], dq = A[A_RHOK2 + f][ip];
                if (st == 1) A[A_RHO2 + f][ip] = q1 + a[0] * dq;
                else A[A_RHO2 + f][ip] += a[st - 1] * dq;
                if (st < 4) A[A_RHOK + f][ip] = q1 + b[st - 1] * dq;
            }
    }
}

/* ------------------------------------------------------------------ */
/* filterConservedData (CSolver_AWS.cpp:1682-1893), updateNonConservedData */
/* (:1895-1935)                                                           */
/* ------------------------------------------------------------------ */
static void filter_conserved(or_solver *s) {
    double **A = s->a;
    if (s->timeStep % s->cfg.filter_step == 0) {
        s->filterTimeStep++;
        int order[3];
        int m = s->filterTimeStep % 3;
        if (m == 1) { order[0] = 0; order[1] = 1; order[2] = 2; }
        else if (m == 2) { order[0] = 1; order[1] = 2; order[2] = 0; }
        else { order[0] = 2; order[1] = 0; order[2] = 1; }
        for (int f = 0; f < 5; f++) {
            field_apply(s, order[0], 3, A[A_RHO2 + f], A[A_F1]);
            field_apply(s, order[1], 3, A[A_F1], A[A_F2]);
            field_apply(s, order[2], 3, A[A_F2], A[A_RHO1 + f]);
        }
    } else {
        for (int f = 0; f < 5; f++) memcpy(A[A_RHO1 + f], A[A_RHO2 + f], s->N * sizeof(double));
    }
}

static void update_nonconserved(or_solver *s) {
    double **A = s->a;
    int base = s->rkLast ? A_RHO1 : A_RHOK;
    const gas_t *g = &s->g;
#pragma omp parallel for schedule(static)
    for (long ip = 0; ip < (long)s->N; ip++) {
        double rho = A[base][ip];
        A[A_U][ip] = A[base + 1][ip] / rho;
        A[A_V][ip] = A[base + 2][ip] / rho;
        A[A_W][ip] = A[base + 3][ip] / rho;
        A[A_P][ip] = g_p(g, rho, A[base + 4][ip], A[A_U][ip], A[A_V][ip], A[A_W][ip]);
        A[A_T][ip] = g_T(g, rho, A[A_P][ip]);
        A[A_MU][ip] = g_mu(g, A[A_T][ip]);
        A[A_AMU][ip] = g_amu(g, A[A_T][ip]);
        A[A_SOS][ip] = g_sos(g, rho, A[A_P][ip]);
    }
}

/* ------------------------------------------------------------------ */
/* Public entry points                                                  */
/* ------------------------------------------------------------------ */

/* setInitialConditions, CSolver_AWS.cpp:199-504 */
int or_set_initial_conditions(or_solver *s, const double *rho0, const double *p0, const double *U0,
                              const double *V0, const double *W0) {
    double **A = s->a;
    const gas_t *g = &s->g;
    long N = (long)s->N;
#pragma omp parallel for schedule(static)
    for (long ip = 0; ip < N; ip++) {
        A[A_RHO1][ip] = rho0[ip];
        A[A_U][ip] = U0[ip];
        A[A_V][ip] = V0[ip];
        A[A_W][ip] = W0[ip];
        A[A_P][ip] = p0[ip];
        A[A_RHOU1][ip] = A[A_RHO1][ip] * A[A_U][ip];
        A[A_RHOV1][ip] = A[A_RHO1][ip] * A[A_V][ip];
        A[A_RHOW1][ip] = A[A_RHO1][ip] * A[A_W][ip];
    }
#pragma omp parallel for schedule(static)
    for (long ip = 0; ip < N; ip++) {
        A[A_RHOE1][ip] = g_rhoE(g, A[A_RHO1][ip], A[A_P][ip], A[A_U][ip], A[A_V][ip], A[A_W][ip]);
        A[A_T][ip] = g_T(g, A[A_RHO1][ip], A[A_P][ip]);
        A[A_MU][ip] = g_mu(g, A[A_T][ip]);
        A[A_AMU][ip] = g_amu(g, A[A_T][ip]);
        A[A_SOS][ip] = g_sos(g, A[A_RHO1][ip], A[A_P][ip]);
    }
    /* walls: velocity, momentum and Neumann temperature (:258-472) */
    int wall = 0;
    s->rkStep = 1; /* so the wall writes below target q1 */
    for (int pass = 0; pass < 2; pass++) {
        int kind = pass == 0 ? CS3D_ADIABATIC_WALL : CS3D_MOVING_ADIABATIC_WALL;
        for (int f = 0; f < 6; f++) {
            if (s->cfg.bc_kind[f] != kind) continue;
            wall = 1;
            int dir = f / 2;
            double uw[3];
            wall_velocity(s, f, kind, uw);
            int Nd = dir == 0 ? s->Nx : dir == 1 ? s->Ny : s->Nz;
            int fix = (f % 2) ? Nd - 1 : 0, sgn = (f % 2) ? -1 : 1;
            for (int k = 0; k < s->Nz; k++)
                for (int j = 0; j < s->Ny; j++)
                    for (int i = 0; i < s->Nx; i++) {
                        int idx3[3] = {i, j, k};
                        if (idx3[dir] != fix) continue;
                        size_t ip = IDX(i, j, k);
                        A[A_U][ip] = uw[0]; A[A_V][ip] = uw[1]; A[A_W][ip] = uw[2];
                        A[A_RHOU1][ip] = dir == 0 ? 0.0 : A[A_RHO1][ip] * uw[0];
                        A[A_RHOV1][ip] = dir == 1 ? 0.0 : A[A_RHO1][ip] * uw[1];
                        A[A_RHOW1][ip] = dir == 2 ? 0.0 : A[A_RHO1][ip] * uw[2];
                        double Tn[6];
                        for (int m = 0; m < 6; m++) {
                            int o = sgn * (m + 1);
                            size_t nb = dir == 0 ? IDX(i + o, j, k) : dir == 1 ? IDX(i, j + o, k) : IDX(i, j, k + o);
                            Tn[m] = A[A_T][nb];
                        }
                        A[A_T][ip] = neumann6(Tn[0], Tn[1], Tn[2], Tn[3], Tn[4], Tn[5]);
                    }
        }
    }
    if (wall) {
#pragma omp parallel for schedule(static)
        for (long ip = 0; ip < N; ip++) {
            A[A_P][ip] = g_p_ideal(g, A[A_RHO1][ip], A[A_T][ip]);
            A[A_SOS][ip] = g_sos(g, A[A_RHO1][ip], A[A_P][ip]);
            A[A_RHOE1][ip] = g_rhoE(g, A[A_RHO1][ip], A[A_P][ip], A[A_U][ip], A[A_V][ip], A[A_W][ip]);
        }
    }
    if (s->sponge_flag)
        for (int f = 0; f < 5; f++) memcpy(A[A_SRHO + f], A[A_RHO1 + f], s->N * sizeof(double));
    s->time = 0.0;
    s->timeStep = 0;
    s->filterTimeStep = 0;
    return 0;
}

/* calcDtFromCFL, CSolver_AWS.cpp:507-551 (always the constant-CFL branch,
 * :530; a positive dt_fixed freezes dt instead) */
void or_pre_step(or_solver *s) {
    double **A = s->a;
    double mx = -100000.0;
    double dx = s->dx, dy = s->dy, dz = s->dz;
#pragma omp parallel for reduction(max : mx) schedule(static)
    for (long ip = 0; ip < (long)s->N; ip++) {
        double v = (fabs(A[A_U][ip]) + A[A_SOS][ip]) / dx + (fabs(A[A_V][ip]) + A[A_SOS][ip]) / dy +
                   (fabs(A[A_W][ip]) + A[A_SOS][ip]) / dz;
        if (v > mx) mx = v;
    }
    s->dt = s->cfg.dt_fixed > 0.0 ? s->cfg.dt_fixed : s->cfg.CFL / mx;
    if (s->timeStep == 0) {
        s->timeStep++;
        s->time = 0.0;
    } else {
        s->timeStep++;
        s->time += s->dt;
    }
}

/* one RK stage: preSubStep, solveEqnSet, postSubStep, updateConservedData,
 * updateData (RK4.hpp:133-137) */
void or_sub_step(or_solver *s, int rk_step, int rk_last) {
    s->rkStep = rk_step;
    s->rkLast = rk_last;
    pre_bc(s);
    pre_derivatives(s);
    solve_eqn_set(s);
    post_bc(s);
    rk_update(s);
    if (s->rkLast) filter_conserved(s);
    update_nonconserved(s);
}

/* updateSponge, CSolver_AWS.cpp:1937-2031 */
void or_post_step(or_solver *s) {
    if (!s->sponge_flag) return;
    double **A = s->a;
    const gas_t *g = &s->g;
    double eps = 1.0 / (s->avgT / s->dt + 1.0);
#pragma omp parallel for schedule(static)
    for (long ip = 0; ip < (long)s->N; ip++) {
        for (int f = 0; f < 5; f++) A[A_SRHO + f][ip] += eps * (A[A_RHO1 + f][ip] - A[A_SRHO + f][ip]);
        A[A_SRHOE][ip] = s->epsP * A[A_SRHOE][ip] +
                         (1.0 - s->epsP) * (s->spongeP / (g->gamma - 1.0) +
                                            0.5 *
                                                (A[A_SRHOU][ip] * A[A_SRHOU][ip] + A[A_SRHOV][ip] * A[A_SRHOV][ip] +
                                                 A[A_SRHOW][ip] * A[A_SRHOW][ip]) /
                                                A[A_SRHO][ip]);
    }
    for (int f = 0; f < 6; f++) {
        if (s->cfg.bc_kind[f] != CS3D_SPONGE) continue;
        int dir = f / 2;
        int Nd = dir == 0 ? s->Nx : dir == 1 ? s->Ny : s->Nz;
        int fix = (f % 2) ? Nd - 1 : 0;
        for (int k = 0; k < s->Nz; k++)
            for (int j = 0; j < s->Ny; j++)
                for (int i = 0; i < s->Nx; i++) {
                    int idx3[3] = {i, j, k};
                    if (idx3[dir] != fix) continue;
                    size_t ip = IDX(i, j, k);
                    for (int q = 0; q < 5; q++) A[A_RHO1 + q][ip] = A[A_SRHO + q][ip];
                }
    }
}

void or_step(or_solver *s) {
    s->rkLast = 0;
    or_pre_step(s);
    for (int st = 1; st <= s->nstages; st++) or_sub_step(s, st, st == s->nstages);
    or_post_step(s);
}

void or_run(or_solver *s, int n) {
    for (int i = 0; i < n; i++) or_step(s);
}

/* field access by the name used in the reference's member list */
int or_get_named(or_solver *s, const char *name, double *out) {
    for (int f = 0; f < A_COUNT; f++)
        if (!strcmp(A_NAMES[f], name)) {
            memcpy(out, s->a[f], s->N * sizeof(double));
            return 0;
        }
    return 1;
}

int or_set_named(or_solver *s, const char *name, const double *in) {
    for (int f = 0; f < A_COUNT; f++)
        if (!strcmp(A_NAMES[f], name)) {
            memcpy(s->a[f], in, s->N * sizeof(double));
            return 0;
        }
    return 1;
}

void or_get_scalars(or_solver *s, double *dt, double *time, int *time_step) {
    *dt = s->dt;
    *time = s->time;
    *time_step = s->timeStep;
}

/* calcTaylorGreenQuantities sums, CSolver_AWS.cpp:2175-2236, over the
 * derivative fields of the last stage and the primitives of q1. */
void or_tgv_quantities(or_solver *s, double out[7]) {
    double **A = s->a;
    double ens = 0, ens2mu = 0, diss = 0, ke = 0, dil = 0, mmu = 0;
    double Ntot = (double)(s->Nx * s->Ny * s->Nz);
#pragma omp parallel for reduction(+ : ens, ens2mu, diss, ke, dil, mmu) schedule(static)
    for (long ip = 0; ip < (long)s->N; ip++) {
        double Ux = A[A_UX][ip], Uy = A[A_UY][ip], Uz = A[A_UZ][ip];
        double Vx = A[A_VX][ip], Vy = A[A_VY][ip], Vz = A[A_VZ][ip];
        double Wx = A[A_WX][ip], Wy = A[A_WY][ip], Wz = A[A_WZ][ip];
        double S[3][3];
        double tr = (1.0 / 3.0) * (Ux + Vy + Wz);
        S[0][0] = 0.5 * (Ux + Ux) - tr;
        S[1][1] = 0.5 * (Vy + Vy) - tr;
        S[2][2] = 0.5 * (Wz + Wz) - tr;
        S[0][1] = S[1][0] = 0.5 * (Uy + Vx);
        S[0][2] = S[2][0] = 0.5 * (Uz + Wx);
        S[1][2] = S[2][1] = 0.5 * (Vz + Wy);
        double td = S[0][0] * Ux;
        td += S[0][1] * Uy;
        td += S[0][2] * Uz;
        td += S[1][0] * Vx;
        td += S[1][1] * Vy;
        td += S[1][2] * Vz;
        td += S[2][0] * Wx;
        td += S[2][1] * Wy;
        td += S[2][2] * Wz;
        td *= 2 * A[A_MU][ip];
        double U = A[A_U][ip], V = A[A_V][ip], W = A[A_W][ip], r1 = A[A_RHO1][ip];
        double uvar = U * U + V * V + W * W;
        double wx = Wy - Vz, wy = Uz - Wx, wz = Vx - Uy;
        ens += (1.0 / 2.0) * r1 * (wx * wx + wy * wy + wz * wz);
        ens2mu += A[A_MU][ip] * r1 * (wx * wx + wy * wy + wz * wz);
        diss += td;
        ke += r1 * uvar / 2.0;
        dil += ((Ux + Vy + Wz) * (Ux + Vy + Wz)) / Ntot;
        mmu += A[A_MU][ip] / Ntot;
    }
    out[0] = s->time;
    out[1] = ke;
    out[2] = diss;
    out[3] = ens;
    out[4] = ens2mu;
    out[5] = mmu;
    out[6] = sqrt(dil);
}

/* calcTurbulenceQuantities (CSolver_AWS.cpp:2033-2173): the row of
 * turbdata.out -- time, tau, taylorReyn3, turbMach, meanTurbDiss, uprime,
 * kolNu, rhoprime, dilprime, vortprime, meanKineticEng -- over the derivative
 * fields of the last stage and the primitives of q1. */
void or_turbulence_quantities(or_solver *s, double out[11]) {
    double **A = s->a;
    const double Ntot = (double)(s->Nx * s->Ny * s->Nz);
    double meanRho = 0, meanMu = 0, meanTurbDiss = 0, uprime = 0, uiprime = 0, urms = 0, meanSOS = 0,
           taylor2_denom = 0, meanKineticEng = 0;
#pragma omp parallel for reduction(+ : meanRho, meanMu, meanTurbDiss, uprime, uiprime, urms, meanSOS, \
                                   taylor2_denom, meanKineticEng) schedule(static)
    for (long ip = 0; ip < (long)s->N; ip++) {
        double Ux = A[A_UX][ip], Uy = A[A_UY][ip], Uz = A[A_UZ][ip];
        double Vx = A[A_VX][ip], Vy = A[A_VY][ip], Vz = A[A_VZ][ip];
        double Wx = A[A_WX][ip], Wy = A[A_WY][ip], Wz = A[A_WZ][ip];
        double S[3][3];
        S[0][0] = 0.5 * (Ux + Ux) - (1.0 / 3.0) * (Ux + Vy + Wz);
        S[1][1] = 0.5 * (Vy + Vy) - (1.0 / 3.0) * (Ux + Vy + Wz);
        S[2][2] = 0.5 * (Wz + Wz) - (1.0 / 3.0) * (Ux + Vy + Wz);
        S[0][1] = S[1][0] = 0.5 * (Uy + Vx);
        S[0][2] = S[2][0] = 0.5 * (Uz + Wx);
        S[1][2] = S[2][1] = 0.5 * (Vz + Wy);
        double td = S[0][0] * Ux;
        td += S[0][1] * Uy;
        td += S[0][2] * Uz;
        td += S[1][0] * Vx;
        td += S[1][1] * Vy;
        td += S[1][2] * Vz;
        td += S[2][0] * Wx;
        td += S[2][1] * Wy;
        td += S[2][2] * Wz;
        td *= 2 * A[A_MU][ip];
        double U = A[A_U][ip], V = A[A_V][ip], W = A[A_W][ip];
        double up2 = (U * U + V * V + W * W) / 3.0;
        double uvar = (U * U + V * V + W * W);
        double uip2 = (Ux * Ux + Vy * Vy + Wz * Wz) / 3.0;
        double ke = A[A_RHO1][ip] * uvar;
        meanRho += A[A_RHO1][ip] / Ntot;
        meanMu += A[A_MU][ip] / Ntot;
        meanTurbDiss += td / Ntot;
        uprime += up2 / Ntot;
        uiprime += uip2 / Ntot;
        urms += uvar / Ntot;
        meanSOS += A[A_SOS][ip] / Ntot;
        taylor2_denom += (Ux * Ux) / Ntot;
        meanKineticEng += ke / Ntot / 2.0;
    }
    double rhoprime = 0, dilprime = 0, vortprime = 0;
#pragma omp parallel for reduction(+ : rhoprime, dilprime, vortprime) schedule(static)
    for (long ip = 0; ip < (long)s->N; ip++) {
        double r = A[A_RHO1][ip];
        double Ux = A[A_UX][ip], Uy = A[A_UY][ip], Uz = A[A_UZ][ip];
        double Vx = A[A_VX][ip], Vy = A[A_VY][ip], Vz = A[A_VZ][ip];
        double Wx = A[A_WX][ip], Wy = A[A_WY][ip], Wz = A[A_WZ][ip];
        rhoprime += ((r - meanRho) * (r - meanRho)) / Ntot;
        dilprime += ((Ux + Vy + Wz) * (Ux + Vy + Wz)) / Ntot;
        double wx = Wy - Vz, wy = Uz - Wx, wz = Vx - Uy;
        vortprime += ((wx * wx + wy * wy + wz * wz)) / Ntot;
    }
    (void)taylor2_denom;
    rhoprime = sqrt(rhoprime);
    dilprime = sqrt(dilprime);
    vortprime = sqrt(vortprime);
    double meanNu = meanMu / meanRho;
    meanTurbDiss /= meanRho;
    uprime = sqrt(uprime);
    uiprime = sqrt(uiprime);
    urms = sqrt(urms);
    double turbMach = urms / meanSOS;
    double taylorMicro2 = uprime / uiprime;
    double taylorReyn3 = uprime * taylorMicro2 / meanNu;
    double k0 = 8.0;
    const double pi = 3.14159265358979323846; /* M_PI of the reference's <cmath> */
    double tau = sqrt(2.0 * pi) / k0 / uprime;
    double kolNu = pow(pow(meanNu, 3.0) / meanTurbDiss, 0.25);
    out[0] = s->time;
    out[1] = tau;
    out[2] = taylorReyn3;
    out[3] = turbMach;
    out[4] = meanTurbDiss;
    out[5] = uprime;
    out[6] = kolNu;
    out[7] = rhoprime;
    out[8] = dilprime;
    out[9] = vortprime;
    out[10] = meanKineticEng;
}

/* shearLayerInfoCalc (CSolver_AWS.cpp:2259-2456): per y plane, the x-z means
 * and second moments of rho, U, V, W, p, T of q1.  out[k*Ny + j] with k =
 * 0 rhoAvg, 1 uAvg, 2 vAvg, 3 wAvg, 4 pAvg, 5 tAvg, 6 rhoprime2, 7 uprime2,
 * 8 vprime2, 9 wprime2, 10 pprime2, 11 tprime2, 12 uvprime, 13 uwprime as the
 * reference writes it (the u'w' and v'w' sums both, :2317-2318), 14 vwprime
 * as the reference writes it (0), 15 u'w' and 16 v'w' each on its own. */
void or_shear_layer_info(or_solver *s, double *out) {
    double **A = s->a;
    const int Nx = s->Nx, Ny = s->Ny, Nz = s->Nz;
    const double nxz = (double)(Nx * Nz);
    double *o = out;
    for (long m = 0; m < 17L * Ny; m++) o[m] = 0.0;
    const double *F[6] = {A[A_RHO1], A[A_U], A[A_V], A[A_W], A[A_P], A[A_T]};
    for (int k = 0; k < Nz; k++)
        for (int j = 0; j < Ny; j++)
            for (int i = 0; i < Nx; i++) {
                size_t ii = IDX(i, j, k);
                for (int f = 0; f < 6; f++) o[f * Ny + j] += F[f][ii] / nxz;
            }
    for (int k = 0; k < Nz; k++)
        for (int j = 0; j < Ny; j++)
            for (int i = 0; i < Nx; i++) {
                size_t ii = IDX(i, j, k);
                double d[6];
                for (int f = 0; f < 6; f++) {
                    d[f] = F[f][ii] - o[f * Ny + j];
                    o[(6 + f) * Ny + j] += d[f] * d[f] / nxz;
                }
                o[12 * Ny + j] += d[1] * d[2] / nxz;
                o[13 * Ny + j] += d[1] * d[3] / nxz;
                o[13 * Ny + j] += d[2] * d[3] / nxz;
                o[15 * Ny + j] += d[1] * d[3] / nxz;
                o[16 * Ny + j] += d[2] * d[3] / nxz;
            }
}

/* linearInterpolation with getBaseNodeIndex (Utils.cpp:242-331), the base
 * index kept at most N-2 per direction (the reference would read one plane
 * past its arrays when a point lies exactly on the last plane, where its
 * weight for that plane is 0). */
static double ao_interp(const or_solver *s, const double *f, const double xp[3]) {
    int b[3];
    b[0] = (int)(xp[0] / s->dx);
    b[1] = (int)(xp[1] / s->dy);
    b[2] = (int)(xp[2] / s->dz);
    if (b[0] > s->Nx - 2) b[0] = s->Nx - 2;
    if (b[1] > s->Ny - 2) b[1] = s->Ny - 2;
    if (b[2] > s->Nz - 2) b[2] = s->Nz - 2;
    double x0 = s->x[b[0]], x1 = s->x[b[0] + 1], y0 = s->y[b[1]], y1 = s->y[b[1] + 1];
    double z0 = s->z[b[2]], z1 = s->z[b[2] + 1];
    double xd = (xp[0] - x0) / (x1 - x0), yd = (xp[1] - y0) / (y1 - y0), zd = (xp[2] - z0) / (z1 - z0);
    int i = b[0], j = b[1], k = b[2];
    double c000 = f[IDX(i, j, k)], c001 = f[IDX(i, j, k + 1)], c010 = f[IDX(i, j + 1, k)];
    double c011 = f[IDX(i, j + 1, k + 1)], c100 = f[IDX(i + 1, j, k)], c101 = f[IDX(i + 1, j, k + 1)];
    double c110 = f[IDX(i + 1, j + 1, k)], c111 = f[IDX(i + 1, j + 1, k + 1)];
    double c00 = c000 * (1 - xd) + c100 * xd;
    double c01 = c001 * (1 - xd) + c101 * xd;
    double c10 = c010 * (1 - xd) + c110 * xd;
    double c11 = c011 * (1 - xd) + c111 * xd;
    double c0 = c00 * (1 - yd) + c10 * yd;
    double c1 = c01 * (1 - yd) + c11 * yd;
    return c0 * (1 - zd) + c1 * zd;
}

/* AeroOptics::computeAO (AeroOptics.cpp:45-93) with generateBaseBeamDiff
 * (:3-22): for each angle and x-z position, the trapezoidal integral of the
 * density along a ray from y = 0.2 Ly to 0.8 Ly tilted by the angle in x
 * (periodic in x), sampled at spacing about min(dx, dy, dz).
 * OPL[ap*Nx*Nz + k*Nx + i].  The density is that of the state q1.  The
 * reference hands its AeroOptics object rho2 (CSolver_AWS.hpp:165), which
 * holds the state on steps without filtering; on filtered steps
 * filterConservedData has used rho2 as a transposition buffer
 * (CSolver_AWS.cpp:1697-1710), and the reference integrates that. */
void or_aero_optics(or_solver *s, int numAngles, double maxAngle, double *OPL) {
    const double *rho = s->a[A_RHO1];
    const double Lx = s->cfg.Lx, Ly = s->cfg.Ly;
    const double lower = 0.2 * Ly, upper = 0.8 * Ly, totalDY = upper - lower;
    const double ds = fmin(s->dx, fmin(s->dy, s->dz));
    const double pi = 3.14159265358979323846;
    for (int ap = 0; ap < numAngles; ap++) {
        double minAngle = 0.0;
        double ang = minAngle + ((double)ap / ((double)(numAngles - 1))) * (maxAngle - minAngle);
        ang *= pi / 180.0;
        double Ldiag = totalDY / cos(ang);
        double totalDX = Ldiag * sin(ang);
        int Nline = (int)ceil(Ldiag / ds) + 1;
        double dsLine = Ldiag / (double)(Nline - 1);
        double dxLine = totalDX / (double)(Nline - 1);
        double dyLine = totalDY / (double)(Nline - 1);
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 0; k < s->Nz; k++)
            for (int i = 0; i < s->Nx; i++) {
                double b[2];
                for (int e = 0; e < 2; e++) {
                    int sp = e == 0 ? 0 : Nline - 1;
                    double xp[3] = {fmod(s->x[i] + (double)(sp * dxLine), Lx), lower + (double)(sp * dyLine),
                                    s->z[k]};
                    b[e] = ao_interp(s, rho, xp);
                }
                /* the reference's order: both ends, then the interior points */
                double opl = b[0] * dsLine / 2.0 + b[1] * dsLine / 2.0;
                for (int sp = 1; sp < Nline - 1; sp++) {
                    double xp[3] = {fmod(s->x[i] + (double)(sp * dxLine), Lx), lower + (double)(sp * dyLine),
                                    s->z[k]};
                    opl += ao_interp(s, rho, xp) * dsLine;
                }
                OPL[(size_t)ap * s->Nx * s->Nz + (size_t)k * s->Nx + i] = opl;
            }
    }
}

/* The vorticity magnitude and Q-criterion of the post-processor
 * (PostProcess.cpp:190-310) for the state q1: U, V, W = rhoU/rho, ...; the
 * nine first derivatives with the solver's operators; per point
 * |curl u| and Q = |W|^2/2 - |S|^2/2 with S and W the symmetric and
 * antisymmetric parts of grad u. */
void or_vorticity_q(or_solver *s, double *vort, double *qcrit) {
    const size_t n = s->N;
    double *vel[3], *d[3][3];
    for (int c = 0; c < 3; c++) {
        vel[c] = (double *)malloc(n * sizeof(double));
        for (int e = 0; e < 3; e++) d[c][e] = (double *)malloc(n * sizeof(double));
    }
    for (size_t ip = 0; ip < n; ip++)
        for (int c = 0; c < 3; c++) vel[c][ip] = s->a[A_RHOU1 + c][ip] / s->a[A_RHO1][ip];
    for (int c = 0; c < 3; c++)
        for (int e = 0; e < 3; e++) field_apply(s, e, 1, vel[c], d[c][e]);
#pragma omp parallel for schedule(static)
    for (long ip = 0; ip < (long)n; ip++) {
        double Ux = d[0][0][ip], Uy = d[0][1][ip], Uz = d[0][2][ip];
        double Vx = d[1][0][ip], Vy = d[1][1][ip], Vz = d[1][2][ip];
        double Wx = d[2][0][ip], Wy = d[2][1][ip], Wz = d[2][2][ip];
        double vx = Wy - Vz, vy = Uz - Wx, vz = Vx - Uy;
        vort[ip] = sqrt(vx * vx + vy * vy + vz * vz);
        double sij[3][3], wij[3][3];
        sij[0][0] = Ux; sij[1][1] = Vy; sij[2][2] = Wz;
        sij[0][1] = 0.5 * (Uy + Vx); sij[1][2] = 0.5 * (Vz + Wy); sij[0][2] = 0.5 * (Uz + Wx);
        wij[0][0] = 0.0; wij[1][1] = 0.0; wij[2][2] = 0.0;
        wij[0][1] = 0.5 * (Uy - Vx); wij[1][2] = 0.5 * (Vz - Wy); wij[0][2] = 0.5 * (Uz - Wx);
        sij[1][0] = sij[0][1]; sij[2][1] = sij[1][2]; sij[2][0] = sij[0][2];
        wij[1][0] = -wij[0][1]; wij[2][1] = -wij[1][2]; wij[2][0] = -wij[0][2];
        double om2 = 0.5 * (wij[0][0] * wij[0][0] + wij[0][1] * wij[0][1] + wij[0][2] * wij[0][2] +
                            wij[1][0] * wij[1][0] + wij[1][1] * wij[1][1] + wij[1][2] * wij[1][2] +
                            wij[2][0] * wij[2][0] + wij[2][1] * wij[2][1] + wij[2][2] * wij[2][2]);
        double st2 = 0.5 * (sij[0][0] * sij[0][0] + sij[0][1] * sij[0][1] + sij[0][2] * sij[0][2] +
                            sij[1][0] * sij[1][0] + sij[1][1] * sij[1][1] + sij[1][2] * sij[1][2] +
                            sij[2][0] * sij[2][0] + sij[2][1] * sij[2][1] + sij[2][2] * sij[2][2]);
        qcrit[ip] = om2 - st2;
    }
    for (int c = 0; c < 3; c++) {
        free(vel[c]);
        for (int e = 0; e < 3; e++) free(d[c][e]);
    }
}

/* Single operator on contiguous lines: kind 1/2/3 as line_apply, nlines
 * lines of length N with spacing dh. */
void or_line_op(int kind, int bc_type, int N, double dh, double alphaF, long nlines, const double *in,
                double *out) {
    lineop_t op;
    lineop_init(&op, N, bc_type, dh, alphaF);
#pragma omp parallel
    {
        double *work = (double *)malloc(sizeof(double) * 6 * (size_t)N);
#pragma omp for schedule(static)
        for (long l = 0; l < nlines; l++) line_apply(&op, kind, in + l * N, out + l * N, work);
        free(work);
    }
    lineop_free(&op);
}

int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
