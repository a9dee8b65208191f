/*
 * mara_oracle.c -- CPU restatement of Mara2's finite-volume time step.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product).  Each function
 * names the reference file:line it restates.  Floating-point expressions keep
 * the reference's operation order because the FP64 GPU path is required to
 * match the reference to a relative L1 of 1e-12 and in practice does so
 * bit-for-bit; build with -ffp-contract=off so no fused multiply-add changes
 * a rounding.
 *
 * Structure: the restatement follows the reference's whole-array passes
 * (godunov sweep -> optional flux CT -> divergence -> RK combine ->
 * primitive recovery -> guard fill) so that each intermediate array can be
 * compared with the reference build.  Loops over independent zones carry
 * OpenMP pragmas; results do not depend on the thread count.
 */
#include "mara_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NSLOT 10 /* MARA_NUM_FIELDS, src/Mara.hpp:15 */

typedef struct {
    double P[NSLOT], U[NSLOT], F[NSLOT], A[NSLOT];
    int nf;
} mstate;

typedef struct {
    int N[3];        /* cells per axis including guards           */
    int nq;
    double dx[3], dA[3], dV, lmin;
    double nrm[3][3];
} mgeom;

/* ------------------------------------------------------------------------ */
/* threads                                                                   */
/* ------------------------------------------------------------------------ */
int mo_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void mo_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void) n;
#endif
}

/* ------------------------------------------------------------------------ */
/* geometry: CartesianMeshGeometry::cacheSpacing (CartesianMeshGeometry.cpp: */
/* 145-157), UnitVector::getCartesianComponents (UnitVector.cpp:32-39)       */
/* ------------------------------------------------------------------------ */
static void unit_vector(double mu, double phi, double out[3])
{
    const double sin_theta = sqrt(1 - mu * mu);
    out[0] = sin_theta * cos(phi);
    out[1] = sin_theta * sin(phi);
    out[2] = mu;
}

void mo_face_normals(double n[3][3])
{
    unit_vector(0, 0, n[0]);          /* xhat (0, 0)      */
    unit_vector(0, M_PI / 2, n[1]);   /* yhat (0, pi/2)   */
    unit_vector(1, 0, n[2]);          /* zhat (1, 0)      */
}

int mo_num_fields(const mo_config* c)
{
    switch (c->law) {
        case MO_LAW_HYDRO: return 5;
        case MO_LAW_MHD: return c->cooling_rate > 0.0 ? 9 : 8;  /* numAuxiliary, ConservationLaws.cpp:355-358 */
        case MO_LAW_RMHD: return 8;
        default: return 0;
    }
}

static int mhd_aux(const mo_config* c) { return c->law == MO_LAW_MHD && c->cooling_rate > 0.0; }

int mo_stencil_size(const mo_config* c)
{
    switch (c->recon) {
        case MO_RECON_PCM: return 1;   /* MethodOfLines::getStencilSize      */
        case MO_RECON_PLM: return 2;   /* MethodOfLinesPlm::getStencilSize   */
        case MO_RECON_WENO5: return 3; /* stencil of the WENO5 composition   */
        default: return 0;
    }
}

static int make_geom_chk(const mo_config* c, mgeom* g, int check_stencil)
{
    const int n[3] = {c->ni, c->nj, c->nk};
    const int s = mo_stencil_size(c);
    g->nq = mo_num_fields(c);
    if (g->nq == 0 || s == 0) return MO_ERR_CONFIG;
    if (c->rk_order < 1 || c->rk_order > 3) return MO_ERR_CONFIG;
    for (int a = 0; a < 3; ++a) {
        if (n[a] < 1 || c->ng[a] < 0) return MO_ERR_CONFIG;
        if (n[a] == 1 && c->ng[a] != 0) return MO_ERR_CONFIG;
        /* SchemeHelpers::makeFootprint (SolutionSchemes.cpp:17-49) */
        if (check_stencil && n[a] > 1 && c->ng[a] < s) return MO_ERR_GUARD_TOO_SMALL;
        g->N[a] = n[a] + 2 * c->ng[a];
        g->dx[a] = (c->upper[a] - c->lower[a]) / n[a];
    }
    g->dA[0] = g->dx[1] * g->dx[2];
    g->dA[1] = g->dx[2] * g->dx[0];
    g->dA[2] = g->dx[0] * g->dx[1];
    g->dV = g->dx[0] * g->dx[1] * g->dx[2];
    /* MeshOperator::linearCellDimension: first smallest of (dx, dy, dz) */
    g->lmin = g->dx[0];
    if (g->dx[1] < g->lmin) g->lmin = g->dx[1];
    if (g->dx[2] < g->lmin) g->lmin = g->dx[2];
    mo_face_normals(g->nrm);
    return MO_OK;
}

/* geometry for whole-array passes; the stencil footprint is checked only
 * where a flux sweep runs (SchemeHelpers::makeFootprint is called by
 * MethodOfLinesTVD::advance alone) */
static int make_geom(const mo_config* c, mgeom* g) { return make_geom_chk(c, g, 0); }

static inline long cidx(const mgeom* g, int i, int j, int k)
{
    return (((long) i * g->N[1] + j) * g->N[2] + k) * g->nq;
}

/* flux array (N0+1, N1+1, N2+1, nq, 3) */
static inline long fidx(const mgeom* g, int i, int j, int k, int q, int a)
{
    return ((((long) i * (g->N[1] + 1) + j) * (g->N[2] + 1) + k) * g->nq + q) * 3 + a;
}

/* ------------------------------------------------------------------------ */
/* NewtonianHydro::fromPrimitive (ConservationLaws.cpp:253-290)              */
/* ------------------------------------------------------------------------ */
static int hydro_prim(double gamma, const double* P, const double* n, mstate* S)
{
    const double gm0 = gamma;
    const double gm1 = gamma - 1.0;
    const double cs = sqrt(gm0 * P[4] / P[0]);
    const double vv = P[1] * P[1] + P[2] * P[2] + P[3] * P[3];
    const double vn = P[1] * n[0] + P[2] * n[1] + P[3] * n[2];
    memset(S, 0, sizeof(*S));
    S->nf = 5;
    for (int q = 0; q < 5; ++q) S->P[q] = P[q];
    S->U[0] = P[0];
    S->U[1] = P[0] * P[1];
    S->U[2] = P[0] * P[2];
    S->U[3] = P[0] * P[3];
    S->U[4] = P[0] * 0.5 * vv + P[4] / gm1;
    S->F[0] = vn * S->U[0];
    S->F[1] = vn * S->U[1] + P[4] * n[0];
    S->F[2] = vn * S->U[2] + P[4] * n[1];
    S->F[3] = vn * S->U[3] + P[4] * n[2];
    S->F[4] = vn * S->U[4] + P[4] * vn;
    S->A[0] = vn - cs;
    S->A[1] = vn;
    S->A[2] = vn;
    S->A[3] = vn;
    S->A[4] = vn + cs;
    return MO_OK;
}

/* NewtonianHydro::fromConserved (ConservationLaws.cpp:238-251) */
static int hydro_cons(double gamma, const double* U, double* P)
{
    const double gm1 = gamma - 1.0;
    const double pp = U[1] * U[1] + U[2] * U[2] + U[3] * U[3];
    P[0] = U[0];
    P[4] = (U[4] - 0.5 * pp / U[0]) * gm1;
    P[1] = U[1] / U[0];
    P[2] = U[2] / U[0];
    P[3] = U[3] / U[0];
    return MO_OK;
}

/* ------------------------------------------------------------------------ */
/* NewtonianMHD::fromPrimitive (ConservationLaws.cpp:416-487), Jameson's     */
/* fast / Alfven / slow speeds                                               */
/* ------------------------------------------------------------------------ */
static int mhd_prim(double gamma, int naux, const double* P, const double* n, mstate* S)
{
    const double gm0 = gamma;
    const double gm1 = gamma - 1.0;
    const double cs2 = gm0 * P[4] / P[0];
    const double vv = P[1] * P[1] + P[2] * P[2] + P[3] * P[3];
    const double BB = P[5] * P[5] + P[6] * P[6] + P[7] * P[7];
    const double Bv = P[5] * P[1] + P[6] * P[2] + P[7] * P[3];
    const double vn = P[1] * n[0] + P[2] * n[1] + P[3] * n[2];
    const double Bn = P[5] * n[0] + P[6] * n[1] + P[7] * n[2];
    const double ps = P[4] + 0.5 * BB;
    memset(S, 0, sizeof(*S));
    S->nf = 8;
    for (int q = 0; q < 8; ++q) S->P[q] = P[q];
    S->U[0] = P[0];
    S->U[1] = P[0] * P[1];
    S->U[2] = P[0] * P[2];
    S->U[3] = P[0] * P[3];
    S->U[4] = P[0] * 0.5 * vv + 0.5 * BB + P[4] / gm1;
    S->U[5] = P[5];
    S->U[6] = P[6];
    S->U[7] = P[7];
    S->F[0] = vn * S->U[0];
    S->F[1] = vn * S->U[1] - Bn * P[5] + ps * n[0];
    S->F[2] = vn * S->U[2] - Bn * P[6] + ps * n[1];
    S->F[3] = vn * S->U[3] - Bn * P[7] + ps * n[2];
    S->F[4] = vn * S->U[4] - Bn * Bv + ps * vn;
    S->F[5] = vn * S->U[5] - Bn * P[1];
    S->F[6] = vn * S->U[6] - Bn * P[2];
    S->F[7] = vn * S->U[7] - Bn * P[3];
    {
        const double Bn2 = Bn * Bn;
        const double ca2 = BB / P[0];
        const double cn2 = Bn2 / P[0];
        const double cw4 = (cs2 + ca2) * (cs2 + ca2);
        const double cF2 = 0.5 * (cs2 + ca2 + sqrt(cw4 - 4 * cs2 * cn2));
        const double cS2 = 0.5 * (cs2 + ca2 - sqrt(cw4 - 4 * cs2 * cn2));
        S->A[0] = vn - sqrt(cF2);
        S->A[1] = vn - sqrt(cn2);
        S->A[2] = vn - sqrt(cS2);
        S->A[3] = vn;
        S->A[4] = vn;
        S->A[5] = vn + sqrt(cS2);
        S->A[6] = vn + sqrt(cn2);
        S->A[7] = vn + sqrt(cF2);
    }
    /* auxiliary fields: carried, no flux, zero eigenvalue (:479-485) */
    for (int q = 8; q < 8 + naux; ++q) {
        S->P[q] = P[q];
        S->U[q] = P[q];
        S->F[q] = 0.0;
        S->A[q] = 0.0;
    }
    S->nf = 8 + naux;
    return MO_OK;
}

/* NewtonianMHD::fromConserved incl. bad-state detection and pressure floor
 * (ConservationLaws.cpp:370-414).  Returns MO_ERR_INVERSION_FAILURE for a
 * StateFailure. */
static int mhd_cons(double gamma, double pfloor, int naux, const double* U, double* P, int* health)
{
    const double gm1 = gamma - 1.0;
    const double pp = U[1] * U[1] + U[2] * U[2] + U[3] * U[3];
    const double BB = U[5] * U[5] + U[6] * U[6] + U[7] * U[7];
    double Q[9];
    const int nf = 8 + naux;
    Q[0] = U[0];
    Q[4] = (U[4] - 0.5 * pp / U[0] - 0.5 * BB) * gm1;
    Q[1] = U[1] / U[0];
    Q[2] = U[2] / U[0];
    Q[3] = U[3] / U[0];
    Q[5] = U[5];
    Q[6] = U[6];
    Q[7] = U[7];
    for (int q = 8; q < nf; ++q) Q[q] = U[q];
    *health = 0;
    if (Q[4] < 0.0 || Q[0] < 0.0 || U[0] < 0.0 || U[4] < 0.0) {
        if (Q[4] < 0.0 && pfloor > 0.0) {
            Q[4] = pfloor * Q[0];
            *health = 1;
        } else {
            for (int q = 0; q < nf; ++q) P[q] = Q[q];
            return MO_ERR_INVERSION_FAILURE;
        }
    }
    for (int q = 0; q < nf; ++q) P[q] = Q[q];
    return MO_OK;
}

/* ------------------------------------------------------------------------ */
/* QuarticPolynomial (QuarticPolynomial.cpp:19-144): real roots through the  */
/* resolvent cubic (Ferrari).                                                */
/* ------------------------------------------------------------------------ */
static void solve_cubic(double c3, double c2, double c1, double c0,
                        double* x1, double* x2, double* x3, int* nr)
{
    const double a2 = c2 / c3;
    const double a1 = c1 / c3;
    const double a0 = c0 / c3;
    const double q = a1 / 3.0 - a2 * a2 / 9.0;
    const double r = (a1 * a2 - 3.0 * a0) / 6.0 - a2 * a2 * a2 / 27.0;
    const double delta = q * q * q + r * r;

    if (delta > 0.0) {
        double s1 = r + sqrt(delta);
        double s2 = r - sqrt(delta);
        s1 = (s1 >= 0.0) ? pow(s1, 1. / 3) : -pow(-s1, 1. / 3);
        s2 = (s2 >= 0.0) ? pow(s2, 1. / 3) : -pow(-s2, 1. / 3);
        *x1 = (s1 + s2) - a2 / 3.0;
        *x2 = *x3 = -0.5 * (s1 + s2) - a2 / 3.0;
        *nr = 1;
    } else if (delta < 0.0) {
        const double theta = acos(r / sqrt(-q * q * q)) / 3.0;
        const double costh = cos(theta);
        const double sinth = sin(theta);
        const double sq = sqrt(-q);
        *x1 = 2.0 * sq * costh - a2 / 3.0;
        *x2 = -sq * costh - a2 / 3.0 - sqrt(3) * sq * sinth;
        *x3 = -sq * costh - a2 / 3.0 + sqrt(3) * sq * sinth;
        *nr = 3;
    } else {
        const double s = (r >= 0.0) ? pow(r, 1. / 3) : -pow(-r, 1. / 3);
        *x1 = 2.0 * s - a2 / 3.0;
        *x2 = *x3 = -s - a2 / 3.0;
        *nr = 3;
    }
}

int mo_quartic(double d4, double d3, double d2, double d1, double d0, double roots[4])
{
    const double a3 = d3 / d4;
    const double a2 = d2 / d4;
    const double a1 = d1 / d4;
    const double a0 = d0 / d4;
    const double au2 = -a2;
    const double au1 = (a1 * a3 - 4 * a0);
    const double au0 = 4.0 * a0 * a2 - a1 * a1 - a0 * a3 * a3;
    int nr, nr12, nr34;
    double r1, r2, r3, r4, x1, x2, x3, u1, D2, E2;

    solve_cubic(1.0, au2, au1, au0, &x1, &x2, &x3, &nr);
    u1 = (nr == 1) ? x1 : ((x1 > x3) ? x1 : x3);

    const double R2 = 0.25 * a3 * a3 + u1 - a2;
    const double R = (R2 > 0.0) ? sqrt(R2) : 0.0;

    if (R != 0.0) {
        const double foo1 = 0.75 * a3 * a3 - R2 - 2.0 * a2;
        const double foo2 = 0.25 * (4.0 * a3 * a2 - 8.0 * a1 - a3 * a3 * a3) / R;
        D2 = foo1 + foo2;
        E2 = foo1 - foo2;
    } else {
        const double foo1 = 0.75 * a3 * a3 - 2.0 * a2;
        const double foo2 = 2.00 * sqrt(u1 * u1 - 4.0 * a0);
        D2 = foo1 + foo2;
        E2 = foo1 - foo2;
    }
    if (D2 >= 0.0) {
        const double D = sqrt(D2);
        r1 = -0.25 * a3 + 0.5 * R - 0.5 * D;
        r2 = -0.25 * a3 + 0.5 * R + 0.5 * D;
        nr12 = 2;
    } else {
        r1 = r2 = -0.25 * a3 + 0.5 * R;
        nr12 = 0;
    }
    if (E2 >= 0.0) {
        const double E = sqrt(E2);
        r3 = -0.25 * a3 - 0.5 * R - 0.5 * E;
        r4 = -0.25 * a3 - 0.5 * R + 0.5 * E;
        nr34 = 2;
    } else {
        r3 = r4 = -0.25 * a3 - 0.5 * R;
        nr34 = 0;
    }
    {
        int m = 0;
        if (nr12 != 0) { roots[m++] = r1; roots[m++] = r2; }
        if (nr34 != 0) { roots[m++] = r3; roots[m++] = r4; }
        /* ascending insertion sort (the reference sorts with std::sort) */
        for (int a = 1; a < m; ++a) {
            const double v = roots[a];
            int b = a - 1;
            while (b >= 0 && v < roots[b]) { roots[b + 1] = roots[b]; --b; }
            roots[b + 1] = v;
        }
    }
    return nr12 + nr34;
}

/* ------------------------------------------------------------------------ */
/* RelativisticMHD::fromPrimitive (ConservationLaws.cpp:659-836)             */
/* ------------------------------------------------------------------------ */
static int rmhd_prim(double gamma, const double* P, const double* n, mstate* S)
{
    const double gm0 = gamma;
    const double gm1 = gamma - 1.0;
    const double vv = P[1] * P[1] + P[2] * P[2] + P[3] * P[3];
    const double BB = P[5] * P[5] + P[6] * P[6] + P[7] * P[7];
    const double Bv = P[5] * P[1] + P[6] * P[2] + P[7] * P[3];
    const double vn = P[1] * n[0] + P[2] * n[1] + P[3] * n[2];
    const double Bn = P[5] * n[0] + P[6] * n[1] + P[7] * n[2];
    const double W2 = 1.0 / (1.0 - vv);
    const double W0 = sqrt(W2);
    const double b0 = W0 * Bv;
    const double bb = (BB + b0 * b0) / W2;
    const double b1 = (P[5] + b0 * W0 * P[1]) / W0;
    const double b2 = (P[6] + b0 * W0 * P[2]) / W0;
    const double b3 = (P[7] + b0 * W0 * P[3]) / W0;
    const double bn = b1 * n[0] + b2 * n[1] + b3 * n[2];
    const double e0 = (P[4] / P[0]) / gm1;
    const double es = e0 + 0.5 * bb / P[0];
    const double p0 = P[4];
    const double ps = p0 + 0.5 * bb;
    const double h0 = 1.0 + e0 + p0 / P[0];
    const double hs = 1.0 + es + ps / P[0];

    if (vv >= 1) return MO_ERR_SUPERLUMINAL;

    memset(S, 0, sizeof(*S));
    S->nf = 8;
    for (int q = 0; q < 8; ++q) S->P[q] = P[q];
    S->U[0] = P[0] * W0;
    S->U[4] = P[0] * hs * W2 - ps - b0 * b0 - S->U[0];
    S->U[1] = P[0] * hs * W2 * P[1] - b0 * b1;
    S->U[2] = P[0] * hs * W2 * P[2] - b0 * b2;
    S->U[3] = P[0] * hs * W2 * P[3] - b0 * b3;
    S->U[5] = P[5];
    S->U[6] = P[6];
    S->U[7] = P[7];
    S->F[0] = vn * S->U[0];
    S->F[1] = vn * S->U[1] - Bn * b1 / W0 + ps * n[0];
    S->F[2] = vn * S->U[2] - Bn * b2 / W0 + ps * n[1];
    S->F[3] = vn * S->U[3] - Bn * b3 / W0 + ps * n[2];
    S->F[4] = vn * S->U[4] - Bn * b0 / W0 + ps * vn;
    S->F[5] = vn * S->U[5] - Bn * P[1];
    S->F[6] = vn * S->U[6] - Bn * P[2];
    S->F[7] = vn * S->U[7] - Bn * P[3];

    {
        const double cs2 = gm0 * p0 / (P[0] * h0);
        const double W4 = W2 * W2;
        const double v2 = vn * vn;
        const double v3 = vn * v2;
        const double v4 = vn * v3;

        if (BB == 0.0) { /* SRHD eigenvalues */
            const double K = sqrt(cs2 * (1 - vv) * (1 - vv * cs2 - v2 * (1 - cs2)));
            S->A[0] = (vn * (1 - cs2) - K) / (1 - vv * cs2);
            S->A[1] = vn;
            S->A[2] = vn;
            S->A[3] = vn;
            S->A[4] = vn;
            S->A[5] = vn;
            S->A[6] = vn;
            S->A[7] = (vn * (1 - cs2) + K) / (1 - vv * cs2);
            return MO_OK;
        }
        {
            const double K = W4 * (P[0] * h0 * (1. / cs2 - 1.));
            const double L = -W2 * (P[0] * h0 + bb / cs2);
            const double A4 = K - L - b0 * b0;
            const double A3 = -4 * K * vn + L * vn * 2 + 2 * b0 * bn;
            const double A2 = 6 * K * v2 + L * (1. - v2) + b0 * b0 - bn * bn;
            const double A1 = -4 * K * v3 - L * vn * 2 - 2 * b0 * bn;
            const double A0 = K * v4 + L * v2 + bn * bn;
            double roots[4];
            const int nr = mo_quartic(A4, A3, A2, A1, A0, roots);
            const double C = sqrt(h0 + bb);

            if (nr == 4) {
                S->A[0] = roots[0];
                S->A[1] = (bn - C * vn * W0) / (b0 - C * W0);
                S->A[2] = roots[1];
                S->A[3] = vn;
                S->A[4] = vn;
                S->A[5] = roots[2];
                S->A[6] = (bn + C * vn * W0) / (b0 + C * W0);
                S->A[7] = roots[3];
            } else if (nr == 2) {
                S->A[0] = roots[0];
                S->A[1] = (bn - C * vn * W0) / (b0 - C * W0);
                S->A[2] = vn;
                S->A[3] = vn;
                S->A[4] = vn;
                S->A[5] = vn;
                S->A[6] = (bn + C * vn * W0) / (b0 + C * W0);
                S->A[7] = roots[1];
            } else {
                return MO_ERR_BAD_EIGENVALUES;
            }
        }
    }
    return MO_OK;
}

/* ------------------------------------------------------------------------ */
/* ConsToPrimRMHD (ConsToPrimRMHD.cpp:77-323): Anton+2006 2-D Newton in      */
/* (Z, W), then Noble+2006 1-D Newton in Z.                                  */
/* ------------------------------------------------------------------------ */
typedef struct {
    double gamf, pfloor;
    double D, Tau, S2, B2, BS, BS2, Cons[8];
    double Z_start, W_start;
} c2p_rmhd;

enum { RM_MAXITER = 250 };
static const double RM_TOL = 1e-12, RM_BIGZ = 1e20, RM_BIGW = 1e12, RM_SMLZ = 0.0, RM_SMLW = 1.0;

static void rm_new_state(c2p_rmhd* s, const double* U)
{
    s->D = U[0];
    s->Tau = U[4];
    s->S2 = U[1] * U[1] + U[2] * U[2] + U[3] * U[3];
    s->B2 = U[5] * U[5] + U[6] * U[6] + U[7] * U[7];
    s->BS = U[5] * U[1] + U[6] * U[2] + U[7] * U[3];
    s->BS2 = s->BS * s->BS;
    memcpy(s->Cons, U, 8 * sizeof(double));
    /* estimate_from_cons */
    s->Z_start = sqrt(s->S2 + s->D * s->D);
    s->W_start = s->Z_start / s->D;
}

static int rm_check_cons(const double* U)
{
    if (U[0] < 0.0) return MO_C2P_CONS_NEGATIVE_DENSITY;
    if (U[4] < 0.0) return MO_C2P_CONS_NEGATIVE_ENERGY;
    for (int i = 0; i < 8; ++i)
        if (!isfinite(U[i])) return MO_C2P_CONS_CONTAINS_NAN;
    return MO_OK;
}

static int rm_check_prim(const double* P)
{
    const double v2 = P[1] * P[1] + P[2] * P[2] + P[3] * P[3];
    if (v2 >= 1.0) return MO_C2P_PRIM_SUPERLUMINAL;
    if (P[4] < 0.0) return MO_C2P_PRIM_NEGATIVE_PRESSURE;
    if (P[0] < 0.0) return MO_C2P_PRIM_NEGATIVE_RESTMASS;
    for (int i = 0; i < 8; ++i)
        if (!isfinite(P[i])) return MO_C2P_PRIM_CONTAINS_NAN;
    return MO_OK;
}

static int rm_reconstruct(const c2p_rmhd* s, double Z, double W, double* Pout)
{
    double P[8];
    const double b0 = s->BS * W / Z;
    P[0] = s->D / W;
    P[4] = (s->D / W) * (Z / (s->D * W) - 1.0) * s->gamf;
    P[1] = (s->Cons[1] + b0 * s->Cons[5] / W) / (Z + s->B2);
    P[2] = (s->Cons[2] + b0 * s->Cons[6] / W) / (Z + s->B2);
    P[3] = (s->Cons[3] + b0 * s->Cons[7] / W) / (Z + s->B2);
    P[5] = s->Cons[5];
    P[6] = s->Cons[6];
    P[7] = s->Cons[7];
    if (P[4] <= 0.0 && s->pfloor > 0.0) P[4] = P[0] * s->pfloor;
    {
        const int err = rm_check_prim(P);
        if (err) return err;
    }
    memcpy(Pout, P, 8 * sizeof(double));
    return MO_OK;
}

static int rm_anton2dzw(const c2p_rmhd* s, double* P)
{
    const int bad = rm_check_cons(s->Cons);
    if (bad) return bad;
    int it = 0;
    double error = 1.0, W = s->W_start, Z = s->Z_start;
    const double D = s->D, Tau = s->Tau, S2 = s->S2, B2 = s->B2, BS2 = s->BS2, gamf = s->gamf;

    while (error > RM_TOL) {
        const double Z2 = Z * Z;
        const double Z3 = Z * Z2;
        const double W2 = W * W;
        const double W3 = W * W2;
        const double Pre = (D / W) * (Z / (D * W) - 1.0) * gamf;
        const double df0dZ = 2 * (B2 + Z) * (BS2 * W2 + (W2 - 1) * Z3) / (W2 * Z3);
        const double df0dW = 2 * (B2 + Z) * (B2 + Z) / W3;
        const double df1dZ = 1.0 + BS2 / Z3 - gamf / W2;
        const double df1dW = B2 / W3 + (2 * Z - D * W) / W3 * gamf;
        const double f0 = -S2 + (Z + B2) * (Z + B2) * (W2 - 1) / W2 - (2 * Z + B2) * BS2 / Z2;
        const double f1 = -Tau + Z + B2 - Pre - 0.5 * B2 / W2 - 0.5 * BS2 / Z2 - D;
        const double J0 = df0dZ, J1 = df0dW, J2 = df1dZ, J3 = df1dW;
        const double det = J0 * J3 - J1 * J2;
        const double G0 = J3 / det, G1 = -J1 / det, G2 = -J2 / det, G3 = J0 / det;
        const double dZ = -(G0 * f0 + G1 * f1);
        const double dW = -(G2 * f0 + G3 * f1);
        double Z_new = Z + dZ;
        double W_new = W + dW;
        Z_new = (Z_new > RM_SMLZ) ? Z_new : -Z_new;
        Z_new = (Z_new < RM_BIGZ) ? Z_new : Z;
        W_new = (W_new > RM_SMLW) ? W_new : RM_SMLW;
        W_new = (W_new < RM_BIGW) ? W_new : RM_BIGW;
        Z = Z_new;
        W = W_new;
        error = fabs(dZ / Z) + fabs(dW / W);
        ++it;
        if (it == RM_MAXITER) return MO_C2P_MAXITER;
    }
    return rm_reconstruct(s, Z, W, P);
}

static int rm_noble1dw(const c2p_rmhd* s, double* P)
{
    const int bad = rm_check_cons(s->Cons);
    if (bad) return bad;
    int it = 0;
    double error = 1.0, Z = s->Z_start;
    const double D = s->D, Tau = s->Tau, S2 = s->S2, B2 = s->B2, BS2 = s->BS2, gamf = s->gamf;

    while (error > RM_TOL) {
        const double Z2 = Z * Z;
        const double Z3 = Z * Z2;
        const double a = S2 * Z2 + BS2 * (B2 + 2 * Z);
        const double b = (B2 + Z) * (B2 + Z) * Z2;
        const double ap = 2 * (S2 * Z + BS2);
        const double bp = 2 * Z * (B2 + Z) * (B2 + 2 * Z);
        const double V2 = a / b;
        const double W2 = 1.0 / (1.0 - V2);
        const double W = sqrt(W2);
        const double W3 = W * W2;
        const double Pre = (D / W) * (Z / (D * W) - 1.0) * gamf;
        const double dv2dZ = (ap * b - bp * a) / (b * b);
        const double delPdelZ = gamf / W2;
        const double delPdelW = gamf * (D / W2 - 2 * Z / W3);
        const double dWdv2 = 0.5 * W3;
        const double dPdZ = delPdelW * dWdv2 * dv2dZ + delPdelZ;
        const double f = Tau + D - 0.5 * B2 * (1 + V2) + 0.5 * BS2 / Z2 - Z + Pre;
        const double g = -0.5 * B2 * dv2dZ - BS2 / Z3 - 1.0 + dPdZ;
        const double dZ = -f / g;
        double Z_new = Z + dZ;
        Z_new = (Z_new > RM_SMLZ) ? Z_new : -Z_new;
        Z_new = (Z_new < RM_BIGZ) ? Z_new : Z;
        Z = Z_new;
        error = fabs(dZ / Z);
        ++it;
        if (it == RM_MAXITER) return MO_C2P_MAXITER;
    }
    {
        const double Z2 = Z * Z;
        const double a = S2 * Z2 + BS2 * (B2 + 2 * Z);
        const double b = (B2 + Z) * (B2 + Z) * Z2;
        const double V2 = a / b;
        const double W2 = 1.0 / (1.0 - V2);
        const double W = sqrt(W2);
        return rm_reconstruct(s, Z, W, P);
    }
}

/* RelativisticMHD::fromConserved (ConservationLaws.cpp:627-657); the
 * eigenvalue evaluation of the final fromPrimitive call may raise "bad
 * eigenvalues", which aborts the caller. */
static int rmhd_cons(double gamma, double pfloor, const double* U, double* P, int* health)
{
    c2p_rmhd s;
    double Q[8];
    int err;
    s.gamf = (gamma - 1.0) / gamma;
    s.pfloor = pfloor;
    rm_new_state(&s, U);
    *health = 0;
    err = rm_anton2dzw(&s, Q);
    if (err != MO_OK) err = rm_noble1dw(&s, Q);
    if (err != MO_OK) return MO_ERR_INVERSION_FAILURE;
    {
        static const double xhat[3] = {1.0, 0.0, 0.0}; /* Request() default areaElement */
        mstate S;
        const int e2 = rmhd_prim(gamma, Q, xhat, &S);
        if (e2 != MO_OK) return e2;
    }
    for (int q = 0; q < 8; ++q) P[q] = Q[q];
    return MO_OK;
}

/* ------------------------------------------------------------------------ */
/* law dispatch                                                              */
/* ------------------------------------------------------------------------ */
static int from_prim(const mo_config* c, const double* P, const double* n, mstate* S)
{
    switch (c->law) {
        case MO_LAW_HYDRO: return hydro_prim(c->gamma, P, n, S);
        case MO_LAW_MHD: return mhd_prim(c->gamma, mhd_aux(c), P, n, S);
        case MO_LAW_RMHD: return rmhd_prim(c->gamma, P, n, S);
        default: return MO_ERR_CONFIG;
    }
}

static int from_cons(const mo_config* c, const double* U, double* P, int* health)
{
    *health = 0;
    switch (c->law) {
        case MO_LAW_HYDRO: return hydro_cons(c->gamma, U, P);
        case MO_LAW_MHD: return mhd_cons(c->gamma, c->pressure_floor, mhd_aux(c), U, P, health);
        case MO_LAW_RMHD: return rmhd_cons(c->gamma, c->pressure_floor, U, P, health);
        default: return MO_ERR_CONFIG;
    }
}

int mo_from_primitive(const mo_config* c, const double* P, const double n[3],
                      double* U, double* F, double* A)
{
    mstate S;
    const int err = from_prim(c, P, n, &S);
    if (err) return err;
    for (int q = 0; q < NSLOT; ++q) {
        if (U) U[q] = S.U[q];
        if (F) F[q] = S.F[q];
        if (A) A[q] = S.A[q];
    }
    return MO_OK;
}

int mo_from_conserved(const mo_config* c, const double* U, double* P, int* health)
{
    int h = 0;
    const int err = from_cons(c, U, P, &h);
    if (health) *health = h;
    return err;
}

/* ------------------------------------------------------------------------ */
/* Reconstruction (Reconstruction.cpp:55-169)                                */
/* ------------------------------------------------------------------------ */
#define SGN(x) (((x) > 0) - ((x) < 0))

static inline double min2(double a, double b) { return a < b ? a : b; }
static inline double min3(double a, double b, double c) { return a < b ? min2(a, c) : min2(b, c); }
static inline double max2(double a, double b) { return a > b ? a : b; }
static inline double max3(double a, double b, double c) { return a > b ? max2(a, c) : max2(b, c); }

/* generalized minmod limiter, Reconstruction.cpp:55-61 */
static inline double minmod(double theta, double ul, double u0, double ur)
{
    const double a = theta * (u0 - ul);
    const double b = 0.5 * (ur - ul);
    const double c = theta * (ur - u0);
    return 0.25 * fabs((double) (SGN(a) + SGN(b))) * (double) (SGN(a) + SGN(c))
         * min3(fabs(a), fabs(b), fabs(c));
}

/* WENO5 tables (Jiang & Shu 1996): finite-difference point values at the
 * right (C2R) and left (C2L) cell edge, Reconstruction.cpp:272-287 */
static const double W_C2R[3][3] = {{1. / 3., 5. / 6., -1. / 6.}, {-1. / 6., 5. / 6., 1. / 3.}, {1. / 3., -7. / 6., 11. / 6.}};
static const double W_C2L[3][3] = {{11. / 6., -7. / 6., 1. / 3.}, {1. / 3., 5. / 6., -1. / 6.}, {-1. / 6., 5. / 6., 1. / 3.}};
static const double W_D_C2R[3] = {0.3, 0.6, 0.1};
static const double W_D_C2L[3] = {0.1, 0.6, 0.3};

#define SQU(x) ((x) * (x))

/* Reconstruction::weno5, Reconstruction.cpp:68-132; v points at the centre */
static double weno5(const double* v, const double c[3][3], const double d[3], int mode, double A)
{
    double eps, eps_prime, w[3];
    const double vs[3] = {
        c[0][0] * v[+0] + c[0][1] * v[+1] + c[0][2] * v[2],
        c[1][0] * v[-1] + c[1][1] * v[+0] + c[1][2] * v[1],
        c[2][0] * v[-2] + c[2][1] * v[-1] + c[2][2] * v[0],
    };
    double B[3] = {
        (13. / 12.) * SQU(1 * v[+0] - 2 * v[+1] + 1 * v[+2]) + (1. / 4.) * SQU(3 * v[+0] - 4 * v[+1] + 1 * v[+2]),
        (13. / 12.) * SQU(1 * v[-1] - 2 * v[+0] + 1 * v[+1]) + (1. / 4.) * SQU(1 * v[-1] - 0 * v[+0] - 1 * v[+1]),
        (13. / 12.) * SQU(1 * v[-2] - 2 * v[-1] + 1 * v[+0]) + (1. / 4.) * SQU(1 * v[-2] - 4 * v[-1] + 3 * v[+0]),
    };
    switch (mode) {
        case MO_WENO_BORGES08: {
            eps = 1e-14;
            const double tau5 = fabs(B[0] - B[2]);
            w[0] = d[0] * (1.0 + (tau5 / (B[0] + eps)));
            w[1] = d[1] * (1.0 + (tau5 / (B[1] + eps)));
            w[2] = d[2] * (1.0 + (tau5 / (B[2] + eps)));
            break;
        }
        case MO_WENO_SHENZHA10: {
            eps_prime = 1e-10;
            const double minB = min3(B[0], B[1], B[2]);
            const double maxB = max3(B[0], B[1], B[2]);
            const double R0 = minB / (maxB + eps_prime);
            B[0] = R0 * A * minB + B[0];
            B[1] = R0 * A * minB + B[1];
            B[2] = R0 * A * minB + B[2];
            w[0] = d[0] / SQU(eps_prime + B[0]);
            w[1] = d[1] / SQU(eps_prime + B[1]);
            w[2] = d[2] / SQU(eps_prime + B[2]);
            break;
        }
        default: {
            eps_prime = 1e-6;
            w[0] = d[0] / SQU(eps_prime + B[0]);
            w[1] = d[1] / SQU(eps_prime + B[1]);
            w[2] = d[2] / SQU(eps_prime + B[2]);
            break;
        }
    }
    {
        const double wtot = w[0] + w[1] + w[2];
        return (w[0] * vs[0] + w[1] * vs[1] + w[2] * vs[2]) / wtot;
    }
}

/* ------------------------------------------------------------------------ */
/* Riemann solvers (RiemannSolvers.cpp:38-118)                               */
/* ------------------------------------------------------------------------ */
static inline double max_slot(const double* A)
{
    double m = A[0];
    for (int n = 1; n < NSLOT; ++n) if (m < A[n]) m = A[n];
    return m;
}

static inline double min_slot(const double* A)
{
    double m = A[0];
    for (int n = 1; n < NSLOT; ++n) if (A[n] < m) m = A[n];
    return m;
}

static void hlle(const mstate* L, const mstate* R, int nq, double* F)
{
    const double epl = max_slot(L->A), eml = min_slot(L->A);
    const double epr = max_slot(R->A), emr = min_slot(R->A);
    const double ap = max3(0.0, epl, epr);
    const double am = min3(0.0, eml, emr);
    for (int q = 0; q < nq; ++q)
        F[q] = (ap * L->F[q] - am * R->F[q] + ap * am * (R->U[q] - L->U[q])) / (ap - am);
}

static void hllc(const mstate* L, const mstate* R, const double* dA, int nq, double* F)
{
    const double epl = max_slot(L->A), eml = min_slot(L->A);
    const double epr = max_slot(R->A), emr = min_slot(R->A);
    const double ap = max3(0.0, epl, epr);
    const double am = min3(0.0, eml, emr);
    const double* Pl = L->P;
    const double* Pr = R->P;
    const double* Ul = L->U;
    const double* Ur = R->U;
    const double vnr = Pr[1] * dA[0] + Pr[2] * dA[1] + Pr[3] * dA[2];
    const double vnl = Pl[1] * dA[0] + Pl[2] * dA[1] + Pl[3] * dA[2];
    double Uls[5], Urs[5];
    const double lc = (+(Pr[4] - Pr[0] * vnr * (ap - vnr)) - (Pl[4] - Pl[0] * vnl * (am - vnl)))
                    / (Pl[0] * (am - vnl) - Pr[0] * (ap - vnr));
    const double fl = Pl[0] * (am - vnl) / (am - lc);
    const double fr = Pr[0] * (ap - vnr) / (ap - lc);
    const double s = 0.0;

    Uls[0] = fl;
    Uls[4] = fl * (Ul[4] / Pl[0] + (lc - vnl) * (lc + Pl[4] / (Pl[0] * (am - vnl))));
    Uls[1] = fl * ((lc - vnl) * dA[0] + Pl[1]);
    Uls[2] = fl * ((lc - vnl) * dA[1] + Pl[2]);
    Uls[3] = fl * ((lc - vnl) * dA[2] + Pl[3]);
    Urs[0] = fr;
    Urs[4] = fr * (Ur[4] / Pr[0] + (lc - vnr) * (lc + Pr[4] / (Pr[0] * (ap - vnr))));
    Urs[1] = fr * ((lc - vnr) * dA[0] + Pr[1]);
    Urs[2] = fr * ((lc - vnr) * dA[1] + Pr[2]);
    Urs[3] = fr * ((lc - vnr) * dA[2] + Pr[3]);

    for (int q = 0; q < nq; ++q) F[q] = 0.0;
    if (s <= am)                 for (int i = 0; i < 5; ++i) F[i] = L->F[i];
    else if (am < s && s <= lc)  for (int i = 0; i < 5; ++i) F[i] = L->F[i] + am * (Uls[i] - Ul[i]);
    else if (lc < s && s <= ap)  for (int i = 0; i < 5; ++i) F[i] = R->F[i] + ap * (Urs[i] - Ur[i]);
    else if (ap < s)             for (int i = 0; i < 5; ++i) F[i] = R->F[i];
}

/* ------------------------------------------------------------------------ */
/* intercell flux: MethodOfLines (IntercellFluxSchemes.cpp:75-88),           */
/* MethodOfLinesPlm (:115-142) and the WENO5 composition (same shape as      */
/* MethodOfLinesPlm with WENO5 C2R/C2L reconstructions on a 6-cell stencil)  */
/* stencil[n] points at cell n's nq primitives; fp = 2 * stencil size.       */
/* ------------------------------------------------------------------------ */
static int face_flux(const mo_config* c, int nq, const double* const* st, const double* n, double* F)
{
    double PL[NSLOT] = {0}, PR[NSLOT] = {0};
    mstate L, R;
    int err;

    switch (c->recon) {
        case MO_RECON_PCM:
            for (int q = 0; q < nq; ++q) { PL[q] = st[0][q]; PR[q] = st[1][q]; }
            break;
        case MO_RECON_PLM:
            for (int q = 0; q < nq; ++q) {
                const double p0 = st[0][q], p1 = st[1][q], p2 = st[2][q], p3 = st[3][q];
                PL[q] = p1 + +1.0 * 0.5 * minmod(c->plm_theta, p0, p1, p2);
                PR[q] = p2 + -1.0 * 0.5 * minmod(c->plm_theta, p1, p2, p3);
            }
            break;
        case MO_RECON_WENO5:
            for (int q = 0; q < nq; ++q) {
                const double v[6] = {st[0][q], st[1][q], st[2][q], st[3][q], st[4][q], st[5][q]};
                PL[q] = weno5(&v[2], W_C2R, W_D_C2R, c->weno_is, c->shenzha_A);
                PR[q] = weno5(&v[3], W_C2L, W_D_C2L, c->weno_is, c->shenzha_A);
            }
            break;
        default:
            return MO_ERR_CONFIG;
    }
    if ((err = from_prim(c, PL, n, &L))) return err;
    if ((err = from_prim(c, PR, n, &R))) return err;
    if (c->riemann == MO_RIEMANN_HLLC) hllc(&L, &R, n, nq, F);
    else hlle(&L, &R, nq, F);
    return MO_OK;
}

/* ------------------------------------------------------------------------ */
/* MeshOperator::godunov (MeshOperator.cpp:443-525)                          */
/* ------------------------------------------------------------------------ */
static int godunov_sweeps(const mo_config* c, const mgeom* g, const double* P, double* F)
{
    const int fp = 2 * mo_stencil_size(c);
    const int nq = g->nq;
    const long fsize = (long) (g->N[0] + 1) * (g->N[1] + 1) * (g->N[2] + 1) * nq * 3;
    int status = MO_OK;

    memset(F, 0, fsize * sizeof(double));

    for (int a = 0; a < 3; ++a) {
        int S[3] = {g->N[0], g->N[1], g->N[2]};
        if (g->N[a] == 1) continue; /* zero footprint on flat axes */
        S[a] -= fp - 1;
        if (S[a] <= 0) continue;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int i = 0; i < S[0]; ++i) {
            const double* st[6];
            double Fh[NSLOT];
            for (int j = 0; j < S[1]; ++j)
                for (int k = 0; k < S[2]; ++k) {
                    int e;
                    for (int n = 0; n < fp; ++n) {
                        const int ii = i + (a == 0 ? n : 0);
                        const int jj = j + (a == 1 ? n : 0);
                        const int kk = k + (a == 2 ? n : 0);
                        st[n] = P + cidx(g, ii, jj, kk);
                    }
                    e = face_flux(c, nq, st, g->nrm[a], Fh);
                    if (e) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
                        status = e;
                        continue;
                    }
                    {
                        const int fi = i + (a == 0 ? fp / 2 : 0);
                        const int fj = j + (a == 1 ? fp / 2 : 0);
                        const int fk = k + (a == 2 ? fp / 2 : 0);
                        for (int q = 0; q < nq; ++q) F[fidx(g, fi, fj, fk, q, a)] = Fh[q];
                    }
                }
        }
        if (status) return status;
    }
    return MO_OK;
}

/* CellCenteredFieldCT::correctGodunovFluxes (CellCenteredFieldCT.cpp:14-134):
 * Toth (2000) flux-CT, eq. 25 */
void mo_ct_correct(double* F, int n0, int n1, int n2, int nq, int ib)
{
    const long total = (long) n0 * n1 * n2 * nq * 3;
    double* G = (double*) malloc(total * sizeof(double));
    const int B0 = ib + 0, B1 = ib + 1, B2 = ib + 2;
#define FI(i, j, k, q, a) (((((long) (i) * n1 + (j)) * n2 + (k)) * nq + (q)) * 3 + (a))
#define FF(i, j, k, q, a) F[FI(i, j, k, q, a)]
    memcpy(G, F, total * sizeof(double));

    for (int i = 0; i < n0; ++i)
        for (int j = 0; j < n1; ++j)
            for (int k = 0; k < n2; ++k) {
                G[FI(i, j, k, B0, 0)] = 0.0;
                G[FI(i, j, k, B1, 1)] = 0.0;
                G[FI(i, j, k, B2, 2)] = 0.0;
            }

    if (n0 >= 3) {
        for (int i = 1; i < n0; ++i)
            for (int j = 1; j < n1 - 1; ++j)
                for (int k = 0; k < n2; ++k)
                    G[FI(i, j, k, B1, 0)] = 0.125 * (
                        + 2 * FF(i + 0, j + 0, k + 0, B1, 0)
                        + 1 * FF(i + 0, j + 1, k + 0, B1, 0)
                        + 1 * FF(i + 0, j - 1, k + 0, B1, 0)
                        - 1 * FF(i + 0, j + 1, k + 0, B0, 1)
                        - 1 * FF(i - 1, j + 1, k + 0, B0, 1)
                        - 1 * FF(i + 0, j + 0, k + 0, B0, 1)
                        - 1 * FF(i - 1, j + 0, k + 0, B0, 1));
        for (int i = 1; i < n0; ++i)
            for (int j = 0; j < n1; ++j)
                for (int k = 1; k < n2 - 1; ++k)
                    G[FI(i, j, k, B2, 0)] = 0.125 * (
                        + 2 * FF(i + 0, j + 0, k + 0, B2, 0)
                        + 1 * FF(i + 0, j + 0, k + 1, B2, 0)
                        + 1 * FF(i + 0, j + 0, k - 1, B2, 0)
                        - 1 * FF(i + 0, j + 0, k + 1, B0, 2)
                        - 1 * FF(i - 1, j + 0, k + 1, B0, 2)
                        - 1 * FF(i + 0, j + 0, k + 0, B0, 2)
                        - 1 * FF(i - 1, j + 0, k + 0, B0, 2));
    }
    if (n1 >= 3) {
        for (int i = 0; i < n0; ++i)
            for (int j = 1; j < n1; ++j)
                for (int k = 1; k < n2 - 1; ++k)
                    G[FI(i, j, k, B2, 1)] = 0.125 * (
                        + 2 * FF(i + 0, j + 0, k + 0, B2, 1)
                        + 1 * FF(i + 0, j + 0, k + 1, B2, 1)
                        + 1 * FF(i + 0, j + 0, k - 1, B2, 1)
                        - 1 * FF(i + 0, j + 0, k + 1, B1, 2)
                        - 1 * FF(i + 0, j - 1, k + 1, B1, 2)
                        - 1 * FF(i + 0, j + 0, k + 0, B1, 2)
                        - 1 * FF(i + 0, j - 1, k + 0, B1, 2));
        for (int i = 1; i < n0 - 1; ++i)
            for (int j = 1; j < n1; ++j)
                for (int k = 0; k < n2; ++k)
                    G[FI(i, j, k, B0, 1)] = 0.125 * (
                        + 2 * FF(i + 0, j + 0, k + 0, B0, 1)
                        + 1 * FF(i + 1, j + 0, k + 0, B0, 1)
                        + 1 * FF(i - 1, j + 0, k + 0, B0, 1)
                        - 1 * FF(i + 1, j + 0, k + 0, B1, 0)
                        - 1 * FF(i + 1, j - 1, k + 0, B1, 0)
                        - 1 * FF(i + 0, j + 0, k + 0, B1, 0)
                        - 1 * FF(i + 0, j - 1, k + 0, B1, 0));
    }
    if (n2 >= 3) {
        for (int i = 1; i < n0 - 1; ++i)
            for (int j = 0; j < n1; ++j)
                for (int k = 1; k < n2; ++k)
                    G[FI(i, j, k, B0, 2)] = 0.125 * (
                        + 2 * FF(i + 0, j + 0, k + 0, B0, 2)
                        + 1 * FF(i + 1, j + 0, k + 0, B0, 2)
                        + 1 * FF(i - 1, j + 0, k + 0, B0, 2)
                        - 1 * FF(i + 1, j + 0, k + 0, B2, 0)
                        - 1 * FF(i + 1, j + 0, k - 1, B2, 0)
                        - 1 * FF(i + 0, j + 0, k + 0, B2, 0)
                        - 1 * FF(i + 0, j + 0, k - 1, B2, 0));
        for (int i = 0; i < n0; ++i)
            for (int j = 1; j < n1 - 1; ++j)
                for (int k = 1; k < n2; ++k)
                    G[FI(i, j, k, B1, 2)] = 0.125 * (
                        + 2 * FF(i + 0, j + 0, k + 0, B1, 2)
                        + 1 * FF(i + 0, j + 1, k + 0, B1, 2)
                        + 1 * FF(i + 0, j - 1, k + 0, B1, 2)
                        - 1 * FF(i + 0, j + 1, k + 0, B2, 1)
                        - 1 * FF(i + 0, j + 1, k - 1, B2, 1)
                        - 1 * FF(i + 0, j + 0, k + 0, B2, 1)
                        - 1 * FF(i + 0, j + 0, k - 1, B2, 1));
    }
    memcpy(F, G, total * sizeof(double));
    free(G);
#undef FF
#undef FI
}

static int use_ct(const mo_config* c)
{
    return (c->law == MO_LAW_MHD || c->law == MO_LAW_RMHD) && !c->disable_ct;
}

int mo_godunov(const mo_config* c, const double* P, double* F)
{
    mgeom g;
    int err = make_geom_chk(c, &g, 1);
    if (err) return err;
    if ((err = godunov_sweeps(c, &g, P, F))) return err;
    if (use_ct(c)) mo_ct_correct(F, g.N[0] + 1, g.N[1] + 1, g.N[2] + 1, g.nq, 5);
    return MO_OK;
}

/* ------------------------------------------------------------------------ */
/* boundary conditions (BoundaryConditions.cpp:8-176)                        */
/* ------------------------------------------------------------------------ */
static void copy_layer(const mgeom* g, double* P, int axis, int dst, int src, int flip_axis)
{
    const int nq = g->nq;
    int lo[3] = {0, 0, 0}, hi[3] = {g->N[0], g->N[1], g->N[2]};
    lo[axis] = 0;
    hi[axis] = 1;
    for (int i = lo[0]; i < hi[0]; ++i)
        for (int j = lo[1]; j < hi[1]; ++j)
            for (int k = lo[2]; k < hi[2]; ++k) {
                int d[3] = {i, j, k}, s[3] = {i, j, k};
                d[axis] = dst;
                s[axis] = src;
                {
                    double* pd = P + cidx(g, d[0], d[1], d[2]);
                    const double* ps = P + cidx(g, s[0], s[1], s[2]);
                    for (int q = 0; q < nq; ++q) pd[q] = ps[q];
                    if (flip_axis >= 0) pd[1 + flip_axis] *= -1;
                }
            }
}

static int apply_bc(const mo_config* c, const mgeom* g, double* P)
{
    for (int a = 0; a < 3; ++a) {
        const int ng = c->ng[a];
        const int N = g->N[a];
        if (ng <= 0) continue;
        /* left, then right */
        for (int side = 0; side < 2; ++side) {
            for (int n = 0; n < ng; ++n) {
                switch (c->bc) {
                    case MO_BC_PERIODIC:
                        /* guard [0,ng) <- [N-2ng, N-ng); guard [N-ng, N) <- [ng, 2ng) */
                        if (side == 0) copy_layer(g, P, a, n, N - 2 * ng + n, -1);
                        else copy_layer(g, P, a, N - ng + n, ng + n, -1);
                        break;
                    case MO_BC_OUTFLOW:
                        if (side == 0) copy_layer(g, P, a, n, ng, -1);
                        else copy_layer(g, P, a, N - n - 1, N - ng - 1, -1);
                        break;
                    case MO_BC_REFLECTING:
                        if (side == 0) copy_layer(g, P, a, n, 2 * ng - n - 1, a);
                        else copy_layer(g, P, a, N - n - 1, N - 2 * ng + n, a);
                        break;
                    default:
                        return MO_ERR_CONFIG;
                }
            }
        }
    }
    return MO_OK;
}

int mo_apply_bc(const mo_config* c, double* P)
{
    mgeom g;
    const int err = make_geom(c, &g);
    if (err) return err;
    return apply_bc(c, &g, P);
}

/* ------------------------------------------------------------------------ */
/* FieldOperator::generateConserved (FieldOperator.cpp:91-116)               */
/* ------------------------------------------------------------------------ */
int mo_generate_conserved(const mo_config* c, const double* P, double* U)
{
    mgeom g;
    static const double xhat[3] = {1.0, 0.0, 0.0};
    int err = make_geom(c, &g), status = MO_OK;
    const long ncell = (long) g.N[0] * g.N[1] * g.N[2];
    if (err) return err;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long n = 0; n < ncell; ++n) {
        mstate S;
        const int e = from_prim(c, P + n * g.nq, xhat, &S);
        if (e) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
            status = e;
            continue;
        }
        for (int q = 0; q < g.nq; ++q) U[n * g.nq + q] = S.U[q];
    }
    return status;
}

/* ------------------------------------------------------------------------ */
/* FieldOperator::getCourantTimestep (FieldOperator.cpp:125-169) with        */
/* ConservationLaw::maxEigenvalueMagnitude (ConservationLaws.cpp:114-127)    */
/* ------------------------------------------------------------------------ */
static double max_eigen_magnitude(const mstate* S, int nq)
{
    double m = 0.0;
    for (int n = 0; n < nq; ++n)
        if (m < fabs(S->A[n])) m = fabs(S->A[n]);
    return m;
}

int mo_courant(const mo_config* c, const double* P, double* dt_out)
{
    mgeom g;
    int err = make_geom(c, &g);
    double dtmin = 1.7976931348623157e308; /* numeric_limits<double>::max */
    int status = MO_OK;
    static const double ax[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    double nrm[3][3];
    if (err) return err;
    /* the Courant requests are oriented with UnitVector::xhat/yhat/zhat */
    mo_face_normals(nrm);
    (void) ax;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(min : dtmin)
#endif
    for (int i = c->ng[0]; i < g.N[0] - c->ng[0]; ++i)
        for (int j = c->ng[1]; j < g.N[1] - c->ng[1]; ++j)
            for (int k = c->ng[2]; k < g.N[2] - c->ng[2]; ++k) {
                const double* p = P + cidx(&g, i, j, k);
                mstate S0, S1, S2;
                double lam[3], lmax, dt;
                int e0 = from_prim(c, p, nrm[0], &S0);
                int e1 = e0 ? e0 : from_prim(c, p, nrm[1], &S1);
                int e2 = e1 ? e1 : from_prim(c, p, nrm[2], &S2);
                if (e2) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
                    status = e2;
                    continue;
                }
                lam[0] = max_eigen_magnitude(&S0, g.nq);
                lam[1] = max_eigen_magnitude(&S1, g.nq);
                lam[2] = max_eigen_magnitude(&S2, g.nq);
                lmax = lam[0];
                if (lmax < lam[1]) lmax = lam[1];
                if (lmax < lam[2]) lmax = lam[2];
                dt = g.lmin / lmax;
                if (dt < dtmin) dtmin = dt;
            }
    *dt_out = dtmin;
    return status;
}

/* ------------------------------------------------------------------------ */
/* MethodOfLinesTVD::advance (SolutionSchemes.cpp:108-275)                   */
/* ------------------------------------------------------------------------ */
/* ------------------------------------------------------------------------ */
/* MethodOfLinesTVD::setSourceTermsFunction (SolutionSchemes.hpp:36) and     */
/* MeshOperator::generateSourceTerms (MeshOperator.cpp:197-218): a per-cell  */
/* function of the cell centre, the auxiliary data (zeros: no star           */
/* particles) and the primitives, evaluated over every cell of the array     */
/* with guards and added to L (SolutionSchemes.cpp:219-228)                  */
/* ------------------------------------------------------------------------ */
static mo_source_fn g_src_fn = NULL;
static void* g_src_user = NULL;

void mo_set_source_terms(mo_source_fn fn, void* user)
{
    g_src_fn = fn;
    g_src_user = user;
}

static void add_source_terms(const mo_config* c, const mgeom* g, const double* P, double* L)
{
    static const double aux[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = 0; i < g->N[0]; ++i)
        for (int j = 0; j < g->N[1]; ++j)
            for (int k = 0; k < g->N[2]; ++k) {
                /* CartesianMeshGeometry::coordinateAtIndex (CartesianMeshGeometry.
                 * cpp:61-67) at the index plus the start index -ng of
                 * SchemeHelpers::makeFootprint */
                const double x = c->lower[0] + g->dx[0] * ((double) (i - c->ng[0]) + 0.5);
                const double y = c->lower[1] + g->dx[1] * ((double) (j - c->ng[1]) + 0.5);
                const double z = c->lower[2] + g->dx[2] * ((double) (k - c->ng[2]) + 0.5);
                double p[NSLOT], S[NSLOT];
                const long o = cidx(g, i, j, k);
                for (int q = 0; q < NSLOT; ++q) {
                    p[q] = q < g->nq ? P[o + q] : 0.0;
                    S[q] = 0.0;
                }
                g_src_fn(g_src_user, x, y, z, aux, p, S);
                for (int q = 0; q < g->nq; ++q) L[o + q] += S[q];
            }
}

int mo_advance(const mo_config* c, double* P, double t0, double dt, mo_failure* fail)
{
    static const double b1[1] = {1.0};
    static const double b2[2] = {1.0, 0.5};
    static const double b3[3] = {1.0, 1. / 4, 2. / 3};
    const double* b;
    mgeom g;
    int err = make_geom_chk(c, &g, 1);
    long ncell, nelem, fsize;
    double *U0, *U, *F, *L;
    (void) t0;
    if (fail) memset(fail, 0, sizeof(*fail));
    if (err) return err;
    b = c->rk_order == 1 ? b1 : c->rk_order == 2 ? b2 : b3;
    ncell = (long) g.N[0] * g.N[1] * g.N[2];
    nelem = ncell * g.nq;
    fsize = (long) (g.N[0] + 1) * (g.N[1] + 1) * (g.N[2] + 1) * g.nq * 3;
    U0 = (double*) malloc(nelem * sizeof(double));
    U = (double*) malloc(nelem * sizeof(double));
    L = (double*) malloc(nelem * sizeof(double));
    F = (double*) malloc(fsize * sizeof(double));
    if (!U0 || !U || !L || !F) { free(U0); free(U); free(L); free(F); return MO_ERR_CONFIG; }

    if ((err = mo_generate_conserved(c, P, U0))) goto done;
    memcpy(U, U0, nelem * sizeof(double));

    for (int rk = 0; rk < c->rk_order; ++rk) {
        if ((err = godunov_sweeps(c, &g, P, F))) goto done;
        if (use_ct(c)) mo_ct_correct(F, g.N[0] + 1, g.N[1] + 1, g.N[2] + 1, g.nq, 5);

        /* MeshOperator::divergence (MeshOperator.cpp:323-381), factor -1 */
        {
            const double factor = -1.0;
            const double A1000 = g.dA[0], A0000 = g.dA[0];
            const double A0101 = g.dA[1], A0001 = g.dA[1];
            const double A0012 = g.dA[2], A0002 = g.dA[2];
            const double vol = g.dV;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
            for (int i = 0; i < g.N[0]; ++i)
                for (int j = 0; j < g.N[1]; ++j)
                    for (int k = 0; k < g.N[2]; ++k)
                        for (int q = 0; q < g.nq; ++q)
                            L[cidx(&g, i, j, k) + q] = factor / vol * (
                                + F[fidx(&g, i + 1, j, k, q, 0)] * A1000
                                - F[fidx(&g, i, j, k, q, 0)] * A0000
                                + F[fidx(&g, i, j + 1, k, q, 1)] * A0101
                                - F[fidx(&g, i, j, k, q, 1)] * A0001
                                + F[fidx(&g, i, j, k + 1, q, 2)] * A0012
                                - F[fidx(&g, i, j, k, q, 2)] * A0002);
        }

        /* ConservationLaw::addSourceTerms (SolutionSchemes.cpp:201):
         * NewtonianMHD cooling (ConservationLaws.cpp:489-501) over every cell */
        if (mhd_aux(c)) {
            const double gm1 = c->gamma - 1.0;
            for (long n = 0; n < ncell; ++n) {
                const double p = P[n * g.nq + 4];
                L[n * g.nq + 4] -= p / gm1 * c->cooling_rate;
                L[n * g.nq + 8] += p / gm1 * c->cooling_rate;
            }
        }
        if (g_src_fn) add_source_terms(c, &g, P, L);

        /* RK combine over every element (SolutionSchemes.cpp:232-235) */
        {
            const double br = b[rk];
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
            for (long n = 0; n < nelem; ++n)
                U[n] = U0[n] * (1 - br) + (U[n] + dt * L[n]) * br;
        }

        /* FieldOperator::recoverPrimitive over the interior
         * (FieldOperator.cpp:41-82): failures are gathered over all zones,
         * then reported; "bad eigenvalues" aborts at once */
        {
            int nfail = 0, abort_code = MO_OK;
            for (int i = c->ng[0]; i < g.N[0] - c->ng[0] && !abort_code; ++i)
                for (int j = c->ng[1]; j < g.N[1] - c->ng[1] && !abort_code; ++j)
                    for (int k = c->ng[2]; k < g.N[2] - c->ng[2]; ++k) {
                        const long o = cidx(&g, i, j, k);
                        int health = 0;
                        double Pn[NSLOT];
                        const int e = from_cons(c, U + o, Pn, &health);
                        if (e == MO_ERR_INVERSION_FAILURE) {
                            if (nfail == 0 && fail) {
                                fail->first[0] = i - c->ng[0];
                                fail->first[1] = j - c->ng[1];
                                fail->first[2] = k - c->ng[2];
                                fail->code = e;
                            }
                            ++nfail;
                            continue;
                        }
                        if (e) { abort_code = e; break; }
                        for (int q = 0; q < g.nq; ++q) P[o + q] = Pn[q];
                    }
            if (fail) fail->count = nfail;
            if (abort_code) { err = abort_code; goto done; }
            if (nfail) { err = MO_ERR_INVERSION_FAILURE; goto done; }
        }
        if ((err = apply_bc(c, &g, P))) goto done;
    }
done:
    free(U0);
    free(U);
    free(L);
    free(F);
    return err;
}

/* ------------------------------------------------------------------------ */
/* CellCenteredFieldCT::monopole, MeshLocation::cell                         */
/* (CellCenteredFieldCT.cpp:159-223)                                         */
/* ------------------------------------------------------------------------ */
void mo_monopole_cell(const double* B, int n0, int n1, int n2, double h, double* Mc)
{
    const int r = n0 > 1 ? 1 : 0, s = n1 > 1 ? 1 : 0, t = n2 > 1 ? 1 : 0;
    const int m0 = n0 + 1, m1 = n1 + 1, m2 = n2 + 1;
    double* M = (double*) calloc((size_t) m0 * m1 * m2, sizeof(double));
#define BI(i, j, k, c) B[(((long) (i) * n1 + (j)) * n2 + (k)) * 3 + (c)]
#define MI(i, j, k) M[((long) (i) * m1 + (j)) * m2 + (k)]
    for (int i = 0; i < n0 - r; ++i)
        for (int j = 0; j < n1 - s; ++j)
            for (int k = 0; k < n2 - t; ++k) {
                const double Bx0 = BI(i, j, k, 0) + BI(i, j, k + t, 0) + BI(i, j + s, k, 0) + BI(i, j + s, k + t, 0);
                const double Bx1 = BI(i + r, j, k, 0) + BI(i + r, j, k + t, 0) + BI(i + r, j + s, k, 0) + BI(i + r, j + s, k + t, 0);
                const double By0 = BI(i, j, k, 1) + BI(i + r, j, k, 1) + BI(i, j, k + t, 1) + BI(i + r, j, k + t, 1);
                const double By1 = BI(i, j + s, k, 1) + BI(i + r, j + s, k, 1) + BI(i, j + s, k + t, 1) + BI(i + r, j + s, k + t, 1);
                const double Bz0 = BI(i, j, k, 2) + BI(i, j + s, k, 2) + BI(i + r, j, k, 2) + BI(i + r, j + s, k, 2);
                const double Bz1 = BI(i, j, k + t, 2) + BI(i, j + s, k + t, 2) + BI(i + r, j, k + t, 2) + BI(i + r, j + s, k + t, 2);
                MI(i + 1, j + 1, k + 1) = 0.25 * ((Bx1 - Bx0) + (By1 - By0) + (Bz1 - Bz0)) / h;
            }
    for (int i = 0; i < n0; ++i)
        for (int j = 0; j < n1; ++j)
            for (int k = 0; k < n2; ++k) {
                const double Mi = MI(i, j, k) + MI(i + 1, j, k);
                const double Mj = MI(i, j, k) + MI(i, j + 1, k);
                const double Mk = MI(i, j, k) + MI(i, j, k + 1);
                Mc[((long) i * n1 + j) * n2 + k] = 1. / 6 * (Mi + Mj + Mk);
            }
    free(M);
#undef BI
#undef MI
}

/* ------------------------------------------------------------------------ */
/* ConservationLaw::makeDiagnostics of one primitive state                   */
/* (NewtonianHydro ConservationLaws.cpp:321-330, NewtonianMHD :536-574 with  */
/* no auxiliary fields, RelativisticMHD :874-922); the state comes from      */
/* fromPrimitive with the default Request (area element x-hat,               */
/* ConservationLaws.cpp:146-157)                                             */
/* ------------------------------------------------------------------------ */
int mo_num_diagnostics(const mo_config* c)
{
    switch (c->law) {
        case MO_LAW_HYDRO: return 5;
        case MO_LAW_MHD: return 17 + mhd_aux(c);
        case MO_LAW_RMHD: return 17;
        default: return 0;
    }
}

static int make_diagnostics(const mo_config* c, const double* P, double* D)
{
    static const double xhat[3] = {1.0, 0.0, 0.0};
    mstate S;
    const int err = from_prim(c, P, xhat, &S);
    if (err) return err;
    if (c->law == MO_LAW_HYDRO) {
        for (int q = 0; q < 5; ++q) D[q] = S.U[q];
        return MO_OK;
    }
    const double gm = c->gamma;
    const double vv = P[1] * P[1] + P[2] * P[2] + P[3] * P[3];
    const double BB = P[5] * P[5] + P[6] * P[6] + P[7] * P[7];
    const double Bv = P[5] * P[1] + P[6] * P[2] + P[7] * P[3];
    const double cs = sqrt(gm * P[4] / P[0]);
    const double ca = sqrt(BB / P[0]);
    const double s0 = P[4] / pow(P[0], gm);
    const double Ms = sqrt(vv) / cs;
    const double Ma = sqrt(vv) / ca;
    for (int q = 0; q < 8; ++q) D[q] = S.U[q];
    if (c->law == MO_LAW_MHD) {
        D[8] = 0.5 * vv * P[0];     /* kinetic energy  */
        D[9] = P[4] / (gm - 1.0);   /* internal energy */
        D[10] = 0.5 * BB;           /* magnetic energy */
    } else {
        const double v1 = P[1], v2 = P[2], v3 = P[3];
        const double B1 = P[5], B2 = P[6], B3 = P[7];
        const double E1 = -(v2 * B3 - v3 * B2);
        const double E2 = -(v3 * B1 - v1 * B3);
        const double E3 = -(v1 * B2 - v2 * B1);
        const double EE = (E1 * E1 + E2 * E2 + E3 * E3);
        const double g0 = 1.0 / sqrt(1 - vv);
        const double d0 = P[0];
        const double p0 = P[4];
        const double e0 = p0 / d0 / (gm - 1);
        const double h0 = 1.0 + e0 + p0 / d0;
        D[8] = g0 * (g0 - 1) * d0 * h0;
        D[9] = p0 * (g0 - 1) + d0 * e0 * g0;
        D[10] = 0.5 * (BB + EE);
    }
    D[11] = cs;
    D[12] = ca;
    D[13] = Ms;
    D[14] = Ma;
    D[15] = s0;
    D[16] = Bv;
    if (mhd_aux(c)) D[17] = S.U[8];
    return MO_OK;
}

/* ------------------------------------------------------------------------ */
/* FieldOperator::volumeIntegratedDiagnostics (FieldOperator.cpp:171-205)    */
/* over the interior of P with the cell volumes of MeshOperator::measure:    */
/* the per-zone terms summed in the reference's iteration order (k fastest). */
/* Dabs (optional) receives the sum of the terms' magnitudes.                */
/* ------------------------------------------------------------------------ */
int mo_volume_diagnostics(const mo_config* c, const double* P, double* D, double* Dabs)
{
    mgeom g;
    int err = make_geom(c, &g);
    const int nd = mo_num_diagnostics(c);
    if (err) return err;
    for (int n = 0; n < nd; ++n) {
        D[n] = 0.0;
        if (Dabs) Dabs[n] = 0.0;
    }
    for (int i = c->ng[0]; i < c->ng[0] + c->ni; ++i)
        for (int j = c->ng[1]; j < c->ng[1] + c->nj; ++j)
            for (int k = c->ng[2]; k < c->ng[2] + c->nk; ++k) {
                double d[18];
                err = make_diagnostics(c, P + cidx(&g, i, j, k), d);
                if (err) return err;
                for (int n = 0; n < nd; ++n) {
                    D[n] += d[n] * g.dV;
                    if (Dabs) Dabs[n] += fabs(d[n] * g.dV);
                }
            }
    return MO_OK;
}

/* ------------------------------------------------------------------------ */
/* CellCenteredFieldCT::current (CellCenteredFieldCT.cpp:231-257): centred   */
/* curl of the cell field B (n0, n1, n2, 3); J has the same shape and is     */
/* zero on the outermost layer of each fleshed axis.                         */
/* ------------------------------------------------------------------------ */
void mo_current_cell(const double* B, int n0, int n1, int n2, double h, double* J)
{
    const int r = n0 > 1 ? 1 : 0, s = n1 > 1 ? 1 : 0, t = n2 > 1 ? 1 : 0;
#define BI(i, j, k, c) B[(((long) (i) * n1 + (j)) * n2 + (k)) * 3 + (c)]
#define JI(i, j, k, c) J[(((long) (i) * n1 + (j)) * n2 + (k)) * 3 + (c)]
    memset(J, 0, sizeof(double) * (size_t) n0 * n1 * n2 * 3);
    for (int i = 0; i < n0 - 2 * r; ++i)
        for (int j = 0; j < n1 - 2 * s; ++j)
            for (int k = 0; k < n2 - 2 * t; ++k) {
                const double d0B1 = BI(i + 2 * r, j, k, 1) - BI(i, j, k, 1);
                const double d0B2 = BI(i + 2 * r, j, k, 2) - BI(i, j, k, 2);
                const double d1B2 = BI(i, j + 2 * s, k, 2) - BI(i, j, k, 2);
                const double d1B0 = BI(i, j + 2 * s, k, 0) - BI(i, j, k, 0);
                const double d2B0 = BI(i, j, k + 2 * t, 0) - BI(i, j, k, 0);
                const double d2B1 = BI(i, j, k + 2 * t, 1) - BI(i, j, k, 1);
                JI(i + r, j + s, k + t, 0) = (d1B2 - d2B1) / h / 2;
                JI(i + r, j + s, k + t, 1) = (d2B0 - d0B2) / h / 2;
                JI(i + r, j + s, k + t, 2) = (d0B1 - d1B0) / h / 2;
            }
#undef BI
#undef JI
}

/* ------------------------------------------------------------------------ */
/* UniformCartesianCT (src/ConstrainedTransport.cpp), the reference's only   */
/* implementation of the ConstrainedTransport interface (src/Mara.hpp:341-  */
/* 349): a cell-centred field with one guard zone on every axis             */
/* (setMeshGeometry :13-76), filled by the boundary condition axis by axis  */
/* (setCellBC :400-420; periodic and outflow images, numGuard = 1).         */
/* ------------------------------------------------------------------------ */
static double* uct_guarded_b(const double* Bc, int n0, int n1, int n2, int bc)
{
    const int m0 = n0 + 2, m1 = n1 + 2, m2 = n2 + 2;
    double* B = (double*) calloc((size_t) m0 * m1 * m2 * 3, sizeof(double));
    if (!B) return NULL;
#define GB(i, j, k, c) B[(((long) (i) * m1 + (j)) * m2 + (k)) * 3 + (c)]
    for (int i = 0; i < n0; ++i)
        for (int j = 0; j < n1; ++j)
            for (int k = 0; k < n2; ++k)
                for (int c = 0; c < 3; ++c)
                    GB(i + 1, j + 1, k + 1, c) = Bc[(((long) i * n1 + j) * n2 + k) * 3 + c];
    const int n[3] = {n0, n1, n2};
    for (int axis = 0; axis < 3; ++axis) {
        /* left guard 0 and right guard n + 1 from their images: periodic
         * n and 1, outflow 1 and n */
        const int lsrc = bc == MO_BC_PERIODIC ? n[axis] : 1;
        const int rsrc = bc == MO_BC_PERIODIC ? 1 : n[axis];
        for (int a = 0; a < (axis == 0 ? 1 : m0); ++a)
            for (int b = 0; b < (axis == 1 ? 1 : m1); ++b)
                for (int e = 0; e < (axis == 2 ? 1 : m2); ++e)
                    for (int c = 0; c < 3; ++c) {
                        int gl[3] = {a, b, e}, gr[3] = {a, b, e}, sl[3] = {a, b, e}, sr[3] = {a, b, e};
                        gl[axis] = 0;
                        gr[axis] = n[axis] + 1;
                        sl[axis] = lsrc;
                        sr[axis] = rsrc;
                        GB(gl[0], gl[1], gl[2], c) = GB(sl[0], sl[1], sl[2], c);
                        GB(gr[0], gr[1], gr[2], c) = GB(sr[0], sr[1], sr[2], c);
                    }
    }
#undef GB
    return B;
}

int mo_uct_monopole(const double* Bc, int n0, int n1, int n2, int bc, int location, double* M)
{
    if (bc != MO_BC_PERIODIC && bc != MO_BC_OUTFLOW) return MO_ERR_CONFIG;
    const int m1 = n1 + 2, m2 = n2 + 2;
    const int v0 = n0 + 1, v1 = n1 + 1, v2 = n2 + 1;
    double* B = uct_guarded_b(Bc, n0, n1, n2, bc);
    double* Mv = (double*) calloc((size_t) v0 * v1 * v2, sizeof(double));
    if (!B || !Mv) { free(B); free(Mv); return MO_ERR_CONFIG; }
#define GB(i, j, k, c) B[(((long) (i) * m1 + (j)) * m2 + (k)) * 3 + (c)]
#define MV(i, j, k) Mv[((long) (i) * v1 + (j)) * v2 + (k)]
    /* computeMonopoleVert (ConstrainedTransport.cpp:302-356) */
    for (int i = 0; i < v0; ++i)
        for (int j = 0; j < v1; ++j)
            for (int k = 0; k < v2; ++k) {
                const double Bx0 = GB(i, j, k, 0) + GB(i, j, k + 1, 0) + GB(i, j + 1, k, 0) + GB(i, j + 1, k + 1, 0);
                const double Bx1 = GB(i + 1, j, k, 0) + GB(i + 1, j, k + 1, 0) + GB(i + 1, j + 1, k, 0) + GB(i + 1, j + 1, k + 1, 0);
                const double By0 = GB(i, j, k, 1) + GB(i + 1, j, k, 1) + GB(i, j, k + 1, 1) + GB(i + 1, j, k + 1, 1);
                const double By1 = GB(i, j + 1, k, 1) + GB(i + 1, j + 1, k, 1) + GB(i, j + 1, k + 1, 1) + GB(i + 1, j + 1, k + 1, 1);
                const double Bz0 = GB(i, j, k, 2) + GB(i, j + 1, k, 2) + GB(i + 1, j, k, 2) + GB(i + 1, j + 1, k, 2);
                const double Bz1 = GB(i, j, k + 1, 2) + GB(i, j + 1, k + 1, 2) + GB(i + 1, j, k + 1, 2) + GB(i + 1, j + 1, k + 1, 2);
                MV(i, j, k) = 0.25 * ((Bx1 - Bx0) + (By1 - By0) + (Bz1 - Bz0));
            }
    if (location == 0) {
        memcpy(M, Mv, sizeof(double) * (size_t) v0 * v1 * v2);
    } else {
        /* computeMonopoleCell (ConstrainedTransport.cpp:358-377) */
        for (int i = 0; i < n0; ++i)
            for (int j = 0; j < n1; ++j)
                for (int k = 0; k < n2; ++k) {
                    const double Mi = 0.5 * (MV(i, j, k) + MV(i + 1, j, k));
                    const double Mj = 0.5 * (MV(i, j, k) + MV(i, j + 1, k));
                    const double Mk = 0.5 * (MV(i, j, k) + MV(i, j, k + 1));
                    M[((long) i * n1 + j) * n2 + k] = 1. / 3 * (Mi + Mj + Mk);
                }
    }
#undef GB
#undef MV
    free(B);
    free(Mv);
    return MO_OK;
}

int mo_uct_current(const double* Bc, int n0, int n1, int n2, int bc, double h, double* J)
{
    if (bc != MO_BC_PERIODIC && bc != MO_BC_OUTFLOW) return MO_ERR_CONFIG;
    const int m0 = n0 + 2, m1 = n1 + 2, m2 = n2 + 2;
    double* B = uct_guarded_b(Bc, n0, n1, n2, bc);
    double* Jg = (double*) malloc(sizeof(double) * (size_t) m0 * m1 * m2 * 3);
    if (!B || !Jg) { free(B); free(Jg); return MO_ERR_CONFIG; }
    /* CellCenteredFieldCT::current (CellCenteredFieldCT.cpp:231-257) of the
     * guarded field, kept at the interior cells */
    mo_current_cell(B, m0, m1, m2, h, Jg);
    for (int i = 0; i < n0; ++i)
        for (int j = 0; j < n1; ++j)
            for (int k = 0; k < n2; ++k)
                for (int c = 0; c < 3; ++c)
                    J[(((long) i * n1 + j) * n2 + k) * 3 + c] = Jg[(((long) (i + 1) * m1 + (j + 1)) * m2 + (k + 1)) * 3 + c];
    free(B);
    free(Jg);
    return MO_OK;
}

/* ------------------------------------------------------------------------ */
/* The divergence-free initial field of src/Problems.cpp:660-667:           */
/* CellCenteredFieldCT::vectorPotentialToFluxes (CellCenteredFieldCT.cpp:   */
/* 136-150), generateGodunovFluxes (:152-157, flux CT with magnetic index   */
/* 0), MeshOperator::divergence with factor 1 (MeshOperator.cpp:323-381),   */
/* every cell with guards; each result times `scale`.  A has shape          */
/* (N0+1, N1+1, N2+1, 3, 3) (component, face axis); B (N0, N1, N2, 3).       */
/* ------------------------------------------------------------------------ */
int mo_vector_potential_to_cell_b_scaled(const mo_config* c, const double* A, double scale, double* B)
{
    mgeom g;
    int err = make_geom(c, &g);
    if (err) return err;
    const int f0 = g.N[0] + 1, f1 = g.N[1] + 1, f2 = g.N[2] + 1;
    const long nf = (long) f0 * f1 * f2;
    double* F = (double*) calloc((size_t) nf * 9, sizeof(double));
    if (!F) return MO_ERR_CONFIG;
#define AI(n, q, a) A[(n) * 9 + (q) * 3 + (a)]
#define FX(n, q, a) F[(n) * 9 + (q) * 3 + (a)]
    for (long n = 0; n < nf; ++n) {
        FX(n, 1, 0) = -AI(n, 2, 0);
        FX(n, 2, 0) = +AI(n, 1, 0);
        FX(n, 2, 1) = -AI(n, 0, 1);
        FX(n, 0, 1) = +AI(n, 2, 1);
        FX(n, 0, 2) = -AI(n, 1, 2);
        FX(n, 1, 2) = +AI(n, 0, 2);
    }
#undef AI
    mo_ct_correct(F, f0, f1, f2, 3, 0);
    const double factor = 1.0;
    const double vol = g.dV;
    for (int i = 0; i < g.N[0]; ++i)
        for (int j = 0; j < g.N[1]; ++j)
            for (int k = 0; k < g.N[2]; ++k) {
#define FI(i, j, k) (((long) (i) * f1 + (j)) * f2 + (k))
                for (int q = 0; q < 3; ++q)
                    B[(((long) i * g.N[1] + j) * g.N[2] + k) * 3 + q] = factor / vol * (
                        + FX(FI(i + 1, j, k), q, 0) * g.dA[0]
                        - FX(FI(i, j, k), q, 0) * g.dA[0]
                        + FX(FI(i, j + 1, k), q, 1) * g.dA[1]
                        - FX(FI(i, j, k), q, 1) * g.dA[1]
                        + FX(FI(i, j, k + 1), q, 2) * g.dA[2]
                        - FX(FI(i, j, k), q, 2) * g.dA[2]) * scale;
#undef FI
            }
#undef FX
    free(F);
    return MO_OK;
}
