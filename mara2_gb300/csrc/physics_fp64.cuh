// physics_fp64.cuh -- FP64 device physics of the plain path.
//
// Every function restates the reference routine it names with the same
// floating-point operation order, and the translation units that include
// this header are compiled with --fmad=false, so the plain path rounds
// exactly as the reference's CPU build (-ffp-contract=off) does.  Divisions
// and square roots are IEEE round-to-nearest in CUDA FP64.  The quartic's
// pow(x, 1/3), acos, cos and sin are the correctly rounded evaluations of
// crmath.cuh; the reference's libm (glibc) returns the correctly rounded
// value on all but ~0.1 % of arguments, the one place where the plain path
// may differ from the reference by a rounding.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "crmath.cuh"

namespace mara {

// LAW_MHD_COOL: NewtonianMHD with a positive cooling rate, which carries one
// auxiliary field (index 8) fed by the cooling source terms
// (ConservationLaws.cpp:355-358, 489-501)
enum { LAW_HYDRO = 0, LAW_MHD = 1, LAW_RMHD = 2, LAW_MHD_COOL = 3 };
enum { RECON_PCM = 0, RECON_PLM = 1, RECON_WENO5 = 2 };
enum { RIEMANN_HLLE = 0, RIEMANN_HLLC = 1 };
enum { BC_PERIODIC = 0, BC_OUTFLOW = 1, BC_REFLECTING = 2 };
enum { WENO_JS96 = 0, WENO_BORGES08 = 1, WENO_SHENZHA10 = 2 };

enum {
    ST_OK = 0,
    ST_C2P_CONS_CONTAINS_NAN = 1,
    ST_C2P_CONS_NEGATIVE_DENSITY = 2,
    ST_C2P_CONS_NEGATIVE_ENERGY = 3,
    ST_C2P_PRIM_CONTAINS_NAN = 4,
    ST_C2P_PRIM_NEGATIVE_PRESSURE = 5,
    ST_C2P_PRIM_NEGATIVE_RESTMASS = 6,
    ST_C2P_PRIM_SUPERLUMINAL = 7,
    ST_C2P_MAXITER = 8,
    ST_INVERSION_FAILURE = 16,
    ST_SUPERLUMINAL = 17,
    ST_BAD_EIGENVALUES = 18,
};

template <int LAW> struct LawInfo;
template <> struct LawInfo<LAW_HYDRO> { static constexpr int NQ = 5; };
template <> struct LawInfo<LAW_MHD> { static constexpr int NQ = 8; };
template <> struct LawInfo<LAW_RMHD> { static constexpr int NQ = 8; };
template <> struct LawInfo<LAW_MHD_COOL> { static constexpr int NQ = 9; };

// Physics parameters shared by every kernel of a handle.
struct PhysParams {
    double gamma;
    double plm_theta;
    double shenzha_A;
    double pressure_floor;
    int weno_is;
    double cooling_rate;  // NewtonianMHD::setCoolingRate (LAW_MHD_COOL)
};

// A ConservationLaw::State restricted to the law's NQ fields; the reference's
// remaining slots up to MARA_NUM_FIELDS = 10 hold zeros, which the Riemann
// solvers' max/min over all slots still see (see slot_max below).
template <int NQ> struct StateD {
    double P[NQ], U[NQ], F[NQ], A[NQ];
};

// IEEE comparison of doubles done on their bit patterns (integer pipe): the
// FP64 pipe of this GPU runs at 1/64 of the FP32 rate and a compare takes a
// slot there like a multiply.  Mapping a double to sign ? -|bits| : |bits|
// orders every non-NaN value, with -0 and +0 equal; a NaN operand makes the
// comparison false, as in IEEE arithmetic.  (Measured: it pays in the
// Courant reduction and in minmod, not in the Riemann solvers' slot max/min.)
__device__ __forceinline__ long long dkey(long long b)
{
    const long long m = b & 0x7fffffffffffffffll;
    return b < 0 ? -m : m;
}

__device__ __forceinline__ bool dnan(long long b) { return (b & 0x7fffffffffffffffll) > 0x7ff0000000000000ll; }

__device__ __forceinline__ bool dlt(double a, double b)  // a < b
{
    const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
    return !dnan(x) && !dnan(y) && dkey(x) < dkey(y);
}

__device__ __forceinline__ double dmin2(double a, double b) { return a < b ? a : b; }
__device__ __forceinline__ double dmax2(double a, double b) { return a > b ? a : b; }
__device__ __forceinline__ double dmin3(double a, double b, double c) { return a < b ? dmin2(a, c) : dmin2(b, c); }
__device__ __forceinline__ double dmax3(double a, double b, double c) { return a > b ? dmax2(a, c) : dmax2(b, c); }

// ---------------------------------------------------------------------------
// NewtonianHydro::fromPrimitive (ConservationLaws.cpp:253-290)
__device__ __forceinline__ void hydro_prim(const PhysParams& pp, const double* P, const double* n, StateD<5>& S)
{
    const double gm0 = pp.gamma;
    const double gm1 = pp.gamma - 1.0;
    const double cs = sqrt(gm0 * P[4] / P[0]);
    const double vv = P[1] * P[1] + P[2] * P[2] + P[3] * P[3];
    const double vn = P[1] * n[0] + P[2] * n[1] + P[3] * n[2];
#pragma unroll
    for (int q = 0; q < 5; ++q) S.P[q] = P[q];
    S.U[0] = P[0];
    S.U[1] = P[0] * P[1];
    S.U[2] = P[0] * P[2];
    S.U[3] = P[0] * P[3];
    S.U[4] = P[0] * 0.5 * vv + P[4] / gm1;
    S.F[0] = vn * S.U[0];
    S.F[1] = vn * S.U[1] + P[4] * n[0];
    S.F[2] = vn * S.U[2] + P[4] * n[1];
    S.F[3] = vn * S.U[3] + P[4] * n[2];
    S.F[4] = vn * S.U[4] + P[4] * vn;
    S.A[0] = vn - cs;
    S.A[1] = vn;
    S.A[2] = vn;
    S.A[3] = vn;
    S.A[4] = vn + cs;
}

// conserved densities of NewtonianHydro::fromPrimitive only
__device__ __forceinline__ void hydro_p2u(const PhysParams& pp, const double* P, double* U)
{
    const double gm1 = pp.gamma - 1.0;
    const double vv = P[1] * P[1] + P[2] * P[2] + P[3] * P[3];
    U[0] = P[0];
    U[1] = P[0] * P[1];
    U[2] = P[0] * P[2];
    U[3] = P[0] * P[3];
    U[4] = P[0] * 0.5 * vv + P[4] / gm1;
}

// NewtonianHydro::fromConserved (ConservationLaws.cpp:238-251)
__device__ __forceinline__ int hydro_cons(const PhysParams& pp, const double* U, double* P)
{
    const double gm1 = pp.gamma - 1.0;
    const double p2 = U[1] * U[1] + U[2] * U[2] + U[3] * U[3];
    P[0] = U[0];
    P[4] = (U[4] - 0.5 * p2 / U[0]) * gm1;
    P[1] = U[1] / U[0];
    P[2] = U[2] / U[0];
    P[3] = U[3] / U[0];
    return ST_OK;
}

// ---------------------------------------------------------------------------
// NewtonianMHD::fromPrimitive (ConservationLaws.cpp:416-487)
template <int NQ>
__device__ __forceinline__ void mhd_prim(const PhysParams& pp, const double* P, const double* n, StateD<NQ>& S)
{
    const double gm0 = pp.gamma;
    const double gm1 = pp.gamma - 1.0;
    const double cs2 = gm0 * P[4] / P[0];
    const double vv = P[1] * P[1] + P[2] * P[2] + P[3] * P[3];
    const double BB = P[5] * P[5] + P[6] * P[6] + P[7] * P[7];
    const double Bv = P[5] * P[1] + P[6] * P[2] + P[7] * P[3];
    const double vn = P[1] * n[0] + P[2] * n[1] + P[3] * n[2];
    const double Bn = P[5] * n[0] + P[6] * n[1] + P[7] * n[2];
    const double ps = P[4] + 0.5 * BB;
#pragma unroll
    for (int q = 0; q < 8; ++q) S.P[q] = P[q];
    S.U[0] = P[0];
    S.U[1] = P[0] * P[1];
    S.U[2] = P[0] * P[2];
    S.U[3] = P[0] * P[3];
    S.U[4] = P[0] * 0.5 * vv + 0.5 * BB + P[4] / gm1;
    S.U[5] = P[5];
    S.U[6] = P[6];
    S.U[7] = P[7];
    S.F[0] = vn * S.U[0];
    S.F[1] = vn * S.U[1] - Bn * P[5] + ps * n[0];
    S.F[2] = vn * S.U[2] - Bn * P[6] + ps * n[1];
    S.F[3] = vn * S.U[3] - Bn * P[7] + ps * n[2];
    S.F[4] = vn * S.U[4] - Bn * Bv + ps * vn;
    S.F[5] = vn * S.U[5] - Bn * P[1];
    S.F[6] = vn * S.U[6] - Bn * P[2];
    S.F[7] = vn * S.U[7] - Bn * P[3];
    const double Bn2 = Bn * Bn;
    const double ca2 = BB / P[0];
    const double cn2 = Bn2 / P[0];
    const double cw4 = (cs2 + ca2) * (cs2 + ca2);
    const double cF2 = 0.5 * (cs2 + ca2 + sqrt(cw4 - 4 * cs2 * cn2));
    const double cS2 = 0.5 * (cs2 + ca2 - sqrt(cw4 - 4 * cs2 * cn2));
    S.A[0] = vn - sqrt(cF2);
    S.A[1] = vn - sqrt(cn2);
    S.A[2] = vn - sqrt(cS2);
    S.A[3] = vn;
    S.A[4] = vn;
    S.A[5] = vn + sqrt(cS2);
    S.A[6] = vn + sqrt(cn2);
    S.A[7] = vn + sqrt(cF2);
    // auxiliary fields: carried, no flux, zero eigenvalue (:479-485)
#pragma unroll
    for (int q = 8; q < NQ; ++q) {
        S.P[q] = P[q];
        S.U[q] = P[q];
        S.F[q] = 0.0;
        S.A[q] = 0.0;
    }
}

template <int NQ>
__device__ __forceinline__ void mhd_p2u(const PhysParams& pp, const double* P, double* U)
{
    const double gm1 = pp.gamma - 1.0;
    const double vv = P[1] * P[1] + P[2] * P[2] + P[3] * P[3];
    const double BB = P[5] * P[5] + P[6] * P[6] + P[7] * P[7];
    U[0] = P[0];
    U[1] = P[0] * P[1];
    U[2] = P[0] * P[2];
    U[3] = P[0] * P[3];
    U[4] = P[0] * 0.5 * vv + 0.5 * BB + P[4] / gm1;
    U[5] = P[5];
    U[6] = P[6];
    U[7] = P[7];
#pragma unroll
    for (int q = 8; q < NQ; ++q) U[q] = P[q];
}

// NewtonianMHD::fromConserved with bad-state detection and the optional
// pressure floor (ConservationLaws.cpp:370-414)
template <int NQ>
__device__ __forceinline__ int mhd_cons(const PhysParams& pp, const double* U, double* P)
{
    const double gm1 = pp.gamma - 1.0;
    const double p2 = U[1] * U[1] + U[2] * U[2] + U[3] * U[3];
    const double BB = U[5] * U[5] + U[6] * U[6] + U[7] * U[7];
    P[0] = U[0];
    P[4] = (U[4] - 0.5 * p2 / U[0] - 0.5 * BB) * gm1;
    P[1] = U[1] / U[0];
    P[2] = U[2] / U[0];
    P[3] = U[3] / U[0];
    P[5] = U[5];
    P[6] = U[6];
    P[7] = U[7];
#pragma unroll
    for (int q = 8; q < NQ; ++q) P[q] = U[q];
    if (P[4] < 0.0 || P[0] < 0.0 || U[0] < 0.0 || U[4] < 0.0) {
        if (P[4] < 0.0 && pp.pressure_floor > 0.0) {
            P[4] = pp.pressure_floor * P[0];
            return ST_OK;
        }
        return ST_INVERSION_FAILURE;
    }
    return ST_OK;
}

// ---------------------------------------------------------------------------
// QuarticPolynomial::solve and its resolvent cubic (QuarticPolynomial.cpp:
// 19-144)
__device__ __forceinline__ void solve_cubic(double c3, double c2, double c1, double c0,
                                            double& x1, double& x2, double& x3, int& nr)
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
        s1 = (s1 >= 0.0) ? crm::pow_third(s1) : -crm::pow_third(-s1);
        s2 = (s2 >= 0.0) ? crm::pow_third(s2) : -crm::pow_third(-s2);
        x1 = (s1 + s2) - a2 / 3.0;
        x2 = x3 = -0.5 * (s1 + s2) - a2 / 3.0;
        nr = 1;
    } else if (delta < 0.0) {
        const double theta = crm::acos_cr(r / sqrt(-q * q * q)) / 3.0;
        const double costh = crm::cos_cr(theta);
        const double sinth = crm::sin_cr(theta);
        const double sq = sqrt(-q);
        const double rt3 = 1.7320508075688772; // sqrt(3), correctly rounded
        x1 = 2.0 * sq * costh - a2 / 3.0;
        x2 = -sq * costh - a2 / 3.0 - rt3 * sq * sinth;
        x3 = -sq * costh - a2 / 3.0 + rt3 * sq * sinth;
        nr = 3;
    } else {
        const double s = (r >= 0.0) ? crm::pow_third(r) : -crm::pow_third(-r);
        x1 = 2.0 * s - a2 / 3.0;
        x2 = x3 = -s - a2 / 3.0;
        nr = 3;
    }
}

__device__ __forceinline__ int quartic_roots(double d4, double d3, double d2, double d1, double d0, double roots[4])
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

    solve_cubic(1.0, au2, au1, au0, x1, x2, x3, nr);
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
    int m = 0;
    if (nr12 != 0) { roots[m++] = r1; roots[m++] = r2; }
    if (nr34 != 0) { roots[m++] = r3; roots[m++] = r4; }
    // ascending insertion sort
    for (int a = 1; a < m; ++a) {
        const double v = roots[a];
        int b = a - 1;
        while (b >= 0 && v < roots[b]) { roots[b + 1] = roots[b]; --b; }
        roots[b + 1] = v;
    }
    return nr12 + nr34;
}

// ---------------------------------------------------------------------------
// RelativisticMHD::fromPrimitive (ConservationLaws.cpp:659-836).  With
// EIGEN false only P, U, F are produced (the superluminal check stays).
template <bool EIGEN>
__device__ __forceinline__ int rmhd_prim(const PhysParams& pp, const double* P, const double* n, StateD<8>& S)
{
    const double gm0 = pp.gamma;
    const double gm1 = pp.gamma - 1.0;
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

    if (vv >= 1) return ST_SUPERLUMINAL;

#pragma unroll
    for (int q = 0; q < 8; ++q) S.P[q] = P[q];
    S.U[0] = P[0] * W0;
    S.U[4] = P[0] * hs * W2 - ps - b0 * b0 - S.U[0];
    S.U[1] = P[0] * hs * W2 * P[1] - b0 * b1;
    S.U[2] = P[0] * hs * W2 * P[2] - b0 * b2;
    S.U[3] = P[0] * hs * W2 * P[3] - b0 * b3;
    S.U[5] = P[5];
    S.U[6] = P[6];
    S.U[7] = P[7];
    S.F[0] = vn * S.U[0];
    S.F[1] = vn * S.U[1] - Bn * b1 / W0 + ps * n[0];
    S.F[2] = vn * S.U[2] - Bn * b2 / W0 + ps * n[1];
    S.F[3] = vn * S.U[3] - Bn * b3 / W0 + ps * n[2];
    S.F[4] = vn * S.U[4] - Bn * b0 / W0 + ps * vn;
    S.F[5] = vn * S.U[5] - Bn * P[1];
    S.F[6] = vn * S.U[6] - Bn * P[2];
    S.F[7] = vn * S.U[7] - Bn * P[3];
    if (!EIGEN) return ST_OK;

    const double cs2 = gm0 * p0 / (P[0] * h0);
    const double W4 = W2 * W2;
    const double v2 = vn * vn;
    const double v3 = vn * v2;
    const double v4 = vn * v3;

    if (BB == 0.0) {
        const double K = sqrt(cs2 * (1 - vv) * (1 - vv * cs2 - v2 * (1 - cs2)));
        S.A[0] = (vn * (1 - cs2) - K) / (1 - vv * cs2);
        S.A[1] = vn;
        S.A[2] = vn;
        S.A[3] = vn;
        S.A[4] = vn;
        S.A[5] = vn;
        S.A[6] = vn;
        S.A[7] = (vn * (1 - cs2) + K) / (1 - vv * cs2);
        return ST_OK;
    }
    const double K = W4 * (P[0] * h0 * (1. / cs2 - 1.));
    const double L = -W2 * (P[0] * h0 + bb / cs2);
    const double A4 = K - L - b0 * b0;
    const double A3 = -4 * K * vn + L * vn * 2 + 2 * b0 * bn;
    const double A2 = 6 * K * v2 + L * (1. - v2) + b0 * b0 - bn * bn;
    const double A1 = -4 * K * v3 - L * vn * 2 - 2 * b0 * bn;
    const double A0 = K * v4 + L * v2 + bn * bn;
    double roots[4] = {0, 0, 0, 0};
    const int nr = quartic_roots(A4, A3, A2, A1, A0, roots);
    const double C = sqrt(h0 + bb);

    if (nr == 4) {
        S.A[0] = roots[0];
        S.A[1] = (bn - C * vn * W0) / (b0 - C * W0);
        S.A[2] = roots[1];
        S.A[3] = vn;
        S.A[4] = vn;
        S.A[5] = roots[2];
        S.A[6] = (bn + C * vn * W0) / (b0 + C * W0);
        S.A[7] = roots[3];
    } else if (nr == 2) {
        S.A[0] = roots[0];
        S.A[1] = (bn - C * vn * W0) / (b0 - C * W0);
        S.A[2] = vn;
        S.A[3] = vn;
        S.A[4] = vn;
        S.A[5] = vn;
        S.A[6] = (bn + C * vn * W0) / (b0 + C * W0);
        S.A[7] = roots[1];
    } else {
        return ST_BAD_EIGENVALUES;
    }
    return ST_OK;
}

// ---------------------------------------------------------------------------
// ConsToPrimRMHD (ConsToPrimRMHD.cpp:77-323): Anton et al. (2006) 2-D Newton
// in (Z, W), then Noble et al. (2006) 1-D Newton in Z.  Both loops are
// bounded by 250 iterations; a NaN error ends the loop as in the reference.
struct C2pRmhd {
    double gamf, pfloor;
    double D, Tau, S2, B2, BS, BS2, Cons[8];
    double Z_start, W_start;
};

__device__ __forceinline__ int rm_check_cons(const double* U)
{
    if (U[0] < 0.0) return ST_C2P_CONS_NEGATIVE_DENSITY;
    if (U[4] < 0.0) return ST_C2P_CONS_NEGATIVE_ENERGY;
    for (int i = 0; i < 8; ++i)
        if (!isfinite(U[i])) return ST_C2P_CONS_CONTAINS_NAN;
    return ST_OK;
}

__device__ __forceinline__ int rm_check_prim(const double* P)
{
    const double v2 = P[1] * P[1] + P[2] * P[2] + P[3] * P[3];
    if (v2 >= 1.0) return ST_C2P_PRIM_SUPERLUMINAL;
    if (P[4] < 0.0) return ST_C2P_PRIM_NEGATIVE_PRESSURE;
    if (P[0] < 0.0) return ST_C2P_PRIM_NEGATIVE_RESTMASS;
    for (int i = 0; i < 8; ++i)
        if (!isfinite(P[i])) return ST_C2P_PRIM_CONTAINS_NAN;
    return ST_OK;
}

__device__ __forceinline__ int rm_reconstruct(const C2pRmhd& s, double Z, double W, double* Pout)
{
    double P[8];
    const double b0 = s.BS * W / Z;
    P[0] = s.D / W;
    P[4] = (s.D / W) * (Z / (s.D * W) - 1.0) * s.gamf;
    P[1] = (s.Cons[1] + b0 * s.Cons[5] / W) / (Z + s.B2);
    P[2] = (s.Cons[2] + b0 * s.Cons[6] / W) / (Z + s.B2);
    P[3] = (s.Cons[3] + b0 * s.Cons[7] / W) / (Z + s.B2);
    P[5] = s.Cons[5];
    P[6] = s.Cons[6];
    P[7] = s.Cons[7];
    if (P[4] <= 0.0 && s.pfloor > 0.0) P[4] = P[0] * s.pfloor;
    const int err = rm_check_prim(P);
    if (err) return err;
#pragma unroll
    for (int q = 0; q < 8; ++q) Pout[q] = P[q];
    return ST_OK;
}

__device__ __forceinline__ int rm_anton2dzw(const C2pRmhd& s, double* P)
{
    const int bad = rm_check_cons(s.Cons);
    if (bad) return bad;
    int it = 0;
    double error = 1.0, W = s.W_start, Z = s.Z_start;
    const double D = s.D, Tau = s.Tau, S2 = s.S2, B2 = s.B2, BS2 = s.BS2, gamf = s.gamf;
    while (error > 1e-12) {
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
        const double det = df0dZ * df1dW - df0dW * df1dZ;
        const double G0 = df1dW / det, G1 = -df0dW / det, G2 = -df1dZ / det, G3 = df0dZ / det;
        const double dZ = -(G0 * f0 + G1 * f1);
        const double dW = -(G2 * f0 + G3 * f1);
        double Z_new = Z + dZ;
        double W_new = W + dW;
        Z_new = (Z_new > 0.0) ? Z_new : -Z_new;
        Z_new = (Z_new < 1e20) ? Z_new : Z;
        W_new = (W_new > 1.0) ? W_new : 1.0;
        W_new = (W_new < 1e12) ? W_new : 1e12;
        Z = Z_new;
        W = W_new;
        error = fabs(dZ / Z) + fabs(dW / W);
        ++it;
        if (it == 250) return ST_C2P_MAXITER;
    }
    return rm_reconstruct(s, Z, W, P);
}

__device__ __forceinline__ int rm_noble1dw(const C2pRmhd& s, double* P)
{
    const int bad = rm_check_cons(s.Cons);
    if (bad) return bad;
    int it = 0;
    double error = 1.0, Z = s.Z_start;
    const double D = s.D, Tau = s.Tau, S2 = s.S2, B2 = s.B2, BS2 = s.BS2, gamf = s.gamf;
    while (error > 1e-12) {
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
        Z_new = (Z_new > 0.0) ? Z_new : -Z_new;
        Z_new = (Z_new < 1e20) ? Z_new : Z;
        Z = Z_new;
        error = fabs(dZ / Z);
        ++it;
        if (it == 250) return ST_C2P_MAXITER;
    }
    const double Z2 = Z * Z;
    const double a = S2 * Z2 + BS2 * (B2 + 2 * Z);
    const double b = (B2 + Z) * (B2 + Z) * Z2;
    const double V2 = a / b;
    const double W2 = 1.0 / (1.0 - V2);
    const double W = sqrt(W2);
    return rm_reconstruct(s, Z, W, P);
}

// RelativisticMHD::fromConserved (ConservationLaws.cpp:627-657).  *code gets
// the Newton failure status when both solvers fail; the eigenvalue check of
// the reference's closing fromPrimitive call is kept (it can raise "bad
// eigenvalues").
__device__ __forceinline__ int rmhd_cons(const PhysParams& pp, const double* U, double* P, int* code)
{
    C2pRmhd s;
    s.gamf = (pp.gamma - 1.0) / pp.gamma;
    s.pfloor = pp.pressure_floor;
    s.D = U[0];
    s.Tau = U[4];
    s.S2 = U[1] * U[1] + U[2] * U[2] + U[3] * U[3];
    s.B2 = U[5] * U[5] + U[6] * U[6] + U[7] * U[7];
    s.BS = U[5] * U[1] + U[6] * U[2] + U[7] * U[3];
    s.BS2 = s.BS * s.BS;
#pragma unroll
    for (int q = 0; q < 8; ++q) s.Cons[q] = U[q];
    s.Z_start = sqrt(s.S2 + s.D * s.D);
    s.W_start = s.Z_start / s.D;
    double Q[8];
    int err = rm_anton2dzw(s, Q);
    if (err != ST_OK) err = rm_noble1dw(s, Q);
    if (err != ST_OK) { *code = err; return ST_INVERSION_FAILURE; }
    {
        const double xhat[3] = {1.0, 0.0, 0.0};
        StateD<8> S;
        const int e2 = rmhd_prim<true>(pp, Q, xhat, S);
        if (e2 != ST_OK) return e2;
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) P[q] = Q[q];
    return ST_OK;
}

// ---------------------------------------------------------------------------
// law dispatch
template <int LAW, bool EIGEN = true>
__device__ __forceinline__ int law_prim(const PhysParams& pp, const double* P, const double* n,
                                        StateD<LawInfo<LAW>::NQ>& S)
{
    if constexpr (LAW == LAW_HYDRO) { hydro_prim(pp, P, n, S); return ST_OK; }
    else if constexpr (LAW == LAW_MHD || LAW == LAW_MHD_COOL) { mhd_prim<LawInfo<LAW>::NQ>(pp, P, n, S); return ST_OK; }
    else { return rmhd_prim<EIGEN>(pp, P, n, S); }
}

template <int LAW>
__device__ __forceinline__ int law_p2u(const PhysParams& pp, const double* P, double* U)
{
    if constexpr (LAW == LAW_HYDRO) { hydro_p2u(pp, P, U); return ST_OK; }
    else if constexpr (LAW == LAW_MHD || LAW == LAW_MHD_COOL) { mhd_p2u<LawInfo<LAW>::NQ>(pp, P, U); return ST_OK; }
    else {
        // FieldOperator::generateConserved calls the full fromPrimitive, whose
        // eigenvalue evaluation can raise "bad eigenvalues"
        const double xhat[3] = {1.0, 0.0, 0.0};
        StateD<8> S;
        const int e = rmhd_prim<true>(pp, P, xhat, S);
#pragma unroll
        for (int q = 0; q < 8; ++q) U[q] = S.U[q];
        return e;
    }
}

template <int LAW>
__device__ __forceinline__ int law_cons(const PhysParams& pp, const double* U, double* P, int* code)
{
    if constexpr (LAW == LAW_HYDRO) return hydro_cons(pp, U, P);
    else if constexpr (LAW == LAW_MHD || LAW == LAW_MHD_COOL) {
        const int e = mhd_cons<LawInfo<LAW>::NQ>(pp, U, P);
        *code = e;
        return e;
    }
    else return rmhd_cons(pp, U, P, code);
}

// ---------------------------------------------------------------------------
// Reconstruction (Reconstruction.cpp:55-169)
__device__ __forceinline__ int dsgn(double x) { return (x > 0) - (x < 0); }

// The sign tests, MIN3 and the small factor 0.25 |SGN(a) + SGN(b)| (SGN(a) +
// SGN(c)) of the generalised minmod are done on the bit patterns, so that
// only the arithmetic reaches the FP64 pipe (a compare costs as much there as
// a multiply); the results are the reference's bit for bit:
//  * SGN(x) = (x > 0) - (x < 0) is 0 for +-0 and NaN;
//  * for |x|, |y| (sign bit clear) x < y is false when either is NaN and is
//    otherwise the order of the bit patterns;
//  * with s = SGN(a) + SGN(b) and t = SGN(a) + SGN(c) in -2..2, the product
//    (0.25 |s|) t is exactly 0, 0.25, 0.5 or 1 in magnitude (0.25 |s| |t|)
//    and carries the sign bit exactly when t < 0 (a zero times a negative t
//    is -0), so its bits are assembled directly; the last factor, times
//    MIN3, is the reference's multiply on the same operands.
__device__ __forceinline__ int bsgn(long long b)
{
    const long long m = b & 0x7fffffffffffffffll;
    return (m == 0 || m > 0x7ff0000000000000ll) ? 0 : (b < 0 ? -1 : 1);
}

__device__ __forceinline__ double minmod(double theta, double ul, double u0, double ur)
{
    const double a = theta * (u0 - ul);
    const double b = 0.5 * (ur - ul);
    const double c = theta * (ur - u0);
    const long long ba = __double_as_longlong(a), bb = __double_as_longlong(b), bc = __double_as_longlong(c);
    const int sa = bsgn(ba), sb = bsgn(bb), sc = bsgn(bc);
    const int s = sa + sb, t = sa + sc;
    const int p = (s < 0 ? -s : s) * (t < 0 ? -t : t);  // 0, 1, 2 or 4
    const long long mag = p == 0 ? 0ll : p == 1 ? 0x3fd0000000000000ll : p == 2 ? 0x3fe0000000000000ll
                                                                        : 0x3ff0000000000000ll;
    const double k = __longlong_as_double(mag | (t < 0 ? (long long) 0x8000000000000000ull : 0ll));
    // MIN3(|a|, |b|, |c|) = |a| < |b| ? MIN2(|a|, |c|) : MIN2(|b|, |c|)
    const long long INF = 0x7ff0000000000000ll;
    const long long xa = ba & 0x7fffffffffffffffll, xb = bb & 0x7fffffffffffffffll, xc = bc & 0x7fffffffffffffffll;
    auto lt = [INF](long long x, long long y) { return x < y && y <= INF; };
    const long long m = lt(xa, xb) ? (lt(xa, xc) ? xa : xc) : (lt(xb, xc) ? xb : xc);
    return k * __longlong_as_double(m);
}

#define MARA_SQU(x) ((x) * (x))

// WENO5 point-value reconstruction at the right (RIGHT = true, tables C2R)
// or left cell edge (tables C2L) of the centre value v[0] (Jiang & Shu 1996).
template <bool RIGHT>
__device__ __forceinline__ double weno5(const double* v, int mode, double Ash)
{
    const double c00 = RIGHT ? 1. / 3. : 11. / 6., c01 = RIGHT ? 5. / 6. : -7. / 6., c02 = RIGHT ? -1. / 6. : 1. / 3.;
    const double c10 = RIGHT ? -1. / 6. : 1. / 3., c11 = 5. / 6., c12 = RIGHT ? 1. / 3. : -1. / 6.;
    const double c20 = RIGHT ? 1. / 3. : -1. / 6., c21 = RIGHT ? -7. / 6. : 5. / 6., c22 = RIGHT ? 11. / 6. : 1. / 3.;
    const double d0 = RIGHT ? 0.3 : 0.1, d1 = 0.6, d2 = RIGHT ? 0.1 : 0.3;
    const double vs0 = c00 * v[+0] + c01 * v[+1] + c02 * v[2];
    const double vs1 = c10 * v[-1] + c11 * v[+0] + c12 * v[1];
    const double vs2 = c20 * v[-2] + c21 * v[-1] + c22 * v[0];
    double B0 = (13. / 12.) * MARA_SQU(1 * v[+0] - 2 * v[+1] + 1 * v[+2]) + (1. / 4.) * MARA_SQU(3 * v[+0] - 4 * v[+1] + 1 * v[+2]);
    double B1 = (13. / 12.) * MARA_SQU(1 * v[-1] - 2 * v[+0] + 1 * v[+1]) + (1. / 4.) * MARA_SQU(1 * v[-1] - 0 * v[+0] - 1 * v[+1]);
    double B2 = (13. / 12.) * MARA_SQU(1 * v[-2] - 2 * v[-1] + 1 * v[+0]) + (1. / 4.) * MARA_SQU(1 * v[-2] - 4 * v[-1] + 3 * v[+0]);
    double w0, w1, w2;
    if (mode == WENO_BORGES08) {
        const double eps = 1e-14;
        const double tau5 = fabs(B0 - B2);
        w0 = d0 * (1.0 + (tau5 / (B0 + eps)));
        w1 = d1 * (1.0 + (tau5 / (B1 + eps)));
        w2 = d2 * (1.0 + (tau5 / (B2 + eps)));
    } else if (mode == WENO_SHENZHA10) {
        const double ep = 1e-10;
        const double minB = dmin3(B0, B1, B2);
        const double maxB = dmax3(B0, B1, B2);
        const double R0 = minB / (maxB + ep);
        B0 = R0 * Ash * minB + B0;
        B1 = R0 * Ash * minB + B1;
        B2 = R0 * Ash * minB + B2;
        w0 = d0 / MARA_SQU(ep + B0);
        w1 = d1 / MARA_SQU(ep + B1);
        w2 = d2 / MARA_SQU(ep + B2);
    } else {
        const double ep = 1e-6;
        w0 = d0 / MARA_SQU(ep + B0);
        w1 = d1 / MARA_SQU(ep + B1);
        w2 = d2 / MARA_SQU(ep + B2);
    }
    const double wtot = w0 + w1 + w2;
    return (w0 * vs0 + w1 * vs1 + w2 * vs2) / wtot;
}

// ---------------------------------------------------------------------------
// Riemann solvers (RiemannSolvers.cpp:38-118).  The max/min run over the
// law's NQ slots and then over the zero slots up to MARA_NUM_FIELDS.
template <int NQ>
__device__ __forceinline__ double slot_max(const double* A)
{
    double m = A[0];
#pragma unroll
    for (int n = 1; n < NQ; ++n) if (m < A[n]) m = A[n];
    if (NQ < 10) { if (m < 0.0) m = 0.0; }
    return m;
}

template <int NQ>
__device__ __forceinline__ double slot_min(const double* A)
{
    double m = A[0];
#pragma unroll
    for (int n = 1; n < NQ; ++n) if (A[n] < m) m = A[n];
    if (NQ < 10) { if (0.0 < m) m = 0.0; }
    return m;
}

template <int NQ>
__device__ __forceinline__ void hlle(const StateD<NQ>& L, const StateD<NQ>& R, double* F)
{
    const double epl = slot_max<NQ>(L.A), eml = slot_min<NQ>(L.A);
    const double epr = slot_max<NQ>(R.A), emr = slot_min<NQ>(R.A);
    const double ap = dmax3(0.0, epl, epr);
    const double am = dmin3(0.0, eml, emr);
#pragma unroll
    for (int q = 0; q < NQ; ++q)
        F[q] = (ap * L.F[q] - am * R.F[q] + ap * am * (R.U[q] - L.U[q])) / (ap - am);
}

template <int NQ>
__device__ __forceinline__ void hllc(const StateD<NQ>& L, const StateD<NQ>& R, const double* dA, double* F)
{
    const double epl = slot_max<NQ>(L.A), eml = slot_min<NQ>(L.A);
    const double epr = slot_max<NQ>(R.A), emr = slot_min<NQ>(R.A);
    const double ap = dmax3(0.0, epl, epr);
    const double am = dmin3(0.0, eml, emr);
    const double* Pl = L.P;
    const double* Pr = R.P;
    const double* Ul = L.U;
    const double* Ur = R.U;
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
#pragma unroll
    for (int q = 0; q < NQ; ++q) F[q] = 0.0;
    if (s <= am) {
#pragma unroll
        for (int i = 0; i < 5; ++i) F[i] = L.F[i];
    } else if (am < s && s <= lc) {
#pragma unroll
        for (int i = 0; i < 5; ++i) F[i] = L.F[i] + am * (Uls[i] - Ul[i]);
    } else if (lc < s && s <= ap) {
#pragma unroll
        for (int i = 0; i < 5; ++i) F[i] = R.F[i] + ap * (Urs[i] - Ur[i]);
    } else if (ap < s) {
#pragma unroll
        for (int i = 0; i < 5; ++i) F[i] = R.F[i];
    }
}

// ConservationLaw::maxEigenvalueMagnitude (ConservationLaws.cpp:114-127)
template <int NQ>
__device__ __forceinline__ double max_eigen_magnitude(const double* A)
{
    double m = 0.0;
#pragma unroll
    for (int n = 0; n < NQ; ++n)
        if (dlt(m, fabs(A[n]))) m = fabs(A[n]);
    return m;
}

// image number idx of interior coordinate ii on one axis, or false where
// there is none: 0 is the zone's own cell, then the guard cells that hold its
// image (periodic: the copy across the grid; outflow: the whole guard layer
// beside an edge zone; reflecting: the mirror cell, whose normal momentum
// flips), as BoundaryCondition::applySimple fills them
__device__ __forceinline__ bool guard_image(int idx, int ii, int n, int g, int bc, int& o, int& f)
{
    f = 0;
    if (idx == 0) { o = ii + g; return true; }
    if (g == 0) return false;
    int c = 1;
    if (bc == BC_PERIODIC) {
        if (ii < g) { if (idx == c) { o = ii + g + n; return true; } ++c; }
        if (ii >= n - g) { if (idx == c) { o = ii + g - n; return true; } ++c; }
    } else if (bc == BC_OUTFLOW) {
        if (ii == 0)
            for (int m = 0; m < g; ++m) { if (idx == c) { o = m; return true; } ++c; }
        if (ii == n - 1)
            for (int m = 0; m < g; ++m) { if (idx == c) { o = n + g + m; return true; } ++c; }
    } else {
        if (ii < g) { if (idx == c) { o = g - 1 - ii; f = 1; return true; } ++c; }
        if (ii >= n - g) { if (idx == c) { o = 2 * n + g - 1 - ii; f = 1; return true; } ++c; }
    }
    return false;
}

} // namespace mara
