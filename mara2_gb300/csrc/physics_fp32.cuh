// physics_fp32.cuh -- device physics of the mixed-precision path.
//
// Reconstruction, equation-of-state, flux, eigenvalue and Riemann arithmetic
// run in FP32 (mixed.cu is compiled with approximate FP32 division and
// square root and flush-to-zero); the conserved-state accumulator is an
// unevaluated FP32 pair (hi + lo, about 48 significant bits) updated with
// error-free transformations (Knuth's TwoSum, FMA-based TwoProd; pair
// arithmetic after Dekker 1971 and the double-double library of Hida, Li and
// Bailey); the relativistic primitive recovery forms its Newton residuals in
// that pair arithmetic and falls back to FP64 (the plain path's routines)
// where the pair iteration cannot finish.  The formulas are those of the reference
// routines named beside each function; only the operation order and the
// precision differ.
#pragma once

#include <cuda_runtime.h>

#include "physics_fp64.cuh"

namespace mara {

// ---------------------------------------------------------------------------
// FP32-pair ("double-float") arithmetic
struct df {
    float hi, lo;
};

// every operation explicitly rounded: no multiply-add contraction can break
// the error-free transformations, and every kernel computes the same bits
__device__ __forceinline__ df two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

__device__ __forceinline__ df fast_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float e = __fsub_rn(b, __fsub_rn(s, a));
    return {s, e};
}

__device__ __forceinline__ df df_add_f(df a, float b)
{
    df s = two_sum(a.hi, b);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}

__device__ __forceinline__ df df_add(df a, df b)
{
    df s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ df df_mul_f(df a, float b)
{
    const float p = __fmul_rn(a.hi, b);
    float e = __fmaf_rn(a.hi, b, -p);
    e = __fmaf_rn(a.lo, b, e);
    return fast_two_sum(p, e);
}

// hardware approximations (about one unit in the last place), the seeds of
// the pair reciprocal and square root below
__device__ __forceinline__ float rcp_approx(float a)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
}

__device__ __forceinline__ float sqrt_approx(float a)
{
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
}

// exact product of two floats as a pair (FMA-based TwoProd)
__device__ __forceinline__ df two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}

// pair x pair (Dekker's product with FMA; about 2^-47 relative)
__device__ __forceinline__ df df_mul(df a, df b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}

__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
// multiplication by a power of two: exact on both words
__device__ __forceinline__ df df_pow2(df a, float p) { return {__fmul_rn(a.hi, p), __fmul_rn(a.lo, p)}; }

// 1 / a: one Newton-Raphson step r + r (1 - a r) on the hardware seed, the
// residual 1 - a r formed from the exact pair product (1 - (a r).hi is exact
// by Sterbenz's lemma); about 2^-46 relative
__device__ __forceinline__ df df_rcp(df a)
{
    const float r = rcp_approx(a.hi);
    const df p = df_mul_f(a, r);
    const float e = __fsub_rn(__fsub_rn(1.0f, p.hi), p.lo);
    return fast_two_sum(r, __fmul_rn(r, e));
}

// sqrt(a) for a > 0: one Newton step s + (a - s^2) / (2 s) on the seed
__device__ __forceinline__ df df_sqrt(df a)
{
    const float s = sqrt_approx(a.hi);
    const df s2 = two_prod(s, s);
    const float d = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, s2.hi), s2.lo), a.lo);
    return fast_two_sum(s, __fmul_rn(d, __fmul_rn(0.5f, rcp_approx(s))));
}

// ---- FP32 <-> FP64 conversions on the integer pipes -----------------------------
// The FP64 pipe executes two operations per clock per SM on this GPU, a
// conversion like an add, and the FP64-accumulator form and the host
// boundary's FP64 <-> FP32-pair conversions convert per field and zone.
// These give, bit for bit, the conversion instructions as the FP32
// translation units compile them (-ftz=true: round to nearest even,
// subnormal inputs and results as signed zeros), from integer operations.

// float -> double, exact
__device__ __forceinline__ double f2d_exact(float f)
{
    const unsigned b = __float_as_uint(f);
    const unsigned e = (b >> 23) & 0xffu;
    const unsigned sign = b & 0x80000000u;
    const unsigned ehi = e == 0xffu ? 0x7ff00000u : (e + 896u) << 20;   // rebias 127 -> 1023
    return __hiloint2double((int) (e == 0 ? sign : sign | ehi | ((b & 0x7fffffu) >> 3)), (int) (e == 0 ? 0u : b << 29));
}

// double -> float, round to nearest even; below 2^-126 to signed zero, above
// the float range to infinity
__device__ __forceinline__ float d2f_rn_ftz(double d)
{
    const unsigned hi = (unsigned) __double2hiint(d), lo = (unsigned) __double2loint(d);
    const unsigned sign = hi & 0x80000000u;
    const unsigned ed = (hi >> 20) & 0x7ffu;
    const int e = (int) ed - 896;
    const unsigned mant = ((hi & 0xfffffu) << 3) | (lo >> 29);   // the 23 kept mantissa bits
    const unsigned rest = lo & 0x1fffffffu;                      // the 29 dropped ones
    const unsigned up = rest > 0x10000000u || (rest == 0x10000000u && (mant & 1u));
    unsigned bits = ((unsigned) e << 23) + mant + up;            // a carry moves into the exponent
    if (e <= 0) bits = 0u;
    if (e >= 255 || bits >= 0x7f800000u) bits = 0x7f800000u;
    if (ed == 0x7ffu && ((hi & 0xfffffu) | lo)) bits = 0x7fffffffu;   // NaN
    return __uint_as_float(sign | bits);
}

// x / 2, exact: the exponent less one while the result stays normal, else the
// FP64 multiply
__device__ __forceinline__ double half_exact(double x)
{
    const int hi = __double2hiint(x);
    const unsigned e = ((unsigned) hi >> 20) & 0x7ffu;
    if (e > 1u && e < 0x7ffu) return __hiloint2double(hi - 0x00100000, __double2loint(x));
    return __dmul_rn(0.5, x);
}

__device__ __forceinline__ df df_from_double(double x)
{
    const float hi = d2f_rn_ftz(x);
    const float lo = d2f_rn_ftz(x - f2d_exact(hi));
    return {hi, lo};
}

__device__ __forceinline__ double df_to_double(df a) { return f2d_exact(a.hi) + f2d_exact(a.lo); }

// U_new = U0 (1 - b) + (U + dt L) b, the RK combine of SolutionSchemes.cpp:
// 232-235, on FP32 pairs.  b is 1, 1/2, 1/4 or 2/3.
__device__ __forceinline__ df rk_combine(df U0, df U, float dtL, float b, float one_minus_b)
{
    const df s = df_add_f(U, dtL);
    if (one_minus_b == 0.0f) return s;
    if (b == 0.5f) {  // (U0 + s) / 2: halving is exact on both words
        const df t = df_add(U0, s);
        return {__fmul_rn(0.5f, t.hi), __fmul_rn(0.5f, t.lo)};
    }
    return df_add(df_mul_f(U0, one_minus_b), df_mul_f(s, b));
}

// ---------------------------------------------------------------------------
__device__ __forceinline__ float fmin3(float a, float b, float c) { return fminf(a, fminf(b, c)); }
__device__ __forceinline__ float fmax3(float a, float b, float c) { return fmaxf(a, fmaxf(b, c)); }

// generalized minmod of Reconstruction.cpp:55-61.  With a = theta (u0 - ul),
// b = (ur - ul) / 2, c = theta (ur - u0), the reference's
// 0.25 |sgn a + sgn b| (sgn a + sgn c) min(|a|, |b|, |c|) is non-zero only
// when a and c share a sign (b is then a positive combination of the same
// two differences and shares it too), and then equals sgn(a) min(|a|,|b|,|c|).
__device__ __forceinline__ float minmod_f(float theta, float ul, float u0, float ur)
{
    const float a = theta * (u0 - ul);
    const float b = 0.5f * (ur - ul);
    const float c = theta * (ur - u0);
    const float m = fmin3(fabsf(a), fabsf(b), fabsf(c));
    return a * c > 0.0f ? copysignf(m, a) : 0.0f;
}

// WENO5 point value at the right / left edge (Reconstruction.cpp:68-169)
template <bool RIGHT>
__device__ __forceinline__ float weno5_f(const float* v, int mode, float Ash)
{
    const float c00 = RIGHT ? 1.f / 3.f : 11.f / 6.f, c01 = RIGHT ? 5.f / 6.f : -7.f / 6.f, c02 = RIGHT ? -1.f / 6.f : 1.f / 3.f;
    const float c10 = RIGHT ? -1.f / 6.f : 1.f / 3.f, c11 = 5.f / 6.f, c12 = RIGHT ? 1.f / 3.f : -1.f / 6.f;
    const float c20 = RIGHT ? 1.f / 3.f : -1.f / 6.f, c21 = RIGHT ? -7.f / 6.f : 5.f / 6.f, c22 = RIGHT ? 11.f / 6.f : 1.f / 3.f;
    const float d0 = RIGHT ? 0.3f : 0.1f, d1 = 0.6f, d2 = RIGHT ? 0.1f : 0.3f;
    const float vs0 = c00 * v[0] + c01 * v[1] + c02 * v[2];
    const float vs1 = c10 * v[-1] + c11 * v[0] + c12 * v[1];
    const float vs2 = c20 * v[-2] + c21 * v[-1] + c22 * v[0];
    const float t0 = v[0] - 2.f * v[1] + v[2], u0 = 3.f * v[0] - 4.f * v[1] + v[2];
    const float t1 = v[-1] - 2.f * v[0] + v[1], u1 = v[-1] - v[1];
    const float t2 = v[-2] - 2.f * v[-1] + v[0], u2 = v[-2] - 4.f * v[-1] + 3.f * v[0];
    float B0 = (13.f / 12.f) * t0 * t0 + 0.25f * u0 * u0;
    float B1 = (13.f / 12.f) * t1 * t1 + 0.25f * u1 * u1;
    float B2 = (13.f / 12.f) * t2 * t2 + 0.25f * u2 * u2;
    float w0, w1, w2;
    if (mode == WENO_BORGES08) {
        // eps 1e-14 is below FP32 resolution of typical B; keep it as given
        const float eps = 1e-14f;
        const float tau5 = fabsf(B0 - B2);
        w0 = d0 * (1.f + tau5 / (B0 + eps));
        w1 = d1 * (1.f + tau5 / (B1 + eps));
        w2 = d2 * (1.f + tau5 / (B2 + eps));
    } else if (mode == WENO_SHENZHA10) {
        const float ep = 1e-10f;
        const float minB = fmin3(B0, B1, B2), maxB = fmax3(B0, B1, B2);
        const float R0 = minB / (maxB + ep);
        const float add = R0 * Ash * minB;
        B0 += add; B1 += add; B2 += add;
        const float e0 = ep + B0, e1 = ep + B1, e2 = ep + B2;
        w0 = d0 / (e0 * e0);
        w1 = d1 / (e1 * e1);
        w2 = d2 / (e2 * e2);
    } else {
        const float ep = 1e-6f;
        const float e0 = ep + B0, e1 = ep + B1, e2 = ep + B2;
        w0 = d0 / (e0 * e0);
        w1 = d1 / (e1 * e1);
        w2 = d2 / (e2 * e2);
    }
    return (w0 * vs0 + w1 * vs1 + w2 * vs2) / (w0 + w1 + w2);
}

// ---------------------------------------------------------------------------
// States: P, U, F and the extreme wave speeds (all the Riemann solvers use).
template <int NQ> struct StateF {
    float P[NQ], U[NQ], F[NQ];
    float amax, amin;  // max / min eigenvalue over the reference's 10 slots
};

// A face normal: a coordinate axis fixed at compile time (the Cartesian
// faces of the flux kernels; the 6e-17 x-component of the reference's yhat
// lies far below FP32 rounding) or a general unit vector.  add(d, x, t) is
// x + t n_d, without the multiplications by zero of an axis.
template <int AXIS> struct AxisNormal {
    __device__ __forceinline__ float dot(float x, float y, float z) const { return AXIS == 0 ? x : AXIS == 1 ? y : z; }
    __device__ __forceinline__ float add(int d, float x, float t) const { return d == AXIS ? x + t : x; }
};
struct VecNormal {
    const float* n;
    __device__ __forceinline__ float dot(float x, float y, float z) const { return x * n[0] + y * n[1] + z * n[2]; }
    __device__ __forceinline__ float add(int d, float x, float t) const { return x + t * n[d]; }
};

// NewtonianHydro::fromPrimitive (ConservationLaws.cpp:253-290)
template <class N>
__device__ __forceinline__ void hydro_prim_f(float gamma, const float* P, const N& n, StateF<5>& S)
{
    const float gm1 = gamma - 1.0f;
    const float cs = sqrtf(gamma * P[4] / P[0]);
    const float vv = P[1] * P[1] + P[2] * P[2] + P[3] * P[3];
    const float vn = n.dot(P[1], P[2], P[3]);
#pragma unroll
    for (int q = 0; q < 5; ++q) S.P[q] = P[q];
    S.U[0] = P[0];
    S.U[1] = P[0] * P[1];
    S.U[2] = P[0] * P[2];
    S.U[3] = P[0] * P[3];
    S.U[4] = 0.5f * P[0] * vv + P[4] / gm1;
    S.F[0] = vn * S.U[0];
    S.F[1] = n.add(0, vn * S.U[1], P[4]);
    S.F[2] = n.add(1, vn * S.U[2], P[4]);
    S.F[3] = n.add(2, vn * S.U[3], P[4]);
    S.F[4] = vn * (S.U[4] + P[4]);
    S.amax = fmaxf(vn + cs, 0.0f);
    S.amin = fminf(vn - cs, 0.0f);
}

__device__ __forceinline__ void hydro_cons_f(float gamma, const float* U, float* P)
{
    const float gm1 = gamma - 1.0f;
    const float ir = 1.0f / U[0];
    P[0] = U[0];
    P[1] = U[1] * ir;
    P[2] = U[2] * ir;
    P[3] = U[3] * ir;
    P[4] = (U[4] - 0.5f * (U[1] * U[1] + U[2] * U[2] + U[3] * U[3]) * ir) * gm1;
}

// NewtonianMHD::fromPrimitive (ConservationLaws.cpp:416-487)
template <class N>
__device__ __forceinline__ void mhd_prim_f(float gamma, const float* P, const N& n, StateF<8>& S)
{
    const float gm1 = gamma - 1.0f;
    const float ir = 1.0f / P[0];
    const float cs2 = gamma * P[4] * ir;
    const float vv = P[1] * P[1] + P[2] * P[2] + P[3] * P[3];
    const float BB = P[5] * P[5] + P[6] * P[6] + P[7] * P[7];
    const float Bv = P[5] * P[1] + P[6] * P[2] + P[7] * P[3];
    const float vn = n.dot(P[1], P[2], P[3]);
    const float Bn = n.dot(P[5], P[6], P[7]);
    const float ps = P[4] + 0.5f * BB;
#pragma unroll
    for (int q = 0; q < 8; ++q) S.P[q] = P[q];
    S.U[0] = P[0];
    S.U[1] = P[0] * P[1];
    S.U[2] = P[0] * P[2];
    S.U[3] = P[0] * P[3];
    S.U[4] = 0.5f * (P[0] * vv + BB) + P[4] / gm1;
    S.U[5] = P[5];
    S.U[6] = P[6];
    S.U[7] = P[7];
    S.F[0] = vn * S.U[0];
    S.F[1] = n.add(0, vn * S.U[1] - Bn * P[5], ps);
    S.F[2] = n.add(1, vn * S.U[2] - Bn * P[6], ps);
    S.F[3] = n.add(2, vn * S.U[3] - Bn * P[7], ps);
    S.F[4] = vn * (S.U[4] + ps) - Bn * Bv;
    S.F[5] = vn * S.U[5] - Bn * P[1];
    S.F[6] = vn * S.U[6] - Bn * P[2];
    S.F[7] = vn * S.U[7] - Bn * P[3];
    const float ca2 = BB * ir, cn2 = Bn * Bn * ir;
    const float s = cs2 + ca2;
    const float cF2 = 0.5f * (s + sqrtf(fmaxf(s * s - 4.f * cs2 * cn2, 0.f)));
    const float cF = sqrtf(cF2);
    S.amax = fmaxf(vn + cF, 0.0f);
    S.amin = fminf(vn - cF, 0.0f);
}

// NewtonianMHD::fromConserved with the bad-state test (ConservationLaws.cpp:
// 370-414); returns ST_INVERSION_FAILURE where the reference throws
__device__ __forceinline__ int mhd_cons_f(float gamma, float pfloor, const float* U, float* P)
{
    const float gm1 = gamma - 1.0f;
    const float ir = 1.0f / U[0];
    P[0] = U[0];
    P[1] = U[1] * ir;
    P[2] = U[2] * ir;
    P[3] = U[3] * ir;
    P[5] = U[5];
    P[6] = U[6];
    P[7] = U[7];
    P[4] = (U[4] - 0.5f * (U[1] * U[1] + U[2] * U[2] + U[3] * U[3]) * ir
            - 0.5f * (U[5] * U[5] + U[6] * U[6] + U[7] * U[7])) * gm1;
    if (P[4] < 0.f || P[0] < 0.f || U[4] < 0.f) {
        if (P[4] < 0.f && pfloor > 0.f) { P[4] = pfloor * P[0]; return ST_OK; }
        return ST_INVERSION_FAILURE;
    }
    return ST_OK;
}

// QuarticPolynomial::solve in FP32 (QuarticPolynomial.cpp:19-144)
__device__ __forceinline__ int quartic_roots_f(float d4, float d3, float d2, float d1, float d0, float roots[4])
{
    const float id4 = 1.0f / d4;
    const float a3 = d3 * id4, a2 = d2 * id4, a1 = d1 * id4, a0 = d0 * id4;
    // resolvent cubic u^3 - a2 u^2 + (a1 a3 - 4 a0) u + (4 a0 a2 - a1^2 - a0 a3^2)
    const float c2 = -a2, c1 = a1 * a3 - 4.f * a0, c0 = 4.f * a0 * a2 - a1 * a1 - a0 * a3 * a3;
    const float q = c1 / 3.f - c2 * c2 / 9.f;
    const float r = (c1 * c2 - 3.f * c0) / 6.f - c2 * c2 * c2 / 27.f;
    const float delta = q * q * q + r * r;
    float u1;
    if (delta > 0.f) {
        const float sd = sqrtf(delta);
        const float s1 = cbrtf(r + sd), s2 = cbrtf(r - sd);
        u1 = (s1 + s2) - c2 / 3.f;
    } else if (delta < 0.f) {
        const float th = acosf(fminf(fmaxf(r / sqrtf(-q * q * q), -1.f), 1.f)) / 3.f;
        const float sq = sqrtf(-q);
        float sn, cs;
        sincosf(th, &sn, &cs);
        const float x1 = 2.f * sq * cs - c2 / 3.f;
        const float x3 = -sq * cs - c2 / 3.f + 1.7320508f * sq * sn;
        u1 = fmaxf(x1, x3);
    } else {
        u1 = 2.f * cbrtf(r) - c2 / 3.f;
    }
    const float R2 = 0.25f * a3 * a3 + u1 - a2;
    const float R = R2 > 0.f ? sqrtf(R2) : 0.f;
    float D2, E2;
    if (R != 0.f) {
        const float f1 = 0.75f * a3 * a3 - R2 - 2.f * a2;
        const float f2 = 0.25f * (4.f * a3 * a2 - 8.f * a1 - a3 * a3 * a3) / R;
        D2 = f1 + f2;
        E2 = f1 - f2;
    } else {
        const float f1 = 0.75f * a3 * a3 - 2.f * a2;
        const float f2 = 2.f * sqrtf(fmaxf(u1 * u1 - 4.f * a0, 0.f));
        D2 = f1 + f2;
        E2 = f1 - f2;
    }
    int m = 0;
    if (D2 >= 0.f) {
        const float D = sqrtf(D2);
        roots[m++] = -0.25f * a3 + 0.5f * R - 0.5f * D;
        roots[m++] = -0.25f * a3 + 0.5f * R + 0.5f * D;
    }
    if (E2 >= 0.f) {
        const float E = sqrtf(E2);
        roots[m++] = -0.25f * a3 - 0.5f * R - 0.5f * E;
        roots[m++] = -0.25f * a3 - 0.5f * R + 0.5f * E;
    }
    return m;
}

// RelativisticMHD::fromPrimitive in FP32 (ConservationLaws.cpp:659-836).
// The wave-speed extremes come from the quartic roots, the Alfven pair and
// vn, as in the reference's eigenvalue table.
template <class N>
__device__ __forceinline__ int rmhd_prim_f(float gamma, const float* P, const N& n, StateF<8>& S)
{
    const float gm1 = gamma - 1.0f;
    const float vv = P[1] * P[1] + P[2] * P[2] + P[3] * P[3];
    if (vv >= 1.f) return ST_SUPERLUMINAL;
    const float BB = P[5] * P[5] + P[6] * P[6] + P[7] * P[7];
    const float Bv = P[5] * P[1] + P[6] * P[2] + P[7] * P[3];
    const float vn = n.dot(P[1], P[2], P[3]);
    const float Bn = n.dot(P[5], P[6], P[7]);
    const float W2 = 1.0f / (1.0f - vv);
    const float W0 = sqrtf(W2);
    const float iW0 = 1.0f / W0;
    const float b0 = W0 * Bv;
    const float bb = (BB + b0 * b0) / W2;
    const float b1 = (P[5] + b0 * W0 * P[1]) * iW0;
    const float b2 = (P[6] + b0 * W0 * P[2]) * iW0;
    const float b3 = (P[7] + b0 * W0 * P[3]) * iW0;
    const float bn = n.dot(b1, b2, b3);
    const float ir = 1.0f / P[0];
    const float e0 = P[4] * ir / gm1;
    const float p0 = P[4];
    const float ps = p0 + 0.5f * bb;
    const float h0 = 1.0f + e0 + p0 * ir;
    const float hs = h0 + bb * ir;
#pragma unroll
    for (int q = 0; q < 8; ++q) S.P[q] = P[q];
    const float rhw = P[0] * hs * W2;
    S.U[0] = P[0] * W0;
    S.U[4] = rhw - ps - b0 * b0 - S.U[0];
    S.U[1] = rhw * P[1] - b0 * b1;
    S.U[2] = rhw * P[2] - b0 * b2;
    S.U[3] = rhw * P[3] - b0 * b3;
    S.U[5] = P[5];
    S.U[6] = P[6];
    S.U[7] = P[7];
    S.F[0] = vn * S.U[0];
    S.F[1] = n.add(0, vn * S.U[1] - Bn * b1 * iW0, ps);
    S.F[2] = n.add(1, vn * S.U[2] - Bn * b2 * iW0, ps);
    S.F[3] = n.add(2, vn * S.U[3] - Bn * b3 * iW0, ps);
    S.F[4] = vn * S.U[4] - Bn * b0 * iW0 + ps * vn;
    S.F[5] = vn * S.U[5] - Bn * P[1];
    S.F[6] = vn * S.U[6] - Bn * P[2];
    S.F[7] = vn * S.U[7] - Bn * P[3];

    const float cs2 = gamma * p0 / (P[0] * h0);
    const float v2 = vn * vn;
    float amax = vn, amin = vn;
    if (BB == 0.f) {
        const float K = sqrtf(fmaxf(cs2 * (1.f - vv) * (1.f - vv * cs2 - v2 * (1.f - cs2)), 0.f));
        const float id = 1.0f / (1.f - vv * cs2);
        amin = fminf(amin, (vn * (1.f - cs2) - K) * id);
        amax = fmaxf(amax, (vn * (1.f - cs2) + K) * id);
    } else {
        const float W4 = W2 * W2;
        const float v3 = vn * v2, v4 = vn * v3;
        const float K = W4 * (P[0] * h0 * (1.f / cs2 - 1.f));
        const float L = -W2 * (P[0] * h0 + bb / cs2);
        const float A4 = K - L - b0 * b0;
        const float A3 = -4.f * K * vn + 2.f * L * vn + 2.f * b0 * bn;
        const float A2 = 6.f * K * v2 + L * (1.f - v2) + b0 * b0 - bn * bn;
        const float A1 = -4.f * K * v3 - 2.f * L * vn - 2.f * b0 * bn;
        const float A0 = K * v4 + L * v2 + bn * bn;
        float roots[4];
        const int nr = quartic_roots_f(A4, A3, A2, A1, A0, roots);
        if (nr != 2 && nr != 4) return ST_BAD_EIGENVALUES;
        for (int m = 0; m < nr; ++m) { amin = fminf(amin, roots[m]); amax = fmaxf(amax, roots[m]); }
        const float C = sqrtf(h0 + bb);
        const float am1 = (bn - C * vn * W0) / (b0 - C * W0);
        const float ap1 = (bn + C * vn * W0) / (b0 + C * W0);
        amin = fminf(amin, fminf(am1, ap1));
        amax = fmaxf(amax, fmaxf(am1, ap1));
    }
    // the relativistic wave speeds are bounded by c = 1
    S.amax = fmaxf(fminf(amax, 1.f), 0.0f);
    S.amin = fminf(fmaxf(amin, -1.f), 0.0f);
    return ST_OK;
}

// ---------------------------------------------------------------------------
template <int LAW, class N>
__device__ __forceinline__ int law_prim_f(float gamma, const float* P, const N& n, StateF<LawInfo<LAW>::NQ>& S)
{
    if constexpr (LAW == LAW_HYDRO) { hydro_prim_f(gamma, P, n, S); return ST_OK; }
    else if constexpr (LAW == LAW_MHD) { mhd_prim_f(gamma, P, n, S); return ST_OK; }
    else return rmhd_prim_f(gamma, P, n, S);
}

// HlleRiemannSolver::solve (RiemannSolvers.cpp:38-57)
template <int NQ>
__device__ __forceinline__ void hlle_f(const StateF<NQ>& L, const StateF<NQ>& R, float* F)
{
    const float ap = fmaxf(L.amax, R.amax);
    const float am = fminf(L.amin, R.amin);
    const float id = 1.0f / (ap - am);
    const float apam = ap * am;
#pragma unroll
    for (int q = 0; q < NQ; ++q)
        F[q] = (ap * L.F[q] - am * R.F[q] + apam * (R.U[q] - L.U[q])) * id;
}

// HllcNewtonianHydroRiemannSolver::solve (RiemannSolvers.cpp:63-118)
template <int NQ, class N>
__device__ __forceinline__ void hllc_f(const StateF<NQ>& L, const StateF<NQ>& R, const N& n, float* F)
{
    const float ap = fmaxf(L.amax, R.amax);
    const float am = fminf(L.amin, R.amin);
    const float* Pl = L.P;
    const float* Pr = R.P;
    const float vnr = n.dot(Pr[1], Pr[2], Pr[3]);
    const float vnl = n.dot(Pl[1], Pl[2], Pl[3]);
    const float ml = Pl[0] * (am - vnl), mr = Pr[0] * (ap - vnr);
    const float lc = ((Pr[4] - mr * vnr) - (Pl[4] - ml * vnl)) / (ml - mr);
#pragma unroll
    for (int q = 0; q < NQ; ++q) F[q] = 0.0f;
    if (0.0f <= am) {
#pragma unroll
        for (int i = 0; i < 5; ++i) F[i] = L.F[i];
    } else if (0.0f <= lc) {
        const float fl = ml / (am - lc);
        const float il = 1.0f / Pl[0];
        float Us[5];
        Us[0] = fl;
        Us[4] = fl * (L.U[4] * il + (lc - vnl) * (lc + Pl[4] / ml));
        Us[1] = fl * n.add(0, Pl[1], lc - vnl);
        Us[2] = fl * n.add(1, Pl[2], lc - vnl);
        Us[3] = fl * n.add(2, Pl[3], lc - vnl);
#pragma unroll
        for (int i = 0; i < 5; ++i) F[i] = L.F[i] + am * (Us[i] - L.U[i]);
    } else if (0.0f <= ap) {
        const float fr = mr / (ap - lc);
        const float ir = 1.0f / Pr[0];
        float Us[5];
        Us[0] = fr;
        Us[4] = fr * (R.U[4] * ir + (lc - vnr) * (lc + Pr[4] / mr));
        Us[1] = fr * n.add(0, Pr[1], lc - vnr);
        Us[2] = fr * n.add(1, Pr[2], lc - vnr);
        Us[3] = fr * n.add(2, Pr[3], lc - vnr);
#pragma unroll
        for (int i = 0; i < 5; ++i) F[i] = R.F[i] + ap * (Us[i] - R.U[i]);
    } else {
#pragma unroll
        for (int i = 0; i < 5; ++i) F[i] = R.F[i];
    }
}

} // namespace mara
