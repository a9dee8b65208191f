// crmath.cuh -- correctly rounded FP64 evaluations of the transcendental
// functions in the RMHD quartic eigenvalue solver (QuarticPolynomial.cpp:
// 19-144): pow(x, 1/3), acos, cos and sin.
//
// The plain FP64 path must reproduce the reference's CPU run, whose libm
// (glibc) returns the correctly rounded result of these functions on all but
// a vanishing fraction of arguments.  CUDA's own pow / acos / cos / sin are
// accurate to 1-2 ulp and so differ from it in the last bit now and then.
// Each function below therefore evaluates its result to about 100 bits in
// double-double arithmetic and rounds that once, so it returns the
// correctly rounded value unless the exact result lies within ~2^-100
// (relative) of a rounding boundary.
//
// Methods (all published; no library internals are reproduced):
//   * double-double arithmetic: Dekker, "A floating-point technique for
//     extending the available precision", Numer. Math. 18 (1971), with
//     Knuth's TwoSum (TAOCP vol. 2, 4.2.2) and the exact product by fused
//     multiply-add;
//   * cube root: one Newton step x1 = x0 - (x0^3 - a) / (3 x0^2) in
//     double-double from a library cube root, then the factor
//     a^(y - 1/3) = exp((y - 1/3) ln a) = 1 + e + e^2/2 for the exponent
//     y = fl(1/3) = (1 - 2^-54) / 3 that the reference passes to pow;
//   * arc cosine: one Newton step on cos(t) = z from a library acos, with
//     cos(t) - z formed from half-angle identities near z = +-1 so that no
//     cancellation loses the step;
//   * sine and cosine: reduction by k pi/2 with pi/2 held in three doubles
//     (Cody and Waite's method), then the Taylor series in double-double
//     (terms below 2^-53 relative summed in double).
// The constants are the mathematical values of ln 2, pi/2 and 1/n!, split
// into double-double (or triple) parts.
//
// Every operation is explicitly rounded (__dadd_rn, __dmul_rn, __fma_rn on
// the device; the host build uses -ffp-contract=off), so the same source
// gives the same bits on the host and on the device for the same starting
// approximations.
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define CRM_FN __host__ __device__ __forceinline__
#else
#define CRM_FN static inline
#endif

namespace crm {

CRM_FN double add(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
CRM_FN double sub(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}
CRM_FN double mul(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
CRM_FN double fmad(double a, double b, double c)
{
#if defined(__CUDA_ARCH__)
    return __fma_rn(a, b, c);
#else
    return fma(a, b, c);
#endif
}
CRM_FN double quot(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __ddiv_rn(a, b);
#else
    return a / b;
#endif
}

struct dd {
    double hi, lo;
};

// s + e = a + b exactly (Knuth)
CRM_FN dd two_sum(double a, double b)
{
    const double s = add(a, b);
    const double bb = sub(s, a);
    return {s, add(sub(a, sub(s, bb)), sub(b, bb))};
}
// the same for |a| >= |b| (Dekker)
CRM_FN dd fast_two_sum(double a, double b)
{
    const double s = add(a, b);
    return {s, sub(b, sub(s, a))};
}
// p + e = a b exactly
CRM_FN dd two_prod(double a, double b)
{
    const double p = mul(a, b);
    return {p, fmad(a, b, -p)};
}
CRM_FN dd dd_neg(dd a) { return {-a.hi, -a.lo}; }
CRM_FN dd dd_add(dd a, dd b)
{
    dd s = two_sum(a.hi, b.hi);
    const dd t = two_sum(a.lo, b.lo);
    s.lo = add(s.lo, t.hi);
    s = fast_two_sum(s.hi, s.lo);
    s.lo = add(s.lo, t.lo);
    return fast_two_sum(s.hi, s.lo);
}
CRM_FN dd dd_add_d(dd a, double b)
{
    dd s = two_sum(a.hi, b);
    s.lo = add(s.lo, a.lo);
    return fast_two_sum(s.hi, s.lo);
}
CRM_FN dd dd_mul(dd a, dd b)
{
    dd p = two_prod(a.hi, b.hi);
    p.lo = fmad(a.hi, b.lo, p.lo);
    p.lo = fmad(a.lo, b.hi, p.lo);
    return fast_two_sum(p.hi, p.lo);
}
CRM_FN dd dd_mul_d(dd a, double b)
{
    dd p = two_prod(a.hi, b);
    p.lo = fmad(a.lo, b, p.lo);
    return fast_two_sum(p.hi, p.lo);
}

// ---- pow(x, 1/3) -------------------------------------------------------------
// pow(x, y) for x >= 0 (or -0) and y = fl(1/3), as the resolvent cubic calls
// it.  Zero, infinity and NaN follow pow's special cases.
CRM_FN double pow_third(double x)
{
    if (x == 0.0) return 0.0;             // pow(+-0, y > 0, not an odd integer) = +0
    if (!(x < INFINITY)) return x;        // +inf, NaN
    // keep x^3-sized intermediates inside the normal range
    double s = x, back = 1.0, lnscale = 0.0;
    if (x < 0x1p-900) { s = mul(x, 0x1p+900); back = 0x1p-300; lnscale = -900.0; }
    else if (x > 0x1p+900) { s = mul(x, 0x1p-900); back = 0x1p+300; lnscale = 900.0; }
    // the cube root c of s to ~104 bits: one Newton step from cbrt
    const double c0 = cbrt(s);
    const dd c2 = two_prod(c0, c0);
    const dd c3 = dd_mul_d(c2, c0);
    const dd r = dd_add_d(c3, -s);                       // c0^3 - s
    const double corr = quot(add(r.hi, r.lo), mul(3.0, mul(c0, c0)));
    dd c = two_sum(c0, -corr);
    // s^(y - 1/3) with y - 1/3 = -2^-54 / 3: 1 + e + e^2 / 2, e = -(2^-54/3) ln x
    const double lnx = add(log(s), mul(lnscale, 0x1.62e42fefa39efp-1));
    const double e = mul(mul(-0x1p-54, lnx), 0x1.5555555555555p-2);
    const double f = fmad(mul(0.5, e), e, e);
    c = dd_add_d(c, fmad(c.lo, f, mul(c.hi, f)));
    return mul(add(c.hi, c.lo), back);
}

// ---- sine and cosine -----------------------------------------------------------
// pi/2 in three parts and 2/pi
#define CRM_PIO2_0 0x1.921fb54442d18p+0
#define CRM_PIO2_1 0x1.1a62633145c07p-54
#define CRM_PIO2_2 (-0x1.f1976b7ed8fbcp-110)
#define CRM_TWO_OVER_PI 0x1.45f306dc9c883p-1

// one Horner step p <- 1/n! - r2 p in double-double
CRM_FN dd horner_alt(dd r2, dd p, double inv_hi, double inv_lo)
{
    return dd_add(dd{inv_hi, inv_lo}, dd_neg(dd_mul(r2, p)));
}

// sin(r) and cos(r) of a double-double |r| <= pi/4 (+ a little), to ~104 bits
CRM_FN void sincos_taylor(dd r, dd& s, dd& c)
{
    const dd r2 = dd_mul(r, r);
    const double x2 = r2.hi;
    // the terms below 2^-53 of the leading one, summed in double:
    // sin: r^17/17! .. r^27/27!,  cos: r^18/18! .. r^28/28!
    double ts = 0x1.d1ab1c2dccea3p-94;                  // 1/27!
    ts = fmad(ts, -x2, 0x1.3f3ccdd165fa9p-84);          // 1/25!
    ts = fmad(ts, -x2, 0x1.761b41316381ap-75);          // 1/23!
    ts = fmad(ts, -x2, 0x1.71b8ef6dcf572p-66);          // 1/21!
    ts = fmad(ts, -x2, 0x1.2f49b46814157p-57);          // 1/19!
    ts = fmad(ts, -x2, 0x1.952c77030ad4ap-49);          // 1/17!
    double tc = 0x1.0a18a2635085dp-98;                  // 1/28!
    tc = fmad(tc, -x2, 0x1.88e85fc6a4e5ap-89);          // 1/26!
    tc = fmad(tc, -x2, 0x1.f2cf01972f578p-80);          // 1/24!
    tc = fmad(tc, -x2, 0x1.0ce396db7f853p-70);          // 1/22!
    tc = fmad(tc, -x2, 0x1.e542ba4020225p-62);          // 1/20!
    tc = fmad(tc, -x2, 0x1.6827863b97d97p-53);          // 1/18!
    // the rest in double-double, p_n = 1/n! - r^2 p_{n+2}:
    // sin = r (1 - r^2 p_3), cos = 1 - r^2 p_2
    dd ps = {ts, 0.0};
    ps = horner_alt(r2, ps, 0x1.ae7f3e733b81fp-41, 0x1.1d8656b0ee8cbp-97);   // 1/15!
    ps = horner_alt(r2, ps, 0x1.6124613a86d09p-33, 0x1.f28e0cc748ebep-87);   // 1/13!
    ps = horner_alt(r2, ps, 0x1.ae64567f544e4p-26, -0x1.c062e06d1f209p-80);  // 1/11!
    ps = horner_alt(r2, ps, 0x1.71de3a556c734p-19, -0x1.c154f8ddc6c00p-73);  // 1/9!
    ps = horner_alt(r2, ps, 0x1.a01a01a01a01ap-13, 0x1.a01a01a01a01ap-73);   // 1/7!
    ps = horner_alt(r2, ps, 0x1.1111111111111p-7, 0x1.1111111111111p-63);    // 1/5!
    ps = horner_alt(r2, ps, 0x1.5555555555555p-3, 0x1.5555555555555p-57);    // 1/3!
    dd pc = {tc, 0.0};
    pc = horner_alt(r2, pc, 0x1.ae7f3e733b81fp-45, 0x1.1d8656b0ee8cbp-101);  // 1/16!
    pc = horner_alt(r2, pc, 0x1.93974a8c07c9dp-37, 0x1.05d6f8a2efd1fp-92);   // 1/14!
    pc = horner_alt(r2, pc, 0x1.1eed8eff8d898p-29, -0x1.2aec959e14c06p-83);  // 1/12!
    pc = horner_alt(r2, pc, 0x1.27e4fb7789f5cp-22, 0x1.cbbc05b4fa99ap-76);   // 1/10!
    pc = horner_alt(r2, pc, 0x1.a01a01a01a01ap-16, 0x1.a01a01a01a01ap-76);   // 1/8!
    pc = horner_alt(r2, pc, 0x1.6c16c16c16c17p-10, -0x1.f49f49f49f49fp-65);  // 1/6!
    pc = horner_alt(r2, pc, 0x1.5555555555555p-5, 0x1.5555555555555p-59);    // 1/4!
    pc = horner_alt(r2, pc, 0.5, 0.0);                                       // 1/2!
    s = dd_mul(r, dd_add_d(dd_neg(dd_mul(r2, ps)), 1.0));
    c = dd_add_d(dd_neg(dd_mul(r2, pc)), 1.0);
}

// sin and cos of x (|x| <= 8) to ~104 bits
CRM_FN void sincos_dd(double x, dd& s, dd& c)
{
    const double k = rint(mul(x, CRM_TWO_OVER_PI));
    dd r = dd_add_d(dd_neg(two_prod(k, CRM_PIO2_0)), x);
    r = dd_add(r, dd_neg(two_prod(k, CRM_PIO2_1)));
    r = dd_add_d(r, -mul(k, CRM_PIO2_2));
    dd sr, cr;
    sincos_taylor(r, sr, cr);
    const int q = ((int) k) & 3;
    if (q == 0) { s = sr; c = cr; }
    else if (q == 1) { s = cr; c = dd_neg(sr); }
    else if (q == 2) { s = dd_neg(sr); c = dd_neg(cr); }
    else { s = dd_neg(cr); c = sr; }
}

CRM_FN double cos_cr(double x)
{
    if (!(fabs(x) <= 8.0)) return cos(x);   // outside the quartic's range
    dd s, c;
    sincos_dd(x, s, c);
    return add(c.hi, c.lo);
}

CRM_FN double sin_cr(double x)
{
    if (!(fabs(x) <= 8.0)) return sin(x);
    if (x == 0.0) return x;                 // keeps the sign of zero
    dd s, c;
    sincos_dd(x, s, c);
    return add(s.hi, s.lo);
}

// ---- arc cosine ----------------------------------------------------------------
// acos(w) for 1/2 < w < 1 as a double-double: one Newton step from the library
// value u0 with cos(u0) - w = (1 - w) - 2 sin^2(u0 / 2) (1 - w is exact)
CRM_FN dd acos_upper(double w)
{
    const double u0 = acos(w);
    dd s, c;
    sincos_dd(mul(0.5, u0), s, c);
    const dd d = dd_add_d(dd_neg(dd_mul_d(dd_mul(s, s), 2.0)), sub(1.0, w));
    return two_sum(u0, quot(add(d.hi, d.lo), sin(u0)));
}

CRM_FN double acos_cr(double z)
{
    if (!(fabs(z) < 1.0)) return acos(z);   // +-1 (exact cases), NaN, |z| > 1
    if (z > 0.5) {
        const dd u = acos_upper(z);
        return add(u.hi, u.lo);
    }
    if (z < -0.5) {                          // acos(z) = pi - acos(-z)
        const dd u = acos_upper(-z);
        const dd t = dd_add(dd{mul(2.0, CRM_PIO2_0), mul(2.0, CRM_PIO2_1)}, dd_neg(u));
        return add(t.hi, t.lo);
    }
    // |z| <= 1/2: Newton t1 = t0 + (cos t0 - z) / sin t0 from the library value
    const double t0 = acos(z);
    dd s, c;
    sincos_dd(t0, s, c);
    const dd d = dd_add_d(c, -z);
    return add(t0, quot(add(d.hi, d.lo), sin(t0)));
}

} // namespace crm
