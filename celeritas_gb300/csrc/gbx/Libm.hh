// Elementary functions of the FP64 stepping loop, identical on host and device.
//
// The stepping loop's outcome depends on the last bit of exp and log: the
// field driver scales each Runge-Kutta step by exp(p * log(err^2))
// (src/corecel/math/Algorithms.hh:481-485, src/celeritas/field/
// FieldDriver.hh:424), and a one-bit change of a step length changes every
// later position and, after enough steps, a boundary decision. CUDA's device
// library and the host C library round differently (and the C library is not
// correctly rounded either), so this header gives the FP64 build one set of
// functions that compiles to the same IEEE operations everywhere (add, mul,
// div, fma and rint, no contraction): the device kernels, the CPU
// restatement and, through oracle/ref/pinned_libm.cc, the reference itself.
//
// Methods (all in double-double arithmetic, Dekker 1971 / Knuth TAOCP 4.2.2):
// * exp: Tang's table-driven method (ACM TOMS 15(2), 1989) with N = 128:
//   x = (128 m + j) ln2/128 + r, exp(x) = 2^m 2^(j/128) exp(r), |r| <= ln2/256,
//   exp(r) - 1 by its Taylor series. Correctly rounded: a fast evaluation
//   with a proven error bound, a rounding test (Ziv 1991), and a more precise
//   evaluation (about 2^-100 relative) when the test fails.
// * log: Tang's table-driven method (ACM TOMS 16(4), 1990): x = 2^e m,
//   m in [1, 2), m/c - 1 = z exactly (as a double-double) for the center c of
//   m's 1/128 interval, log(x) = e ln2 - log(1/c) + log1p(z), log1p by its
//   Taylor series; |x - 1| < 2^-7 directly by log1p(x - 1). Correctly
//   rounded in the same way.
// * sin, cos: Cody-Waite reduction by pi/2 in three parts (exact enough for
//   |x| < 2^20 pi/2), Taylor series of sin and cos on [-pi/4, pi/4] with the
//   leading terms in double-double, the rounding test, and the series in
//   double-double when it fails.
// * expm1, log1p, tanh, cbrt: from the double-double forms of the above
//   (tanh = E / (E + 2) with E = expm1(2|x|); cbrt by one Newton step in
//   double-double from exp(log(x)/3), then the cubes of the two rounding
//   midpoints against x), with rounding tests where a fast form is used.
//
// "Correctly rounded" holds except possibly for the few inputs whose exact
// result lies within about 2^-100 (relative) of a rounding midpoint, which
// the accurate paths cannot separate; sin and cos additionally need
// |x| < 2^20 pi/2 (the stepping loop's angles are below 2 pi).
//
// The float overloads (mixed-precision physics) forward to the C++ library:
// nothing compares FP32 results bit for bit. Defining GBX_SYSTEM_LIBM makes
// the double overloads forward too (the CPU restatement built that way
// reproduces the reference linked against the host C library).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#include "LibmTables.hh"
#include "Macros.hh"

namespace gbx
{
namespace libm
{
namespace detail
{
// Each table twice: in device global memory (read through the read-only
// cache) and in host memory, with the same values
#if defined(__CUDACC__)
__device__ const double d_exp_table[] = {GBX_LIBM_EXP_TABLE};
__device__ const double d_log_table[] = {GBX_LIBM_LOG_TABLE};
__device__ const double d_inv_fact[] = {GBX_LIBM_INV_FACT};
__device__ const double d_inv_int[] = {GBX_LIBM_INV_INT};
#endif
inline constexpr double h_exp_table[] = {GBX_LIBM_EXP_TABLE};
inline constexpr double h_log_table[] = {GBX_LIBM_LOG_TABLE};
inline constexpr double h_inv_fact[] = {GBX_LIBM_INV_FACT};
inline constexpr double h_inv_int[] = {GBX_LIBM_INV_INT};
#if defined(__CUDA_ARCH__)
#    define GBX_LIBM_LOAD(table, i) __ldg(&detail::d_##table[i])
#else
#    define GBX_LIBM_LOAD(table, i) detail::h_##table[i]
#endif
// Three-part constants as scalars (usable in device code)
struct Parts3
{
    double v0, v1, v2;
};
constexpr Parts3 ln2_n_parts{GBX_LIBM_LN2_N};
constexpr Parts3 ln2_parts{GBX_LIBM_LN2};
constexpr Parts3 pio2_parts{GBX_LIBM_PIO2};
constexpr double ln2_n0 = ln2_n_parts.v0, ln2_n1 = ln2_n_parts.v1, ln2_n2 = ln2_n_parts.v2;
constexpr double ln2_0 = ln2_parts.v0, ln2_1 = ln2_parts.v1, ln2_2 = ln2_parts.v2;
constexpr double pio2_0 = pio2_parts.v0, pio2_1 = pio2_parts.v1, pio2_2 = pio2_parts.v2;
constexpr double inv_ln2_n = GBX_LIBM_INV_LN2_N;
constexpr double two_over_pi = GBX_LIBM_TWO_OVER_PI;

//! Fast-path relative error bounds of exp and log: at least eight times the
//! largest errors measured against 250-bit evaluations (2^-65.5 and
//! 2^-67.1)
constexpr double exp_fast_err = 0x1p-62;
constexpr double log_fast_err = 0x1p-63;

GBX_FORCEINLINE double fma_(double a, double b, double c)
{
    return std::fma(a, b, c);
}

GBX_FORCEINLINE std::uint64_t bits(double x)
{
#if defined(__CUDA_ARCH__)
    return static_cast<std::uint64_t>(__double_as_longlong(x));
#else
    std::uint64_t u;
    std::memcpy(&u, &x, sizeof(u));
    return u;
#endif
}

GBX_FORCEINLINE double from_bits(std::uint64_t u)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double(static_cast<long long>(u));
#else
    double x;
    std::memcpy(&x, &u, sizeof(x));
    return x;
#endif
}

//! 2^e for -1022 <= e <= 1023
GBX_FORCEINLINE double pow2(int e)
{
    return from_bits(static_cast<std::uint64_t>(e + 1023) << 52);
}

//! Double-double value hi + lo, |lo| <= ulp(hi) / 2 when normalized
struct DD
{
    double hi;
    double lo;
};

//! a + b exactly (Knuth)
GBX_FORCEINLINE DD two_sum(double a, double b)
{
    double s = a + b;
    double bb = s - a;
    double e = (a - (s - bb)) + (b - bb);
    return {s, e};
}

//! a + b exactly for |a| >= |b| (Dekker)
GBX_FORCEINLINE DD fast_two_sum(double a, double b)
{
    double s = a + b;
    double e = b - (s - a);
    return {s, e};
}

//! a * b exactly
GBX_FORCEINLINE DD two_prod(double a, double b)
{
    double p = a * b;
    return {p, fma_(a, b, -p)};
}

GBX_FORCEINLINE DD dd_add(DD a, DD b)
{
    DD s = two_sum(a.hi, b.hi);
    DD t = two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = fast_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return fast_two_sum(s.hi, s.lo);
}

GBX_FORCEINLINE DD dd_mul(DD a, DD b)
{
    DD p = two_prod(a.hi, b.hi);
    p.lo += a.hi * b.lo + a.lo * b.hi;
    return fast_two_sum(p.hi, p.lo);
}

GBX_FORCEINLINE DD dd_mul_d(DD a, double b)
{
    DD p = two_prod(a.hi, b);
    p.lo += a.lo * b;
    return fast_two_sum(p.hi, p.lo);
}

//! Quotient of double-doubles to about 2^-104 (one correction step)
GBX_FORCEINLINE DD dd_div(DD a, DD b)
{
    double q1 = a.hi / b.hi;
    DD r = dd_add(a, dd_mul_d(b, -q1));
    double q2 = r.hi / b.hi;
    r = dd_add(r, dd_mul_d(b, -q2));
    double q3 = r.hi / b.hi;
    DD q = fast_two_sum(q1, q2);
    return dd_add(q, DD{q3, 0});
}

//! Whether hi + lo rounds to the same double as every value within
//! err * |hi| of it
GBX_FORCEINLINE bool rounds_surely(double hi, double lo, double err)
{
    double e = err * std::fabs(hi);
    return hi + (lo + e) == hi + (lo - e);
}

//---------------------------------------------------------------------------//
// exp
//---------------------------------------------------------------------------//
//! Reduced argument of exp: x = (k / 128) ln2 + r with r as a double-double
struct ExpReduced
{
    int k;
    DD r;
};

GBX_FORCEINLINE ExpReduced exp_reduce(double x)
{
    double kd = std::rint(x * inv_ln2_n);
    // kd times either of the 35-bit parts is exact (|k| < 2^18), and so is
    // the first subtraction (Sterbenz); the third part's product error is
    // below 2^-120 of the result
    double r1 = fma_(-kd, ln2_n0, x);
    DD r = two_sum(r1, -kd * ln2_n1);
    r.lo = fma_(-kd, ln2_n2, r.lo);
    return {static_cast<int>(kd), r};
}

//! 2^(j/128) as a double-double
GBX_FORCEINLINE DD exp_table_entry(int j)
{
    return {GBX_LIBM_LOAD(exp_table, 2 * j), GBX_LIBM_LOAD(exp_table, 2 * j + 1)};
}

//! exp(r) for |r| <= ln2/256, relative error below 2^-67, as hi + lo
//! multiplied by 2^(j/128)
GBX_FORCEINLINE DD exp_core_fast(DD r, DD t)
{
    double const x = r.hi;
    // r^2 (1/2 + r/6 + ... + r^5/7!) plus the r_hi r_lo cross term
    double q = fma_(x, GBX_LIBM_LOAD(inv_fact, 14), GBX_LIBM_LOAD(inv_fact, 12));
    q = fma_(x, q, GBX_LIBM_LOAD(inv_fact, 10));
    q = fma_(x, q, GBX_LIBM_LOAD(inv_fact, 8));
    q = fma_(x, q, GBX_LIBM_LOAD(inv_fact, 6));
    q = fma_(x, q, GBX_LIBM_LOAD(inv_fact, 4));
    // exp(r) - 1 = x + (r.lo + x r.lo + x^2 q), the parenthesis below
    // 2^-16 of the result
    double const tail = fma_(x * x, q, fma_(x, r.lo, r.lo));
    // t (1 + x + tail): t.hi x exactly, the rest to double precision
    DD m = two_prod(t.hi, x);
    DD out = fast_two_sum(t.hi, m.hi);
    out.lo += m.lo + fma_(t.hi, tail, fma_(t.lo, x, t.lo));
    return out;
}

//! The same to about 2^-100: Horner in double-double to r^11/11!
GBX_FORCEINLINE DD exp_core_accurate(DD r, DD t)
{
    DD p{GBX_LIBM_LOAD(inv_fact, 22), GBX_LIBM_LOAD(inv_fact, 23)};
    for (int k = 10; k >= 1; --k)
    {
        p = dd_mul(p, r);
        p = dd_add(p, DD{GBX_LIBM_LOAD(inv_fact, 2 * k), GBX_LIBM_LOAD(inv_fact, 2 * k + 1)});
    }
    p = dd_mul(p, r);  // exp(r) - 1
    DD tp = dd_mul(t, p);
    return dd_add(t, tp);
}

//! Round hi + lo (value in [0.7, 1.5)) times 2^m to a double, correctly
//! when 'sure'; 'ok' is false when the rounding is not decided by an error
//! of err * |hi|
GBX_FORCEINLINE double exp_scale(DD v, int m, double err, bool* ok)
{
    if (m >= -1021)
    {
        *ok = rounds_surely(v.hi, v.lo, err);
        double y = v.hi + v.lo;
        if (m > 1023)
            return y * 2.0 * pow2(m - 1);
        return y * pow2(m);
    }
    // Subnormal result: round (hi + lo) 2^(m + 1074) to an integer n and
    // return n 2^-1074 (exact)
    int const s = m + 1074;
    if (s < -2)
    {
        *ok = true;
        return 0.0;
    }
    double const scale = s >= -1022 ? pow2(s) : 0.0;
    v = fast_two_sum(v.hi, v.lo);  // |lo| <= ulp(hi) / 2 for the test below
    double uh = v.hi * scale;
    double ul = v.lo * scale;
    double n = std::rint(uh);
    double d = (uh - n) + ul;
    double e = err * uh;
    *ok = std::fabs(std::fabs(d) - 0.5) > e;
    if (d > 0.5)
        n += 1;
    else if (d < -0.5)
        n -= 1;
    return n * 0x1p-1074;
}

//! exp as a double-double hi + lo times 2^m (for expm1 and tanh)
GBX_FORCEINLINE DD exp_dd(double x, int* m)
{
    ExpReduced red = exp_reduce(x);
    int j = red.k & 127;
    *m = (red.k - j) / 128;
    return exp_core_accurate(red.r, exp_table_entry(j));
}

//! exp of a finite x in range by the accurate path (rarely taken)
GBX_NOINLINE double exp_accurate(double x)
{
    ExpReduced red = exp_reduce(x);
    int const j = red.k & 127;
    int const m = (red.k - j) / 128;
    bool ok = false;
    return exp_scale(exp_core_accurate(red.r, exp_table_entry(j)), m, 0.0, &ok);
}
}  // namespace detail

//! exp(x), correctly rounded
GBX_FORCEINLINE double exp(double x)
{
#if defined(GBX_SYSTEM_LIBM)
    return std::exp(x);
#else
    using namespace detail;
    if (!(x == x))
        return x + x;
    if (x > 0x1.62e42fefa39efp+9)
        return x * 0x1p1023 * 2.0;  // +inf (or the infinite input)
    if (x < -0x1.74910d52d3052p+9)
        return 0.0;  // below half the smallest subnormal: exp(x) rounds to 0
    if (std::fabs(x) < 0x1p-54)
        return 1.0 + x;
    ExpReduced red = exp_reduce(x);
    int const j = red.k & 127;
    int const m = (red.k - j) / 128;
    bool ok = false;
    double y = exp_scale(exp_core_fast(red.r, exp_table_entry(j)), m, exp_fast_err, &ok);
    if (ok)
        return y;
    return exp_accurate(x);
#endif
}

namespace detail
{
//---------------------------------------------------------------------------//
// log
//---------------------------------------------------------------------------//
//! log1p(z) for a double-double z = zh + zl, |z| < 2^-7: the Taylor series
//! with -z^2/2 exact and the rest in double; relative error below 2^-66
GBX_FORCEINLINE DD log1p_small_fast(double zh, double zl)
{
    // z^3 (1/3 - z/4 + ... - z^9/12)
    double p = fma_(zh, -GBX_LIBM_LOAD(inv_int, 24), GBX_LIBM_LOAD(inv_int, 22));
    p = fma_(zh, p, -GBX_LIBM_LOAD(inv_int, 20));
    p = fma_(zh, p, GBX_LIBM_LOAD(inv_int, 18));
    p = fma_(zh, p, -GBX_LIBM_LOAD(inv_int, 16));
    p = fma_(zh, p, GBX_LIBM_LOAD(inv_int, 14));
    p = fma_(zh, p, -GBX_LIBM_LOAD(inv_int, 12));
    p = fma_(zh, p, GBX_LIBM_LOAD(inv_int, 10));
    p = fma_(zh, p, -GBX_LIBM_LOAD(inv_int, 8));
    p = fma_(zh, p, GBX_LIBM_LOAD(inv_int, 6));
    p *= zh * zh * zh;
    // -z^2/2 exactly (zh times the exact zh/2), then the first-order term
    // of zl: log1p(zh + zl) = log1p(zh) + zl (1 - zh + zh^2) + O(zl zh^3)
    DD h = two_prod(zh, 0.5 * zh);
    DD s = fast_two_sum(zh, -h.hi);
    s.lo += fma_(zl, fma_(zh, zh, -zh), zl) - h.lo + p;
    return s;
}

//! log1p(z) to about 2^-100 relative: Horner in double-double to z^18/18
GBX_FORCEINLINE DD log1p_small_accurate(DD z)
{
    DD p{-GBX_LIBM_LOAD(inv_int, 36), -GBX_LIBM_LOAD(inv_int, 37)};
    for (int k = 17; k >= 1; --k)
    {
        p = dd_mul(p, z);
        double sign = (k % 2) ? 1.0 : -1.0;
        p = dd_add(p,
                   DD{sign * GBX_LIBM_LOAD(inv_int, 2 * k),
                      sign * GBX_LIBM_LOAD(inv_int, 2 * k + 1)});
    }
    return dd_mul(p, z);
}

//! Reduced argument of log: x = 2^e m, m in [1, 2), table row j of m's
//! 1/128 interval, z = m / c_j - 1 exactly as a double-double
struct LogReduced
{
    int e;
    int j;
    DD z;
    bool near_one;  //!< |x - 1| < 2^-7: z = x - 1 (exact), no table term
};

GBX_FORCEINLINE LogReduced log_reduce(double x)
{
    LogReduced red;
    if (std::fabs(x - 1.0) < 0x1p-7)
    {
        red.e = 0;
        red.j = 0;
        red.z = DD{x - 1.0, 0.0};
        red.near_one = true;
        return red;
    }
    int bias = 0;
    if (x < 0x1p-1022)
    {
        x *= 0x1p54;  // subnormal input: normalize
        bias = -54;
    }
    std::uint64_t const u = bits(x);
    red.e = static_cast<int>((u >> 52) & 0x7ff) - 1023 + bias;
    red.j = static_cast<int>((u >> 45) & 127);
    double const m = from_bits((u & 0x000fffffffffffffull) | 0x3ff0000000000000ull);
    double const inv_c = GBX_LIBM_LOAD(log_table, 3 * red.j);
    // m inv_c - 1: the product exactly as p + pe, p - 1 exact (Sterbenz);
    // z = (p - 1) + pe is kept as that unnormalized pair (|pe| <= 2^-54)
    DD p = two_prod(m, inv_c);
    red.z = DD{p.hi - 1.0, p.lo};
    red.near_one = false;
    return red;
}

//! e ln2 - log(inv_c_j) + log1p(z) from its parts, fast path
GBX_FORCEINLINE DD log_fast(LogReduced const& red)
{
    DD l = log1p_small_fast(red.z.hi, red.z.lo);
    if (red.near_one)
        return l;
    double const ed = red.e;
    double const th = GBX_LIBM_LOAD(log_table, 3 * red.j + 1);
    double const tl = GBX_LIBM_LOAD(log_table, 3 * red.j + 2);
    // e ln2_0 is exact and at least ln 2 > th when e != 0 (th < 0.6913)
    DD s = fast_two_sum(ed * ln2_0, th);
    DD t = two_sum(s.hi, l.hi);
    double const lo = fma_(ed, ln2_2, fma_(ed, ln2_1, (s.lo + t.lo) + (l.lo + tl)));
    return {t.hi, lo};
}

GBX_NOINLINE DD log_accurate(LogReduced const& red)
{
    DD l = log1p_small_accurate(red.z);
    if (red.near_one)
        return l;
    double const ed = red.e;
    DD t{GBX_LIBM_LOAD(log_table, 3 * red.j + 1), GBX_LIBM_LOAD(log_table, 3 * red.j + 2)};
    DD el = two_sum(ed * ln2_0, ed * ln2_1);  // both products exact
    el = dd_add(el, two_prod(ed, ln2_2));
    return dd_add(dd_add(el, t), l);
}
}  // namespace detail

//! log(x), correctly rounded
GBX_FORCEINLINE double log(double x)
{
#if defined(GBX_SYSTEM_LIBM)
    return std::log(x);
#else
    using namespace detail;
    if (!(x > 0) || x > 0x1.fffffffffffffp+1023)
    {
        if (x == 0)
            return -HUGE_VAL;
        if (x < 0)
            return (x - x) / (x - x);  // NaN
        return x + x;  // NaN or +inf
    }
    if (x == 1.0)
        return 0.0;
    LogReduced red = log_reduce(x);
    DD v = log_fast(red);
    if (rounds_surely(v.hi, v.lo, log_fast_err))
        return v.hi + v.lo;
    v = log_accurate(red);
    return v.hi + v.lo;
#endif
}

namespace detail
{
//! log(x) as a double-double for x > 0 finite (accurate path)
GBX_FORCEINLINE DD log_dd(double x)
{
    return log_accurate(log_reduce(x));
}

//---------------------------------------------------------------------------//
// sin, cos
//---------------------------------------------------------------------------//
//! x = q pi/2 + r, r as a double-double, |r| <= pi/4 (plus rounding)
GBX_FORCEINLINE DD trig_reduce(double x, int* q)
{
    double kd = std::rint(x * two_over_pi);
    double r1 = x - kd * pio2_0;  // exact for |k| < 2^20
    DD r = two_sum(r1, -kd * pio2_1);  // kd * pio2_1 exact
    DD p3 = two_prod(kd, pio2_2);
    r.lo -= p3.hi;
    r.lo -= p3.lo;
    r = fast_two_sum(r.hi, r.lo);
    *q = static_cast<int>(static_cast<long long>(kd) & 3);
    return r;
}

//! sin(r) for |r| <= pi/4 + a little, as hi + lo (relative error below
//! 2^-60)
GBX_FORCEINLINE DD sin_core(DD r)
{
    double const x = r.hi;
    DD z = two_prod(x, x);
    // r^5 (1/5! - r^2/7! + ... ) in double
    double zz = z.hi;
    double p = -GBX_LIBM_LOAD(inv_fact, 2 * 23);
    for (int k = 21; k >= 5; k -= 2)
    {
        double c = ((k - 1) / 2) % 2 ? -GBX_LIBM_LOAD(inv_fact, 2 * k)
                                     : GBX_LIBM_LOAD(inv_fact, 2 * k);
        p = fma_(zz, p, c);
    }
    // x^3 times (-1/6 + z p), both factors as double-doubles
    DD c3{x * z.hi, fma_(x, z.hi, -(x * z.hi)) + x * z.lo};
    DD zp = two_prod(zz, p);
    DD f = two_sum(-GBX_LIBM_LOAD(inv_fact, 6), zp.hi);
    f.lo += zp.lo - GBX_LIBM_LOAD(inv_fact, 7);
    DD u = dd_mul(c3, f);
    // sin(rh + rl) = sin(rh) + rl cos(rh), cos(rh) to its quartic term
    DD s = two_sum(x, u.hi);
    double const corr = r.lo * (1.0 - zz * (0.5 - zz * GBX_LIBM_LOAD(inv_fact, 8)));
    return {s.hi, s.lo + u.lo + corr};
}

//! cos(r) for |r| <= pi/4 + a little, as hi + lo (relative error below
//! 2^-60)
GBX_FORCEINLINE DD cos_core(DD r)
{
    double const x = r.hi;
    DD z = two_prod(x, x);
    double zz = z.hi;
    // -1/6! + z/8! - ... (the terms after z^2/4!)
    double p = -GBX_LIBM_LOAD(inv_fact, 2 * 22);
    for (int k = 20; k >= 6; k -= 2)
    {
        double c = (k / 2) % 2 ? -GBX_LIBM_LOAD(inv_fact, 2 * k) : GBX_LIBM_LOAD(inv_fact, 2 * k);
        p = fma_(zz, p, c);
    }
    // z^2 (1/4! + z p) with z^2 and its 1/24 in double-double
    DD w = two_prod(zz, zz);
    w.lo += 2.0 * zz * z.lo;
    double const c4h = GBX_LIBM_LOAD(inv_fact, 8);
    double const c4l = GBX_LIBM_LOAD(inv_fact, 9);
    DD u = two_prod(w.hi, c4h);
    u.lo += w.lo * c4h + w.hi * (c4l + zz * p);
    DD s = two_sum(1.0, -0.5 * z.hi);
    DD t = two_sum(s.hi, u.hi);
    // cos(rh + rl) = cos(rh) - rl sin(rh), sin(rh) to its cubic term
    double const corr = x * r.lo * (1.0 - zz * GBX_LIBM_LOAD(inv_fact, 6));
    return {t.hi, t.lo + s.lo + u.lo - 0.5 * z.lo - corr};
}

//! sin(r) (odd) or cos(r) (even) to about 2^-100: Horner in double-double
//! over r^2 to the r^27 (r^26) term
GBX_NOINLINE DD trig_accurate(DD r, bool odd)
{
    DD z = dd_mul(r, r);
    int const top = odd ? 27 : 26;
    double sign = ((top / 2) % 2) ? -1.0 : 1.0;
    DD p{sign * GBX_LIBM_LOAD(inv_fact, 2 * top), sign * GBX_LIBM_LOAD(inv_fact, 2 * top + 1)};
    for (int k = top - 2; k >= 0; k -= 2)
    {
        p = dd_mul(p, z);
        sign = ((k / 2) % 2) ? -1.0 : 1.0;
        p = dd_add(p, DD{sign * GBX_LIBM_LOAD(inv_fact, 2 * k), sign * GBX_LIBM_LOAD(inv_fact, 2 * k + 1)});
    }
    return odd ? dd_mul(p, r) : p;
}

//! sin (quadrant offset 0) or cos (offset 1) of x, correctly rounded
GBX_FORCEINLINE double sin_cos(double x, int offset)
{
    int q;
    DD r = trig_reduce(x, &q);
    q = (q + offset) & 3;
    bool const odd = (q & 1) == 0;
    DD v = odd ? sin_core(r) : cos_core(r);
    double y;
    // Fast-path error: below 2^-60.4 measured, bound taken 4x larger
    if (rounds_surely(v.hi, v.lo, 0x1p-58))
    {
        y = v.hi + v.lo;
    }
    else
    {
        v = trig_accurate(r, odd);
        y = v.hi + v.lo;
    }
    return (q & 2) ? -y : y;
}
}  // namespace detail

//! sin(x), correctly rounded for |x| < 2^20 pi/2
GBX_NOINLINE double sin(double x)
{
#if defined(GBX_SYSTEM_LIBM)
    return std::sin(x);
#else
    if (!(std::fabs(x) <= 0x1.fffffffffffffp+1023))
        return (x - x) / (x - x);
    if (std::fabs(x) < 0x1p-26)
        return x;
    return detail::sin_cos(x, 0);
#endif
}

//! cos(x), correctly rounded for |x| < 2^20 pi/2
GBX_NOINLINE double cos(double x)
{
#if defined(GBX_SYSTEM_LIBM)
    return std::cos(x);
#else
    if (!(std::fabs(x) <= 0x1.fffffffffffffp+1023))
        return (x - x) / (x - x);
    if (std::fabs(x) < 0x1p-27)
        return 1.0;
    return detail::sin_cos(x, 1);
#endif
}

namespace detail
{
//! expm1(x) as a double-double for |x| <= 0.35 (Taylor series)
GBX_FORCEINLINE DD expm1_small(double x)
{
    // x^3 (1/3! + x (1/4! + ... + x^13/17!)), x^3 and its 1/6 in
    // double-double
    double p = GBX_LIBM_LOAD(inv_fact, 2 * 17);
    for (int k = 16; k >= 4; --k)
        p = fma_(x, p, GBX_LIBM_LOAD(inv_fact, 2 * k));
    DD h = two_prod(x, x);
    DD c3{x * h.hi, fma_(x, h.hi, -(x * h.hi)) + x * h.lo};
    DD xp = two_prod(x, p);
    DD f = two_sum(GBX_LIBM_LOAD(inv_fact, 6), xp.hi);
    f.lo += xp.lo + GBX_LIBM_LOAD(inv_fact, 7);
    DD u = dd_mul(c3, f);
    h.hi *= 0.5;
    h.lo *= 0.5;
    DD s = two_sum(x, h.hi);
    DD t = two_sum(s.hi, u.hi);
    t.lo += s.lo + h.lo + u.lo;
    return fast_two_sum(t.hi, t.lo);
}

//! expm1(x) to about 2^-100 for |x| <= 0.35: Horner in double-double to
//! x^27/27!
GBX_NOINLINE DD expm1_small_accurate(double x)
{
    DD p{GBX_LIBM_LOAD(inv_fact, 54), GBX_LIBM_LOAD(inv_fact, 55)};
    for (int k = 26; k >= 1; --k)
    {
        p = dd_mul_d(p, x);
        p = dd_add(p, DD{GBX_LIBM_LOAD(inv_fact, 2 * k), GBX_LIBM_LOAD(inv_fact, 2 * k + 1)});
    }
    return dd_mul_d(p, x);
}

//! expm1(x) as a double-double, any finite x above -745; 'accurate' selects
//! the slower series near zero
GBX_FORCEINLINE DD expm1_dd(double x, bool accurate = false)
{
    if (std::fabs(x) <= 0.35)
        return accurate ? expm1_small_accurate(x) : expm1_small(x);
    int m;
    DD e = exp_dd(x, &m);
    if (m > 1000)
        return {(e.hi + e.lo) * 2.0 * pow2(m - 1), 0.0};  // exp(x) - 1 = exp(x)
    double const sc = m >= -1022 ? pow2(m) : 0.0;
    DD s = two_sum(e.hi * sc, -1.0);
    s.lo += e.lo * sc;
    return fast_two_sum(s.hi, s.lo);
}
}  // namespace detail

//! exp(x) - 1, correctly rounded
GBX_NOINLINE double expm1(double x)
{
#if defined(GBX_SYSTEM_LIBM)
    return std::expm1(x);
#else
    using namespace detail;
    if (!(x == x))
        return x + x;
    if (x > 0x1.62e42fefa39efp+9)
        return x * 0x1p1023 * 2.0;
    if (x < -40.0)
        return -1.0;
    if (std::fabs(x) < 0x1p-54)
        return x;
    DD v = expm1_dd(x);
    // Series error near zero: below 2^-61.5 measured, bound taken 4x larger
    if (std::fabs(x) <= 0.35 && !rounds_surely(v.hi, v.lo, 0x1p-59))
        v = expm1_small_accurate(x);
    return v.hi + v.lo;
#endif
}

//! log(1 + x), correctly rounded
GBX_NOINLINE double log1p(double x)
{
#if defined(GBX_SYSTEM_LIBM)
    return std::log1p(x);
#else
    using namespace detail;
    if (!(x > -1.0) || x > 0x1.fffffffffffffp+1023)
    {
        if (x == -1.0)
            return -HUGE_VAL;
        if (x < -1.0)
            return (x - x) / (x - x);
        return x + x;
    }
    if (std::fabs(x) < 0x1p-54)
        return x;
    if (std::fabs(x) < 0x1p-7)
    {
        DD v = log1p_small_accurate(DD{x, 0.0});
        return v.hi + v.lo;
    }
    // 1 + x as a double-double; log(uh + ul) = log(uh) + ul / uh
    DD u = two_sum(1.0, x);
    DD v = log_dd(u.hi);
    v = dd_add(v, DD{u.lo / u.hi, 0.0});
    return v.hi + v.lo;
#endif
}

//! tanh(x), correctly rounded
GBX_NOINLINE double tanh(double x)
{
#if defined(GBX_SYSTEM_LIBM)
    return std::tanh(x);
#else
    using namespace detail;
    if (!(x == x))
        return x + x;
    double const ax = std::fabs(x);
    if (ax < 0x1p-27)
        return x;
    double y;
    if (ax >= 22.0)
    {
        y = 1.0;
    }
    else
    {
        // tanh |x| = E / (E + 2), E = expm1(2 |x|)
        DD e = expm1_dd(2 * ax);
        DD q = dd_div(e, dd_add(e, DD{2.0, 0.0}));
        if (!rounds_surely(q.hi, q.lo, 0x1p-58))
        {
            e = expm1_dd(2 * ax, true);
            q = dd_div(e, dd_add(e, DD{2.0, 0.0}));
        }
        y = q.hi + q.lo;
    }
    return x < 0 ? -y : y;
#endif
}

//! Cube root, correctly rounded
GBX_NOINLINE double cbrt(double x)
{
#if defined(GBX_SYSTEM_LIBM)
    return std::cbrt(x);
#else
    using namespace detail;
    if (!(std::fabs(x) <= 0x1.fffffffffffffp+1023) || x == 0)
        return x + x;
    double ax = std::fabs(x);
    int bias = 0;
    if (ax < 0x1p-1022)
    {
        ax *= 0x1p54;
        bias = -18;
    }
    // ax = 2^(3k) w, w in [1, 8)
    std::uint64_t const u = bits(ax);
    int const e = static_cast<int>((u >> 52) & 0x7ff) - 1023;
    int k = e >= 0 ? e / 3 : -((-e + 2) / 3);
    // 2^(-3k) in two factors: -3k reaches -1023
    double const w = ax * pow2(-3 * k / 2) * pow2(-3 * k - (-3 * k / 2));
    double y = exp(log(w) / 3.0);
    // One Newton step in double-double: y - (y^3 - w) / (3 y^2)
    DD y2 = two_prod(y, y);
    DD y3 = dd_mul_d(y2, y);
    DD d = dd_add(y3, DD{-w, 0.0});
    y = y - d.hi / (3.0 * y2.hi);
    // Correct rounding: y in [1, 2) is the nearest double to cbrt(w) when
    // (y - 2^-53)^3 < w < (y + 2^-53)^3, the cubes of the midpoints in
    // double-double
    auto cube_minus_w = [w](double hi, double lo) {
        DD m{hi, lo};
        DD c = dd_mul(dd_mul(m, m), m);
        return dd_add(c, DD{-w, 0.0}).hi;
    };
    if (cube_minus_w(y, 0x1p-53) < 0)
        y = from_bits(bits(y) + 1);
    else if (cube_minus_w(y, -0x1p-53) > 0)
        y = from_bits(bits(y) - 1);
    double r = y * pow2(k + bias);
    return x < 0 ? -r : r;
#endif
}

//! FP32 overloads: the C++ library's functions (mixed-precision physics)
GBX_FORCEINLINE float exp(float x)
{
    return std::exp(x);
}
GBX_FORCEINLINE float log(float x)
{
    return std::log(x);
}
GBX_FORCEINLINE float sin(float x)
{
    return std::sin(x);
}
GBX_FORCEINLINE float cos(float x)
{
    return std::cos(x);
}
GBX_FORCEINLINE float expm1(float x)
{
    return std::expm1(x);
}
GBX_FORCEINLINE float log1p(float x)
{
    return std::log1p(x);
}
GBX_FORCEINLINE float tanh(float x)
{
    return std::tanh(x);
}
GBX_FORCEINLINE float cbrt(float x)
{
    return std::cbrt(x);
}

}  // namespace libm
}  // namespace gbx
