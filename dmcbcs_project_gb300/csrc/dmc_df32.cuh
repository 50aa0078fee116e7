// Double-float ("double-word") arithmetic on the FP32 pipe.
//
// A value is hi + lo with |lo| <= ulp(hi)/2: about 48 significant bits,
// i.e. a unit roundoff near 2^-47 (7e-15) against 2^-53 for FP64, with the
// FP32 exponent range.  GB300 issues 128 FP32 FMAs per SM per cycle against 2
// FP64 FMAs, so a double-float multiply-add at ~11 FP32 instructions is ~5x
// cheaper than an FP64 one.
//
// Building blocks (error-free transformations): TwoSum (Knuth), FastTwoSum
// (Dekker, |a| >= |b|), TwoProd with FMA; the double-word sum and product
// follow the "accurate" algorithms analysed by Joldes, Muller and Popescu
// (ACM TOMS 44(2), 2017): DWPlusDW (relative error <= 3u^2) and DWTimesDW with
// FMA (<= 5u^2), u = 2^-24.  The GEMM accumulator `dfacc` keeps the running
// sum's leading part exact with TwoSum and adds all low-order terms into a
// plain FP32 tail, renormalised once at the end.
#pragma once

#include <cuda_runtime.h>

namespace dmc {

struct __align__(8) df {
    float hi, lo;
};

// The error-free transformations below spell their roundings with the _rn
// intrinsics, which the compiler never fuses into an FMA: a contracted
// s = fma(a, b, c) in place of s = fl(fl(a*b) + c) would break the identities
// the error terms rely on.
__device__ __forceinline__ df mkdf(float h, float l) { return df{h, l}; }
__device__ __forceinline__ df two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return df{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ df fast_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return df{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return df{p, fmaf(a, b, -p)};
}

__device__ __forceinline__ df operator+(df x, df y)
{
    const df s = two_sum(x.hi, y.hi);
    const df t = two_sum(x.lo, y.lo);
    const df v = fast_two_sum(s.hi, s.lo + t.hi);
    return fast_two_sum(v.hi, t.lo + v.lo);
}
__device__ __forceinline__ df operator-(df x) { return df{-x.hi, -x.lo}; }
__device__ __forceinline__ df operator-(df x, df y) { return x + (-y); }
__device__ __forceinline__ df operator*(df x, df y)
{
    const df c = two_prod(x.hi, y.hi);
    const float t = fmaf(x.lo, y.hi, fmaf(x.hi, y.lo, x.lo * y.lo));
    return fast_two_sum(c.hi, c.lo + t);
}
// double-float times float
__device__ __forceinline__ df operator*(df x, float y)
{
    const df c = two_prod(x.hi, y);
    return fast_two_sum(c.hi, fmaf(x.lo, y, c.lo));
}
__device__ __forceinline__ df& operator+=(df& a, df b) { return a = a + b; }
__device__ __forceinline__ df& operator-=(df& a, df b) { return a = a - b; }

__device__ __forceinline__ df fma(df a, df b, df c) { return a * b + c; }
using ::fma;   // keep the double overloads visible next to the double-float one

// reciprocal: one Newton step from the FP32 reciprocal of the leading part.
// For the correctly rounded y = 1/x.hi the residual 1 - x.hi*y is exact in
// FP32 (one FMA); the low part contributes -x.lo*y.
__device__ __forceinline__ df rcp(df x)
{
    const float y = __frcp_rn(x.hi);
    const float e = fmaf(-x.lo, y, fmaf(-x.hi, y, 1.0f));
    return fast_two_sum(y, y * e);
}
__device__ __forceinline__ df operator/(df a, df b) { return a * rcp(b); }

// square root: one Newton-like correction of sqrtf of the leading part
__device__ __forceinline__ df dsqrt(df x)
{
    if (x.hi <= 0.0f) return df{0.0f, 0.0f};
    const float s = sqrtf(x.hi);
    const df ss = two_prod(s, s);
    const float r = ((x.hi - ss.hi) - ss.lo + x.lo) / (2.0f * s);
    return fast_two_sum(s, r);
}

__device__ __forceinline__ df dabs(df x) { return x.hi < 0.0f ? -x : x; }
// |a| > |b| (ties broken by the low parts)
__device__ __forceinline__ bool abs_gt(df a, df b)
{
    const df x = dabs(a), y = dabs(b);
    return x.hi > y.hi || (x.hi == y.hi && x.lo > y.lo);
}
// a < b for normalised values (|lo| <= ulp(hi)/2): the leading parts
// decide unless they are equal
__device__ __forceinline__ bool lt(df a, df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool is_zero(df a) { return a.hi == 0.0f; }
__device__ __forceinline__ bool is_neg(df a) { return a.hi < 0.0f || (a.hi == 0.0f && a.lo < 0.0f); }
__host__ __device__ __forceinline__ double to_double(df a) { return (double)a.hi + (double)a.lo; }
__host__ __device__ __forceinline__ df from_double(double d)
{
    const float h = (float)d;
    return df{h, (float)(d - (double)h)};
}

// Accumulator for long dot products: hi is kept exact with TwoSum, every
// rounding error and low-order product goes into the FP32 tail.
struct dfacc {
    float hi, lo;
};
__device__ __forceinline__ void acc_init(dfacc& a) { a.hi = a.lo = 0.0f; }
__device__ __forceinline__ void acc_madd(dfacc& a, df x, df y)
{
    const float p = __fmul_rn(x.hi, y.hi);
    float pe = fmaf(x.hi, y.hi, -p);
    pe = fmaf(x.hi, y.lo, pe);
    pe = fmaf(x.lo, y.hi, pe);
    const float s = __fadd_rn(a.hi, p);
    const float bb = __fsub_rn(s, a.hi);
    const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    a.hi = s;
    a.lo += e + pe;
}
__device__ __forceinline__ void acc_add(dfacc& a, df x)
{
    const float s = __fadd_rn(a.hi, x.hi);
    const float bb = __fsub_rn(s, a.hi);
    const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(x.hi, bb));
    a.hi = s;
    a.lo += e + x.lo;
}
__device__ __forceinline__ df acc_value(const dfacc& a) { return fast_two_sum(a.hi, a.lo); }

// Dot products with a known bound on sum |x_j y_j|, after Rump, Ogita and
// Oishi's ExtractScalar (Accurate floating-point summation part I, SIAM J.
// Sci. Comput. 31(1), 2008).  With sigma = 2^k >= 4 sum |x_j y_j|, the
// running value T = sigma + (partial sum) stays in [3 sigma/4, 5 sigma/4]:
// each step T' = fl(T + x*y) is one FMA, its change q = T' - T is exact by
// Sterbenz's lemma, and the remainder x*y - q (one FMA, one rounding) goes
// into an FP32 tail; the products with the low parts go into a second tail.
// At the end T - sigma is exact.  6 FP32 instructions per multiply-add (12
// for dfacc); error of order n 2^-48 sigma for n terms.
struct bacc {
    float t, e, c;
};
__device__ __forceinline__ void bacc_init(bacc& a, float sigma)
{
    a.t = sigma;
    a.e = a.c = 0.0f;
}
__device__ __forceinline__ void bacc_madd(bacc& a, df x, df y)
{
    const float t = fmaf(x.hi, y.hi, a.t);
    const float q = __fsub_rn(t, a.t);
    a.t = t;
    a.e = __fadd_rn(a.e, fmaf(x.hi, y.hi, -q));
    a.c = fmaf(x.hi, y.lo, a.c);
    a.c = fmaf(x.lo, y.hi, a.c);
}
__device__ __forceinline__ df bacc_value(const bacc& a, float sigma)
{
    return two_sum(__fsub_rn(a.t, sigma), __fadd_rn(a.e, a.c));
}
// smallest power of two >= v for finite v > 0 (2^-100 for v = 0)
__device__ __forceinline__ float pow2_ceil(float v)
{
    if (!(v > 0.0f)) return 7.8886091e-31f;
    const int b = __float_as_int(v);
    return __int_as_float((b + 0x007fffff) & 0x7f800000);
}

// ---- the same interface for double, so kernels can be written once --------

__device__ __forceinline__ double rcp(double x) { return 1.0 / x; }
__device__ __forceinline__ double dsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ double dabs(double x) { return fabs(x); }
// magnitude comparisons on the bit patterns (integer pipe, finite values)
__device__ __forceinline__ bool abs_gt(double a, double b)
{
    const unsigned long long m = 0x7fffffffffffffffull;
    return ((unsigned long long)__double_as_longlong(a) & m) > ((unsigned long long)__double_as_longlong(b) & m);
}
__device__ __forceinline__ bool is_zero(double a) { return ((unsigned long long)__double_as_longlong(a) << 1) == 0ull; }
__device__ __forceinline__ bool is_neg(double a) { return __double_as_longlong(a) < 0 && !is_zero(a); }
__host__ __device__ __forceinline__ double to_double(double a) { return a; }

struct dacc64 {
    double v;
};
__device__ __forceinline__ void acc_init(dacc64& a) { a.v = 0.0; }
__device__ __forceinline__ void acc_madd(dacc64& a, double x, double y) { a.v = fma(x, y, a.v); }
__device__ __forceinline__ void acc_add(dacc64& a, double x) { a.v += x; }
__device__ __forceinline__ double acc_value(const dacc64& a) { return a.v; }

template <class R>
struct AccOf;
template <>
struct AccOf<double> {
    using type = dacc64;
};
template <>
struct AccOf<df> {
    using type = dfacc;
};

template <class R>
__device__ __forceinline__ R rzero();
template <>
__device__ __forceinline__ double rzero<double>() { return 0.0; }
template <>
__device__ __forceinline__ df rzero<df>() { return df{0.0f, 0.0f}; }

template <class R>
__device__ __forceinline__ R rone();
template <>
__device__ __forceinline__ double rone<double>() { return 1.0; }
template <>
__device__ __forceinline__ df rone<df>() { return df{1.0f, 0.0f}; }

}  // namespace dmc
