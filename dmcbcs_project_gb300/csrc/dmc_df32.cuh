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

__device__ __forceinline__ df mkdf(float h, float l) { return df{h, l}; }
__device__ __forceinline__ df two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    return df{s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ df fast_two_sum(float a, float b)
{
    const float s = a + b;
    return df{s, b - (s - a)};
}
__device__ __forceinline__ df two_prod(float a, float b)
{
    const float p = a * b;
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

// reciprocal: one Newton step from the FP32 reciprocal of the leading part
__device__ __forceinline__ df rcp(df x)
{
    const float y = __frcp_rn(x.hi);
    const df e = df{1.0f, 0.0f} - x * y;          // 1 - x*y, exact to double-float accuracy
    return fast_two_sum(y, y * e.hi);
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
    const float p = x.hi * y.hi;
    float pe = fmaf(x.hi, y.hi, -p);
    pe = fmaf(x.hi, y.lo, pe);
    pe = fmaf(x.lo, y.hi, pe);
    const float s = a.hi + p;
    const float bb = s - a.hi;
    const float e = (a.hi - (s - bb)) + (p - bb);
    a.hi = s;
    a.lo += e + pe;
}
__device__ __forceinline__ void acc_add(dfacc& a, df x)
{
    const float s = a.hi + x.hi;
    const float bb = s - a.hi;
    const float e = (a.hi - (s - bb)) + (x.hi - bb);
    a.hi = s;
    a.lo += e + x.lo;
}
__device__ __forceinline__ df acc_value(const dfacc& a) { return fast_two_sum(a.hi, a.lo); }

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
