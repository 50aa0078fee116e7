// Elementary functions in double-float arithmetic for the mixed path: sin and
// cos of pi*a, and the natural logarithm, evaluated on the FP32 pipe.
//
// GB300 runs FP64 at 2 FMAs per SM per cycle, so one FP64 warp instruction
// holds an SM sub-partition's FP64 pipe for about 64 cycles; the library
// sincospi/log in FP64 cost a few thousand cycles per warp.  These versions
// use truncated series with exact rational coefficients (the Taylor series
// of sin and cos, the atanh series of log), not fitted approximations:
//   sin x = x sum_k (-1)^k y^k / (2k+1)!,   cos x = sum_k (-1)^k y^k / (2k)!,
//   y = x^2, |x| <= pi/4 after reduction by quarter turns;
//   log m = 2 z sum_k z^(2k) / (2k+1),  z = (m-1)/(m+1),  m in [sqrt(1/2), sqrt(2)).
// The high-order terms, whose sum is below 2^-24 of the result, are summed
// in FP32; the rest in double-float.  Accuracy is a few units of 2^-48
// relative (absolute for sin/cos), checked against the FP64 library
// functions by the GPU tests.
#pragma once

#include "dmc_df32.cuh"

namespace dmc {
namespace dfm {

// compile-time split of a double constant into a double-float
struct dfc {
    float hi, lo;
};
constexpr dfc split(double v) { return dfc{(float)v, (float)(v - (double)(float)v)}; }
constexpr double inv_fact(int n) { return n <= 1 ? 1.0 : inv_fact(n - 1) / (double)n; }

__device__ __forceinline__ df mk(dfc c) { return df{c.hi, c.lo}; }

// double-float plus float
__device__ __forceinline__ df add_f(df x, float y)
{
    const df s = two_sum(x.hi, y);
    return fast_two_sum(s.hi, s.lo + x.lo);
}

constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr double kLn2 = 0.693147180559945309417232121458176568;

// series coefficients (compile-time constants)
constexpr dfc kPiDf = split(kPi);
constexpr dfc kLn2Df = split(kLn2);
// sin: (-1)^k / (2k+1)!
constexpr float kS8 = (float)inv_fact(17), kS7 = (float)(-inv_fact(15)), kS6 = (float)inv_fact(13),
                kS5 = (float)(-inv_fact(11));
constexpr dfc kS4 = split(inv_fact(9)), kS3 = split(-inv_fact(7)), kS2 = split(inv_fact(5)),
              kS1 = split(-1.0 / 6.0);
// cos, as 1 - y sum_k (-1)^k y^k / (2k+2)!
constexpr float kC9 = (float)inv_fact(18), kC8 = (float)(-inv_fact(16)), kC7 = (float)inv_fact(14),
                kC6 = (float)(-inv_fact(12)), kC5 = (float)inv_fact(10);
constexpr dfc kC4 = split(-inv_fact(8)), kC3 = split(inv_fact(6)), kC2 = split(-inv_fact(4)), kC1 = split(0.5);
// atanh: 1 / (2k+1)
constexpr float kL10 = (float)(1.0 / 21.0), kL9 = (float)(1.0 / 19.0), kL8 = (float)(1.0 / 17.0),
                kL7 = (float)(1.0 / 15.0), kL6 = (float)(1.0 / 13.0), kL5 = (float)(1.0 / 11.0);
constexpr dfc kL4 = split(1.0 / 9.0), kL3 = split(1.0 / 7.0), kL2 = split(1.0 / 5.0), kL1 = split(1.0 / 3.0);

// sin(x), cos(x) for |x| <= pi/4 + a few ulp
__device__ __forceinline__ void sincos_small(df x, df& s, df& c)
{
    const df y = x * x;
    const float yh = y.hi;
    // sin: x * S(y); terms k >= 5 in FP32 (|c_5 y^5| < 2.3e-9)
    float sf = kS8;
    sf = fmaf(sf, yh, kS7);
    sf = fmaf(sf, yh, kS6);
    sf = fmaf(sf, yh, kS5);
    df sp = df{sf, 0.0f};
    sp = sp * y + mk(kS4);
    sp = sp * y + mk(kS3);
    sp = sp * y + mk(kS2);
    sp = sp * y + mk(kS1);
    sp = sp * y;   // S(y) - 1
    s = x + x * sp;
    // cos: terms k >= 5 in FP32 (|y^5 / 10!| < 2.5e-8)
    float cf = kC9;
    cf = fmaf(cf, yh, kC8);
    cf = fmaf(cf, yh, kC7);
    cf = fmaf(cf, yh, kC6);
    cf = fmaf(cf, yh, kC5);
    df cp = df{cf, 0.0f};
    cp = cp * y + mk(kC4);
    cp = cp * y + mk(kC3);
    cp = cp * y + mk(kC2);
    cp = cp * y + mk(kC1);
    // cos = 1 - y (1/2 - y/4! + ...)
    c = add_f(-(cp * y), 1.0f);
}

// quarter-turn rotation: (sin, cos) of r*pi + k*pi/2 from those of r*pi
__device__ __forceinline__ void rotate(int k, df sr, df cr, df& s, df& c)
{
    switch (k & 3) {
        case 0: s = sr; c = cr; break;
        case 1: s = cr; c = -sr; break;
        case 2: s = -sr; c = -cr; break;
        default: s = -cr; c = sr; break;
    }
}

// sin(pi a), cos(pi a) for |a| < 2^22
__device__ __forceinline__ void sincospi_df(df a, df& s, df& c)
{
    const float k = rintf(2.0f * a.hi);
    // a.hi - k/2 is exact (Sterbenz: a.hi and k/2 are within a factor of two
    // whenever k != 0)
    const df r = two_sum(__fsub_rn(a.hi, 0.5f * k), a.lo);
    df sr, cr;
    sincos_small(r * mk(kPiDf), sr, cr);
    rotate((int)k, sr, cr, s, c);
}

// sin(2 pi u), cos(2 pi u) for the uniform deviate u = m 2^-48, 0 < m < 2^48,
// reduced exactly in integer arithmetic: 2u = m 2^-47 = k/2 + d 2^-47 with
// |d| <= 2^45, so r = d 2^-47 is exact in double-float
__device__ __forceinline__ void sincos2pi_u48(unsigned long long m, df& s, df& c)
{
    const long long k = (long long)((m + (1ull << 45)) >> 46);
    const long long d = (long long)m - (k << 46);
    const long long dh = d >> 23;                       // |dh| <= 2^22
    const long long dl = d - (dh << 23);                // 0 <= dl < 2^23
    const df r = two_sum((float)dh * 5.9604644775390625e-8f, (float)dl * 7.105427357601002e-15f);
    df sr, cr;
    sincos_small(r * mk(kPiDf), sr, cr);
    rotate((int)k, sr, cr, s, c);
}

// the uniform deviate m 2^-48 as an exact double-float
__device__ __forceinline__ df u48(unsigned long long m)
{
    const float h = (float)(unsigned)(m >> 24) * 5.9604644775390625e-8f;       // 2^-24
    const float l = (float)(unsigned)(m & 0xffffffull) * 3.552713678800501e-15f;  // 2^-48
    return two_sum(h, l);
}

// natural logarithm of a positive normal double-float
__device__ __forceinline__ df log_df(df x)
{
    // x.hi = f 2^e with f in [1/2, 1); choose e so that m = x 2^-e is in
    // [sqrt(1/2), sqrt(2))
    const int bits = __float_as_int(x.hi);
    int e = ((bits >> 23) & 0xff) - 126;
    const float f = __int_as_float((bits & 0x007fffff) | (126 << 23));
    if (f < 0.70710678f) e -= 1;
    const float sc = __int_as_float((127 - e) << 23);   // 2^-e, exact
    const df m = df{x.hi * sc, x.lo * sc};
    const df num = add_f(m, -1.0f);   // exact leading part: Sterbenz
    const df den = add_f(m, 1.0f);
    const df z = num / den;
    const df y = z * z;
    const float yh = y.hi;
    // terms k >= 5 of sum y^k / (2k+1) in FP32 (y <= 0.0295: c_5 y^5 < 2.1e-9)
    float pf = kL10;
    pf = fmaf(pf, yh, kL9);
    pf = fmaf(pf, yh, kL8);
    pf = fmaf(pf, yh, kL7);
    pf = fmaf(pf, yh, kL6);
    pf = fmaf(pf, yh, kL5);
    df p = df{pf, 0.0f};
    p = p * y + mk(kL4);
    p = p * y + mk(kL3);
    p = p * y + mk(kL2);
    p = p * y + mk(kL1);
    p = p * y;                            // sum - 1
    const df lm = z + z * p;              // log(m) / 2
    const df ln2e = mk(kLn2Df) * (float)e;
    return ln2e + df{2.0f * lm.hi, 2.0f * lm.lo};
}

// deterministic warp sum (xor butterfly) in double-float
__device__ __forceinline__ df warp_sum(df v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const df w = df{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
        v = v + w;
    }
    return v;
}

}  // namespace dfm
}  // namespace dmc
