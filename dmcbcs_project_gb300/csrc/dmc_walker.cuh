// Walker kernel stages of the GB300 DMCBS path, templated on the arithmetic
// of the determinant part:
//   R = double : the plain FP64 path,
//   R = df     : the mixed path (pair matrix, inverse and contractions in
//                double-float on the FP32 pipe; Jastrow and potential in FP32).
//
// One CTA of 256 threads owns one walker at a time (persistent grid over
// the population).  The whole wavefunction evaluation of a walker stays on
// chip: positions, k-vector records, the nd x nd pair matrix and its
// inverse, the pair-orbital matrices U (up x K) and D (down x K), the beta
// pair terms and the reduction scratch.  Global memory is touched only to
// read the walker, the tables (L2-resident) and to write the results.
//
// The reference computes the determinant drift and Laplacian from five
// GEMMs (psislaterbcs.f90:278-281) and the contractions with the inverse
// (:211-223).  Here the same quantities come from three products:
//   S = U D^T (+ beta),  G = D^T-rows . S^-1 (up drift/Laplacian),
//   H = S^-1 . U (down drift/Laplacian),
// using that the orbital derivatives are the orbitals of the partner column
// times k (cos' = -k sin, sin' = k cos) and that the Laplacian is -|k|^2
// times the orbital: 3 nd^2 K instead of 5 nd^2 K multiply-adds.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "dmc_device.cuh"
#include "dmc_dfmath.cuh"

namespace dmc {
namespace walker {

constexpr unsigned long long kMask48 = (1ull << 48) - 1ull;
constexpr double kTwoM48 = 1.0 / 281474976710656.0;

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Deterministic block sum of NV values (fixed tree); the result is returned
// in v on every thread.
template <int NV, int NT = kThreads>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* red)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = warp_sum(v[q]);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) red[w * NV + q] = v[q];
    __syncthreads();
    if (threadIdx.x < NV) {
        double s = 0.0;
        for (int k = 0; k < (NT / 32); ++k) s += red[k * NV + threadIdx.x];
        red[(NT / 32) * NV + threadIdx.x] = s;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = red[(NT / 32) * NV + q];
    __syncthreads();
}

// Deterministic block sum of NV values held by the first nw warps (the
// other warps hold zeros and skip the shuffles), in the value type T
// (double, or double-float on the FP32 pipe).  The result is returned in v
// on every thread.
__device__ __forceinline__ double wsum(double v) { return warp_sum(v); }
__device__ __forceinline__ df wsum(df v) { return dfm::warp_sum(v); }
template <int NV, int NT, class T>
__device__ __forceinline__ void block_sum_t(T (&v)[NV], T* red, int nw = NT / 32)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (w < nw) {
#pragma unroll
        for (int q = 0; q < NV; ++q) v[q] = wsum(v[q]);
        if (lane == 0)
#pragma unroll
            for (int q = 0; q < NV; ++q) red[w * NV + q] = v[q];
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        T s = red[threadIdx.x];
        for (int k = 1; k < nw; ++k) s = s + red[k * NV + threadIdx.x];
        red[(NT / 32) * NV + threadIdx.x] = s;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = red[(NT / 32) * NV + q];
    __syncthreads();
}

// 48-bit LCG state after t steps of ran1 (ran.f90:8-27), from jump tables:
// state_t = A_t * state_0 + C_t (mod 2^48).
__device__ __forceinline__ unsigned long long lcg_jump(unsigned long long s0, const unsigned long long* A,
                                                       const unsigned long long* Cc, int t)
{
    return (A[t] * s0 + Cc[t]) & kMask48;
}
__device__ __forceinline__ double lcg_uniform(unsigned long long s) { return (double)(s | 1ull) * kTwoM48; }

// minimum-image separation component
// Division of loop indices by a runtime divisor d >= 1 with one multiply-high:
// q = umulhi(e, m), m = floor((2^32 - 1) / d) + 1, is e / d for every
// e * d < 2^32 (here e <= 256^2 and d <= 256); the divider is built once per loop.
struct UDiv {
    unsigned d, m;
    __device__ __forceinline__ explicit UDiv(int dd) : d((unsigned)dd), m(dd > 1 ? 0xffffffffu / (unsigned)dd + 1u : 0u) {}
    __device__ __forceinline__ int quo(int e) const { return d > 1 ? (int)__umulhi((unsigned)e, m) : e; }
};

__device__ __forceinline__ double min_image(double d, const DevParams& p) { return d - p.el * rint(d * p.eli); }
__device__ __forceinline__ df min_image(df d, const DevParams& p)
{
    const float m = rintf(d.hi * p.eli_f);
    // |m| <= 2 (positions in or next to the box): m L is exact in double-float
    const df ml = fabsf(m) <= 2.0f ? df{p.el_df.hi * m, p.el_df.lo * m} : p.el_df * m;
    return d - ml;
}
// |d|^2 of a displacement: one accumulator for the double-float path
__device__ __forceinline__ double norm2(double a, double b, double c) { return a * a + b * b + c * c; }
__device__ __forceinline__ df norm2(df a, df b, df c)
{
    dfacc s;
    acc_init(s);
    acc_madd(s, a, a);
    acc_madd(s, b, b);
    acc_madd(s, c, c);
    return acc_value(s);
}

// ---- precision traits --------------------------------------------------------

template <class R>
struct Prec;
template <>
struct Prec<double> {
    using J = double;   // Jastrow / potential arithmetic
    using Tab = TabUD;
    using TabS = TabSS;
    using KV = KVecDev;
    static __device__ const Tab* tud(const KernelArgs& a) { return a.tud; }
    static __device__ const TabS* tss(const KernelArgs& a) { return a.tss; }
    static __device__ const KV* kv(const KernelArgs& a) { return a.kv; }
};
template <>
struct Prec<df> {
    using J = df;
    using Tab = TabUDmp;
    using TabS = TabSSmp;
    using KV = KVecMP;
    static __device__ const Tab* tud(const KernelArgs& a) { return a.tud_mp; }
    static __device__ const TabS* tss(const KernelArgs& a) { return a.tss_mp; }
    static __device__ const KV* kv(const KernelArgs& a) { return a.kv_mp; }
};

template <class T>
struct is_df {
    static constexpr bool value = false;
};
template <>
struct is_df<df> {
    static constexpr bool value = true;
};

// convert a double (positions, sincos results) into the arithmetic type
template <class R>
__device__ __forceinline__ R from_dbl(double d);
template <>
__device__ __forceinline__ double from_dbl<double>(double d) { return d; }
template <>
__device__ __forceinline__ df from_dbl<df>(double d) { return from_double(d); }

// x - a*b
__device__ __forceinline__ double fms(double x, double a, double b) { return fma(-a, b, x); }
__device__ __forceinline__ df fms(df x, df a, df b)
{
    dfacc t{x.hi, x.lo};
    acc_madd(t, -a, b);
    return acc_value(t);
}

// 4-point Lagrange weights on a uniform grid (coshpot.f90:172-179)
template <class T>
struct Lagrange {
    int idx;
    T c1, c2, c3, c4;
};
__device__ __forceinline__ Lagrange<double> lagrange(double r, double scale, int ntab)
{
    Lagrange<double> L;
    double dr = scale * r;
    int idx = (int)dr;
    idx = max(1, min(idx, ntab - 2));
    const double t = dr - (double)idx;
    const double tm1 = t - 1.0, tm2 = t - 2.0, tp1 = t + 1.0;
    L.idx = idx;
    L.c1 = -t * tm1 * tm2 / 6.0;
    L.c2 = tp1 * tm1 * tm2 / 2.0;
    L.c3 = -tp1 * t * tm2 / 2.0;
    L.c4 = tp1 * t * tm1 / 6.0;
    return L;
}
// double-float grid position: index and fraction t = scale*r - idx
__device__ __forceinline__ int grid_pos(df r, df scale, int ntab, df& frac)
{
    const df t = r * scale;
    int idx = (int)t.hi;
    df f = fast_two_sum(t.hi - (float)idx, t.lo);
    if (f.hi < 0.0f) {
        idx -= 1;
        f = f + df{1.0f, 0.0f};
    }
    const int ic = max(1, min(idx, ntab - 2));
    if (ic != idx) f = fast_two_sum(t.hi - (float)ic, t.lo);
    frac = f;
    return ic;
}
__device__ __forceinline__ Lagrange<df> lagrange_df(df t, int idx)
{
    Lagrange<df> L;
    const df tm1 = dfm::add_f(t, -1.0f), tm2 = dfm::add_f(t, -2.0f), tp1 = dfm::add_f(t, 1.0f);
    const df sixth = df{0.16666667163372040f, -4.9670538e-09f};
    const df p = t * tm1, q = tp1 * tm2;
    L.idx = idx;
    L.c1 = -(p * tm2) * sixth;
    L.c2 = (q * tm1) * 0.5f;
    L.c3 = -(q * t) * 0.5f;
    L.c4 = (p * tp1) * sixth;
    return L;
}
// 4-point combination c1 a0 + c2 a1 + c3 a2 + c4 a3: the cubic Lagrange
// weights on [0, 1) are at most 1.1 in magnitude, so 1.1 sum |a_k| bounds
// the terms of the bounded accumulator
__device__ __forceinline__ df lag4(const Lagrange<df>& W, df a0, df a1, df a2, df a3)
{
    const float b = (fabsf(a0.hi) + fabsf(a1.hi)) + (fabsf(a2.hi) + fabsf(a3.hi));
    const float sg = pow2_ceil(4.0f * 1.13f * b);
    bacc s;
    bacc_init(s, sg);
    bacc_madd(s, W.c1, a0);
    bacc_madd(s, W.c2, a1);
    bacc_madd(s, W.c3, a2);
    bacc_madd(s, W.c4, a3);
    return bacc_value(s, sg);
}
__device__ __forceinline__ Lagrange<float> lagrange_f(float t, int idx)
{
    Lagrange<float> L;
    const float tm1 = t - 1.0f, tm2 = t - 2.0f, tp1 = t + 1.0f;
    L.idx = idx;
    L.c1 = -t * tm1 * tm2 * (1.0f / 6.0f);
    L.c2 = tp1 * tm1 * tm2 * 0.5f;
    L.c3 = -tp1 * t * tm2 * 0.5f;
    L.c4 = tp1 * t * tm1 * (1.0f / 6.0f);
    return L;
}

template <class R, int NT = kThreads, bool BIG = false>
struct Ctx {
    static constexpr int nt = NT;   // threads of the walker CTA
    const DevParams& p;
    const KernelArgs& a;
    const SmemLayout& L;
    double* sm;
    double* pb;
    double* un;   // BIG: the union region in the CTA's global scratch slice
    // a region of the union (pair vectors, U, D, E, S2): on chip, or (BIG)
    // in the global slice at its offset from the union's start
    template <class T>
    __device__ __forceinline__ T* uat(int off) const
    {
        if constexpr (BIG)
            return reinterpret_cast<T*>(un + (off - L.R));
        else
            return reinterpret_cast<T*>(sm + off);
    }
};

// two consecutive values (16-byte aligned) with one shared-memory load
__device__ __forceinline__ void ld2(const double* p, double& a, double& b)
{
    const double2 v = *reinterpret_cast<const double2*>(p);
    a = v.x;
    b = v.y;
}
__device__ __forceinline__ void ld2(const df* p, df& a, df& b)
{
    const float4 v = *reinterpret_cast<const float4*>(p);
    a = df{v.x, v.y};
    b = df{v.z, v.w};
}

// typed views of the shared-memory regions
template <class T>
__device__ __forceinline__ T* at(double* sm, int off) { return reinterpret_cast<T*>(sm + off); }

// ---------------------------------------------------------------------------
// Stage 1: Jastrow + potential over all pairs (coshpot.f90:154-205) fused with
// the beta pair function (psislaterbcs.f90:283-293, betafun.f90:173-194).
// Up-down pairs are processed in row chunks; each pair stores its Jastrow
// gradient vector g = dx * u'/r, whose row sums (up) and column sums (down)
// are taken in a fixed order.  Writes S[i][j] = beta(r_ij) and the beta pair
// terms (f'/r, lap f) to pb.  Returns per-thread sums of u, v and the pair
// Laplacian part: jt[] for the up-down pairs in the Jastrow type, ss[] for
// the same-spin pairs (FP64 on both paths).
// ---------------------------------------------------------------------------
template <class R, int NT, bool BIG>
__device__ void pair_stage(const Ctx<R, NT, BIG>& c, typename Prec<R>::J (&jt)[3], double (&ss)[3])
{
    using J = typename Prec<R>::J;
    const DevParams& p = c.p;
    double* sm = c.sm;
    const R* x = at<R>(sm, c.L.xr);
    R* S = at<R>(sm, c.L.S);
    J* pv = c.template uat<J>(c.L.R);
    R* pb = reinterpret_cast<R*>(c.pb);
    double* du = sm + c.L.acc + 4 * p.npart;
    const int nup = p.nup, ndn = p.ndn, ldS = p.ldS;
    const auto* tud = Prec<R>::tud(c.a);
    const double imu_ud = 1.0 / (p.mass[0] * p.mass[1] / (p.mass[0] + p.mass[1]));
    const R imu_df = from_dbl<R>(imu_ud);
    (void)imu_df;
    for (int i = threadIdx.x; i < 3 * p.npart; i += NT) du[i] = 0.0;
    // per-thread partial sums in the Jastrow type
    J tu = rzero<J>(), tv = rzero<J>(), td = rzero<J>();
    __syncthreads();
    for (int r0 = 0; r0 < nup; r0 += c.L.rows_jas) {
        const int r1 = min(nup, r0 + c.L.rows_jas);
        const int npc = (r1 - r0) * ndn;
        const UDiv dv(ndn);
        for (int q = threadIdx.x; q < npc; q += NT) {
            const int qi = dv.quo(q);
            const int i = r0 + qi, j = q - qi * ndn;
            const R* xi = x + 3 * i;
            const R* xj = x + 3 * (nup + j);
            const R d0 = min_image(xi[0] - xj[0], p);
            const R d1 = min_image(xi[1] - xj[1], p);
            const R d2 = min_image(xi[2] - xj[2], p);
            const R rb = dsqrt(norm2(d0, d1, d2));
            const R rinv = rcp(rb);
            J g0 = rzero<J>(), g1 = rzero<J>(), g2 = rzero<J>();
            R f = rzero<R>(), dfr = rzero<R>(), d2f = rzero<R>();
            if constexpr (!is_df<R>::value) {
                // FP64: the reference's arithmetic (tiny clamp, separate grids)
                const double r = fmax(rb, 1.0e-14);
                if (r < p.range) {
                    const Lagrange<double> W = lagrange(r, p.scale, p.ntab);
                    const TabUD* T = c.a.tud + (W.idx - 1);
                    const TabUD A0 = T[0], A1 = T[1], A2 = T[2], A3 = T[3];
                    const double vp = W.c1 * A0.v + W.c2 * A1.v + W.c3 * A2.v + W.c4 * A3.v;
                    const double uj = W.c1 * A0.u + W.c2 * A1.u + W.c3 * A2.u + W.c4 * A3.u;
                    const double duj = W.c1 * A0.du + W.c2 * A1.du + W.c3 * A2.du + W.c4 * A3.du;
                    const double d2uj = W.c1 * A0.d2u + W.c2 * A1.d2u + W.c3 * A2.d2u + W.c4 * A3.d2u;
                    const double ri = (r == rb) ? rinv : 1.0 / r;
                    tv += vp;
                    tu += uj;
                    const double gf = duj * ri;
                    g0 = d0 * gf;
                    g1 = d1 * gf;
                    g2 = d2 * gf;
                    td += (d2uj + 2.0 * gf) * imu_ud;
                }
                if (!p.nobeta && !(rb > p.rangeb)) {
                    const Lagrange<double> W = lagrange(rb, p.scaleb, p.ntab);
                    const TabUD* T = c.a.tud + (W.idx - 1);
                    const TabUD A0 = T[0], A1 = T[1], A2 = T[2], A3 = T[3];
                    f = W.c1 * A0.b + W.c2 * A1.b + W.c3 * A2.b + W.c4 * A3.b;
                    const double df_ = W.c1 * A0.db + W.c2 * A1.db + W.c3 * A2.db + W.c4 * A3.db;
                    d2f = W.c1 * A0.d2b + W.c2 * A1.d2b + W.c3 * A2.d2b + W.c4 * A3.d2b;
                    dfr = df_ * rinv;
                }
            } else {
                // mixed: one double-float grid position for beta and Jastrow.
                // Inside the healing distance the Jastrow kinetic term and the
                // potential nearly cancel, so both stay in double-float there;
                // beyond it the Jastrow is exactly zero and only the
                // exponentially small potential tail is left (FP32).
                // full double-float comparisons: a pair within an FP32 ulp of
                // a range end must fall on the same side as in FP64
                const bool in_j = lt(rb, p.range_df);
                const bool in_b = !p.nobeta && !lt(p.rangeb_df, rb);
                if (in_j || in_b) {
                    df t;
                    const int idx = grid_pos(rb, p.scaleb_df, p.ntab, t);
                    const auto* T = tud + (idx - 1);
                    const auto A0 = T[0], A1 = T[1], A2 = T[2], A3 = T[3];
                    const Lagrange<df> W = lagrange_df(t, idx);
                    if (in_j) {
                        if (idx - 1 <= p.ntab0) {
                            const df vp = lag4(W, A0.v, A1.v, A2.v, A3.v);
                            const df uj = lag4(W, A0.u, A1.u, A2.u, A3.u);
                            const df duj = lag4(W, A0.du, A1.du, A2.du, A3.du);
                            const df d2uj = lag4(W, A0.d2u, A1.d2u, A2.d2u, A3.d2u);
                            const df gf = duj * rinv;
                            tv += vp;
                            tu += uj;
                            g0 = d0 * gf;
                            g1 = d1 * gf;
                            g2 = d2 * gf;
                            td += (d2uj + gf * 2.0f) * imu_df;
                        } else {
                            const float vp = W.c1.hi * A0.v.hi + W.c2.hi * A1.v.hi + W.c3.hi * A2.v.hi +
                                             W.c4.hi * A3.v.hi;
                            tv += df{vp, 0.0f};
                        }
                    }
                    if (in_b) {
                        f = lag4(W, A0.b, A1.b, A2.b, A3.b);
                        const df df_ = lag4(W, A0.db, A1.db, A2.db, A3.db);
                        d2f = lag4(W, A0.d2b, A1.d2b, A2.d2b, A3.d2b);
                        dfr = df_ * rinv;
                    }
                }
            }
            S[i * ldS + j] = f;
            R* pbq = pb + 2 * (i * ndn + j);
            pbq[0] = dfr;
            pbq[1] = d2f;
            pv[3 * q + 0] = g0;
            pv[3 * q + 1] = g1;
            pv[3 * q + 2] = g2;
        }
        __syncthreads();
        // row sums -> up particles (+), column sums -> down particles (-);
        // one thread per (particle, component)
        const int nr = r1 - r0;
        for (int tc = threadIdx.x; tc < 3 * (nr + ndn); tc += NT) {
            const int t = tc / 3, cmp = tc % 3;
            typename AccOf<J>::type sacc;
            acc_init(sacc);
            if (t < nr) {
                const J* row = pv + 3 * (t * ndn) + cmp;
                for (int j = 0; j < ndn; ++j) acc_add(sacc, row[3 * j]);
                du[3 * (r0 + t) + cmp] += to_double(acc_value(sacc)) * p.isqm[0];
            } else {
                const int j = t - nr;
                for (int r = 0; r < nr; ++r) acc_add(sacc, pv[3 * (r * ndn + j) + cmp]);
                du[3 * (nup + j) + cmp] -= to_double(acc_value(sacc)) * p.isqm[1];
            }
        }
        __syncthreads();
    }
    jt[0] = tu;
    jt[1] = tv;
    jt[2] = td;
    if (!p.ieq) return;
    double& su = ss[0];
    double& sv = ss[1];
    double& sd2 = ss[2];
    // same-spin pairs (coshpot.f90:167 with cjas(2) != 0): up-up then down-down,
    // in FP64 on both paths (off the benchmark configurations)
    const double* xd = sm + c.L.x;
    for (int blk = 0; blk < 2; ++blk) {
        const int n = blk == 0 ? nup : ndn;
        const int base = blk == 0 ? 0 : nup;
        const double imu = 1.0 / (p.mass[blk] * 0.5);
        const double isq = p.isqm[blk];
        if (n < 2) continue;
        double* pvd = c.template uat<double>(c.L.R);
        const int rows = max(1, c.L.rsize / (3 * n));
        for (int r0 = 0; r0 < n; r0 += rows) {
            const int r1 = min(n, r0 + rows);
            const int npc = (r1 - r0) * n;
            for (int q = threadIdx.x; q < npc; q += NT) {
                const int i = r0 + q / n, j = q % n;
                double g0 = 0.0, g1 = 0.0, g2 = 0.0;
                if (j > i) {
                    const double* xi = xd + 3 * (base + i);
                    const double* xj = xd + 3 * (base + j);
                    const double d0 = min_image(xi[0] - xj[0], p);
                    const double d1 = min_image(xi[1] - xj[1], p);
                    const double d2 = min_image(xi[2] - xj[2], p);
                    const double r = fmax(sqrt(d0 * d0 + d1 * d1 + d2 * d2), 1.0e-14);
                    if (r < p.range) {
                        const Lagrange<double> W = lagrange(r, p.scale, p.ntab);
                        const TabSS* T = c.a.tss + (W.idx - 1);
                        const TabSS A0 = T[0], A1 = T[1], A2 = T[2], A3 = T[3];
                        const double uj = W.c1 * A0.u + W.c2 * A1.u + W.c3 * A2.u + W.c4 * A3.u;
                        const double duj = W.c1 * A0.du + W.c2 * A1.du + W.c3 * A2.du + W.c4 * A3.du;
                        const double d2uj = W.c1 * A0.d2u + W.c2 * A1.d2u + W.c3 * A2.d2u + W.c4 * A3.d2u;
                        const double vp = W.c1 * A0.v + W.c2 * A1.v + W.c3 * A2.v + W.c4 * A3.v;
                        const double ri = 1.0 / r;
                        sv += vp;
                        su += uj;
                        const double gf = duj * ri;
                        g0 = d0 * gf;
                        g1 = d1 * gf;
                        g2 = d2 * gf;
                        sd2 += (d2uj + 2.0 * gf) * imu;
                    }
                }
                pvd[3 * q + 0] = g0;
                pvd[3 * q + 1] = g1;
                pvd[3 * q + 2] = g2;
            }
            __syncthreads();
            // row sums (+) then column sums (-): rows and columns are the
            // same particles here, so the two passes are separated by a
            // barrier (one thread per particle in each)
            const int nr = r1 - r0;
            for (int t = threadIdx.x; t < nr; t += NT) {
                double s0 = 0.0, s1 = 0.0, s2 = 0.0;
                const double* row = pvd + 3 * (t * n);
                for (int j = 0; j < n; ++j) {
                    s0 += row[3 * j];
                    s1 += row[3 * j + 1];
                    s2 += row[3 * j + 2];
                }
                const int i = base + r0 + t;
                du[3 * i + 0] += s0 * isq;
                du[3 * i + 1] += s1 * isq;
                du[3 * i + 2] += s2 * isq;
            }
            __syncthreads();
            for (int j = threadIdx.x; j < n; j += NT) {
                double s0 = 0.0, s1 = 0.0, s2 = 0.0;
                for (int r = 0; r < nr; ++r) {
                    const double* e = pvd + 3 * (r * n + j);
                    s0 += e[0];
                    s1 += e[1];
                    s2 += e[2];
                }
                du[3 * (base + j) + 0] -= s0 * isq;
                du[3 * (base + j) + 1] -= s1 * isq;
                du[3 * (base + j) + 2] -= s2 * isq;
            }
            __syncthreads();
        }
    }
}

// complex product in the arithmetic type
__device__ __forceinline__ void cmul(double ar, double ai, double br, double bi, double& cr, double& ci)
{
    cr = ar * br - ai * bi;
    ci = ar * bi + ai * br;
}
// product of two unit-modulus complex numbers (|a|, |b| <= 1 up to rounding):
// every partial product is below 1 in magnitude, so the bounded accumulator
// with sigma = 4 applies (6 instead of 12 FP32 instructions per term)
__device__ __forceinline__ void cmul_unit(double ar, double ai, double br, double bi, double& cr, double& ci)
{
    cr = ar * br - ai * bi;
    ci = ar * bi + ai * br;
}
__device__ __forceinline__ void cmul_unit(df ar, df ai, df br, df bi, df& cr, df& ci)
{
    bacc r, i;
    bacc_init(r, 4.0f);
    bacc_init(i, 4.0f);
    bacc_madd(r, ar, br);
    bacc_madd(r, -ai, bi);
    bacc_madd(i, ar, bi);
    bacc_madd(i, ai, br);
    cr = bacc_value(r, 4.0f);
    ci = bacc_value(i, 4.0f);
}
__device__ __forceinline__ void cmul(df ar, df ai, df br, df bi, df& cr, df& ci)
{
    dfacc r, i;
    acc_init(r);
    acc_init(i);
    acc_madd(r, ar, br);
    acc_madd(r, -ai, bi);
    acc_madd(i, ar, bi);
    acc_madd(i, ai, br);
    cr = acc_value(r);
    ci = acc_value(i);
}

// ---------------------------------------------------------------------------
// Stage 2: pair orbitals (psislaterbcs.f90:248-277).  exp(i k.x) is built
// from exp(i 2 pi x_c / L) and its integer powers, so each particle needs
// three sincos instead of one per k vector.
// U[i][0] = vorb(1), U[i][2q-1] = v_q cos(k_q.x_i), U[i][2q] = v_q sin(k_q.x_i)
// D[j][0] = 1,       D[j][2q-1] = cos(k_q.x_j),     D[j][2q] = sin(k_q.x_j)
// Then the unpaired plane-wave rows and columns of S (:171-206).
// ---------------------------------------------------------------------------
template <class R, int NT, bool BIG>
__device__ void orbital_stage(const Ctx<R, NT, BIG>& c)
{
    const DevParams& p = c.p;
    double* sm = c.sm;
    const double* x = sm + c.L.x;
    R* U = c.template uat<R>(c.L.U);
    R* D = c.template uat<R>(c.L.D);
    R* E = c.template uat<R>(c.L.E);
    R* S = at<R>(sm, c.L.S);
    const int np1 = p.nmax + 1;
    // powers e^{i m theta_c}, m = 0..nmax, E[(p*3+c)*np1 + m] = (re, im)
    for (int t = threadIdx.x; t < 3 * p.npart; t += NT) {
        R s1, c1;
        if constexpr (is_df<R>::value) {
            // base angle 2 pi x / L in double-float, off the FP64 pipe
            dfm::sincospi_df(at<R>(sm, c.L.xr)[t] * p.eli2_df, s1, c1);
        } else {
            sincospi(2.0 * x[t] * p.eli, &s1, &c1);
        }
        R* e = E + 2 * t * np1;
        e[0] = rone<R>();
        e[1] = rzero<R>();
        if (p.nmax >= 1) {
            e[2] = c1;
            e[3] = s1;
        }
        R cr = c1, ci = s1;
        for (int m = 2; m <= p.nmax; ++m) {
            R nr, ni;
            cmul_unit(cr, ci, c1, s1, nr, ni);
            cr = nr;
            ci = ni;
            e[2 * m] = cr;
            e[2 * m + 1] = ci;
        }
    }
    __syncthreads();
    // columns: (cos, sin) of k vector q at 2(q-1), 2(q-1)+1; the constant
    // term at 2 nq; zero padding up to ldU
    const int nq = p.nk - 1, nk = p.nk;
    // k-vector fields as arrays: lanes with consecutive k read consecutive words
    const R* kv_v = at<R>(sm, c.L.ksoa) + 4 * nk;
    const int* kn = reinterpret_cast<const int*>(at<R>(sm, c.L.ksoa) + 5 * nk);
    // item t = part * (nq + 1) + q; (part, q) advance incrementally.  The
    // product of the three component powers is taken branch-free: a zero
    // component multiplies by e^0 = (1, 0), which is exact.
    const int nq1 = nq + 1, items = p.npart * nq1;
    const int dpart = NT / nq1, dq = NT % nq1;
    int part = (int)threadIdx.x / nq1, q = (int)threadIdx.x % nq1;
    for (int t = threadIdx.x; t < items; t += NT) {
        const bool up = part < p.nup;
        R* row = up ? U + part * p.ldU : D + (part - p.nup) * p.ldU;
        if (q == 0) {
            row[2 * nq] = up ? kv_v[0] : rone<R>();
            for (int z = 2 * nq + 1; z < p.ldU; ++z) row[z] = rzero<R>();
        } else {
            const R* eb = E + 2 * (part * 3 * np1);
            const int n0 = kn[q];
            const R* e0 = eb + 2 * (n0 < 0 ? -n0 : n0);
            R zr = e0[0], zi = n0 < 0 ? -e0[1] : e0[1];
#pragma unroll
            for (int cc = 1; cc < 3; ++cc) {
                const int n = kn[cc * nk + q];
                const R* e = eb + 2 * (cc * np1 + (n < 0 ? -n : n));
                const R er = e[0], ei = n < 0 ? -e[1] : e[1];
                R nr, ni;
                cmul_unit(zr, zi, er, ei, nr, ni);
                zr = nr;
                zi = ni;
            }
            if (up) {
                const R kvq = kv_v[q];
                row[2 * q - 2] = kvq * zr;
                row[2 * q - 1] = kvq * zi;
            } else {
                row[2 * q - 2] = zr;
                row[2 * q - 1] = zi;
            }
        }
        part += dpart;
        q += dq;
        if (q >= nq1) {
            q -= nq1;
            ++part;
        }
    }
    // unpaired plane waves: up columns ndn.., down rows nup.., zero corner
    const int ldS = p.ldS;
    for (int t = threadIdx.x; t < p.nup * p.nexup; t += NT) {
        const int i = t / p.nexup, jj = t % p.nexup;
        const double* xi = x + 3 * i;
        const double arg = p.akup[jj][0] * xi[0] + p.akup[jj][1] * xi[1] + p.akup[jj][2] * xi[2];
        double s, co;
        sincos(arg, &s, &co);
        S[i * ldS + p.ndn + jj] = from_dbl<R>(p.sinup[jj] ? s : co);
    }
    for (int t = threadIdx.x; t < p.ndn * p.nexdn; t += NT) {
        const int j = t / p.nexdn, jj = t % p.nexdn;
        const double* xj = x + 3 * (p.nup + j);
        const double arg = p.akdn[jj][0] * xj[0] + p.akdn[jj][1] * xj[1] + p.akdn[jj][2] * xj[2];
        double s, co;
        sincos(arg, &s, &co);
        S[(p.nup + jj) * ldS + j] = from_dbl<R>(p.sindn[jj] ? s : co);
    }
    for (int t = threadIdx.x; t < p.nexdn * p.nexup; t += NT) {
        const int r = t / p.nexup, cc = t % p.nexup;
        S[(p.nup + r) * ldS + p.ndn + cc] = rzero<R>();
    }
    __syncthreads();
}

// Stage 3: S[i][j] = sum_q U[i][q] D[j][q] + beta (psislaterbcs.f90:278,289)
// A task is one row i and up to kGJ columns j = g, g + ng, ... (ng groups
// per row): one U read feeds kGJ multiply-adds, lanes with consecutive g
// read consecutive D rows (conflict-free), and 33 x 7 tasks fill one round
// of 256 threads at N = 66.  16-byte pair loads over the padded rows (the
// padding is zero).
constexpr int kGJ = 5;
template <class R, int NT, bool BIG>
__device__ void gemm_stage(const Ctx<R, NT, BIG>& c)
{
    using Acc = typename AccOf<R>::type;
    const DevParams& p = c.p;
    double* sm = c.sm;
    const R* U = c.template uat<R>(c.L.U);
    const R* D = c.template uat<R>(c.L.D);
    R* S = at<R>(sm, c.L.S);
    const int ldU = p.ldU;
    const int ng = (p.ndn + kGJ - 1) / kGJ;
    // double-float path: |U[i][q] D[j][q]| <= |v_q| bounds every term (cos and
    // sin columns, |D| <= 1; the k = 0 column holds v_0 and 1), so one bound
    // per walker serves the bounded accumulator (6 FP32 instructions per
    // multiply-add instead of 12; error of order K 2^-48 sigma)
    float sig = 0.0f;
    if constexpr (is_df<R>::value) {
        const R* kv = at<R>(sm, c.L.ksoa) + 4 * p.nk;
        float sv = fabsf(kv[0].hi);
        for (int q = 1; q < p.nk; ++q) sv += 2.0f * fabsf(kv[q].hi);
        sig = pow2_ceil(4.0f * 1.001f * sv);
    }
    const UDiv dg(ng);
    for (int t = threadIdx.x; t < p.nup * ng; t += NT) {
        const int i = dg.quo(t), g = t - i * ng;
        const R* u = U + i * ldU;
        const R* d[kGJ];
        bool ok[kGJ];
#pragma unroll
        for (int m = 0; m < kGJ; ++m) {
            const int j = g + ng * m;
            ok[m] = j < p.ndn;
            d[m] = D + (ok[m] ? j : g) * ldU;
        }
        if constexpr (is_df<R>::value) {
            bacc a[kGJ];
#pragma unroll
            for (int m = 0; m < kGJ; ++m) bacc_init(a[m], sig);
            for (int q = 0; q < ldU; q += 2) {
                R ua, ub;
                ld2(u + q, ua, ub);
#pragma unroll
                for (int m = 0; m < kGJ; ++m) {
                    R xa, xb;
                    ld2(d[m] + q, xa, xb);
                    bacc_madd(a[m], ua, xa);
                    bacc_madd(a[m], ub, xb);
                }
            }
#pragma unroll
            for (int m = 0; m < kGJ; ++m)
                if (ok[m]) {
                    R* sij = S + i * p.ldS + g + ng * m;
                    *sij = bacc_value(a[m], sig) + *sij;
                }
        } else {
            Acc a[kGJ];
#pragma unroll
            for (int m = 0; m < kGJ; ++m) acc_init(a[m]);
            for (int q = 0; q < ldU; q += 2) {
                R ua, ub;
                ld2(u + q, ua, ub);
#pragma unroll
                for (int m = 0; m < kGJ; ++m) {
                    R xa, xb;
                    ld2(d[m] + q, xa, xb);
                    acc_madd(a[m], ua, xa);
                    acc_madd(a[m], ub, xb);
                }
            }
#pragma unroll
            for (int m = 0; m < kGJ; ++m)
                if (ok[m]) {
                    R* sij = S + i * p.ldS + g + ng * m;
                    *sij = acc_value(a[m]) + *sij;
                }
        }
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Stage 4: inverse and log|det| of the pair matrix (matrixlapack.f90:13-41:
// dgetrf + dgetri, log|det| = sum log|pivot|, sign from the pivots and the
// row interchanges).  Partial pivoting, first maximum of |a| wins (idamax).
// On return sm[L.S] holds inv(S) in natural order; returns false for an
// exactly singular matrix.
//
// Main path (nd <= 128): blocked Gauss-Jordan with implicit row pivoting.
// Column blocks of B are factored as n x B panels by warps 0 and 1 in
// registers (REDUX max/min pivot search per warp, the two candidates
// compared through shared memory under a 64-thread barrier, no block barrier
// inside a panel), and each factored panel is applied to the other columns
// as one rank-B update
//     A'[i][j] = [i not a pivot row of the block] A[i][j]
//                + sum_c P[i][c] A[piv(k0+c)][j]
// from one buffer into the other (sm[L.S] <-> sm[L.S2]).  The panel warps
// factor the next panel while warps 2..7 apply the current one: one block
// barrier per B columns.  With pivot row p_k for column k, the final buffer M holds
// M[p_a][b'] = inv(S)[a][p_b'], so inv(S)[a][b] = M[p_a][pos(b)] with
// pos(p_k) = k; the last pass writes it in natural order.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned mag_hi(double v) { return (unsigned)(__double_as_longlong(v) >> 32) & 0x7fffffffu; }
__device__ __forceinline__ unsigned mag_lo(double v) { return (unsigned)(__double_as_longlong(v) & 0xffffffffll); }
__device__ __forceinline__ unsigned mag_hi(df v) { return __float_as_uint(v.hi) & 0x7fffffffu; }
__device__ __forceinline__ unsigned mag_lo(df) { return 0u; }
__device__ __forceinline__ double shfl_r(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ double shfl_x(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ df shfl_x(df v, int o)
{
    return df{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
}
__device__ __forceinline__ df shfl_r(df v, int src)
{
    return df{__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src)};
}

// Named barrier 1 over the whole CTA: the panel warp waits, the others only
// arrive.
template <int NT>
__device__ __forceinline__ void bar1_sync() { asm volatile("bar.sync 1, %0;" ::"n"(NT) : "memory"); }
template <int NT>
__device__ __forceinline__ void bar1_arrive() { asm volatile("bar.arrive 1, %0;" ::"n"(NT) : "memory"); }

constexpr int kPanelWarps = 1;

// Factor columns k0..k0+bw-1 of A (all n rows, rows pivoted in earlier
// blocks excluded from the pivot search) by Gauss-Jordan steps restricted
// to the panel.  Called by warp 0; lane t holds rows t + 32 s (s < RPL) in
// registers, so the pivot search is a warp reduction (REDUX max of the
// magnitude keys, then min of the rows that reach it: the first maximum, as
// idamax) and the pivot row reaches every lane by shuffles.  Records piv[k],
// pvals[k] and rowpos[piv[k]] = k.  Returns false on a zero pivot.
template <class R, int RPL, int B>
__device__ __forceinline__ bool gj_panel(R* A, int ld, int n, int k0, int bw, int* piv, R* pvals, int* rowpos)
{
    const int t = threadIdx.x;
    R v[RPL][B];
    bool done[RPL];
#pragma unroll
    for (int s = 0; s < RPL; ++s) {
        const int r = t + 32 * s;
        const bool ok = r < n;
        done[s] = !ok || rowpos[r] < k0;
#pragma unroll
        for (int c = 0; c < B; ++c) v[s][c] = (ok && c < bw) ? A[r * ld + k0 + c] : rzero<R>();
    }
    // Column steps.  The registers rotate by one column per step, so the
    // active column is always v[.][0] and the step body is compiled once (a
    // rolled loop keeps the kernel's instruction footprint small); after B
    // steps the columns are back in order.
#pragma unroll 1
    for (int c = 0; c < B; ++c) {
        if (c < bw) {
            // largest |a| among rows not yet pivoted; smallest row on ties
            unsigned kh[RPL], mh = 0u;
#pragma unroll
            for (int s = 0; s < RPL; ++s) {
                kh[s] = done[s] ? 0u : mag_hi(v[s][0]);
                mh = kh[s] > mh ? kh[s] : mh;
            }
            const unsigned gh = __reduce_max_sync(0xffffffffu, mh);
            unsigned gl = 0u;
            if constexpr (!is_df<R>::value) {
                unsigned ml = 0u;
#pragma unroll
                for (int s = 0; s < RPL; ++s)
                    if (!done[s] && kh[s] == gh) {
                        const unsigned l = mag_lo(v[s][0]);
                        ml = l > ml ? l : ml;
                    }
                gl = __reduce_max_sync(0xffffffffu, ml);
            }
            if (gh == 0u && gl == 0u) return false;   // no non-zero candidate
            unsigned mine = 0xffffffffu;
#pragma unroll
            for (int s = RPL - 1; s >= 0; --s)
                if (!done[s] && kh[s] == gh && mag_lo(v[s][0]) == gl) mine = (unsigned)(t + 32 * s);
            const int pr = (int)__reduce_min_sync(0xffffffffu, mine);
            // the pivot row from its lane (slot pr / 32 is the same on every lane)
            const int ps = pr >> 5, pl = pr & 31;
            R rr[B];
#pragma unroll
            for (int c2 = 0; c2 < B; ++c2) {
                R own = v[0][c2];
#pragma unroll
                for (int s = 1; s < RPL; ++s)
                    if (ps == s) own = v[s][c2];
                rr[c2] = shfl_r(own, pl);
            }
            // Gauss-Jordan step with the unscaled pivot row p and multiplier
            // m = a_c / p_c per row (m = -1/p_c for the pivot row itself):
            //   a_c2 <- a_c2 - m p_c2   (pivot row: p_c2 / p_c),
            //   a_c  <- -m              (pivot row: 1 / p_c)
            // one multiply per row instead of scaling the pivot row on every lane
            const R pv = rr[0];
            const R pinv = rcp(pv);
#pragma unroll
            for (int s = 0; s < RPL; ++s) {
                const bool isp = t + 32 * s == pr;
                const R m = isp ? -pinv : v[s][0] * pinv;
#pragma unroll
                for (int c2 = 1; c2 < B; ++c2) v[s][c2] = fms(isp ? rzero<R>() : v[s][c2], m, rr[c2]);
                v[s][0] = -m;
                if (isp) done[s] = true;
            }
            if (t == 0) {
                piv[k0 + c] = pr;
                pvals[k0 + c] = pv;
                rowpos[pr] = k0 + c;
            }
        }
        // rotate: the next column becomes v[.][0]
#pragma unroll
        for (int s = 0; s < RPL; ++s) {
            const R f = v[s][0];
#pragma unroll
            for (int c2 = 0; c2 < B - 1; ++c2) v[s][c2] = v[s][c2 + 1];
            v[s][B - 1] = f;
        }
    }
#pragma unroll
    for (int s = 0; s < RPL; ++s) {
        const int r = t + 32 * s;
        if (r < n)
#pragma unroll
            for (int c = 0; c < B; ++c)
                if (c < bw) A[r * ld + k0 + c] = v[s][c];
    }
    return true;
}

// One element of the rank-B update of a factored block (see above).
template <class R, int B>
__device__ __forceinline__ R gj_apply(const R* cur, int ld, int i, int j, int k0, int bw, const int (&prow)[B],
                                      const int* rowpos)
{
    if (bw == 0) return cur[i * ld + j];   // the first pass only copies
    typename AccOf<R>::type a;
    acc_init(a);
    const int rp = rowpos[i];
    if (rp < k0 || rp >= k0 + bw) acc_add(a, cur[i * ld + j]);
    const R* ri = cur + i * ld + k0;
#pragma unroll
    for (int c = 0; c < B; ++c)
        if (c < bw) acc_madd(a, ri[c], cur[prow[c] * ld + j]);
    return acc_value(a);
}

template <class R, int RPL, int B, int NT, bool BIG>
__device__ bool inverse_blocked(const Ctx<R, NT, BIG>& c, double& logdet, int& sgn)
{
    const DevParams& p = c.p;
    double* sm = c.sm;
    R* const A0 = at<R>(sm, c.L.S);
    R* const A1 = c.template uat<R>(c.L.S2);
    int* piv = reinterpret_cast<int*>(sm + c.L.red + 512);                           // nd ints
    R* pvals = reinterpret_cast<R*>(sm + c.L.red + 512 + 2 * DMC_MAX_PART);          // nd pivots
    int* rowpos = reinterpret_cast<int*>(sm + c.L.red + 512 + 4 * DMC_MAX_PART);     // nd ints
    __shared__ int s_sing;
    __shared__ double s_logdet;
    const int n = p.nd, ld = p.ldS;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < n; i += NT) rowpos[i] = n;
    if (threadIdx.x == 0) s_sing = 0;
    __syncthreads();
    // Pass 0 applies no block (it copies S into the second buffer) while the
    // panel warps factor the first panel there; pass p > 0 applies block p-1
    // and factors panel p.  One call site of the (unrolled) panel keeps the
    // kernel's instruction footprint small.
    // With an even number of panels the first pass works in place (the copy
    // writes every element onto itself), so that the last pass lands in S
    // and writes the natural order directly: no final copy.
    const bool inplace = ((n + B - 1) / B) % 2 == 0;
    R* cur = A0;
    R* nxt = inplace ? A0 : A1;
    int k0 = 0, bw = 0;
    for (;;) {
        if (s_sing) break;
        const int k1 = k0 + bw, bw1 = min(B, n - k1);
        int prow[B];
#pragma unroll
        for (int q = 0; q < B; ++q) prow[q] = q < bw ? piv[k0 + q] : 0;
        // the last block writes the natural order directly when it lands in S
        const bool scatter = (bw1 == 0) && (nxt == A0);
        if (bw1 > 0) {
            // columns of the next panel first, by everyone
            const UDiv db(bw1);
            for (int e = threadIdx.x; e < n * bw1; e += NT) {
                const int i = db.quo(e), j = k1 + e - i * bw1;
                nxt[i * ld + j] = gj_apply<R, B>(cur, ld, i, j, k0, bw, prow, rowpos);
            }
            if (warp < kPanelWarps) {
                bar1_sync<NT>();
                if (!gj_panel<R, RPL, B>(nxt, ld, n, k1, bw1, piv, pvals, rowpos) && threadIdx.x == 0) s_sing = 1;
            } else {
                bar1_arrive<NT>();
            }
        }
        if (bw1 == 0 || warp >= kPanelWarps) {
            // every other column: the non-panel warps (all warps in the last block)
            const int nt = bw1 > 0 ? NT - 32 * kPanelWarps : NT;
            const int t0 = bw1 > 0 ? (int)threadIdx.x - 32 * kPanelWarps : (int)threadIdx.x;
            const int nc = n - bw1;
            const UDiv dc(nc);
            for (int e = t0; e < n * nc; e += nt) {
                const int i = dc.quo(e), jj = e - i * nc;
                const int j = jj < k1 ? jj : jj + bw1;
                // the block's own (factored) columns pass through unchanged
                const R val = (j >= k0 && j < k1) ? cur[i * ld + j] : gj_apply<R, B>(cur, ld, i, j, k0, bw, prow, rowpos);
                if (scatter)
                    nxt[rowpos[i] * ld + piv[j]] = val;
                else
                    nxt[i * ld + j] = val;
            }
        }
        __syncthreads();
        R* t = cur;
        cur = nxt;
        nxt = (t == cur) ? (cur == A0 ? A1 : A0) : t;
        if (bw1 == 0) break;
        k0 = k1;
        bw = bw1;
    }
    const bool sing = s_sing != 0;
    // natural order, sign of the row permutation and of the pivots, log|det|
    int odd = 0;
    if (!sing) {
        const bool copy = (cur == A1);
        const UDiv dn(n);
        for (int e = threadIdx.x; e < n * n; e += NT) {
            const int a = dn.quo(e), b = e - a * n;
            if (copy) A0[a * ld + b] = A1[piv[a] * ld + rowpos[b]];
            if (a < b && piv[a] > piv[b]) odd ^= 1;
        }
        for (int q = threadIdx.x; q < n; q += NT)
            if (is_neg(pvals[q])) odd ^= 1;
        if (warp == 0) {
            if constexpr (is_df<R>::value) {
                // double-float logarithms on the FP32 pipe
                df ls = df{0.0f, 0.0f};
                for (int q = lane; q < n; q += 32) ls = ls + dfm::log_df(dabs(pvals[q]));
                ls = dfm::warp_sum(ls);
                if (lane == 0) s_logdet = to_double(ls);
            } else {
                double ls = 0.0;
                for (int q = lane; q < n; q += 32) ls += log(fabs(pvals[q]));
                ls = warp_sum(ls);
                if (lane == 0) s_logdet = ls;
            }
        }
    }
    const int nodd = __syncthreads_count(odd);
    logdet = sing ? 0.0 : s_logdet;
    sgn = (nodd & 1) ? -1 : 1;
    return !sing;
}

// Unblocked in-place Gauss-Jordan with explicit row interchanges, for
// matrices the blocked path does not take (nd > 128 or no second buffer).
// Pivot search by warp 0 one column ahead of the elimination.
__device__ __forceinline__ unsigned long long pivot_key(double v, int row)
{
    const unsigned long long m = ((unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull) >> 12;
    return (m << 12) | (unsigned long long)(4095 - row);
}
__device__ __forceinline__ unsigned long long pivot_key(df v, int row)
{
    const unsigned long long m = (unsigned long long)((unsigned)__float_as_uint(v.hi) & 0x7fffffffu);
    return (m << 32) | (unsigned long long)(0xffffffffu - (unsigned)row);
}

// pivot search over rows k..n-1 of column k by one warp; every lane
// returns the pivot row and its value
template <class R>
__device__ __forceinline__ int warp_pivot(const R* A, int ld, int n, int k, R& pv)
{
    const int lane = threadIdx.x & 31;
    unsigned long long best = 0ull;
    for (int i = k + lane; i < n; i += 32) {
        const unsigned long long key = pivot_key(A[i * ld + k], i);
        best = key > best ? key : best;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long ob = __shfl_xor_sync(0xffffffffu, best, o);
        best = ob > best ? ob : best;
    }
    int bi;
    if constexpr (is_df<R>::value)
        bi = (int)(0xffffffffu - (unsigned)(best & 0xffffffffull));
    else
        bi = 4095 - (int)(best & 4095ull);
    if (best == 0ull || bi < k || bi >= n) bi = k;   // empty column: report row k (its value is zero)
    pv = A[bi * ld + k];
    return bi;
}

template <class R, int NT, bool BIG>
__device__ bool inverse_unblocked(const Ctx<R, NT, BIG>& c, double& logdet, int& sgn)
{
    const DevParams& p = c.p;
    double* sm = c.sm;
    R* A = at<R>(sm, c.L.S);
    R* colk = at<R>(sm, c.L.colk);
    int* piv = reinterpret_cast<int*>(sm + c.L.red + 512);                    // nd ints
    R* pvals = reinterpret_cast<R*>(sm + c.L.red + 512 + 2 * DMC_MAX_PART);   // nd pivots
    __shared__ R s_pinv;
    __shared__ int s_piv;
    __shared__ int s_sing;
    __shared__ double s_logdet;
    __shared__ int s_sgn;
    const int n = p.nd, ld = p.ldS;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        R pv;
        const int bi = warp_pivot<R>(A, ld, n, 0, pv);
        if (lane == 0) {
            s_sing = is_zero(pv) ? 1 : 0;
            s_piv = bi;
            piv[0] = bi;
            pvals[0] = pv;
            if (!is_zero(pv)) s_pinv = rcp(pv);
        }
    }
    __syncthreads();
    const int ew = NT - 32;
    const int e0 = (int)threadIdx.x - 32;
    const int di = ew / n, dc = ew % n;
    for (int k = 0; k < n; ++k) {
        if (s_sing) break;
        const int pr = s_piv;
        const R pinv = s_pinv;
        // save column k (rows in swapped order), swap rows k/pr, scale row k
        for (int t = threadIdx.x; t < n; t += NT) {
            const int src = (t == k) ? pr : ((t == pr) ? k : t);
            const R ck = A[src * ld + k];
            const R a = A[k * ld + t];
            const R b = A[pr * ld + t];
            colk[t] = ck;
            if (t != k) {
                R nk = a;
                if (pr != k) {
                    A[pr * ld + t] = a;
                    nk = b;
                }
                A[k * ld + t] = nk * pinv;
            }
        }
        __syncthreads();
        if (warp == 0) {
            // look-ahead: column k+1 and its pivot
            if (k + 1 < n) {
                const R akn = A[k * ld + k + 1];
                for (int i = lane; i < n; i += 32)
                    if (i != k) A[i * ld + k + 1] = fms(A[i * ld + k + 1], colk[i], akn);
                __syncwarp();
                R pv;
                const int bi = warp_pivot<R>(A, ld, n, k + 1, pv);
                if (lane == 0) {
                    pvals[k + 1] = pv;
                    if (is_zero(pv)) {
                        s_sing = 1;
                    } else {
                        s_piv = bi;
                        piv[k + 1] = bi;
                        s_pinv = rcp(pv);
                    }
                }
            }
        } else {
            int i = e0 / n, cc = e0 % n;
            for (int t = e0; t < n * n; t += ew) {
                if (i != k && cc != k + 1)
                    A[i * ld + cc] = (cc == k) ? -(colk[i] * pinv) : fms(A[i * ld + cc], colk[i], A[k * ld + cc]);
                i += di;
                cc += dc;
                if (cc >= n) {
                    cc -= n;
                    ++i;
                }
            }
            if (threadIdx.x == 32) A[k * ld + k] = pinv;
        }
        __syncthreads();
    }
    const bool sing = s_sing != 0;
    if (!sing) {
        // undo the row interchanges on the columns, last first (dgetri);
        // each thread owns whole rows, so no barrier between swaps
        for (int r = threadIdx.x; r < n; r += NT)
            for (int q = n - 1; q >= 0; --q) {
                const int pq = piv[q];
                if (pq != q) {
                    const R t = A[r * ld + q];
                    A[r * ld + q] = A[r * ld + pq];
                    A[r * ld + pq] = t;
                }
            }
    }
    if (warp == 0) {
        double ls = 0.0;
        int neg = 0, swp = 0;
        if (!sing)
            for (int q = lane; q < n; q += 32) {
                const R v = pvals[q];
                ls += log(fabs(to_double(v)));
                neg += is_neg(v) ? 1 : 0;
                swp += (piv[q] != q) ? 1 : 0;
            }
        ls = warp_sum(ls);
        for (int o = 16; o > 0; o >>= 1) {
            neg += __shfl_xor_sync(0xffffffffu, neg, o);
            swp += __shfl_xor_sync(0xffffffffu, swp, o);
        }
        if (lane == 0) {
            s_logdet = ls;
            s_sgn = ((neg + swp) & 1) ? -1 : 1;
        }
    }
    __syncthreads();
    logdet = s_logdet;
    sgn = s_sgn;
    return !sing;
}

template <class R, int NT, bool BIG>
__device__ bool inverse_stage(const Ctx<R, NT, BIG>& c, double& logdet, int& sgn)
{
    const int n = c.p.nd;
    if (c.L.S2 >= 0) {
        if (n <= 64) return inverse_blocked<R, 2, 6>(c, logdet, sgn);
        if (n <= 96) return inverse_blocked<R, 3, 8>(c, logdet, sgn);
        if (n <= 128) return inverse_blocked<R, 4, 8>(c, logdet, sgn);
    }
    return inverse_unblocked<R>(c, logdet, sgn);
}

// ---------------------------------------------------------------------------
// Stage 5: drift and Laplacian of log det from the inverse.
//  up i:   sum_q k_q (U_c G_s - U_s G_c), lap -|k|^2 (U_c G_c + U_s G_s),
//          G_{c,s} = sum_j D[j][c,s] Sinv[j][i]
//  down j: sum_q k_q (H_s D_c - H_c D_s), lap -|k|^2 (H_c D_c + H_s D_s),
//          H_{c,s} = sum_i Sinv[j][i] U[i][c,s]
// Register-tiled: a task is one particle and kQT k vectors q = g, g + G,
// g + 2G, ... (G = ceil(nq / kQT) groups per particle), so one Sinv load
// feeds 2 kQT multiply-adds and a thread carries 2 kQT independent
// accumulators; lanes of a warp read consecutive k vectors (no bank
// conflicts).  Tasks are split into contiguous per-thread chunks; each
// thread sums its chunk per particle and the partial sums of a particle are
// added in thread order.  Up and down tasks go to disjoint warps (in
// proportion to the particle counts), so that no warp runs both loop bodies
// one after the other.
// ---------------------------------------------------------------------------
constexpr int kQT = 4;

struct DriftSplit {
    int pbeg[2], np[2], tbeg[2], nth[2], chunk[2];
};

// Half 0 = up particles on the first warps, half 1 = down particles on the
// rest.  A chunk must not span more than two particles (chunk <= ng, the
// tasks per particle); when a split cannot guarantee that, half 0 takes
// every particle on all threads.
template <int NT>
__device__ __forceinline__ DriftSplit drift_split(int nup, int ndn, int ng)
{
    DriftSplit s;
    const int P = nup + ndn;
    int wu = P > 0 ? ((NT / 32) * nup + P / 2) / P : 0;
    if (nup > 0 && wu < 1) wu = 1;
    if (ndn > 0 && wu > (NT / 32) - 1) wu = (NT / 32) - 1;
    s.pbeg[0] = 0;
    s.np[0] = nup;
    s.tbeg[0] = 0;
    s.nth[0] = 32 * wu;
    s.pbeg[1] = nup;
    s.np[1] = ndn;
    s.tbeg[1] = 32 * wu;
    s.nth[1] = NT - 32 * wu;
    bool ok = nup > 0 && ndn > 0;
    for (int h = 0; h < 2; ++h) {
        s.chunk[h] = s.nth[h] > 0 ? (s.np[h] * ng + s.nth[h] - 1) / s.nth[h] : 0;
        if (s.chunk[h] > ng) ok = false;
    }
    if (!ok) {
        s.np[0] = P;
        s.nth[0] = NT;
        s.chunk[0] = (P * ng + NT - 1) / NT;
        s.np[1] = 0;
        s.tbeg[1] = NT;
        s.nth[1] = 0;
        s.chunk[1] = 1;
    }
    return s;
}

// one accumulator per (k vector, cos|sin) of a task
template <class R>
struct DriftAcc {
    typename AccOf<R>::type a[2 * kQT];
    __device__ __forceinline__ void init(const float*) {
#pragma unroll
        for (int m = 0; m < 2 * kQT; ++m) acc_init(a[m]);
    }
    __device__ __forceinline__ void madd(int m, R x, R y) { acc_madd(a[m], x, y); }
    __device__ __forceinline__ R value(int m, const float*) const { return acc_value(a[m]); }
};
template <>
struct DriftAcc<df> {
    bacc a[2 * kQT];
    __device__ __forceinline__ void init(const float* sig) {
#pragma unroll
        for (int m = 0; m < 2 * kQT; ++m) bacc_init(a[m], sig[m >> 1]);
    }
    __device__ __forceinline__ void madd(int m, df x, df y) { bacc_madd(a[m], x, y); }
    __device__ __forceinline__ df value(int m, const float* sig) const { return bacc_value(a[m], sig[m >> 1]); }
};

// Warp-tiled form of stage 5 (the main path).  The contractions
// G = Si^T D (up) and H = Si U (down) are GEMMs of nd x nd by nd x 2nq;
// operand reads from shared memory bound them, so each lane keeps a
// register tile of kTR particles x kTS k vectors (cos and sin: 2 kTR kTS
// accumulators) and the lanes of a warp form a kTA x kTB grid: a warp tile
// covers kTA kTR = 8 particles of one spin and kTB kTS = 40 k vectors, each
// Sinv read feeds 2 kTS multiply-adds and each D/U read 2 kTR.  Warps 0-3
// take the up tiles, warps 4-7 the down tiles.  Per particle, the lanes of
// a tile that share it sum their k vectors with a fixed xor tree; particles
// beyond the last full block of 8 are computed one (particle, k) item per
// thread.  Partial sums go to shared memory and are added per particle in
// a fixed order.  Returns false (nothing done) when the partial sums do not
// fit the reduction area.
constexpr int kTR = 2, kTS = 5, kTA = 4, kTB = 8;
static_assert(kTA * kTB == 32, "one warp per tile");

__device__ __forceinline__ float abs_hi(df v) { return fabsf(v.hi); }
__device__ __forceinline__ float abs_hi(double v) { return (float)fabs(v); }

// partial contraction of one (particle, k vector) item over the terms
// k0, k0 + kstep, ...: G (up particle) or H (down particle) for the cos and
// sin parts of k vector q (1-based)
template <class R, int NT, bool BIG>
__device__ __forceinline__ void drift_dots(const Ctx<R, NT, BIG>& c, const float* bound, int pt, int q, int k0, int kstep,
                                           R& vc, R& vs)
{
    const DevParams& p = c.p;
    double* sm = c.sm;
    const R* U = c.template uat<R>(c.L.U);
    const R* D = c.template uat<R>(c.L.D);
    const R* Si = at<R>(sm, c.L.S);
    const R* ks = at<R>(sm, c.L.ksoa);
    const int nk = p.nk, ld = p.ldS, ldU = p.ldU, qc = 2 * q - 2;
    const bool up = pt < p.nup;
    const int j = pt - p.nup;
    typename AccOf<R>::type ac, as;
    bacc bc, bs;
    float sig = 0.0f;
    if constexpr (is_df<R>::value) {
        sig = up ? pow2_ceil(4.0f * bound[pt]) : pow2_ceil(4.0f * fabsf(ks[4 * nk + q].hi) * 1.001f * bound[p.nd + j]);
        bacc_init(bc, sig);
        bacc_init(bs, sig);
    } else {
        acc_init(ac);
        acc_init(as);
    }
    const int nK = up ? p.ndn : p.nup;
    for (int kk = k0; kk < nK; kk += kstep) {
        const R sv = up ? Si[kk * ld + pt] : Si[j * ld + kk];
        R bcv, bsv;
        ld2((up ? D : U) + kk * ldU + qc, bcv, bsv);
        if constexpr (is_df<R>::value) {
            bacc_madd(bc, bcv, sv);
            bacc_madd(bs, bsv, sv);
        } else {
            acc_madd(ac, bcv, sv);
            acc_madd(as, bsv, sv);
        }
    }
    if constexpr (is_df<R>::value) {
        vc = bacc_value(bc, sig);
        vs = bacc_value(bs, sig);
    } else {
        vc = acc_value(ac);
        vs = acc_value(as);
    }
}

// the 4 terms (3 drift components, Laplacian) of k vector q (1-based) for
// particle pt from its contractions vc, vs
template <class R, int NT, bool BIG>
__device__ __forceinline__ void drift_terms(const Ctx<R, NT, BIG>& c, int pt, int q, R vc, R vs, R (&out)[4])
{
    const DevParams& p = c.p;
    double* sm = c.sm;
    const R* ks = at<R>(sm, c.L.ksoa);
    const int nk = p.nk, ldU = p.ldU, qc = 2 * q - 2;
    R t, l;
    if (pt < p.nup) {
        R uc, us;
        ld2(c.template uat<R>(c.L.U) + pt * ldU + qc, uc, us);
        t = uc * vs - us * vc;
        l = uc * vc + us * vs;
    } else {
        R dc, ds;
        ld2(c.template uat<R>(c.L.D) + (pt - p.nup) * ldU + qc, dc, ds);
        t = vs * dc - vc * ds;
        l = vc * dc + vs * ds;
    }
    out[0] = ks[q] * t;
    out[1] = ks[nk + q] * t;
    out[2] = ks[2 * nk + q] * t;
    out[3] = -(ks[3 * nk + q] * l);
}

// one warp tile: particles blk*8 .. blk*8+7 of one spin, k vectors of
// chunk qch; writes the tile's per-particle sums to pbuf.  Both spins share
// the code: up (down = false) contracts Sinv columns with D, down contracts
// Sinv rows with U, and in both cases
//   t = O_c V_s - O_s V_c,  l = O_c V_c + O_s V_s
// with O the particle's own orbital row and V the contraction.
template <class R, int NT, bool BIG>
__device__ __forceinline__ void drift_tile(const Ctx<R, NT, BIG>& c, const float* bound, bool down, int blk, int qch, int nqc,
                                           R* pbuf)
{
    const DevParams& p = c.p;
    double* sm = c.sm;
    const R* Si = at<R>(sm, c.L.S);
    const R* ks = at<R>(sm, c.L.ksoa);
    const R* B = c.template uat<R>(down ? c.L.U : c.L.D);     // contraction operand
    const R* O = c.template uat<R>(down ? c.L.D : c.L.U);     // the particles' own orbital rows
    const int nq = p.nk - 1, nk = p.nk, ld = p.ldS, ldU = p.ldU;
    const int lane = threadIdx.x & 31, ai = lane & (kTA - 1), bi = lane / kTA;
    const int nK = down ? p.nup : p.ndn;
    int pi[kTR];
#pragma unroll
    for (int k = 0; k < kTR; ++k) pi[k] = blk * kTA * kTR + ai + kTA * k;
    int qo[kTS];       // offset of the (cos, sin) pair in an orbital row
    bool okq[kTS];
#pragma unroll
    for (int m = 0; m < kTS; ++m) {
        const int q = qch * kTB * kTS + bi + kTB * m;
        okq[m] = q < nq;
        qo[m] = 2 * (okq[m] ? q : 0);               // a missing k vector reads vector 1 and is dropped
    }
    // bound of the double-float dot products (|D| <= 1, |U[i][q]| <= |v_q|)
    auto sigma = [&](int k, int m) {
        return down ? pow2_ceil(4.0f * abs_hi(ks[4 * nk + qo[m] / 2 + 1]) * 1.001f * bound[p.nd + pi[k]])
                    : pow2_ceil(4.0f * bound[pi[k]]);
    };
    typename AccOf<R>::type a64[kTR][kTS][2];
    bacc adf[kTR][kTS][2];
#pragma unroll
    for (int k = 0; k < kTR; ++k)
#pragma unroll
        for (int m = 0; m < kTS; ++m) {
            if constexpr (is_df<R>::value) {
                const float sg = sigma(k, m);
                bacc_init(adf[k][m][0], sg);
                bacc_init(adf[k][m][1], sg);
            } else {
                acc_init(a64[k][m][0]);
                acc_init(a64[k][m][1]);
            }
        }
    // up: G[i][q] = sum_j Si[j][i] D[j][q];  down: H[j][q] = sum_i Si[j][i] U[i][q]
    // Sinv element (particle pi[k], term kk) at s0 + kk * sstep + k * kTA * pstep
    const int sstep = down ? 1 : ld, pstep = down ? ld : 1;
    const R* s0 = Si + pi[0] * pstep;
    for (int kk = 0; kk < nK; ++kk) {
        R sv[kTR];
#pragma unroll
        for (int k = 0; k < kTR; ++k) sv[k] = s0[kk * sstep + k * kTA * pstep];
        const R* brow = B + kk * ldU;
#pragma unroll
        for (int m = 0; m < kTS; ++m) {
            R bc, bs;
            ld2(brow + qo[m], bc, bs);
#pragma unroll
            for (int k = 0; k < kTR; ++k) {
                if constexpr (is_df<R>::value) {
                    bacc_madd(adf[k][m][0], bc, sv[k]);
                    bacc_madd(adf[k][m][1], bs, sv[k]);
                } else {
                    acc_madd(a64[k][m][0], bc, sv[k]);
                    acc_madd(a64[k][m][1], bs, sv[k]);
                }
            }
        }
    }
    // per particle: sum over this lane's k vectors
    R ts[kTR][4];
#pragma unroll
    for (int k = 0; k < kTR; ++k) {
        typename AccOf<R>::type sx, sy, sz, sl;
        acc_init(sx);
        acc_init(sy);
        acc_init(sz);
        acc_init(sl);
        const R* own = O + pi[k] * ldU;
#pragma unroll
        for (int m = 0; m < kTS; ++m) {
            R vc, vs;
            if constexpr (is_df<R>::value) {
                const float sg = sigma(k, m);
                vc = bacc_value(adf[k][m][0], sg);
                vs = bacc_value(adf[k][m][1], sg);
            } else {
                vc = acc_value(a64[k][m][0]);
                vs = acc_value(a64[k][m][1]);
            }
            if (!okq[m]) continue;
            R oc, os;
            ld2(own + qo[m], oc, os);
            R t, l;
            if constexpr (is_df<R>::value) {
                // |t|, |l| <= |own (cos, sin)| |(vc, vs)|: up |v_q| * colsum,
                // down 1 * |v_q| * rowsum
                const float vq = abs_hi(ks[4 * nk + qo[m] / 2 + 1]) * 1.001f;
                const float sg = down ? sigma(k, m)
                                      : pow2_ceil(4.0f * fmaxf(1.0f, vq) * bound[pi[k]]);
                bacc at_, al_;
                bacc_init(at_, sg);
                bacc_init(al_, sg);
                bacc_madd(at_, oc, vs);
                bacc_madd(at_, -os, vc);
                bacc_madd(al_, oc, vc);
                bacc_madd(al_, os, vs);
                t = bacc_value(at_, sg);
                l = bacc_value(al_, sg);
            } else {
                typename AccOf<R>::type at_, al_;
                acc_init(at_);
                acc_init(al_);
                acc_madd(at_, oc, vs);
                acc_madd(at_, -os, vc);
                acc_madd(al_, oc, vc);
                acc_madd(al_, os, vs);
                t = acc_value(at_);
                l = acc_value(al_);
            }
            const int q1 = qo[m] / 2 + 1;
            acc_madd(sx, ks[q1], t);
            acc_madd(sy, ks[nk + q1], t);
            acc_madd(sz, ks[2 * nk + q1], t);
            acc_madd(sl, -ks[3 * nk + q1], l);
        }
        ts[k][0] = acc_value(sx);
        ts[k][1] = acc_value(sy);
        ts[k][2] = acc_value(sz);
        ts[k][3] = acc_value(sl);
    }
    // fixed xor tree over the lanes that share the particles (lane bits of bi)
#pragma unroll
    for (int o = kTA; o < 32; o <<= 1)
#pragma unroll
        for (int k = 0; k < kTR; ++k)
#pragma unroll
            for (int z = 0; z < 4; ++z) ts[k][z] = ts[k][z] + shfl_x(ts[k][z], o);
    const int pbase = down ? p.nup : 0;
    if (bi == 0)
#pragma unroll
        for (int k = 0; k < kTR; ++k)
#pragma unroll
            for (int z = 0; z < 4; ++z) pbuf[((pbase + pi[k]) * nqc + qch) * 4 + z] = ts[k][z];
}

template <class R, int NT, bool BIG>
__device__ bool drift_tiled(const Ctx<R, NT, BIG>& c, const float* bound)
{
    const DevParams& p = c.p;
    double* sm = c.sm;
    const int P = p.npart, nq = p.nk - 1;
    const int nqc = (nq + kTB * kTS - 1) / (kTB * kTS);   // k-vector chunks of 40
    const int tu = p.nup % (kTA * kTR), td = p.ndn % (kTA * kTR);
    const int ntail = (tu + td) * nq;
    if (p.nup == 0 || p.ndn == 0 || (P * nqc + ntail) * 4 > NT * 8) return false;
    double* acc = sm + c.L.acc;
    R* pbuf = at<R>(sm, c.L.red);              // [P][nqc][4], then tail items [ntail][4]
    R* tbuf = pbuf + P * nqc * 4;
    const int warp = threadIdx.x >> 5;
    const int half = warp >= (NT / 32) / 2 ? 1 : 0, hw = warp & ((NT / 32) / 2 - 1);
    const int n = half ? p.ndn : p.nup;        // particles of this spin
    const int nb = n / (kTA * kTR);            // full blocks of 8
    for (int tau = hw; tau < nb * nqc; tau += (NT / 32) / 2)
        drift_tile<R>(c, bound, half != 0, tau / nqc, tau % nqc, nqc, pbuf);
    // particles beyond the full blocks: (particle, k vector) items, 10 per
    // warp, each contraction split over 3 lanes and added in lane order
    {
        const int lane = threadIdx.x & 31, grp = lane / 3, sub = lane % 3;
        for (int r0 = 0; r0 < ntail; r0 += (NT / 32) * 10) {
            const int it = r0 + warp * 10 + grp;
            const bool act = grp < 10 && it < ntail;
            const int pl = act ? it / nq : 0, q = act ? it % nq + 1 : 1;
            const int pt = pl < tu ? p.nup - tu + pl : p.nup + p.ndn - td + (pl - tu);
            R vc = rzero<R>(), vs = rzero<R>();
            if (act) drift_dots<R>(c, bound, pt, q, sub, 3, vc, vs);
            const int l0 = min(grp, 9) * 3;
            const R c1 = shfl_r(vc, l0 + 1), c2 = shfl_r(vc, l0 + 2);
            const R s1 = shfl_r(vs, l0 + 1), s2 = shfl_r(vs, l0 + 2);
            if (act && sub == 0) {
                R o[4];
                drift_terms<R>(c, pt, q, (vc + c1) + c2, (vs + s1) + s2, o);
                for (int z = 0; z < 4; ++z) tbuf[it * 4 + z] = o[z];
            }
        }
    }
    __syncthreads();
    for (int pt = threadIdx.x; pt < P; pt += NT) {
        const bool dn = pt >= p.nup;
        const int pl = dn ? pt - p.nup : pt, nn = dn ? p.ndn : p.nup, tt = dn ? td : tu;
        R r[4];
        for (int z = 0; z < 4; ++z) r[z] = rzero<R>();
        if (pl < nn - tt) {
            for (int qch = 0; qch < nqc; ++qch)
                for (int z = 0; z < 4; ++z) r[z] = r[z] + pbuf[(pt * nqc + qch) * 4 + z];
        } else {
            const int row = (dn ? tu + (pl - (nn - tt)) : pl - (nn - tt)) * nq;
            for (int q = 0; q < nq; ++q)
                for (int z = 0; z < 4; ++z) r[z] = r[z] + tbuf[(row + q) * 4 + z];
        }
        acc[3 * pt + 0] = to_double(r[0]);
        acc[3 * pt + 1] = to_double(r[1]);
        acc[3 * pt + 2] = to_double(r[2]);
        acc[3 * P + pt] = to_double(r[3]);
    }
    __syncthreads();
    return true;
}

template <class R, int NT, bool BIG>
__device__ void drift_stage(const Ctx<R, NT, BIG>& c)
{
    using KV = typename Prec<R>::KV;
    const DevParams& p = c.p;
    double* sm = c.sm;
    const R* U = c.template uat<R>(c.L.U);
    const R* D = c.template uat<R>(c.L.D);
    const R* Si = at<R>(sm, c.L.S);
    const R* ks = at<R>(sm, c.L.ksoa);      // kx, ky, kz, k^2, v by k vector
    double* acc = sm + c.L.acc;             // drift [3N], lap [N]
    R* part = at<R>(sm, c.L.red);           // per thread: 2 segments x 4 sums
    const int nq = p.nk - 1, nk = p.nk, P = p.npart, ld = p.ldS, ldU = p.ldU;
    const int ng = (nq + kQT - 1) / kQT;    // tasks per particle
    const DriftSplit sp = drift_split<NT>(p.nup, p.ndn, ng);
    // double-float path: abs column sums (bound[i], for G) and row sums
    // (bound[nd + j], for H) of the inverse bound the dot products
    float* bound = reinterpret_cast<float*>(sm + c.L.colk);
    if constexpr (is_df<R>::value) {
        for (int t = threadIdx.x; t < 2 * p.nd; t += NT) {
            float sacc = 0.0f;
            if (t < p.nd)
                for (int j = 0; j < p.nd; ++j) sacc += fabsf(Si[j * ld + t].hi);
            else
                for (int i = 0; i < p.nd; ++i) sacc += fabsf(Si[(t - p.nd) * ld + i].hi);
            bound[t] = sacc * 1.001f;
        }
        __syncthreads();
    }
    if (drift_tiled<R>(c, bound)) return;
    const int h = (int)threadIdx.x >= sp.tbeg[1] ? 1 : 0;
    const int lt = (int)threadIdx.x - sp.tbeg[h];
    const int tasks = sp.np[h] * ng, chunk = sp.chunk[h], pbeg = sp.pbeg[h];
    const int b = lt * chunk, e = min(tasks, b + chunk);
    R s0[4], s1[4];
    for (int k = 0; k < 4; ++k) s0[k] = s1[k] = rzero<R>();
    const int first = b < e ? pbeg + b / ng : -1;
    for (int it = b; it < e; ++it) {
        const int pt = pbeg + it / ng, g = it % ng;
        // k vectors of the task (1-based records); a missing one (q > nq)
        // reads vector g + 1 and is dropped
        int qv[kQT];
        bool ok[kQT];
#pragma unroll
        for (int m = 0; m < kQT; ++m) {
            const int q = g + ng * m;
            ok[m] = q < nq;
            qv[m] = (ok[m] ? q : g) + 1;
        }
        R vc[kQT], vs[kQT];   // G or H of each k vector
        float sig[kQT] = {};
        DriftAcc<R> A;
        const bool up = pt < p.nup;
        if (up) {
            const int i = pt;
            if constexpr (is_df<R>::value) {
                const float sg = pow2_ceil(4.0f * bound[i]);   // |D| <= 1
#pragma unroll
                for (int m = 0; m < kQT; ++m) sig[m] = sg;
            }
            A.init(sig);
            const R* sc = Si + i;
            for (int j = 0; j < p.ndn; ++j) {
                const R sji = sc[j * ld];
                const R* dj = D + j * ldU;
#pragma unroll
                for (int m = 0; m < kQT; ++m) {
                    R dc_, ds_;
                    ld2(dj + 2 * qv[m] - 2, dc_, ds_);
                    A.madd(2 * m, dc_, sji);
                    A.madd(2 * m + 1, ds_, sji);
                }
            }
        } else {
            const int j = pt - p.nup;
            if constexpr (is_df<R>::value) {
#pragma unroll
                for (int m = 0; m < kQT; ++m)   // |U[i][q]| <= |v_q|
                    sig[m] = pow2_ceil(4.0f * fabsf(ks[4 * nk + qv[m]].hi) * 1.001f * bound[p.nd + j]);
            }
            A.init(sig);
            const R* srow = Si + j * ld;
            for (int i = 0; i < p.nup; ++i) {
                const R sji = srow[i];
                const R* ui = U + i * ldU;
#pragma unroll
                for (int m = 0; m < kQT; ++m) {
                    R uc_, us_;
                    ld2(ui + 2 * qv[m] - 2, uc_, us_);
                    A.madd(2 * m, sji, uc_);
                    A.madd(2 * m + 1, sji, us_);
                }
            }
        }
#pragma unroll
        for (int m = 0; m < kQT; ++m) {
            vc[m] = A.value(2 * m, sig);
            vs[m] = A.value(2 * m + 1, sig);
        }
        R ts[4];
        for (int k = 0; k < 4; ++k) ts[k] = rzero<R>();
#pragma unroll
        for (int m = 0; m < kQT; ++m) {
            if (!ok[m]) continue;
            const int qc = 2 * qv[m] - 2;   // (cos, sin) pair of the k vector
            R t, l;
            if (up) {
                R uc, us;
                ld2(U + pt * ldU + qc, uc, us);
                t = uc * vs[m] - us * vc[m];
                l = uc * vc[m] + us * vs[m];
            } else {
                R dc, ds;
                ld2(D + (pt - p.nup) * ldU + qc, dc, ds);
                t = vs[m] * dc - vc[m] * ds;
                l = vc[m] * dc + vs[m] * ds;
            }
            ts[0] = fma(ks[qv[m]], t, ts[0]);
            ts[1] = fma(ks[nk + qv[m]], t, ts[1]);
            ts[2] = fma(ks[2 * nk + qv[m]], t, ts[2]);
            ts[3] = ts[3] - ks[3 * nk + qv[m]] * l;
        }
        if (pt == first) {
            for (int k = 0; k < 4; ++k) s0[k] = s0[k] + ts[k];
        } else {
            for (int k = 0; k < 4; ++k) s1[k] = s1[k] + ts[k];
        }
    }
    // publish the (at most two) particle segments of this thread's chunk;
    // a chunk never spans more than two particles because chunk <= ng
    R* my = part + threadIdx.x * 8;
    for (int k = 0; k < 4; ++k) {
        my[k] = s0[k];
        my[4 + k] = s1[k];
    }
    __syncthreads();
    // particle pl of a half is covered by that half's local threads
    // floor(pl*ng/chunk) .. floor((pl*ng+ng-1)/chunk)
    for (int pt = threadIdx.x; pt < P; pt += NT) {
        const int hh = (sp.nth[1] > 0 && pt >= sp.pbeg[1]) ? 1 : 0;
        const int pl = pt - sp.pbeg[hh], ch = sp.chunk[hh], ni = sp.np[hh] * ng;
        R r[4];
        for (int k = 0; k < 4; ++k) r[k] = rzero<R>();
        const int l0 = (pl * ng) / ch, l1 = (pl * ng + ng - 1) / ch;
        for (int u = l0; u <= l1 && u < sp.nth[hh]; ++u) {
            const int tb = u * ch, te = min(ni, tb + ch);
            if (tb >= te) continue;
            const R* o = part + (sp.tbeg[hh] + u) * 8;
            const int sl = (tb / ng == pl) ? 0 : (((te - 1) / ng == pl) ? 4 : -1);
            if (sl < 0) continue;
            for (int k = 0; k < 4; ++k) r[k] = r[k] + o[sl + k];
        }
        acc[3 * pt + 0] = to_double(r[0]);
        acc[3 * pt + 1] = to_double(r[1]);
        acc[3 * pt + 2] = to_double(r[2]);
        acc[3 * P + pt] = to_double(r[3]);
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Stage 6: beta terms of the drift and Laplacian (psislaterbcs.f90:290-291
// through :213-222): per up-down pair h = Sinv[j][i] f'/r dx, l = Sinv[j][i]
// lap f; row sums go to the up particle, column sums (negated drift) to the
// down particle.  Then the unpaired plane waves.
template <class R, int NT, bool BIG>
__device__ void beta_drift_stage(const Ctx<R, NT, BIG>& c)
{
    const DevParams& p = c.p;
    double* sm = c.sm;
    const R* xr = at<R>(sm, c.L.xr);
    const double* x = sm + c.L.x;
    const R* Si = at<R>(sm, c.L.S);
    R* pv = c.template uat<R>(c.L.R);
    const R* pb = reinterpret_cast<const R*>(c.pb);
    double* acc = sm + c.L.acc;
    const int nup = p.nup, ndn = p.ndn, ld = p.ldS, P = p.npart;
    if (!p.nobeta) {
        for (int r0 = 0; r0 < nup; r0 += c.L.rows_beta) {
            const int r1 = min(nup, r0 + c.L.rows_beta);
            const int npc = (r1 - r0) * ndn;
            const UDiv dv(ndn);
            for (int q = threadIdx.x; q < npc; q += NT) {
                const int qi = dv.quo(q);
                const int i = r0 + qi, j = q - qi * ndn;
                const R* xi = xr + 3 * i;
                const R* xj = xr + 3 * (nup + j);
                const R* pbq = pb + 2 * (i * ndn + j);
                const R sij = Si[j * ld + i];
                const R w = sij * pbq[0];
                pv[4 * q + 0] = w * min_image(xi[0] - xj[0], p);
                pv[4 * q + 1] = w * min_image(xi[1] - xj[1], p);
                pv[4 * q + 2] = w * min_image(xi[2] - xj[2], p);
                pv[4 * q + 3] = sij * pbq[1];
            }
            __syncthreads();
            const int nr = r1 - r0;
            for (int tc = threadIdx.x; tc < 4 * (nr + ndn); tc += NT) {
                const int t = tc / 4, cmp = tc % 4;
                typename AccOf<R>::type sacc;
                acc_init(sacc);
                if (t < nr) {
                    const R* row = pv + 4 * (t * ndn) + cmp;
                    for (int j = 0; j < ndn; ++j) acc_add(sacc, row[4 * j]);
                    const int i = r0 + t;
                    acc[cmp < 3 ? 3 * i + cmp : 3 * P + i] += to_double(acc_value(sacc));
                } else {
                    const int j = t - nr;
                    for (int r = 0; r < nr; ++r) acc_add(sacc, pv[4 * (r * ndn + j) + cmp]);
                    if (cmp < 3)
                        acc[3 * (nup + j) + cmp] -= to_double(acc_value(sacc));
                    else
                        acc[3 * P + nup + j] += to_double(acc_value(sacc));
                }
            }
            __syncthreads();
        }
    }
    // unpaired plane waves (psislaterbcs.f90:171-206 with :211-223)
    if (p.nexup > 0 || p.nexdn > 0) {
        for (int pt = threadIdx.x; pt < P; pt += NT) {
            const double* xp = x + 3 * pt;
            double g0 = 0, g1 = 0, g2 = 0, lp = 0;
            if (pt < nup) {
                for (int jj = 0; jj < p.nexup; ++jj) {
                    const double* k = p.akup[jj];
                    double s, co;
                    sincos(k[0] * xp[0] + k[1] * xp[1] + k[2] * xp[2], &s, &co);
                    const double w = to_double(Si[(ndn + jj) * ld + pt]);
                    // sin: grad k cos, lap -k2 sin; cos: grad -k sin, lap -k2 cos
                    const double gcoef = p.sinup[jj] ? co : -s;
                    const double val = p.sinup[jj] ? s : co;
                    g0 += w * k[0] * gcoef;
                    g1 += w * k[1] * gcoef;
                    g2 += w * k[2] * gcoef;
                    lp += w * (-p.ak2up[jj] * val);
                }
            } else {
                const int j = pt - nup;
                for (int jj = 0; jj < p.nexdn; ++jj) {
                    const double* k = p.akdn[jj];
                    double s, co;
                    sincos(k[0] * xp[0] + k[1] * xp[1] + k[2] * xp[2], &s, &co);
                    const double w = to_double(Si[j * ld + nup + jj]);
                    const double gcoef = p.sindn[jj] ? co : -s;
                    const double val = p.sindn[jj] ? s : co;
                    g0 += w * k[0] * gcoef;
                    g1 += w * k[1] * gcoef;
                    g2 += w * k[2] * gcoef;
                    lp += w * (-p.ak2dn[jj] * val);
                }
            }
            acc[3 * pt + 0] += g0;
            acc[3 * pt + 1] += g1;
            acc[3 * pt + 2] += g2;
            acc[3 * P + pt] += lp;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Long-range Jastrow (getjaslong, jastrowlongrange.f90:22-46), FP64 on both
// paths.  The reference's pair sum is evaluated through the densities
// rho_q = sum_i e^{i q.x_i}:
//   U    = sum_q f_q (|rho_q|^2 - N),          f_q = gamma e^{-beta|q|}/|q|,
//   dU_i = -2 sum_q f_q q Im(e^{i q.x_i} conj(rho_q)),
//   lap  = -2 sum_q f_q |q|^2 (|rho_q|^2 - N)  (before |dU|^2 is added),
// O(N n_q) instead of O(N^2 n_q).  Leaves dU in sm[L.dg] (free until the
// guide-function gradient is written) and uses the union region for rho_q.
// ---------------------------------------------------------------------------
template <int NT>
__device__ inline void jaslong_stage(const DevParams& p, const KernelArgs& a, const SmemLayout& L, double* sm,
                                     double* rho, double& ul, double& d2l)
{
    const double* x = sm + L.x;
    double* dl = sm + L.dg;
    const int P = p.npart;
    for (int q = threadIdx.x; q < p.nql; q += NT) {
        const double* Q = a.jq + 8 * q;
        double re = 0.0, im = 0.0;
        for (int i = 0; i < P; ++i) {
            double sn, cs;
            sincos(Q[0] * x[3 * i] + Q[1] * x[3 * i + 1] + Q[2] * x[3 * i + 2], &sn, &cs);
            re += cs;
            im += sn;
        }
        rho[2 * q] = re;
        rho[2 * q + 1] = im;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < P; i += NT) {
        double g0 = 0.0, g1 = 0.0, g2 = 0.0;
        for (int q = 0; q < p.nql; ++q) {
            const double* Q = a.jq + 8 * q;
            double sn, cs;
            sincos(Q[0] * x[3 * i] + Q[1] * x[3 * i + 1] + Q[2] * x[3 * i + 2], &sn, &cs);
            const double f = -2.0 * Q[4] * (sn * rho[2 * q] - cs * rho[2 * q + 1]);
            g0 = fma(f, Q[0], g0);
            g1 = fma(f, Q[1], g1);
            g2 = fma(f, Q[2], g2);
        }
        dl[3 * i] = g0;
        dl[3 * i + 1] = g1;
        dl[3 * i + 2] = g2;
    }
    double u = 0.0, d2 = 0.0;
    for (int q = 0; q < p.nql; ++q) {
        const double* Q = a.jq + 8 * q;
        const double r2 = rho[2 * q] * rho[2 * q] + rho[2 * q + 1] * rho[2 * q + 1] - (double)P;
        u += Q[4] * r2;
        d2 += -2.0 * Q[4] * Q[3] * r2;
    }
    ul = u;
    d2l = d2;
    __syncthreads();
}

// Scalars of one evaluation.
struct HRes {
    double psil, d2psi, v, vext, psigl, d2psig, u, d2u, logdet, d2phi;
    int is;
    bool singular;
};

// ---------------------------------------------------------------------------
// hpsi (wavefunction.f90:161-201) for the positions in sm[L.x].  Leaves
// dpsi in acc[0..3N) and dpsig in sm[L.dg] when a2 != 0.
// mode MODE_GETPHI stops after the Jastrow; MODE_BCS skips the Jastrow.
// ---------------------------------------------------------------------------
template <class R, int NT, bool BIG>
__device__ HRes hpsi_eval(const Ctx<R, NT, BIG>& c, int mode)
{
    const DevParams& p = c.p;
    double* sm = c.sm;
    const int P = p.npart, n3 = 3 * P;
    double* acc = sm + c.L.acc;
    double* du = acc + 4 * P;
    const double* x = sm + c.L.x;
    {
        R* xr = at<R>(sm, c.L.xr);
        for (int i = threadIdx.x; i < n3; i += NT) xr[i] = from_dbl<R>(x[i]);
        __syncthreads();
    }
    HRes h;
    using J = typename Prec<R>::J;
    J jt[3] = {rzero<J>(), rzero<J>(), rzero<J>()};
    double ss[3] = {0.0, 0.0, 0.0};
    pair_stage<R>(c, jt, ss);   // also fills the beta part of S (needed by MODE_BCS too)
    double su = 0.0, sv = 0.0, sd2 = 0.0;
    if (mode == MODE_BCS) {
        for (int i = threadIdx.x; i < n3; i += NT) du[i] = 0.0;
        __syncthreads();
    } else {
        // Jastrow, potential and pair-Laplacian sums in the Jastrow type
        // (double-float on the mixed path: no FP64 shuffle tree)
        block_sum_t<3, NT>(jt, at<J>(sm, c.L.red));
        if (threadIdx.x < 32) {   // only warp 0 assembles the scalar results
            su = to_double(jt[0]);
            sv = to_double(jt[1]);
            sd2 = to_double(jt[2]);
        }
        if (p.ieq) {
            block_sum_t<3, NT>(ss, sm + c.L.red);
            su += ss[0];
            sv += ss[1];
            sd2 += ss[2];
        }
    }
    // long-range Jastrow: part of hpsi (getphilong, wavefunction.f90:148-159,173),
    // not of getphi or bcs
    const bool jl = p.nql > 0 && (mode == MODE_HPSI || mode == MODE_STEP);
    double ulong = 0.0, d2long = 0.0;
    if (jl) jaslong_stage<NT>(c.p, c.a, c.L, sm, c.template uat<double>(c.L.R), ulong, d2long);
    double logdet = 0.0;
    int sgn = 1;
    bool ok = true;
    if (mode != MODE_GETPHI) {
        orbital_stage<R>(c);
        gemm_stage<R>(c);
        ok = inverse_stage<R>(c, logdet, sgn);
        if (ok) {
            drift_stage<R>(c);
            beta_drift_stage<R>(c);
        } else {
            for (int i = threadIdx.x; i < 4 * P; i += NT) acc[i] = 0.0;
            __syncthreads();
        }
    } else {
        for (int i = threadIdx.x; i < 4 * P; i += NT) acc[i] = 0.0;
        __syncthreads();
    }
    // one-body term (psislaterbcs.f90:378-395) and per-particle combination
    double sums[8] = {su, sv, sd2, 0.0, 0.0, 0.0, 0.0, 0.0};
    // sums[3]: sum lap/m (d2phi), [4]: |du|^2, [5]: du.dphi, [6]: one-body g, [7]: vext
    const bool ob = p.onebody && (mode == MODE_HPSI || mode == MODE_STEP);
    double g1 = 0.0, d2g = 0.0, dudg = 0.0;
    double ll = 0.0, dudl = 0.0, dgdl = 0.0;   // |dUlong|^2, du.dUlong, dg.dUlong
    const double* dl = sm + c.L.dg;
    for (int pt = threadIdx.x; pt < P; pt += NT) {
        const int sp = pt < p.nup ? 0 : 1;
        const double isq = p.isqm[sp], im = p.imass[sp];
        double dph[3], dj[3];
        for (int k = 0; k < 3; ++k) {
            dph[k] = ok ? acc[3 * pt + k] * isq : 0.0;
            dj[k] = du[3 * pt + k];
        }
        sums[3] += (ok ? acc[3 * P + pt] : 0.0) * im;
        sums[4] += dj[0] * dj[0] + dj[1] * dj[1] + dj[2] * dj[2];
        double dg[3] = {0.0, 0.0, 0.0};
        if (ob) {
            double s, co;
            sincos(p.qex[0] * x[3 * pt] + p.qex[1] * x[3 * pt + 1] + p.qex[2] * x[3 * pt + 2], &s, &co);
            sums[7] -= p.v0ex * co;
            g1 -= p.v0exjas * co;
            const double q2 = p.qex[0] * p.qex[0] + p.qex[1] * p.qex[1] + p.qex[2] * p.qex[2];
            d2g += p.v0exjas * q2 * (p.v0exjas * s * s + co);
            for (int k = 0; k < 3; ++k) dg[k] = p.v0exjas * p.qex[k] * s;
            dudg += dj[0] * dg[0] + dj[1] * dg[1] + dj[2] * dg[2];
        }
        double dtot[3];
        for (int k = 0; k < 3; ++k) dtot[k] = dj[k] + dg[k];
        if (jl)
            for (int k = 0; k < 3; ++k) {
                const double l = dl[3 * pt + k];
                ll += l * l;
                dudl += dj[k] * l;
                dgdl += dg[k] * l;
                dtot[k] += l;
            }
        sums[5] += dtot[0] * dph[0] + dtot[1] * dph[1] + dtot[2] * dph[2];
        // the determinant's drift alone replaces this particle's Jastrow
        // gradient (read above) when the caller asks for it
        if (mode == MODE_HPSI && c.a.o_dphi)
            for (int k = 0; k < 3; ++k) du[3 * pt + k] = dph[k];
        // dpsi = dphi + du (+ dg)
        for (int k = 0; k < 3; ++k) acc[3 * pt + k] = dph[k] + dtot[k];
    }
    sums[6] = g1;
    // per-particle sums live on the first ceil(P/32) warps; the one-body
    // and long-range terms are reduced only when present
    const int pw = min((NT / 32), (P + 31) / 32);
    {
        double ps[3] = {sums[3], sums[4], sums[5]};
        block_sum_t<3, NT>(ps, sm + c.L.red, pw);
        sums[3] = ps[0];
        sums[4] = ps[1];
        sums[5] = ps[2];
    }
    double more[5] = {d2g, dudg, ll, dudl, dgdl};
    if (ob || jl) {
        double ex[7] = {sums[6], sums[7], more[0], more[1], more[2], more[3], more[4]};
        block_sum_t<7, NT>(ex, sm + c.L.red, pw);
        sums[6] = ex[0];
        sums[7] = ex[1];
        for (int q = 0; q < 5; ++q) more[q] = ex[2 + q];
    }
    // the scalar results in FP64 on warp 0 only (one FP64 warp instruction
    // holds the sub-partition's FP64 pipe for ~64 cycles), then shared
    __shared__ HRes s_h;
    if (threadIdx.x < 32) {
        const bool extra = ob || jl;
        const double u = extra ? sums[0] + sums[6] + ulong : sums[0];
        const double d2u_j = sums[2] + sums[4];                        // getphi d2u
        // + one-body and long-range terms with their cross terms (wavefunction.f90:178-184)
        const double d2u = extra ? d2u_j + more[0] + (d2long + more[2]) + 2.0 * (more[1] + more[3] + more[4]) : d2u_j;
        h.u = u;
        h.d2u = mode == MODE_GETPHI ? d2u_j : d2u;
        h.v = extra ? sums[1] + sums[7] : sums[1];
        h.vext = sums[7];
        h.logdet = ok ? logdet : DMC_MINUSHUGE;
        h.d2phi = ok ? sums[3] : 0.0;
        h.is = ok ? sgn : 1;
        h.singular = !ok;
        h.psil = h.logdet + u;
        h.d2psi = h.d2phi + d2u + 2.0 * sums[5];
        if (mode == MODE_GETPHI) h.psil = u;
        if (threadIdx.x == 0) s_h = h;
    }
    __syncthreads();
    h = s_h;
    if (p.a2 == 0.0 || (mode != MODE_HPSI && mode != MODE_STEP)) {
        h.psigl = h.psil;
        h.d2psig = h.d2psi;
    } else {
        double sd[1] = {0.0};
        for (int i = threadIdx.x; i < n3; i += NT) sd[0] += acc[i] * acc[i];
        block_sum<1, NT>(sd, sm + c.L.red);
        const double psi = exp(h.psil);
        const double psig2 = psi * psi + p.a2;
        const double f = psi * psi / psig2;
        double* dg = sm + c.L.dg;
        for (int i = threadIdx.x; i < n3; i += NT) dg[i] = f * acc[i];
        h.d2psig = (sd[0] + h.d2psi) * f - psi * psi * psi * psi * sd[0] / (psig2 * psig2);
        h.psigl = 0.5 * log(psig2);
        __syncthreads();
    }
    return h;
}

}  // namespace walker
}  // namespace dmc
