// FP64 walker kernels of the GB300 DMCBS path (sm_103a).
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
// times the orbital.  This is the same algebra with 5*nd^2*K -> 3*nd^2*K
// multiply-adds; FP64 throughput is the bound on GB300.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include "dmc_device.cuh"
#include "dmc_kernels.h"

namespace dmc {

namespace {

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
template <int NV>
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
        for (int k = 0; k < kWarps; ++k) s += red[k * NV + threadIdx.x];
        red[kWarps * NV + threadIdx.x] = s;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = red[kWarps * NV + q];
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

// 4-point Lagrange weights on a uniform grid (coshpot.f90:172-179)
struct Lagrange {
    int idx;
    double c1, c2, c3, c4;
};
__device__ __forceinline__ Lagrange lagrange(double r, double scale, int ntab)
{
    Lagrange L;
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

// minimum-image separation component
__device__ __forceinline__ double min_image(double d, double el, double eli) { return d - el * rint(d * eli); }

struct Ctx {
    const DevParams& p;
    const KernelArgs& a;
    const SmemLayout& L;
    double* sm;
    double* pb;
};

// ---------------------------------------------------------------------------
// Stage 1: Jastrow + potential over all pairs (coshpot.f90:154-205) fused with
// the beta pair function (psislaterbcs.f90:283-293, betafun.f90:173-194).
// Up-down pairs are processed in row chunks; each pair stores its Jastrow
// gradient vector g = dx * u'/r, whose row sums (up) and column sums (down)
// are taken in a fixed order.  Writes S[i][j] = beta(r_ij) and the beta pair
// terms (f'/r, lap f) to pb.  Returns per-thread partial sums of u, v and
// the pair Laplacian part.
// ---------------------------------------------------------------------------
__device__ void pair_stage(const Ctx& c, double& su, double& sv, double& sd2)
{
    const DevParams& p = c.p;
    double* sm = c.sm;
    const double* x = sm + c.L.x;
    double* S = sm + c.L.S;
    double* pv = sm + c.L.R;
    double* du = sm + c.L.acc + 4 * p.npart;
    const int nup = p.nup, ndn = p.ndn, ldS = p.ldS;
    const double el = p.el, eli = p.eli;
    const double imu_ud = 1.0 / (p.mass[0] * p.mass[1] / (p.mass[0] + p.mass[1]));
    for (int i = threadIdx.x; i < 3 * p.npart; i += kThreads) du[i] = 0.0;
    __syncthreads();
    for (int r0 = 0; r0 < nup; r0 += c.L.rows_jas) {
        const int r1 = min(nup, r0 + c.L.rows_jas);
        const int npc = (r1 - r0) * ndn;
        for (int q = threadIdx.x; q < npc; q += kThreads) {
            const int i = r0 + q / ndn, j = q % ndn;
            const double* xi = x + 3 * i;
            const double* xj = x + 3 * (nup + j);
            double d0 = min_image(xi[0] - xj[0], el, eli);
            double d1 = min_image(xi[1] - xj[1], el, eli);
            double d2 = min_image(xi[2] - xj[2], el, eli);
            const double rb = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
            const double rinv = 1.0 / rb;
            double g0 = 0.0, g1 = 0.0, g2 = 0.0;
            // Jastrow and potential, opposite spins (table 1 of the reference)
            {
                const double r = fmax(rb, 1.0e-14);
                if (r < p.range) {
                    const Lagrange W = lagrange(r, p.scale, p.ntab);
                    const TabUD* T = c.a.tud + (W.idx - 1);
                    const TabUD A0 = T[0], A1 = T[1], A2 = T[2], A3 = T[3];
                    const double vp = W.c1 * A0.v + W.c2 * A1.v + W.c3 * A2.v + W.c4 * A3.v;
                    const double uj = W.c1 * A0.u + W.c2 * A1.u + W.c3 * A2.u + W.c4 * A3.u;
                    const double duj = W.c1 * A0.du + W.c2 * A1.du + W.c3 * A2.du + W.c4 * A3.du;
                    const double d2uj = W.c1 * A0.d2u + W.c2 * A1.d2u + W.c3 * A2.d2u + W.c4 * A3.d2u;
                    const double ri = (r == rb) ? rinv : 1.0 / r;
                    sv += vp;
                    su += uj;
                    const double gf = duj * ri;
                    g0 = d0 * gf;
                    g1 = d1 * gf;
                    g2 = d2 * gf;
                    sd2 += (d2uj + 2.0 * gf) * imu_ud;
                }
            }
            // beta(r) of the pair function
            double f = 0.0, dfr = 0.0, d2f = 0.0;
            if (!p.nobeta && !(rb > p.rangeb)) {
                const Lagrange W = lagrange(rb, p.scaleb, p.ntab);
                const TabUD* T = c.a.tud + (W.idx - 1);
                const TabUD A0 = T[0], A1 = T[1], A2 = T[2], A3 = T[3];
                f = W.c1 * A0.b + W.c2 * A1.b + W.c3 * A2.b + W.c4 * A3.b;
                const double df = W.c1 * A0.db + W.c2 * A1.db + W.c3 * A2.db + W.c4 * A3.db;
                d2f = W.c1 * A0.d2b + W.c2 * A1.d2b + W.c3 * A2.d2b + W.c4 * A3.d2b;
                dfr = df * rinv;
            }
            S[i * ldS + j] = f;
            double* pbq = c.pb + 2 * (i * ndn + j);
            pbq[0] = dfr;
            pbq[1] = d2f;
            pv[3 * q + 0] = g0;
            pv[3 * q + 1] = g1;
            pv[3 * q + 2] = g2;
        }
        __syncthreads();
        // row sums -> up particles (+), column sums -> down particles (-)
        const int nr = r1 - r0;
        for (int t = threadIdx.x; t < nr + ndn; t += kThreads) {
            double s0 = 0.0, s1 = 0.0, s2 = 0.0;
            if (t < nr) {
                const double* row = pv + 3 * (t * ndn);
                for (int j = 0; j < ndn; ++j) {
                    s0 += row[3 * j];
                    s1 += row[3 * j + 1];
                    s2 += row[3 * j + 2];
                }
                const int i = r0 + t;
                du[3 * i + 0] += s0 * p.isqm[0];
                du[3 * i + 1] += s1 * p.isqm[0];
                du[3 * i + 2] += s2 * p.isqm[0];
            } else {
                const int j = t - nr;
                for (int r = 0; r < nr; ++r) {
                    const double* e = pv + 3 * (r * ndn + j);
                    s0 += e[0];
                    s1 += e[1];
                    s2 += e[2];
                }
                du[3 * (nup + j) + 0] -= s0 * p.isqm[1];
                du[3 * (nup + j) + 1] -= s1 * p.isqm[1];
                du[3 * (nup + j) + 2] -= s2 * p.isqm[1];
            }
        }
        __syncthreads();
    }
    if (!p.ieq) return;
    // same-spin pairs (coshpot.f90:167 with cjas(2) != 0): up-up then down-down
    for (int blk = 0; blk < 2; ++blk) {
        const int n = blk == 0 ? nup : ndn;
        const int base = blk == 0 ? 0 : nup;
        const double imu = 1.0 / (p.mass[blk] * 0.5);
        const double isq = p.isqm[blk];
        if (n < 2) continue;
        const int rows = max(1, c.L.rsize / (3 * n));
        for (int r0 = 0; r0 < n; r0 += rows) {
            const int r1 = min(n, r0 + rows);
            const int npc = (r1 - r0) * n;
            for (int q = threadIdx.x; q < npc; q += kThreads) {
                const int i = r0 + q / n, j = q % n;
                double g0 = 0.0, g1 = 0.0, g2 = 0.0;
                if (j > i) {
                    const double* xi = x + 3 * (base + i);
                    const double* xj = x + 3 * (base + j);
                    double d0 = min_image(xi[0] - xj[0], el, eli);
                    double d1 = min_image(xi[1] - xj[1], el, eli);
                    double d2 = min_image(xi[2] - xj[2], el, eli);
                    const double r = fmax(sqrt(d0 * d0 + d1 * d1 + d2 * d2), 1.0e-14);
                    if (r < p.range) {
                        const Lagrange W = lagrange(r, p.scale, p.ntab);
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
                pv[3 * q + 0] = g0;
                pv[3 * q + 1] = g1;
                pv[3 * q + 2] = g2;
            }
            __syncthreads();
            const int nr = r1 - r0;
            for (int t = threadIdx.x; t < nr + n; t += kThreads) {
                double s0 = 0.0, s1 = 0.0, s2 = 0.0;
                if (t < nr) {
                    const double* row = pv + 3 * (t * n);
                    for (int j = 0; j < n; ++j) {
                        s0 += row[3 * j];
                        s1 += row[3 * j + 1];
                        s2 += row[3 * j + 2];
                    }
                    const int i = base + r0 + t;
                    du[3 * i + 0] += s0 * isq;
                    du[3 * i + 1] += s1 * isq;
                    du[3 * i + 2] += s2 * isq;
                } else {
                    const int j = t - nr;
                    for (int r = 0; r < nr; ++r) {
                        const double* e = pv + 3 * (r * n + j);
                        s0 += e[0];
                        s1 += e[1];
                        s2 += e[2];
                    }
                    du[3 * (base + j) + 0] -= s0 * isq;
                    du[3 * (base + j) + 1] -= s1 * isq;
                    du[3 * (base + j) + 2] -= s2 * isq;
                }
            }
            __syncthreads();
        }
    }
}

// ---------------------------------------------------------------------------
// Stage 2: pair orbitals (psislaterbcs.f90:248-277).  exp(i k.x) is built
// from exp(i 2 pi x_c / L) and its integer powers, so each particle needs
// three sincos instead of one per k vector.
// U[i][0] = vorb(1), U[i][2q-1] = v_q cos(k_q.x_i), U[i][2q] = v_q sin(k_q.x_i)
// D[j][0] = 1,       D[j][2q-1] = cos(k_q.x_j),     D[j][2q] = sin(k_q.x_j)
// Then the unpaired plane-wave rows and columns of S (:171-206).
// ---------------------------------------------------------------------------
__device__ void orbital_stage(const Ctx& c)
{
    const DevParams& p = c.p;
    double* sm = c.sm;
    const double* x = sm + c.L.x;
    double* U = sm + c.L.U;
    double* D = sm + c.L.D;
    double* E = sm + c.L.E;
    double* S = sm + c.L.S;
    const KVecDev* kq = reinterpret_cast<const KVecDev*>(sm + c.L.kq);
    const int np1 = p.nmax + 1;
    // powers e^{i m theta_c}, m = 0..nmax, E[(p*3+c)*np1 + m] = (re, im)
    for (int t = threadIdx.x; t < 3 * p.npart; t += kThreads) {
        double s1, c1;
        sincospi(2.0 * x[t] * p.eli, &s1, &c1);
        double* e = E + 2 * t * np1;
        e[0] = 1.0;
        e[1] = 0.0;
        if (p.nmax >= 1) {
            e[2] = c1;
            e[3] = s1;
        }
        double cr = c1, ci = s1;
        for (int m = 2; m <= p.nmax; ++m) {
            const double nr = cr * c1 - ci * s1;
            const double ni = cr * s1 + ci * c1;
            cr = nr;
            ci = ni;
            e[2 * m] = cr;
            e[2 * m + 1] = ci;
        }
    }
    __syncthreads();
    const int nq = p.nk - 1;
    const int items = p.npart * (nq + 1);
    for (int t = threadIdx.x; t < items; t += kThreads) {
        const int part = t / (nq + 1), q = t % (nq + 1);
        const bool up = part < p.nup;
        double* row = up ? U + part * p.ldU : D + (part - p.nup) * p.ldU;
        if (q == 0) {
            row[0] = up ? p.vorb1 : 1.0;
            continue;
        }
        const KVecDev& K = kq[q];
        double zr = 1.0, zi = 0.0;
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) {
            const int n = K.n[cc];
            if (n == 0) continue;
            const double* e = E + 2 * ((part * 3 + cc) * np1 + (n < 0 ? -n : n));
            const double er = e[0], ei = n < 0 ? -e[1] : e[1];
            const double nr = zr * er - zi * ei;
            const double ni = zr * ei + zi * er;
            zr = nr;
            zi = ni;
        }
        if (up) {
            row[2 * q - 1] = K.v * zr;
            row[2 * q] = K.v * zi;
        } else {
            row[2 * q - 1] = zr;
            row[2 * q] = zi;
        }
    }
    // unpaired plane waves: up columns ndn.., down rows nup.., zero corner
    const int nd = p.nd, ldS = p.ldS;
    for (int t = threadIdx.x; t < p.nup * p.nexup; t += kThreads) {
        const int i = t / p.nexup, jj = t % p.nexup;
        const double* xi = x + 3 * i;
        const double arg = p.akup[jj][0] * xi[0] + p.akup[jj][1] * xi[1] + p.akup[jj][2] * xi[2];
        double s, co;
        sincos(arg, &s, &co);
        S[i * ldS + p.ndn + jj] = p.sinup[jj] ? s : co;
    }
    for (int t = threadIdx.x; t < p.ndn * p.nexdn; t += kThreads) {
        const int j = t / p.nexdn, jj = t % p.nexdn;
        const double* xj = x + 3 * (p.nup + j);
        const double arg = p.akdn[jj][0] * xj[0] + p.akdn[jj][1] * xj[1] + p.akdn[jj][2] * xj[2];
        double s, co;
        sincos(arg, &s, &co);
        S[(p.nup + jj) * ldS + j] = p.sindn[jj] ? s : co;
    }
    for (int t = threadIdx.x; t < p.nexdn * p.nexup; t += kThreads) {
        const int r = t / p.nexup, cc = t % p.nexup;
        S[(p.nup + r) * ldS + p.ndn + cc] = 0.0;
    }
    __syncthreads();
}

// Stage 3: S[i][j] = sum_q U[i][q] D[j][q] + beta (psislaterbcs.f90:278,289)
__device__ void gemm_stage(const Ctx& c)
{
    const DevParams& p = c.p;
    double* sm = c.sm;
    const double* U = sm + c.L.U;
    const double* D = sm + c.L.D;
    double* S = sm + c.L.S;
    const int ncol = p.ncol, ldU = p.ldU;
    const int nout = p.nup * p.ndn;
    // two outputs of one row per thread (shared U row)
    const int half = (p.ndn + 1) / 2;
    for (int t = threadIdx.x; t < p.nup * half; t += kThreads) {
        const int i = t / half, j0 = t % half, j1 = j0 + half;
        const double* u = U + i * ldU;
        const double* d0 = D + j0 * ldU;
        const bool two = j1 < p.ndn;
        const double* d1 = D + (two ? j1 : j0) * ldU;
        double a0 = 0.0, a1 = 0.0;
#pragma unroll 4
        for (int q = 0; q < ncol; ++q) {
            const double uq = u[q];
            a0 = fma(uq, d0[q], a0);
            a1 = fma(uq, d1[q], a1);
        }
        S[i * p.ldS + j0] = a0 + S[i * p.ldS + j0];
        if (two) S[i * p.ldS + j1] = a1 + S[i * p.ldS + j1];
    }
    (void)nout;
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Stage 4: in-place Gauss-Jordan inverse with partial pivoting (first
// maximum wins, as LAPACK idamax).  The pivot sequence is the one dgetrf
// takes (matrixlapack.f90:20), so log|det| = sum log|pivot| and the sign
// follow matrixlapack.f90:27-33.  Row interchanges are undone on the columns
// of the inverse at the end.  Returns false for an exactly singular matrix.
// ---------------------------------------------------------------------------
__device__ bool inverse_stage(const Ctx& c, double& logdet, int& sgn)
{
    const DevParams& p = c.p;
    double* sm = c.sm;
    double* A = sm + c.L.S;
    double* colk = sm + c.L.colk;
    int* piv = reinterpret_cast<int*>(sm + c.L.red + 512);   // nd ints
    __shared__ double s_pinv;
    __shared__ int s_piv;
    __shared__ int s_sing;
    const int n = p.nd, ld = p.ldS;
    double mant = 1.0;
    int expo = 0;
    int sg = 1;
    __shared__ double s_logdet;
    __shared__ int s_sgn;
    if (threadIdx.x == 0) s_sing = 0;
    for (int k = 0; k < n; ++k) {
        // pivot search in column k, rows k..n-1 (warp 0)
        if (threadIdx.x < 32) {
            double best = -1.0;
            int bi = n;
            for (int i = k + (int)threadIdx.x; i < n; i += 32) {
                const double v = fabs(A[i * ld + k]);
                if (v > best) {
                    best = v;
                    bi = i;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) {
                    best = ob;
                    bi = oi;
                }
            }
            if (threadIdx.x == 0) {
                const double pv = A[bi * ld + k];
                s_piv = bi;
                piv[k] = bi;
                if (pv == 0.0) s_sing = 1;
                s_pinv = 1.0 / pv;
            }
        }
        __syncthreads();
        if (s_sing) break;
        const int pr = s_piv;
        const double pinv = s_pinv;
        // save column k (rows in swapped order), swap rows k/pr, scale row k
        for (int t = threadIdx.x; t < n; t += kThreads) {
            const int src = (t == k) ? pr : ((t == pr) ? k : t);
            colk[t] = A[src * ld + k];
            if (t != k) {
                const double a = A[k * ld + t];
                const double b = A[pr * ld + t];
                double nk = a;
                if (pr != k) {
                    A[pr * ld + t] = a;
                    nk = b;
                }
                A[k * ld + t] = nk * pinv;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            // |det| kept as mantissa * 2^exponent; one log at the end
            int ex;
            const double pvv = colk[k];
            mant = frexp(mant * fabs(pvv), &ex);
            expo += ex;
            sg = (pvv < 0.0) ? -sg : sg;
            if (pr != k) sg = -sg;
        }
        // eliminate column k from every other row
        const int tot = n * n;
        for (int t = threadIdx.x; t < tot; t += kThreads) {
            const int i = t / n, cc = t % n;
            if (i == k) continue;
            if (cc == k)
                A[i * ld + k] = -colk[i] * pinv;
            else
                A[i * ld + cc] = fma(-colk[i], A[k * ld + cc], A[i * ld + cc]);
        }
        if (threadIdx.x == 0) A[k * ld + k] = pinv;
        __syncthreads();
    }
    const bool sing = s_sing != 0;
    if (!sing) {
        // undo the row interchanges on the columns: inv(S) = inv(P S) P
        for (int k = n - 1; k >= 0; --k) {
            const int pr = piv[k];
            if (pr != k)
                for (int t = threadIdx.x; t < n; t += kThreads) {
                    const double a = A[t * ld + k];
                    A[t * ld + k] = A[t * ld + pr];
                    A[t * ld + pr] = a;
                }
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) {
        s_logdet = log(mant) + expo * 0.69314718055994530942;
        s_sgn = sg;
    }
    __syncthreads();
    logdet = s_logdet;
    sgn = s_sgn;
    return !sing;
}

// ---------------------------------------------------------------------------
// Stage 5: drift and Laplacian of log det from the inverse.
//  up i:   sum_q k_q (U_c G_s - U_s G_c), lap -|k|^2 (U_c G_c + U_s G_s),
//          G_{c,s} = sum_j D[j][c,s] Sinv[j][i]
//  down j: sum_q k_q (H_s D_c - H_c D_s), lap -|k|^2 (H_c D_c + H_s D_s),
//          H_{c,s} = sum_i Sinv[j][i] U[i][c,s]
// Work items (particle, k vector) are split into contiguous per-thread
// chunks; each thread sums its chunk per particle and the partial sums of a
// particle are added in thread order.
// ---------------------------------------------------------------------------
__device__ void drift_stage(const Ctx& c)
{
    const DevParams& p = c.p;
    double* sm = c.sm;
    const double* U = sm + c.L.U;
    const double* D = sm + c.L.D;
    const double* Si = sm + c.L.S;
    const KVecDev* kq = reinterpret_cast<const KVecDev*>(sm + c.L.kq);
    double* acc = sm + c.L.acc;             // drift [3N], lap [N]
    double* part = sm + c.L.red;            // per thread: 2 segments x (id, 4 sums)
    const int nq = p.nk - 1, P = p.npart, ld = p.ldS, ldU = p.ldU;
    const int items = P * nq;
    const int chunk = (items + kThreads - 1) / kThreads;
    const int b = threadIdx.x * chunk, e = min(items, b + chunk);
    double s[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
    int seg = 0, cur = b < e ? b / nq : -1, first = cur;
    for (int it = b; it < e; ++it) {
        const int pt = it / nq, q = it % nq + 1;
        if (pt != cur) {
            seg = 1;
            cur = pt;
        }
        const KVecDev& K = kq[q];
        const int qc = 2 * q - 1, qs = 2 * q;
        double t, l;
        if (pt < p.nup) {
            const int i = pt;
            double gc = 0.0, gs = 0.0;
            for (int j = 0; j < p.ndn; ++j) {
                const double sji = Si[j * ld + i];
                gc = fma(D[j * ldU + qc], sji, gc);
                gs = fma(D[j * ldU + qs], sji, gs);
            }
            const double uc = U[i * ldU + qc], us = U[i * ldU + qs];
            t = uc * gs - us * gc;
            l = uc * gc + us * gs;
        } else {
            const int j = pt - p.nup;
            double hc = 0.0, hs = 0.0;
            for (int i = 0; i < p.nup; ++i) {
                const double sji = Si[j * ld + i];
                hc = fma(sji, U[i * ldU + qc], hc);
                hs = fma(sji, U[i * ldU + qs], hs);
            }
            const double dc = D[j * ldU + qc], ds = D[j * ldU + qs];
            t = hs * dc - hc * ds;
            l = hc * dc + hs * ds;
        }
        s[seg][0] = fma(K.k[0], t, s[seg][0]);
        s[seg][1] = fma(K.k[1], t, s[seg][1]);
        s[seg][2] = fma(K.k[2], t, s[seg][2]);
        s[seg][3] = fma(-K.k2, l, s[seg][3]);
    }
    // publish the (at most two) particle segments of this thread's chunk;
    // a chunk never spans more than two particles because chunk <= nq
    double* my = part + threadIdx.x * 8;
    for (int k = 0; k < 4; ++k) {
        my[k] = s[0][k];
        my[4 + k] = s[1][k];
    }
    (void)first;
    __syncthreads();
    // particle pt is covered by threads floor(pt*nq/chunk) .. floor((pt*nq+nq-1)/chunk)
    for (int pt = threadIdx.x; pt < P; pt += kThreads) {
        double r[4] = {0, 0, 0, 0};
        const int t0 = (pt * nq) / chunk, t1 = (pt * nq + nq - 1) / chunk;
        for (int t = t0; t <= t1 && t < kThreads; ++t) {
            const int tb = t * chunk, te = min(items, tb + chunk);
            if (tb >= te) continue;
            const double* o = part + t * 8;
            const int sl = (tb / nq == pt) ? 0 : (((te - 1) / nq == pt) ? 4 : -1);
            if (sl < 0) continue;
            for (int k = 0; k < 4; ++k) r[k] += o[sl + k];
        }
        acc[3 * pt + 0] = r[0];
        acc[3 * pt + 1] = r[1];
        acc[3 * pt + 2] = r[2];
        acc[3 * P + pt] = r[3];
    }
    __syncthreads();
}

// Stage 6: beta terms of the drift and Laplacian (psislaterbcs.f90:290-291
// through :213-222): per up-down pair h = Sinv[j][i] f'/r dx, l = Sinv[j][i]
// lap f; row sums go to the up particle, column sums (negated drift) to the
// down particle.  Then the unpaired plane waves.
__device__ void beta_drift_stage(const Ctx& c)
{
    const DevParams& p = c.p;
    double* sm = c.sm;
    const double* x = sm + c.L.x;
    const double* Si = sm + c.L.S;
    double* pv = sm + c.L.R;
    double* acc = sm + c.L.acc;
    const int nup = p.nup, ndn = p.ndn, ld = p.ldS, P = p.npart;
    if (!p.nobeta) {
        for (int r0 = 0; r0 < nup; r0 += c.L.rows_beta) {
            const int r1 = min(nup, r0 + c.L.rows_beta);
            const int npc = (r1 - r0) * ndn;
            for (int q = threadIdx.x; q < npc; q += kThreads) {
                const int i = r0 + q / ndn, j = q % ndn;
                const double* xi = x + 3 * i;
                const double* xj = x + 3 * (nup + j);
                const double* pbq = c.pb + 2 * (i * ndn + j);
                const double sij = Si[j * ld + i];
                const double w = sij * pbq[0];
                pv[4 * q + 0] = w * min_image(xi[0] - xj[0], p.el, p.eli);
                pv[4 * q + 1] = w * min_image(xi[1] - xj[1], p.el, p.eli);
                pv[4 * q + 2] = w * min_image(xi[2] - xj[2], p.el, p.eli);
                pv[4 * q + 3] = sij * pbq[1];
            }
            __syncthreads();
            const int nr = r1 - r0;
            for (int t = threadIdx.x; t < nr + ndn; t += kThreads) {
                double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
                if (t < nr) {
                    const double* row = pv + 4 * (t * ndn);
                    for (int j = 0; j < ndn; ++j) {
                        s0 += row[4 * j];
                        s1 += row[4 * j + 1];
                        s2 += row[4 * j + 2];
                        s3 += row[4 * j + 3];
                    }
                    const int i = r0 + t;
                    acc[3 * i + 0] += s0;
                    acc[3 * i + 1] += s1;
                    acc[3 * i + 2] += s2;
                    acc[3 * P + i] += s3;
                } else {
                    const int j = t - nr;
                    for (int r = 0; r < nr; ++r) {
                        const double* e = pv + 4 * (r * ndn + j);
                        s0 += e[0];
                        s1 += e[1];
                        s2 += e[2];
                        s3 += e[3];
                    }
                    acc[3 * (nup + j) + 0] -= s0;
                    acc[3 * (nup + j) + 1] -= s1;
                    acc[3 * (nup + j) + 2] -= s2;
                    acc[3 * P + nup + j] += s3;
                }
            }
            __syncthreads();
        }
    }
    // unpaired plane waves (psislaterbcs.f90:171-206 with :211-223)
    if (p.nexup > 0 || p.nexdn > 0) {
        for (int pt = threadIdx.x; pt < P; pt += kThreads) {
            const double* xp = x + 3 * pt;
            double g0 = 0, g1 = 0, g2 = 0, lp = 0;
            if (pt < nup) {
                for (int jj = 0; jj < p.nexup; ++jj) {
                    const double* k = p.akup[jj];
                    double s, co;
                    sincos(k[0] * xp[0] + k[1] * xp[1] + k[2] * xp[2], &s, &co);
                    const double w = Si[(ndn + jj) * ld + pt];
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
                    const double w = Si[j * ld + (nup + jj)];
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

// Scalars of one evaluation.
struct HRes {
    double psil, d2psi, v, vext, psigl, d2psig, u, d2u, logdet, d2phi;
    int is;
    bool singular;
};

// ---------------------------------------------------------------------------
// hpsi (wavefunction.f90:161-201) for the positions in sm[L.x].  Leaves
// dpsi in acc[0..3N) and dpsig in sm[L.drift] when a2 != 0.
// mode MODE_GETPHI stops after the Jastrow; MODE_BCS skips the Jastrow.
// ---------------------------------------------------------------------------
__device__ HRes hpsi_eval(const Ctx& c, int mode)
{
    const DevParams& p = c.p;
    double* sm = c.sm;
    const int P = p.npart, n3 = 3 * P;
    double* acc = sm + c.L.acc;
    double* du = acc + 4 * P;
    const double* x = sm + c.L.x;
    HRes h;
    double su = 0.0, sv = 0.0, sd2 = 0.0;
    pair_stage(c, su, sv, sd2);   // also fills the beta part of S (needed by MODE_BCS too)
    if (mode == MODE_BCS) {
        su = sv = sd2 = 0.0;
        for (int i = threadIdx.x; i < n3; i += kThreads) du[i] = 0.0;
        __syncthreads();
    }
    double logdet = 0.0;
    int sgn = 1;
    bool ok = true;
    if (mode != MODE_GETPHI) {
        orbital_stage(c);
        gemm_stage(c);
        ok = inverse_stage(c, logdet, sgn);
        if (ok) {
            drift_stage(c);
            beta_drift_stage(c);
        } else {
            for (int i = threadIdx.x; i < 4 * P; i += kThreads) acc[i] = 0.0;
            __syncthreads();
        }
    } else {
        for (int i = threadIdx.x; i < 4 * P; i += kThreads) acc[i] = 0.0;
        __syncthreads();
    }
    // one-body term (psislaterbcs.f90:378-395) and per-particle combination
    double sums[8] = {su, sv, sd2, 0.0, 0.0, 0.0, 0.0, 0.0};
    // sums[3]: sum lap/m (d2phi), [4]: |du|^2, [5]: du.dphi, [6]: one-body g, [7]: vext
    double g1 = 0.0, d2g = 0.0, dudg = 0.0, dgdphi = 0.0;
    for (int pt = threadIdx.x; pt < P; pt += kThreads) {
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
        if (p.onebody && (mode == MODE_HPSI || mode == MODE_STEP)) {
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
        sums[5] += dtot[0] * dph[0] + dtot[1] * dph[1] + dtot[2] * dph[2];
        dgdphi += 0.0;
        // dpsi = dphi + du (+ dg)
        for (int k = 0; k < 3; ++k) acc[3 * pt + k] = dph[k] + dtot[k];
    }
    sums[6] = g1;
    double more[2] = {d2g, dudg};
    block_sum<8>(sums, sm + c.L.red);
    block_sum<2>(more, sm + c.L.red);
    const double u = sums[0] + sums[6];
    const double d2u_j = sums[2] + sums[4];                        // getphi d2u
    const double d2u = d2u_j + more[0] + 2.0 * more[1];            // + one-body terms
    h.u = u;
    h.d2u = d2u;
    h.v = sums[1] + sums[7];
    h.vext = sums[7];
    h.logdet = ok ? logdet : DMC_MINUSHUGE;
    h.d2phi = ok ? sums[3] : 0.0;
    h.is = ok ? sgn : 1;
    h.singular = !ok;
    h.psil = h.logdet + u;
    h.d2psi = h.d2phi + d2u + 2.0 * sums[5];
    if (mode == MODE_GETPHI) {
        h.psil = u;
    }
    if (p.a2 == 0.0 || mode != MODE_HPSI && mode != MODE_STEP) {
        h.psigl = h.psil;
        h.d2psig = h.d2psi;
    } else {
        double sd[1] = {0.0};
        for (int i = threadIdx.x; i < n3; i += kThreads) sd[0] += acc[i] * acc[i];
        block_sum<1>(sd, sm + c.L.red);
        const double psi = exp(h.psil);
        const double psig2 = psi * psi + p.a2;
        const double f = psi * psi / psig2;
        double* dg = sm + c.L.dg;
        for (int i = threadIdx.x; i < n3; i += kThreads) dg[i] = f * acc[i];
        h.d2psig = (sd[0] + h.d2psi) * f - psi * psi * psi * psi * sd[0] / (psig2 * psig2);
        h.psigl = 0.5 * log(psig2);
        __syncthreads();
    }
    (void)dgdphi;
    return h;
}

}  // namespace

// ---------------------------------------------------------------------------
// The walker kernel: persistent CTAs, one walker per CTA per iteration.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads, 2)
walker_kernel(const __grid_constant__ DevParams p, const __grid_constant__ KernelArgs a, SmemLayout L)
{
    extern __shared__ __align__(16) double sm[];
    const int P = p.npart, n3 = 3 * P;
    for (int i = threadIdx.x; i < p.nk * 8; i += kThreads) sm[L.kq + i] = reinterpret_cast<const double*>(a.kv)[i];
    double* pb = L.pb_in_smem ? sm + L.pb : a.gscratch + (size_t)blockIdx.x * L.pb_size;
    Ctx c{p, a, L, sm, pb};
    __syncthreads();
    for (int w = blockIdx.x; w < a.nw; w += gridDim.x) {
        double* x = sm + L.x;
        double* xo = sm + L.xo;
        double* dxs = sm + L.dx;
        double* drift = sm + L.drift;
        const int src = a.nw - 1 - w;   // MODE_STEP pops from the top
        unsigned long long s0 = 0;
        if (a.mode == MODE_STEP) {
            // step.f90:59-74: wrap, gaussians, drift, proposal
            s0 = a.in.irn[src] & kMask48;
            const double* x1 = a.in.x + (size_t)src * n3;
            const double* g1 = a.in.dpsig + (size_t)src * n3;
            for (int e = threadIdx.x; e < n3; e += kThreads) xo[e] = min_image(x1[e], p.el, p.eli);
            // Box-Muller pairs (ran.f90:74-104): draws t = 1..nrand from the
            // walker's stream, pair i uses draws 2i-1, 2i
            const int npairs = (n3 + 1) / 2;
            for (int q = threadIdx.x; q < npairs; q += kThreads) {
                const double u1 = lcg_uniform(lcg_jump(s0, a.jumpA, a.jumpC, 2 * q + 1));
                const double u2 = lcg_uniform(lcg_jump(s0, a.jumpA, a.jumpC, 2 * q + 2));
                double sn, cs;
                sincospi(2.0 * u1, &sn, &cs);
                const double r = sqrt(-2.0 * log(u2));
                if (2 * q + 1 < n3) {
                    dxs[2 * q] = sn * r;
                    dxs[2 * q + 1] = cs * r;
                } else {
                    dxs[2 * q] = cs * r;   // odd count: the last one uses cos (ran.f90:95-102)
                }
            }
            __syncthreads();
            for (int e = threadIdx.x; e < n3; e += kThreads) {
                const int sp = (e / 3) < p.nup ? 0 : 1;
                const double sig = p.sigma[sp];
                double d = g1[e] * (sig * sig) * p.sqm[sp];
                if (p.cutdrift) d = fmin(p.dcut[sp], fmax(-p.dcut[sp], d));
                drift[e] = d;
                const double dxe = d + sig * dxs[e];
                dxs[e] = dxe;
                x[e] = min_image(xo[e] + dxe, p.el, p.eli);
            }
        } else {
            for (int e = threadIdx.x; e < n3; e += kThreads) x[e] = a.xin[(size_t)w * n3 + e];
        }
        __syncthreads();
        const int hmode = a.mode == MODE_STEP ? MODE_HPSI : a.mode;
        HRes h = hpsi_eval(c, a.mode == MODE_STEP ? MODE_STEP : hmode);
        double* dpsi = sm + L.acc;
        const double* dpsig = (p.a2 == 0.0) ? dpsi : sm + L.dg;
        if (h.singular && threadIdx.x == 0 && a.status) atomicOr(a.status, 1);
        if (a.mode != MODE_STEP) {
            // ---- batched wavefunction outputs ----
            if (threadIdx.x == 0) {
                if (a.o_psil) a.o_psil[w] = h.psil;
                if (a.o_is) a.o_is[w] = h.is;
                if (a.o_d2psi) a.o_d2psi[w] = a.mode == MODE_GETPHI ? h.d2u : (a.mode == MODE_BCS ? h.d2phi : h.d2psi);
                if (a.o_v) a.o_v[w] = h.v;
                if (a.o_vext) a.o_vext[w] = h.vext;
                if (a.o_psigl) a.o_psigl[w] = h.psigl;
                if (a.o_d2psig) a.o_d2psig[w] = h.d2psig;
            }
            if (a.o_dpsi)
                for (int e = threadIdx.x; e < n3; e += kThreads) {
                    double val = dpsi[e];
                    if (a.mode == MODE_GETPHI) val = sm[L.acc + 4 * P + e];
                    a.o_dpsi[(size_t)w * n3 + e] = val;
                }
            if (a.o_dpsig)
                for (int e = threadIdx.x; e < n3; e += kThreads) a.o_dpsig[(size_t)w * n3 + e] = dpsig[e];
            if (a.o_sinv) {
                const int nd = p.nd;
                // column-major nd x nd as the reference's smati(nd,nd)
                for (int t = threadIdx.x; t < nd * nd; t += kThreads) {
                    const int r = t % nd, cc = t / nd;
                    a.o_sinv[(size_t)w * nd * nd + t] = h.singular ? 0.0 : sm[L.S + r * p.ldS + cc];
                }
            }
            __syncthreads();
            continue;
        }
        // ---- step1 decision (step.f90:76-226) ----
        __shared__ int s_take_new;
        __shared__ double s_prob;
        const double hb = p.hbar;
        const double* pin_psil = a.in.psil;
        const double o_psil = pin_psil[src], o_psigl = a.in.psigl[src], o_d2psi = a.in.d2psi[src];
        const double o_d2psig = a.in.d2psig[src], o_v = a.in.v[src], o_vext = a.in.vext[src];
        const double o_weight = a.in.weight[src];
        const float o_wt0 = a.in.wt0[src];
        const int o_is = a.in.is[src];
        const double eo = -hb * o_d2psi + o_v;
        const double en = -hb * h.d2psi + h.v;
        const int nr = p.nrand;
        unsigned long long irn_out = lcg_jump(s0, a.jumpA, a.jumpC, nr);
        double* est = a.est + (size_t)w * p.nest * 2;
        const bool metro = (p.idmc == -1 || p.idmc == 0 || p.idmc == 2);
        if (metro) {
            // Metropolis with the drift Green's function ratio (step.f90:80-91)
            double acc1[2] = {0.0, 0.0};
            for (int e = threadIdx.x; e < n3; e += kThreads) {
                const int sp = (e / 3) < p.nup ? 0 : 1;
                const double sig = p.sigma[sp];
                double dn = dpsig[e] * (sig * sig) * p.sqm[sp];
                if (p.cutdrift) dn = fmin(p.dcut[sp], fmax(-p.dcut[sp], dn));
                const double d1 = drift[e] + dn;
                const double d2 = drift[e] - dn - 2.0 * dxs[e];
                acc1[0] += d1 * d2 / (2.0 * (sig * sig));
            }
            block_sum<2>(acc1, sm + L.red);
            if (threadIdx.x == 0) {
                double prob = (p.idmc == 2 ? 2.0 * (h.psigl - o_psigl) : 2.0 * (h.psil - o_psil)) + acc1[0];
                prob = exp(fmin(0.0, prob));
                const double rn = lcg_uniform(lcg_jump(s0, a.jumpA, a.jumpC, nr + 1));
                s_take_new = rn < prob;
                s_prob = prob;
            }
            irn_out = lcg_jump(s0, a.jumpA, a.jumpC, nr + 1);
            __syncthreads();
        } else if (threadIdx.x == 0) {
            s_take_new = 1;
        }
        __syncthreads();
        const bool take_new = s_take_new != 0;
        // sum |dpsi|^2/m of the pushed walker for the Jackson-Feenberg energy
        double ejfd[1] = {0.0};
        if (p.idmc == -1 || p.idmc == 0) {
            const double* dsrc = take_new ? dpsi : a.in.dpsi + (size_t)src * n3;
            for (int e = threadIdx.x; e < n3; e += kThreads) {
                const int sp = (e / 3) < p.nup ? 0 : 1;
                ejfd[0] += dsrc[e] * dsrc[e] * p.imass[sp];
            }
            block_sum<1>(ejfd, sm + L.red);
        }
        // scalars of the pushed walker
        const int k = w;   // push order = pop order
        if (threadIdx.x == 0) {
            for (int q = 0; q < 2 * p.nest; ++q) est[q] = 0.0;
            auto add = [&](int i1, double val, double wt) {
                est[2 * (i1 - 1)] = val;
                est[2 * (i1 - 1) + 1] = wt;
            };
            const double nfac = p.nfac;
            double wnew = o_weight;
            float wt0new = o_wt0;
            if (p.idmc == -1 || p.idmc == 0) {
                if (take_new) {
                    const double ejf = -0.5 * hb * (h.d2psi - ejfd[0]) + h.v;
                    add(1, en * nfac, o_weight);
                    add(2, (en - h.v) * nfac, o_weight);
                    add(3, h.v * nfac, o_weight);
                    add(4, h.vext * nfac, o_weight);
                    add(5, ejf * nfac, o_weight);
                    add(6, 1.0, 1.0);
                    wt0new = (float)h.is;
                } else {
                    const double ejf = -0.5 * hb * (o_d2psi - ejfd[0]) + o_v;
                    add(1, eo * nfac, o_weight);
                    add(2, (eo - o_v) * nfac, o_weight);
                    add(3, o_v * nfac, o_weight);
                    add(4, o_vext * nfac, o_weight);
                    add(5, ejf * nfac, o_weight);
                    add(6, 0.0, 1.0);
                }
            } else if (p.idmc == 1 || p.idmc == -2) {
                const double ego = -hb * o_d2psig + o_v;
                const double egn = -hb * h.d2psig + h.v;
                double wt = exp(-(0.5 * (ego + egn) - p.etrial) * p.dt);
                wnew = fmin(p.wtcut, wt);
                if (h.is != o_is) {
                    if (p.fn) {
                        wnew = 0.0;
                        wt = 0.0;
                    }
                    add(5, 1.0, 1.0);
                } else {
                    add(5, 0.0, 1.0);
                }
                const double wtg = wt * exp(h.psil - h.psigl) * h.is * (double)o_wt0;
                if (a.opcomp) {
                    add(1, en * nfac, wtg);
                    add(2, (en - h.v) * nfac, wtg);
                    add(3, h.v * nfac, wtg);
                    add(4, h.vext * nfac, wtg);
                    add(6, 0.5 * (ego + egn) * nfac, 1.0);
                    add(7, exp(h.psil - h.psigl), 1.0);
                    add(8, h.is * exp(h.psil), 1.0);
                    add(9, exp(h.psigl), 1.0);
                    add(10, 1.0 * h.is, 1.0);
                    add(11, wt, 1.0);
                    add(12, wtg, 1.0);
                    add(13, copysign(1.0, wtg), 1.0);
                    add(14, copysign(1.0, wtg), wtg);
                }
            } else {   // idmc == 2
                if (take_new) {
                    double wt = exp(-(0.5 * (eo + en) - p.etrial) * p.dt);
                    wnew = fmin(p.wtcut, wt);
                    if (h.is != o_is) {
                        if (p.fn) {
                            wnew = 0.0;
                            wt = 0.0;
                        }
                        add(4, 1.0, 1.0);
                    } else {
                        add(4, 0.0, 1.0);
                    }
                    const double wtg = wt * exp(h.psil - h.psigl) * h.is * (double)o_wt0;
                    if (a.opcomp) {
                        add(1, en * nfac, wtg);
                        add(2, (en - h.v) * nfac, wtg);
                        add(3, h.v * nfac, wtg);
                        add(6, exp(h.psil - h.psigl), 1.0);
                        add(7, h.is * exp(h.psil), 1.0);
                        add(8, exp(h.psigl), 1.0);
                        add(9, 1.0 * h.is, 1.0);
                        add(10, wt, 1.0);
                        add(11, wtg, 1.0);
                        add(12, copysign(1.0, wtg), 1.0);
                        add(13, copysign(1.0, wtg), wtg);
                    }
                    add(5, 1.0, 1.0);
                } else {
                    const double wt = exp(-(eo - p.etrial) * p.dt);
                    const double wtg = wt * exp(o_psil - o_psigl) * o_is * (double)o_wt0;
                    wnew = fmin(p.wtcut, wt * o_weight);
                    if (a.opcomp) {
                        add(1, eo * nfac, wtg);
                        add(2, (eo - o_v) * nfac, wtg);
                        add(3, o_v * nfac, wtg);
                        add(6, exp(o_psil - o_psigl), 1.0);
                        add(7, o_is * exp(o_psil), 1.0);
                        add(8, exp(o_psigl), 1.0);
                        add(9, 1.0 * o_is, 1.0);
                        add(10, wt, 1.0);
                        add(11, wtg, 1.0);
                        add(12, copysign(1.0, wtg), 1.0);
                        add(13, copysign(1.0, wtg), wtg);
                    }
                    add(5, 0.0, 1.0);
                }
            }
            DevStack o = a.out;
            if (take_new) {
                o.psil[k] = h.psil;
                o.psigl[k] = h.psigl;
                o.d2psi[k] = h.d2psi;
                o.d2psig[k] = h.d2psig;
                o.v[k] = h.v;
                o.vext[k] = h.vext;
                o.is[k] = h.is;
            } else {
                o.psil[k] = o_psil;
                o.psigl[k] = o_psigl;
                o.d2psi[k] = o_d2psi;
                o.d2psig[k] = o_d2psig;
                o.v[k] = o_v;
                o.vext[k] = o_vext;
                o.is[k] = o_is;
            }
            o.weight[k] = wnew;
            o.wt0[k] = wt0new;
            o.irn[k] = irn_out;
            o.psil0[k] = a.in.psil0[src];
            o.psigl0[k] = a.in.psigl0[src];
        }
        if (take_new) {
            for (int e = threadIdx.x; e < n3; e += kThreads) {
                a.out.x[(size_t)k * n3 + e] = x[e];
                a.out.dpsi[(size_t)k * n3 + e] = dpsi[e];
                a.out.dpsig[(size_t)k * n3 + e] = dpsig[e];
            }
        } else {
            for (int e = threadIdx.x; e < n3; e += kThreads) {
                a.out.x[(size_t)k * n3 + e] = xo[e];
                a.out.dpsi[(size_t)k * n3 + e] = a.in.dpsi[(size_t)src * n3 + e];
                a.out.dpsig[(size_t)k * n3 + e] = a.in.dpsig[(size_t)src * n3 + e];
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Estimator block sums (estimator.f90:72-82): est[n][nest][2] -> valblk,
// valblk2, wtblk (accumulated), fixed-order tree per estimator.
// ---------------------------------------------------------------------------
__global__ void estimator_kernel(const double* est, int n, int nest, double* valblk, double* valblk2, double* wtblk)
{
    const int e = blockIdx.x;
    double s[3] = {0.0, 0.0, 0.0};
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const double v = est[((size_t)k * nest + e) * 2], wt = est[((size_t)k * nest + e) * 2 + 1];
        s[0] += v * wt;
        s[1] += v * v * wt;
        s[2] += wt;
    }
    __shared__ double red[3 * 32];
    for (int q = 0; q < 3; ++q) s[q] = warp_sum(s[q]);
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    if (lane == 0)
        for (int q = 0; q < 3; ++q) red[wp * 3 + q] = s[q];
    __syncthreads();
    if (threadIdx.x == 0) {
        double t[3] = {0.0, 0.0, 0.0};
        for (int k = 0; k < (int)(blockDim.x / 32); ++k)
            for (int q = 0; q < 3; ++q) t[q] += red[k * 3 + q];
        valblk[e] += t[0];
        valblk2[e] += t[1];
        wtblk[e] += t[2];
    }
}

// ---------------------------------------------------------------------------
// branch (step.f90:287-315), three passes: copy counts, scan, scatter.
// The input stack is popped from the top: pop index m = n-1-j.
// ---------------------------------------------------------------------------
__global__ void branch_count_kernel(DevStack in, int n, double factor, int* counts,
                                    unsigned long long* irn1, unsigned long long* wtisto)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    const int j = n - 1 - m;
    const double wt = in.weight[j] * factor;
    // ran1 on the walker's own state
    const unsigned long long s = in.irn[j] & kMask48;
    const unsigned long long s1 = (44485709377909ull * s + 96309754297ull) & kMask48;
    const double rn = lcg_uniform(s1);
    const int iwt = (int)(wt + rn);
    counts[m] = iwt > 0 ? iwt : 0;
    irn1[m] = s1;
    if (iwt >= 0 && iwt < DMC_WTISTO) atomicAdd(&wtisto[iwt], 1ull);
}

// single-CTA exclusive scan of counts[0..n) -> offs, total in offs[n]
__global__ void scan_kernel(const int* counts, int n, int* offs)
{
    __shared__ int part[1024];
    const int t = threadIdx.x, T = blockDim.x;
    const int chunk = (n + T - 1) / T;
    const int b = t * chunk, e = min(n, b + chunk);
    int s = 0;
    for (int i = b; i < e; ++i) s += counts[i];
    part[t] = s;
    __syncthreads();
    // Hillis-Steele on the partials
    for (int o = 1; o < T; o <<= 1) {
        const int v = t >= o ? part[t - o] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int run = part[t] - s;
    for (int i = b; i < e; ++i) {
        offs[i] = run;
        run += counts[i];
    }
    if (t == T - 1) offs[n] = part[T - 1];
}

// one warp per source walker; copy c (1-based) advanced by c ran2 steps
__global__ void branch_scatter_kernel(DevStack in, DevStack out, int n, int n3, int cap, const int* counts,
                                      const int* offs, const unsigned long long* irn1)
{
    const int m = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (m >= n) return;
    const int j = n - 1 - m;
    const int cnt = counts[m];
    const int o0 = offs[m];
    unsigned long long s = irn1[m];
    const double wsign = copysign(1.0, in.weight[j]);
    for (int cp = 0; cp < cnt; ++cp) {
        s = (34522712143931ull * s + 55789347517ull) & kMask48;   // ran2 (ran.f90:29-48)
        const int d = o0 + cp;
        if (d >= cap) return;
        for (int e = lane; e < n3; e += 32) {
            out.x[(size_t)d * n3 + e] = in.x[(size_t)j * n3 + e];
            out.dpsi[(size_t)d * n3 + e] = in.dpsi[(size_t)j * n3 + e];
            out.dpsig[(size_t)d * n3 + e] = in.dpsig[(size_t)j * n3 + e];
        }
        if (lane == 0) {
            out.psil[d] = in.psil[j];
            out.psigl[d] = in.psigl[j];
            out.d2psi[d] = in.d2psi[j];
            out.d2psig[d] = in.d2psig[j];
            out.v[d] = in.v[j];
            out.vext[d] = in.vext[j];
            out.weight[d] = wsign;
            out.psil0[d] = in.psil0[j];
            out.psigl0[d] = in.psigl0[j];
            out.wt0[d] = in.wt0[j];
            out.is[d] = in.is[j];
            out.irn[d] = s;
        }
    }
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------

int walker_smem_bytes(const DevParams& p, int limit_bytes, SmemLayout* Lout)
{
    SmemLayout L = make_layout(p, limit_bytes);
    if (Lout) *Lout = L;
    return L.total * 8;
}

cudaError_t launch_walker(const DevParams& p, const KernelArgs& a, const SmemLayout& L, int grid, cudaStream_t st)
{
    const size_t smem = (size_t)L.total * 8;
    cudaError_t e = cudaFuncSetAttribute(walker_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    walker_kernel<<<grid, kThreads, smem, st>>>(p, a, L);
    return cudaGetLastError();
}

cudaError_t launch_estimators(const double* est, int n, int nest, double* vb, double* vb2, double* wb, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    estimator_kernel<<<nest, 256, 0, st>>>(est, n, nest, vb, vb2, wb);
    return cudaGetLastError();
}

cudaError_t launch_branch(const DevStack& in, const DevStack& out, int n, int n3, int cap, double factor, int* counts,
                          int* offs, unsigned long long* irn1, unsigned long long* wtisto, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    branch_count_kernel<<<(n + 255) / 256, 256, 0, st>>>(in, n, factor, counts, irn1, wtisto);
    scan_kernel<<<1, 1024, 0, st>>>(counts, n, offs);
    const int warps = n;
    branch_scatter_kernel<<<(warps * 32 + 255) / 256, 256, 0, st>>>(in, out, n, n3, cap, counts, offs, irn1);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Batched rmatinv (matrixlapack.f90:13-41): one CTA per column-major matrix.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads, 1)
matinv_kernel(const double* a, double* inv, double* detl, int* is, int n, DevParams p, SmemLayout L)
{
    extern __shared__ __align__(16) double sm[];
    const int b = blockIdx.x;
    const size_t n2 = (size_t)n * n;
    for (int t = threadIdx.x; t < n * n; t += kThreads) {
        const int r = t % n, cc = t / n;
        sm[L.S + r * p.ldS + cc] = a[b * n2 + t];
    }
    __syncthreads();
    KernelArgs dummy;
    Ctx ctx{p, dummy, L, sm, nullptr};
    double logdet;
    int sg;
    const bool ok = inverse_stage(ctx, logdet, sg);
    for (int t = threadIdx.x; t < n * n; t += kThreads) {
        const int r = t % n, cc = t / n;
        inv[b * n2 + t] = sm[L.S + r * p.ldS + cc];
    }
    if (threadIdx.x == 0) {
        detl[b] = ok ? logdet : DMC_MINUSHUGE;
        is[b] = ok ? sg : 1;
    }
}

cudaError_t launch_matinv(const double* a, double* inv, double* detl, int* is, int n, int nb, cudaStream_t st)
{
    DevParams p;
    memset(&p, 0, sizeof p);
    p.nd = n;
    p.ldS = n | 1;
    SmemLayout L;
    memset(&L, 0, sizeof L);
    L.S = 0;
    L.colk = round_up(n * p.ldS, 2);
    L.red = L.colk + round_up(n + 2, 2);
    L.total = L.red + kThreads * 8;
    const size_t smem = (size_t)L.total * 8;
    cudaError_t e = cudaFuncSetAttribute(matinv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    matinv_kernel<<<nb, kThreads, smem, st>>>(a, inv, detl, is, n, p, L);
    return cudaGetLastError();
}

// out[k] = in[n-1-k]: one pass of pop/push over a whole stack
__global__ void reverse_kernel(DevStack in, DevStack out, int n, int n3)
{
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (k >= n) return;
    const int j = n - 1 - k;
    for (int e = lane; e < n3; e += 32) {
        out.x[(size_t)k * n3 + e] = in.x[(size_t)j * n3 + e];
        out.dpsi[(size_t)k * n3 + e] = in.dpsi[(size_t)j * n3 + e];
        out.dpsig[(size_t)k * n3 + e] = in.dpsig[(size_t)j * n3 + e];
    }
    if (lane == 0) {
        out.psil[k] = in.psil[j];
        out.psigl[k] = in.psigl[j];
        out.d2psi[k] = in.d2psi[j];
        out.d2psig[k] = in.d2psig[j];
        out.v[k] = in.v[j];
        out.vext[k] = in.vext[j];
        out.weight[k] = in.weight[j];
        out.psil0[k] = in.psil0[j];
        out.psigl0[k] = in.psigl0[j];
        out.wt0[k] = in.wt0[j];
        out.is[k] = in.is[j];
        out.irn[k] = in.irn[j];
    }
}

cudaError_t launch_reverse(const DevStack& in, const DevStack& out, int n, int n3, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    reverse_kernel<<<(n * 32 + 255) / 256, 256, 0, st>>>(in, out, n, n3);
    return cudaGetLastError();
}

}  // namespace dmc
