// Single-particle moves and parameter derivatives of the DMCBS walker path
// (sm_103a):
//  - bcsone   (psislaterbcs.f90:296-376): determinant ratio for one particle
//    moved, from the stored inverse of the pair matrix;
//  - getphione (coshpot.f90:207-264): Jastrow ratio exp(U' - U) for the same
//    move; move1 (wavefunction.f90:393-404) is their product;
//  - getderbcs (psislaterbcs.f90:449-524, optsw on, optbeta off):
//    d log|det| / d vorb(shell) = tr(S^-1 dS/dvorb);
//  - the sums that calder (optimizer.f90:90-116) accumulates over a walker
//    population for the stochastic-reconfiguration step;
//  - the adjoint parameter gradients d log Psi / d theta and d E_L / d theta
//    for theta = (vorb(1..norb), bfact, b, d) of the pair function
//    (psislaterbcs.f90:249-293, betafun.f90:12-125) and the 16 knots of the
//    opt-in Jastrow spline.
// One warp per walker for the ratios (a few hundred flops each); one CTA per
// walker for the derivatives, which contract the whole inverse.
#include <cuda_runtime.h>
#include <math.h>

#include "dmc_device.cuh"
#include "dmc_kernels.h"
#include "dmc_walker.cuh"
#include "dmc_single.cuh"
#include "dmc_spline.h"

namespace dmc {


namespace {

__global__ void bcsone_kernel(const __grid_constant__ DevParams p, const KVecDev* __restrict__ kv,
                              const TabUD* __restrict__ tud, const double* __restrict__ x,
                              const double* __restrict__ smati, const int* __restrict__ ipart,
                              const double* __restrict__ dr, double* __restrict__ ratio, int nw)
{
    const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= nw) return;
    const int P = p.npart, nd = p.nd;
    const double* xw = x + (size_t)w * 3 * P;
    const int i = ipart[w] - 1;   // checked on the host
    const double xi[3] = {xw[3 * i] - dr[3 * w], xw[3 * i + 1] - dr[3 * w + 1], xw[3 * i + 2] - dr[3 * w + 2]};
    const double r = single::warp_bcsone(p, kv, tud, xw, smati + (size_t)w * nd * nd, i, xi);
    if (lane == 0) ratio[w] = r;
}

__global__ void getphione_kernel(const __grid_constant__ DevParams p, const TabUD* __restrict__ tud,
                                 const TabSS* __restrict__ tss, const double* __restrict__ x,
                                 const int* __restrict__ ipart, const double* __restrict__ drr,
                                 double* __restrict__ ratio, int nw)
{
    const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= nw) return;
    const double* xw = x + (size_t)w * 3 * p.npart;
    const double d[3] = {drr[3 * w], drr[3 * w + 1], drr[3 * w + 2]};
    const double r = single::warp_getphione(p, tud, tss, xw, ipart[w] - 1, d);
    if (lane == 0) ratio[w] = r;
}

// d log|det| / d vorb(shell) for one walker per CTA.  smati is the inverse in
// the reference's column-major layout: smati[j + i*nd] = inv(S)[j][i].
//  shell 1: sum over the up-down block of inv(S)[j][i];
//  shell s >= 2: sum_{k in s} 2 sum_i [cos(k.r_i) sum_j inv(S)[j][i] cos(k.r_j)
//                                     + sin(k.r_i) sum_j inv(S)[j][i] sin(k.r_j)]
// (cos(k.(r_i - r_j)) split into the two products).  k vectors are taken in
// chunks of kChunk with the down particles' cos/sin tabulated on chip; the
// per-(k, i) terms are summed per shell in a fixed order.
constexpr int kChunk = 8;

__global__ void __launch_bounds__(kThreads) derbcs_kernel(const __grid_constant__ DevParams p,
                                                         const KVecDev* __restrict__ kv,
                                                         const double* __restrict__ x,
                                                         const double* __restrict__ smati,
                                                         double* __restrict__ dpsi, int nw, int stride, int off)
{
    extern __shared__ __align__(16) double sm[];
    const int nd = p.nd, nup = p.nup, ndn = p.ndn, P = p.npart, norb = p.norb;
    double* Si = sm;                                  // nd*nd, column-major as smati
    double* xs = Si + nd * nd;                        // 3P
    double* cs = xs + 3 * P;                          // [kChunk][ndn][2]
    double* term = cs + kChunk * ndn * 2;             // [kChunk][nup]
    double* dsh = term + kChunk * nup;                // norb
    double* red = dsh + norb;                         // kThreads
    for (int w = blockIdx.x; w < nw; w += gridDim.x) {
        for (int t = threadIdx.x; t < nd * nd; t += kThreads) Si[t] = smati[(size_t)w * nd * nd + t];
        for (int t = threadIdx.x; t < 3 * P; t += kThreads) xs[t] = x[(size_t)w * 3 * P + t];
        for (int t = threadIdx.x; t < norb; t += kThreads) dsh[t] = 0.0;
        __syncthreads();
        // shell 1: block sum of the inverse over up rows i < nup, down cols j < ndn
        {
            double s = 0.0;
            for (int t = threadIdx.x; t < nup * ndn; t += kThreads) {
                const int i = t / ndn, j = t % ndn;
                s += Si[j + i * nd];
            }
            red[threadIdx.x] = s;
            __syncthreads();
            if (threadIdx.x == 0) {
                double tot = 0.0;
                for (int t = 0; t < kThreads; ++t) tot += red[t];
                dsh[0] = tot;
            }
            __syncthreads();
        }
        for (int q0 = 1; q0 < p.nk; q0 += kChunk) {
            const int nq = min(kChunk, p.nk - q0);
            for (int t = threadIdx.x; t < nq * ndn; t += kThreads) {
                const int ql = t / ndn, j = t % ndn;
                const KVecDev& K = kv[q0 + ql];
                const double* xj = xs + 3 * (nup + j);
                double s, c;
                sincos(K.k[0] * xj[0] + K.k[1] * xj[1] + K.k[2] * xj[2], &s, &c);
                cs[2 * (ql * ndn + j)] = c;
                cs[2 * (ql * ndn + j) + 1] = s;
            }
            __syncthreads();
            for (int t = threadIdx.x; t < nq * nup; t += kThreads) {
                const int ql = t / nup, i = t % nup;
                const KVecDev& K = kv[q0 + ql];
                const double* xi = xs + 3 * i;
                double si, ci;
                sincos(K.k[0] * xi[0] + K.k[1] * xi[1] + K.k[2] * xi[2], &si, &ci);
                double gc = 0.0, gs = 0.0;
                const double* col = Si + (size_t)i * nd;
                const double* cq = cs + 2 * ql * ndn;
                for (int j = 0; j < ndn; ++j) {
                    gc = fma(col[j], cq[2 * j], gc);
                    gs = fma(col[j], cq[2 * j + 1], gs);
                }
                term[ql * nup + i] = 2.0 * (ci * gc + si * gs);
            }
            __syncthreads();
            if (threadIdx.x == 0)
                for (int ql = 0; ql < nq; ++ql) {
                    double s = 0.0;
                    for (int i = 0; i < nup; ++i) s += term[ql * nup + i];
                    dsh[kv[q0 + ql].shell - 1] += s;
                }
            __syncthreads();
        }
        for (int t = threadIdx.x; t < norb; t += kThreads) dpsi[(size_t)w * stride + off + t] = dsh[t];
        __syncthreads();
    }
}

// beta(r) with its radial derivative and Laplacian (radialfun,
// betafun.f90:173-194); zero beyond the range
__device__ __forceinline__ void beta_all(const DevParams& p, const TabUD* tud, double r, double& f, double& df,
                                         double& d2f)
{
    f = df = d2f = 0.0;
    if (p.nobeta || r > p.rangeb) return;
    const walker::Lagrange<double> W = walker::lagrange(r, p.scaleb, p.ntab);
    const TabUD* T = tud + (W.idx - 1);
    f = W.c1 * T[0].b + W.c2 * T[1].b + W.c3 * T[2].b + W.c4 * T[3].b;
    df = W.c1 * T[0].db + W.c2 * T[1].db + W.c3 * T[2].db + W.c4 * T[3].db;
    d2f = W.c1 * T[0].d2b + W.c2 * T[1].d2b + W.c3 * T[2].d2b + W.c4 * T[3].d2b;
}

// N sums over the CTA in a fixed order (warp trees, then the warps in
// order); red holds at least kWarps * N doubles; sum k goes to outa[k] for
// k < N/2 and to outb[k - N/2] otherwise
template <int N>
__device__ void block_sum_n(double (&v)[N], double* red, double* outa, double* outb)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        double a = v[k];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0) red[warp * N + k] = a;
    }
    __syncthreads();
    if (threadIdx.x < N) {
        double t = 0.0;
        for (int q = 0; q < kWarps; ++q) t += red[q * N + threadIdx.x];
        if (threadIdx.x < N / 2)
            outa[threadIdx.x] = t;
        else
            outb[threadIdx.x - N / 2] = t;
    }
    __syncthreads();
}

__device__ double block_sum1(double v, double* red)
{
    red[threadIdx.x] = v;
    __syncthreads();
    for (int h = kThreads / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    const double t = red[0];
    __syncthreads();
    return t;
}

// Adjoint parameter gradients, one walker per CTA (FP64).
//
// The determinant's share of the kinetic term of E_L = -hbar d2psi + v is
//   Q = sum_p (1/m_p) [ lap_p Phi / Phi + 2 grad_p log Phi . grad_p J ]
//     = tr(S^-1 M),   M_ij = sum over the particles p that entry (i,j) of the
//                     pair matrix depends on of (1/m_p) lap_p S_ij
//                     + 2 grad_p S_ij . w_p,   w_p = grad_p J / m_p,
// because S is linear in each particle's row or column (psislaterbcs.f90:
// 209-223).  J (Jastrow, one-body and long-range terms) and v do not depend
// on theta, so with S' = dS/dtheta and M' = dM/dtheta
//   d log Psi / d theta = tr(S^-1 S')
//   d Q / d theta       = tr(S^-1 M') - tr(T S'),   T = S^-1 M S^-1
// and d E_L / d theta = -hbar dQ/dtheta: one extra pair of nd^3 products per
// walker gives every parameter.  Only the up-down block depends on the pair
// function's parameters: phi = vorb(1) + sum_k 2 vorb(shell k) cos(k.r) +
// beta(r), beta linear in bfact and given with its b and d derivatives as
// tables on the beta grid (the derivatives of the image-summed, shifted,
// bfact-scaled table that Psi uses).
//
// Per up-down pair (i, j) and shell s >= 2 (all k of a shell have the same
// k^2 and amplitude v_s = 2 vorb(s)), with C_s = sum_{k in s} cos(k.r_ij) and
// H_s = sum_{k in s} k sin(k.r_ij):
//   S_ij  = ... + v_s C_s                      S'_s,ij = 2 C_s
//   M_ij  = ... - v_s (k_s^2 C_s (1/m_i + 1/m_j) + 2 H_s . (w_i - w_j))
//   M'_s,ij = -2 k_s^2 C_s (1/m_i + 1/m_j) - 4 H_s . (w_i - w_j)
// The pass that forms M keeps (S'_s, M'_s) of every pair and shell, so the
// shell parameters' sums after T cost three multiply-adds per pair and shell
// instead of a second pass over the k vectors.
//
// The 16 knots t_k of the opt-in up-down Jastrow spline are Jastrow
// parameters: J = ... + sum_pairs sum_k t_k phi_k(r), so
//   d log Psi / d t_k = sum_pairs phi_k(r)
//   d E_L / d t_k     = -hbar sum_pairs [ (1/m_i + 1/m_j)(phi_k'' + 2 phi_k'/r)
//                        + 2 phi_k'/r d.(g_i - g_j) ],  g_p = grad_p log Psi / m_p,
// with phi_k, phi_k', phi_k'' interpolated from their values on the Jastrow
// table's grid (ktd[k][g]: the values the table itself was built from) with
// the pair's Lagrange weights, exactly as the pair loop interpolates the
// Jastrow table they are added to.
// Inputs per walker: x, the inverse (column-major as smati), the total and
// determinant drifts (grad / sqrt m) whose difference is grad J.  Outputs
// dlog[w*np + t], deloc[w*np + t] for t = vorb(1..norb), then bfact, b, d
// (nbeta = 3 with the beta function on), then the knots (nknot = 16 with the
// spline on).
// Memory: the CTA's core (inverse, M, product buffer, per-particle vectors,
// reductions) in shared memory (in core_g when it does not fit); the axis
// powers e^{i 2 pi m x_a / L}, the plane waves of every k at every particle
// and the per-pair shell derivatives in the CTA's slice of slice_g (L2).
__global__ void __launch_bounds__(kThreads) pgrad_kernel(const __grid_constant__ DevParams p,
                                                         const KVecDev* __restrict__ kv,
                                                         const TabUD* __restrict__ tud, const double* __restrict__ x,
                                                         const double* __restrict__ sinv,
                                                         const double* __restrict__ dpsi,
                                                         const double* __restrict__ dphi, double* __restrict__ dlog,
                                                         double* __restrict__ deloc, int nw, int np, double bfact,
                                                         const PgTab* __restrict__ btd, const PgTab* __restrict__ ktd,
                                                         int nbeta, int nknot, double* core_g, size_t core_per,
                                                         double* slice_g, size_t slice_per)
{
    extern __shared__ __align__(16) double smp[];
    double* base = core_g ? core_g + (size_t)blockIdx.x * core_per : smp;
    const int nd = p.nd, nup = p.nup, ndn = p.ndn, P = p.npart, nq = p.nk - 1, norb = p.norb;
    const size_t nd2 = (size_t)nd * nd;
    double* Si = base;                 // (S^-1)_{rc} = Si[r + c nd]
    double* M = Si + nd2;              // M, later T
    double* B = M + nd2;               // M S^-1
    double* xs = B + nd2;              // [P][3]
    double* w = xs + 3 * P;            // [P][3]: grad J / m
    double* gt = w + 3 * P;            // [P][3]: grad log Psi / m
    double* red = gt + 3 * P;
    double* res = red + kThreads;      // [2][kPgradMax]: d log Psi, then d Q
    int* sh0 = reinterpret_cast<int*>(res + 2 * kPgradMax);   // first k of each shell s >= 2, then the end
    const int np1 = p.nmax + 1, nsh = norb - 1, npairs = nup * ndn;
    double2* E = reinterpret_cast<double2*>(slice_g + (size_t)blockIdx.x * slice_per);   // [P][3][np1]
    double2* cs = E + (size_t)3 * P * np1;                                             // [nq][P]
    double2* dsm = cs + (size_t)P * (nq > 0 ? nq : 1);                                 // [nsh][npairs]
    const int npb = norb + nbeta;      // parameters of the pair function
    const double imu = p.imass[0], imd = p.imass[1], ims = imu + imd;
    if (threadIdx.x == 0) {
        // k vectors are sorted by shell; shell 1 is k = 0
        int q = 1;
        for (int sh = 2; sh <= norb; ++sh) {
            sh0[sh - 2] = q;
            while (q < p.nk && kv[q].shell == sh) ++q;
        }
        sh0[norb - 1] = q;
    }
    for (int wk = blockIdx.x; wk < nw; wk += gridDim.x) {
        for (size_t t = threadIdx.x; t < nd2; t += kThreads) Si[t] = sinv[(size_t)wk * nd2 + t];
        for (int t = threadIdx.x; t < 3 * P; t += kThreads) {
            const size_t g = (size_t)wk * 3 * P + t;
            const double xv = x[g];
            xs[t] = xv;
            const int sp = (t / 3) < nup ? 0 : 1;
            w[t] = (dpsi[g] - dphi[g]) * p.isqm[sp];
            gt[t] = dpsi[g] * p.isqm[sp];
            // powers of e^{i 2 pi x_a / L}, m = 0..nmax
            double s1, c1;
            sincospi(2.0 * xv * p.eli, &s1, &c1);
            double2* e = E + (size_t)t * np1;
            e[0] = make_double2(1.0, 0.0);
            double cr = c1, ci = s1;
            if (np1 > 1) e[1] = make_double2(c1, s1);
            for (int m = 2; m < np1; ++m) {
                const double nr = cr * c1 - ci * s1, ni = cr * s1 + ci * c1;
                cr = nr;
                ci = ni;
                e[m] = make_double2(cr, ci);
            }
        }
        __syncthreads();
        // e^{i k_q . x_p} as the product of the three axis powers
        for (int t = threadIdx.x; t < nq * P; t += kThreads) {
            const int q = t / P + 1, pp = t - (q - 1) * P;
            const KVecDev& K = kv[q];
            const double2* eb = E + (size_t)pp * 3 * np1;
            const int n0 = K.n[0];
            const double2 e0 = eb[n0 < 0 ? -n0 : n0];
            double zr = e0.x, zi = n0 < 0 ? -e0.y : e0.y;
#pragma unroll
            for (int a = 1; a < 3; ++a) {
                const int n = K.n[a];
                const double2 e = eb[a * np1 + (n < 0 ? -n : n)];
                const double er = e.x, ei = n < 0 ? -e.y : e.y;
                const double nr = zr * er - zi * ei, ni = zr * ei + zi * er;
                zr = nr;
                zi = ni;
            }
            cs[t] = make_double2(zr, zi);
        }
        __syncthreads();
        // M (psislaterbcs.f90:171-206, 249-293 for the entries and their
        // derivatives), with every pair's shell derivatives on the side
        for (size_t t = threadIdx.x; t < nd2; t += kThreads) {
            const int i = (int)(t % nd), j = (int)(t / nd);
            double m = 0.0;
            if (i < nup && j < ndn) {
                const int pj = nup + j;
                const double wd0 = w[3 * i] - w[3 * pj], wd1 = w[3 * i + 1] - w[3 * pj + 1];
                const double wd2 = w[3 * i + 2] - w[3 * pj + 2];
                double l = 0.0, g0 = 0.0, g1 = 0.0, g2 = 0.0;
                double2* dp = dsm + (size_t)i * ndn + j;
                for (int s = 0; s < nsh; ++s) {
                    const int q0 = sh0[s], q1 = sh0[s + 1];
                    double cc = 0.0, h0 = 0.0, h1 = 0.0, h2 = 0.0;
                    for (int q = q0; q < q1; ++q) {
                        const KVecDev& K = kv[q];
                        const double2 ci = cs[(size_t)(q - 1) * P + i];
                        const double2 cj = cs[(size_t)(q - 1) * P + pj];
                        const double co = fma(ci.x, cj.x, ci.y * cj.y);
                        const double si = fma(ci.y, cj.x, -ci.x * cj.y);
                        cc += co;
                        h0 = fma(si, K.k[0], h0);
                        h1 = fma(si, K.k[1], h1);
                        h2 = fma(si, K.k[2], h2);
                    }
                    double ds = 0.0, dm = 0.0;
                    if (q1 > q0) {
                        const double v = kv[q0].v, k2c = kv[q0].k2 * cc;
                        const double hw = h0 * wd0 + h1 * wd1 + h2 * wd2;
                        l -= v * k2c;
                        g0 -= v * h0;
                        g1 -= v * h1;
                        g2 -= v * h2;
                        ds = 2.0 * cc;
                        dm = -2.0 * k2c * ims - 4.0 * hw;
                    }
                    dp[(size_t)s * npairs] = make_double2(ds, dm);
                }
                if (!p.nobeta) {
                    double d[3];
                    for (int cc = 0; cc < 3; ++cc) d[cc] = walker::min_image(xs[3 * i + cc] - xs[3 * pj + cc], p);
                    const double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                    double f, df, d2f;
                    beta_all(p, tud, r, f, df, d2f);
                    if (r > 0.0) {
                        const double dr = df / r;
                        g0 += dr * d[0];
                        g1 += dr * d[1];
                        g2 += dr * d[2];
                    }
                    l += d2f;
                }
                m = l * ims + 2.0 * (g0 * wd0 + g1 * wd1 + g2 * wd2);
            } else if (i < nup) {
                // unpaired up plane wave in column j (depends on up particle i)
                const int u = j - ndn;
                const double* k = p.akup[u];
                double sn, c;
                sincos(k[0] * xs[3 * i] + k[1] * xs[3 * i + 1] + k[2] * xs[3 * i + 2], &sn, &c);
                const double a = p.sinup[u] ? c : -sn;        // d/d(k.x) of the entry
                const double e = p.sinup[u] ? sn : c;
                m = -p.ak2up[u] * e * imu + 2.0 * a * (k[0] * w[3 * i] + k[1] * w[3 * i + 1] + k[2] * w[3 * i + 2]);
            } else if (j < ndn) {
                // unpaired down plane wave in row i (depends on down particle j)
                const int u = i - nup, pj = nup + j;
                const double* k = p.akdn[u];
                double sn, c;
                sincos(k[0] * xs[3 * pj] + k[1] * xs[3 * pj + 1] + k[2] * xs[3 * pj + 2], &sn, &c);
                const double a = p.sindn[u] ? c : -sn;
                const double e = p.sindn[u] ? sn : c;
                m = -p.ak2dn[u] * e * imd + 2.0 * a * (k[0] * w[3 * pj] + k[1] * w[3 * pj + 1] + k[2] * w[3 * pj + 2]);
            }
            M[t] = m;
        }
        __syncthreads();
        // B = M S^-1, then T = S^-1 B (into M)
        for (size_t t = threadIdx.x; t < nd2; t += kThreads) {
            const int i = (int)(t % nd), j = (int)(t / nd);
            double s = 0.0;
            for (int k = 0; k < nd; ++k) s = fma(M[i + (size_t)k * nd], Si[k + (size_t)j * nd], s);
            B[t] = s;
        }
        __syncthreads();
        for (size_t t = threadIdx.x; t < nd2; t += kThreads) {
            const int i = (int)(t % nd), j = (int)(t / nd);
            double s = 0.0;
            for (int k = 0; k < nd; ++k) s = fma(Si[i + (size_t)k * nd], B[k + (size_t)j * nd], s);
            M[t] = s;
        }
        __syncthreads();
        // per pair-function shell parameter (eight at a time): sums over the
        // up-down pairs of S^-1_ji S'_ij and S^-1_ji M'_ij - T_ji S'_ij
        for (int th0 = 0; th0 < norb; th0 += 8) {
            double acc[16];
#pragma unroll
            for (int k = 0; k < 16; ++k) acc[k] = 0.0;
            for (int t = threadIdx.x; t < npairs; t += kThreads) {
                const int i = t / ndn, j = t - i * ndn;
                const double a = Si[j + (size_t)i * nd], tt = M[j + (size_t)i * nd];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int th = th0 + u;
                    if (th < norb) {
                        if (th == 0) {   // vorb(1): S' = 1, M' = 0
                            acc[u] += a;
                            acc[8 + u] -= tt;
                        } else {
                            const double2 v = dsm[(size_t)(th - 1) * npairs + t];
                            acc[u] = fma(a, v.x, acc[u]);
                            acc[8 + u] += a * v.y - tt * v.x;
                        }
                    }
                }
            }
            block_sum_n<16>(acc, red, res + th0, res + kPgradMax + th0);
        }
        if (nbeta > 0) {
            // bfact (beta / bfact), b and d (their derivative tables) in one
            // pass: one distance and one set of Lagrange weights per pair
            double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
            const double ib = 1.0 / bfact;
            const PgTab* Tb = btd;
            const PgTab* Td = btd + (size_t)(p.ntab + 1);
            for (int t = threadIdx.x; t < npairs; t += kThreads) {
                const int i = t / ndn, j = t % ndn, pj = nup + j;
                double d[3];
                for (int cc = 0; cc < 3; ++cc) d[cc] = walker::min_image(xs[3 * i + cc] - xs[3 * pj + cc], p);
                const double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                if (p.nobeta || r > p.rangeb) continue;
                const double a = Si[j + (size_t)i * nd], tt = M[j + (size_t)i * nd];
                const walker::Lagrange<double> W = walker::lagrange(r, p.scaleb, p.ntab);
                const double ri = r > 0.0 ? 1.0 / r : 0.0;
                const double gw = d[0] * (w[3 * i] - w[3 * pj]) + d[1] * (w[3 * i + 1] - w[3 * pj + 1]) +
                                  d[2] * (w[3 * i + 2] - w[3 * pj + 2]);
                const int o = W.idx - 1;
                double f[3], df[3], d2f[3];
                {
                    const TabUD* T = tud + o;
                    f[0] = (W.c1 * T[0].b + W.c2 * T[1].b + W.c3 * T[2].b + W.c4 * T[3].b) * ib;
                    df[0] = (W.c1 * T[0].db + W.c2 * T[1].db + W.c3 * T[2].db + W.c4 * T[3].db) * ib;
                    d2f[0] = (W.c1 * T[0].d2b + W.c2 * T[1].d2b + W.c3 * T[2].d2b + W.c4 * T[3].d2b) * ib;
                }
                for (int q = 1; q < 3; ++q) {
                    const PgTab* T = (q == 1 ? Tb : Td) + o;
                    f[q] = W.c1 * T[0].f + W.c2 * T[1].f + W.c3 * T[2].f + W.c4 * T[3].f;
                    df[q] = W.c1 * T[0].df + W.c2 * T[1].df + W.c3 * T[2].df + W.c4 * T[3].df;
                    d2f[q] = W.c1 * T[0].d2f + W.c2 * T[1].d2f + W.c3 * T[2].d2f + W.c4 * T[3].d2f;
                }
                for (int q = 0; q < 3; ++q) {
                    const double dm = d2f[q] * ims + 2.0 * df[q] * ri * gw;
                    acc[q] += a * f[q];
                    acc[3 + q] += a * dm - tt * f[q];
                }
            }
            block_sum_n<6>(acc, red, res + norb, res + kPgradMax + norb);
        }
        if (nknot > 0) {
            // the Jastrow knots, all in one pass over the up-down pairs
            double acc[2 * kJastrowKnots];
#pragma unroll
            for (int k = 0; k < 2 * kJastrowKnots; ++k) acc[k] = 0.0;
            // grid rows in units of the knot spacing (t = r / h): the knots
            // whose support [k - 2, k + 2] (and the mirror image of k = 1
            // below one spacing) reaches the pair's four grid rows
            const double tstep = kJastrowCells / (p.el * p.scale);
            const size_t kstride = (size_t)p.ntab + 1;
            for (int t = threadIdx.x; t < npairs; t += kThreads) {
                const int i = t / ndn, j = t % ndn, pj = nup + j;
                double d[3];
                for (int cc = 0; cc < 3; ++cc) d[cc] = walker::min_image(xs[3 * i + cc] - xs[3 * pj + cc], p);
                const double r = fmax(sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]), 1.0e-14);
                if (!(r < p.range)) continue;
                const walker::Lagrange<double> W = walker::lagrange(r, p.scale, p.ntab);
                const double ri = 1.0 / r;
                const double gd = d[0] * (gt[3 * i] - gt[3 * pj]) + d[1] * (gt[3 * i + 1] - gt[3 * pj + 1]) +
                                  d[2] * (gt[3 * i + 2] - gt[3 * pj + 2]);
                const double cp = 2.0 * ri * (ims + gd);   // weight of phi' (phi'' has ims)
                const int o = W.idx - 1;
                const double t0 = o * tstep;
                const int klo = max(0, (int)t0 - 2);
                const int khi = min(kJastrowKnots - 1, (int)(t0 + 3.0 * tstep) + 2);
#pragma unroll 1
                for (int k = klo; k <= khi; ++k) {
                    const PgTab* T = ktd + k * kstride + o;
                    const double f = W.c1 * T[0].f + W.c2 * T[1].f + W.c3 * T[2].f + W.c4 * T[3].f;
                    const double fp = W.c1 * T[0].df + W.c2 * T[1].df + W.c3 * T[2].df + W.c4 * T[3].df;
                    const double fpp = W.c1 * T[0].d2f + W.c2 * T[1].d2f + W.c3 * T[2].d2f + W.c4 * T[3].d2f;
                    acc[k] += f;
                    acc[kJastrowKnots + k] += ims * fpp + cp * fp;
                }
            }
            block_sum_n<2 * kJastrowKnots>(acc, red, res + npb, res + kPgradMax + npb);
        }
        __syncthreads();
        for (int th = threadIdx.x; th < np; th += kThreads) {
            dlog[(size_t)wk * np + th] = res[th];
            deloc[(size_t)wk * np + th] = -p.hbar * res[kPgradMax + th];
        }
        __syncthreads();
    }
}

// getjasder (jastrowlongrange.f90:63-78) for one walker per CTA: the
// long-range Jastrow at beta + dp, (beta + dp) - 2 dp and back, from the
// densities rho_q; d/d beta by central differences as the reference takes
// them, d/d gamma = U / gamma.  Writes dpsi[w*stride + 0..1].
__global__ void __launch_bounds__(kThreads) jasder_kernel(const __grid_constant__ DevParams p,
                                                         const double* __restrict__ jq,
                                                         const double* __restrict__ x,
                                                         double* __restrict__ dpsi, int nw, int stride)
{
    extern __shared__ __align__(16) double sm[];
    const int P = p.npart;
    double* r2 = sm;   // |rho_q|^2 - N per q
    for (int w = blockIdx.x; w < nw; w += gridDim.x) {
        const double* xw = x + (size_t)w * 3 * P;
        for (int q = threadIdx.x; q < p.nql; q += kThreads) {
            const double* Q = jq + 8 * q;
            double re = 0.0, im = 0.0;
            for (int i = 0; i < P; ++i) {
                double sn, cs;
                sincos(Q[0] * xw[3 * i] + Q[1] * xw[3 * i + 1] + Q[2] * xw[3 * i + 2], &sn, &cs);
                re += cs;
                im += sn;
            }
            r2[q] = re * re + im * im - (double)P;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const double dp = 0.0001;
            const double b1 = p.jbeta + dp, b2 = b1 - 2.0 * dp, b3 = b2 + dp;
            double u1 = 0.0, u2 = 0.0, u3 = 0.0;
            for (int q = 0; q < p.nql; ++q) {
                const double qmod = sqrt(jq[8 * q + 3]);
                u1 += p.jgamma * exp(-b1 * qmod) / qmod * r2[q];
                u2 += p.jgamma * exp(-b2 * qmod) / qmod * r2[q];
                u3 += p.jgamma * exp(-b3 * qmod) / qmod * r2[q];
            }
            dpsi[(size_t)w * stride] = (u1 - u2) / (2.0 * dp);
            dpsi[(size_t)w * stride + 1] = u3 / p.jgamma;
        }
        __syncthreads();
    }
}

// calder sums (optimizer.f90:105-115) over a population, in pop order (the
// top of the stack, index n-1, first): ovec += d, ovecw += d*e, pmat += d d^T,
// esum += e, esum2 += e^2 with e = E_L / eunit / npart.  One thread per
// output, so every sum runs over the walkers in the same order as the
// reference's loop; products are rounded before the add (no contraction).
// ene = (-hbar*d2psi + v)/eunit/npart (dmcbcs.f90:497), once per walker
__global__ void sr_energy_kernel(const double* __restrict__ d2psi, const double* __restrict__ v, int n,
                                 double hbar, double eunit, double npart, double* __restrict__ ene)
{
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < n; w += gridDim.x * blockDim.x)
        ene[w] = __ddiv_rn(__ddiv_rn(__dadd_rn(__dmul_rn(-hbar, d2psi[w]), v[w]), eunit), npart);
}

__global__ void sr_sums_kernel(const double* __restrict__ der, const double* __restrict__ ene, int n, int np,
                               double* __restrict__ sums)
{
    const int nout = np * np + 2 * np + 2;
    for (int t = threadIdx.x; t < nout; t += blockDim.x) {
        double s = sums[t];
        for (int w = n - 1; w >= 0; --w) {
            const double e = ene[w];
            const double* d = der + (size_t)w * np;
            double term;
            if (t < np)
                term = d[t];
            else if (t < 2 * np)
                term = __dmul_rn(d[t - np], e);
            else if (t < 2 * np + np * np) {
                const int q = t - 2 * np, i = q % np, j = q / np;   // column-major pmat(i,j)
                term = __dmul_rn(d[i], d[j]);
            } else if (t == nout - 2)
                term = e;
            else
                term = __dmul_rn(e, e);
            s = __dadd_rn(s, term);
        }
        sums[t] = s;
    }
}

}  // namespace

cudaError_t launch_bcsone(const DevParams& p, const KVecDev* kv, const TabUD* tud, const double* x,
                          const double* smati, const int* ipart, const double* dr, double* ratio, int nw,
                          cudaStream_t st)
{
    if (nw <= 0) return cudaSuccess;
    const int warps = 8;
    bcsone_kernel<<<(nw + warps - 1) / warps, 32 * warps, 0, st>>>(p, kv, tud, x, smati, ipart, dr, ratio, nw);
    return cudaGetLastError();
}

cudaError_t launch_getphione(const DevParams& p, const TabUD* tud, const TabSS* tss, const double* x,
                             const int* ipart, const double* drr, double* ratio, int nw, cudaStream_t st)
{
    if (nw <= 0) return cudaSuccess;
    const int warps = 8;
    getphione_kernel<<<(nw + warps - 1) / warps, 32 * warps, 0, st>>>(p, tud, tss, x, ipart, drr, ratio, nw);
    return cudaGetLastError();
}

size_t derbcs_smem_bytes(const DevParams& p)
{
    return sizeof(double) * ((size_t)p.nd * p.nd + 3 * p.npart + 2 * kChunk * p.ndn + (size_t)kChunk * p.nup +
                             p.norb + kThreads);
}

cudaError_t launch_derbcs(const DevParams& p, const KVecDev* kv, const double* x, const double* smati, double* dpsi,
                          int nw, int grid, cudaStream_t st, int stride, int off)
{
    if (nw <= 0) return cudaSuccess;
    const size_t smem = derbcs_smem_bytes(p);
    cudaError_t e = cudaFuncSetAttribute(derbcs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    derbcs_kernel<<<grid < nw ? grid : nw, kThreads, smem, st>>>(p, kv, x, smati, dpsi, nw, stride < 0 ? p.norb : stride,
                                                                 off);
    return cudaGetLastError();
}

// Layout of one pgrad CTA's core, in doubles: inverse, M, product buffer
// (nd^2 each), positions, grad J / m and grad log Psi / m (3 npart each),
// reduction buffer, results, first k of each shell.
size_t pgrad_doubles(const DevParams& p)
{
    const size_t nd2 = (size_t)p.nd * p.nd;
    return 3 * nd2 + 9 * (size_t)p.npart + kThreads + 2 * (size_t)kPgradMax + (size_t)(p.norb + 2);
}

// The CTA's global slice, in doubles (even): axis powers (3 npart (nmax+1)
// complex), plane waves (npart (nk-1) complex), shell derivatives
// ((norb-1) nup ndn pairs of doubles).
size_t pgrad_slice_doubles(const DevParams& p)
{
    const size_t nq = p.nk > 1 ? (size_t)p.nk - 1 : 1, nsh = p.norb > 1 ? (size_t)p.norb - 1 : 1;
    return 2 * (3 * (size_t)p.npart * (p.nmax + 1) + (size_t)p.npart * nq + nsh * p.nup * p.ndn);
}

// CTAs of one pgrad launch: as many as are resident on the device's SMs
// together, at most one per walker.
int pgrad_grid(const DevParams& p, int nw, int nsm, int smem_limit)
{
    const size_t need = pgrad_doubles(p) * 8;
    const int smem = need <= (size_t)smem_limit ? (int)need : 0;
    int per_sm = 1;
    if (smem > 0 && cudaFuncSetAttribute(pgrad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pgrad_kernel, kThreads, smem) != cudaSuccess)
        return 0;
    const long long g = (long long)(per_sm > 0 ? per_sm : 1) * nsm;
    return (int)(g < nw ? g : (nw > 0 ? nw : 1));
}

cudaError_t launch_pgrad(const DevParams& p, const KVecDev* kv, const TabUD* tud, const double* x, const double* sinv,
                         const double* dpsi, const double* dphi, double* dlog, double* deloc, int nw, int np,
                         double bfact, const PgTab* btd, const PgTab* ktd, int nbeta, int nknot, int grid,
                         double* gscr, double* slices, int smem_limit, cudaStream_t st)
{
    if (np > kPgradMax || nknot > kJastrowKnots || np != p.norb + nbeta + nknot || (nbeta > 1 && !btd) ||
        (nknot > 0 && !ktd) || !slices || grid < 1)
        return cudaErrorInvalidValue;
    if (nw <= 0) return cudaSuccess;
    const size_t need = pgrad_doubles(p);
    const bool on_chip = need * 8 <= (size_t)smem_limit;
    const size_t smem = on_chip ? need * 8 : 0;
    if (on_chip) {
        cudaError_t e = cudaFuncSetAttribute(pgrad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    } else if (!gscr) {
        return cudaErrorInvalidValue;
    }
    pgrad_kernel<<<grid < nw ? grid : nw, kThreads, smem, st>>>(p, kv, tud, x, sinv, dpsi, dphi, dlog, deloc, nw, np,
                                                                bfact, btd, ktd, nbeta, nknot,
                                                                on_chip ? nullptr : gscr, need, slices,
                                                                pgrad_slice_doubles(p));
    return cudaGetLastError();
}

cudaError_t launch_jasder(const DevParams& p, const double* jq, const double* x, double* dpsi, int nw, int grid,
                          cudaStream_t st, int stride)
{
    if (nw <= 0) return cudaSuccess;
    const size_t smem = sizeof(double) * (size_t)(p.nql > 0 ? p.nql : 1);
    jasder_kernel<<<grid < nw ? grid : nw, kThreads, smem, st>>>(p, jq, x, dpsi, nw, stride);
    return cudaGetLastError();
}

cudaError_t launch_sr_sums(const double* der, const double* d2psi, const double* v, int n, int np, double hbar,
                           double eunit, int npart, double* sums, double* ene, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    sr_energy_kernel<<<(n + 255) / 256, 256, 0, st>>>(d2psi, v, n, hbar, eunit, (double)npart, ene);
    sr_sums_kernel<<<1, 1024, 0, st>>>(der, ene, n, np, sums);
    return cudaGetLastError();
}

}  // namespace dmc
