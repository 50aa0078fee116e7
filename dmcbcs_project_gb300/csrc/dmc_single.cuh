// Single-particle ratios as warp-level device functions, shared by the
// bcsone/getphione kernels and the n(k) estimator.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "dmc_device.cuh"
#include "dmc_walker.cuh"

namespace dmc {
namespace single {

// Fortran nint: nearest integer, halves away from zero
__device__ __forceinline__ double fnint(double a) { return round(a); }

// beta(r) (radialfun, betafun.f90:173-194), value only; zero beyond L/2
__device__ __forceinline__ double beta_value(const DevParams& p, const TabUD* tud, double r)
{
    if (p.nobeta || r > p.rangeb) return 0.0;
    const walker::Lagrange<double> W = walker::lagrange(r, p.scaleb, p.ntab);
    const TabUD* T = tud + (W.idx - 1);
    return W.c1 * T[0].b + W.c2 * T[1].b + W.c3 * T[2].b + W.c4 * T[3].b;
}

// Jastrow u(r) of one pair type (coshpot.f90:236-250): 0 beyond the range
__device__ __forceinline__ double jastrow_u(const DevParams& p, const TabUD* tud, const TabSS* tss, bool opposite,
                                            double r)
{
    if (!(r < p.range)) return 0.0;
    const walker::Lagrange<double> W = walker::lagrange(r, p.scale, p.ntab);
    if (opposite) {
        const TabUD* T = tud + (W.idx - 1);
        return W.c1 * T[0].u + W.c2 * T[1].u + W.c3 * T[2].u + W.c4 * T[3].u;
    }
    const TabSS* T = tss + (W.idx - 1);
    return W.c1 * T[0].u + W.c2 * T[1].u + W.c3 * T[2].u + W.c4 * T[3].u;
}

// bcsone (psislaterbcs.f90:296-376) for particle i (0-based) of the walker at
// xw moved to xi; S is the walker's inverse, column-major as smati.  Called
// by a whole warp; every lane returns the ratio.
__device__ __forceinline__ double warp_bcsone(const DevParams& p, const KVecDev* __restrict__ kv,
                                              const TabUD* __restrict__ tud, const double* xw, const double* S, int i,
                                              const double (&xi)[3])
{
    const int lane = threadIdx.x & 31, nd = p.nd;
    const bool isup = i < p.nup;
    const int nloop = isup ? p.npair + p.nexdn : p.npair + p.nexup;
    double acc = 0.0;
    for (int q = lane; q < nd; q += 32) {
        double ph;
        if (q < nloop) {
            // new pair-function entry phi(r_i' - r_jj) (psislaterbcs.f90:318-350)
            const int jj = isup ? q + p.npair + p.nexup : q;
            double d[3];
            for (int c = 0; c < 3; ++c) {
                d[c] = xi[c] - xw[3 * jj + c];
                d[c] = d[c] - p.el * fnint(d[c] / p.el);
            }
            ph = kv[0].v;
            for (int k = 1; k < p.nk; ++k) ph += kv[k].v * cos(kv[k].k[0] * d[0] + kv[k].k[1] * d[1] + kv[k].k[2] * d[2]);
            ph += beta_value(p, tud, sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]));
        } else {
            // unpaired plane wave of the moved particle (psislaterbcs.f90:352-365)
            const int j = q - nloop;
            const double* a = isup ? p.akup[j] : p.akdn[j];
            const int sn = isup ? p.sinup[j] : p.sindn[j];
            const double arg = a[0] * xi[0] + a[1] * xi[1] + a[2] * xi[2];
            ph = sn ? sin(arg) : cos(arg);
        }
        // up: row i of S replaced, ratio = sum_q Sinv(q,i) phi_q; down: column
        const double s = isup ? S[q + (size_t)i * nd] : S[(i - p.nup) + (size_t)q * nd];
        acc = fma(s, ph, acc);
    }
    return walker::warp_sum(acc);
}

// The same ratio with the plane waves from tables: cs[(k-1) npart + j] holds
// (cos, sin) of k.x_j for every particle j and k = 1..nk-1, csn[k-1] holds
// v_k (cos, sin) of k.r' at the moved particle's new position, so each
// pair-function entry is sum_k v_k (cos k.r' cos k.r_j + sin k.r' sin k.r_j)
// = sum_k v_k cos k.(r' - r_j) with two multiply-adds per k instead of a cosine.
__device__ __forceinline__ double warp_bcsone_tab(const DevParams& p, const KVecDev* __restrict__ kv,
                                                  const TabUD* __restrict__ tud, const double* xw, const double* S,
                                                  int i, const double (&xi)[3], const double2* cs,
                                                  const double2* csn)
{
    const int lane = threadIdx.x & 31, nd = p.nd, P = p.npart, nq = p.nk - 1;
    const bool isup = i < p.nup;
    const int nloop = isup ? p.npair + p.nexdn : p.npair + p.nexup;
    double acc = 0.0;
    for (int q = lane; q < nd; q += 32) {
        double ph;
        if (q < nloop) {
            const int jj = isup ? q + p.npair + p.nexup : q;
            double d[3];
            for (int c = 0; c < 3; ++c) {
                d[c] = xi[c] - xw[3 * jj + c];
                d[c] = d[c] - p.el * fnint(d[c] / p.el);
            }
            ph = kv[0].v;
            const double2* cj = cs + jj;
            for (int k = 0; k < nq; ++k) {
                const double2 a = csn[k], b = cj[(size_t)k * P];
                ph = fma(a.x, b.x, fma(a.y, b.y, ph));
            }
            ph += beta_value(p, tud, sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]));
        } else {
            const int j = q - nloop;
            const double* a = isup ? p.akup[j] : p.akdn[j];
            const int sn = isup ? p.sinup[j] : p.sindn[j];
            const double arg = a[0] * xi[0] + a[1] * xi[1] + a[2] * xi[2];
            ph = sn ? sin(arg) : cos(arg);
        }
        const double s = isup ? S[q + (size_t)i * nd] : S[(i - p.nup) + (size_t)q * nd];
        acc = fma(s, ph, acc);
    }
    return walker::warp_sum(acc);
}

// getphione (coshpot.f90:207-264): exp(U' - U) for particle i (0-based)
// displaced by -drr.  Called by a whole warp; every lane returns the ratio.
__device__ __forceinline__ double warp_getphione(const DevParams& p, const TabUD* __restrict__ tud,
                                                 const TabSS* __restrict__ tss, const double* xw, int i,
                                                 const double (&drr)[3])
{
    const int lane = threadIdx.x & 31, P = p.npart;
    const bool upi = i < p.nup;
    double u = 0.0;
    for (int j = lane; j < P; j += 32) {
        if (j == i) continue;
        const bool opposite = upi != (j < p.nup);
        if (!opposite && !p.ieq) continue;   // opposite-spin pairs are always on
        for (int pass = 0; pass < 2; ++pass) {
            double d[3];
            for (int c = 0; c < 3; ++c) {
                d[c] = xw[3 * i + c] - xw[3 * j + c];
                if (pass) d[c] -= drr[c];
                d[c] = d[c] - p.el * fnint(d[c] * p.eli);
            }
            const double r = fmax(sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]), 1.0e-14);
            const double uj = jastrow_u(p, tud, tss, opposite, r);
            u = pass ? u + uj : u - uj;
        }
    }
    return exp(walker::warp_sum(u));
}

// sum over the other particles j of u(|r - x_j|) for particle i (0-based) at
// position r, with the pair rules of getphione (coshpot.f90:218-250); a
// whole warp calls it and every lane returns the sum
__device__ __forceinline__ double warp_jastrow_sum(const DevParams& p, const TabUD* __restrict__ tud,
                                                   const TabSS* __restrict__ tss, const double* xw, int i,
                                                   const double (&r)[3])
{
    const int lane = threadIdx.x & 31, P = p.npart;
    const bool upi = i < p.nup;
    double u = 0.0;
    for (int j = lane; j < P; j += 32) {
        if (j == i) continue;
        const bool opposite = upi != (j < p.nup);
        if (!opposite && !p.ieq) continue;
        double d[3];
        for (int c = 0; c < 3; ++c) {
            d[c] = r[c] - xw[3 * j + c];
            d[c] = d[c] - p.el * fnint(d[c] * p.eli);
        }
        const double rr = fmax(sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]), 1.0e-14);
        u += jastrow_u(p, tud, tss, opposite, rr);
    }
    return walker::warp_sum(u);
}

}  // namespace single
}  // namespace dmc
