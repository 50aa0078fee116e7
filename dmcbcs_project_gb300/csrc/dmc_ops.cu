// Operators of the reference's block loop (operators.f90:90-124) on the GPU:
//  - g(r) of up-down, up-up and down-down pairs and the density profile
//    along x, y, z of each species (gofr.f90:53-92),
//  - S(q) of the up, down and up-down densities (sofq.f90:43-64),
//  - n(k) from single-particle moves (momentum3d.f90:89-124).
// Per walker, one CTA fills integer pair/density histograms and the S(q)
// values; for n(k), one CTA per walker runs the N x nsamp moves over its
// warps (ratios from the walker's inverse, random displacements from the
// walker's own stream by jump-ahead).  A single-CTA pass then adds every
// walker's contributions with its weight, one thread per output, walkers in
// pop order, so the sums are deterministic.
#include <cuda_runtime.h>
#include <math.h>

#include "dmc_device.cuh"
#include "dmc_kernels.h"
#include "dmc_single.cuh"
#include "dmc_walker.cuh"

namespace dmc {

namespace {

__global__ void __launch_bounds__(kThreads) ops_walker_kernel(const __grid_constant__ DevParams p,
                                                             const __grid_constant__ OpsDev o,
                                                             const double* __restrict__ x, int n,
                                                             int* __restrict__ hg, int* __restrict__ hd,
                                                             double* __restrict__ sv)
{
    extern __shared__ __align__(16) double osm[];
    const int P = p.npart, nup = p.nup;
    const int ng = o.ntabg > 0 ? 3 * (o.ntabg + 1) : 0, ndh = o.ntabg > 0 ? 6 * (2 * o.ntabg + 1) : 0;
    double* xs = osm;
    int* g = reinterpret_cast<int*>(xs + 3 * P);
    int* d = g + ng;
    for (int w = blockIdx.x; w < n; w += gridDim.x) {
        for (int t = threadIdx.x; t < 3 * P; t += kThreads) xs[t] = x[(size_t)w * 3 * P + t];
        if (o.ntabg > 0)
            for (int t = threadIdx.x; t < ng + ndh; t += kThreads) g[t] = 0;
        __syncthreads();
        if (o.ntabg > 0) {
            // pairs i < j (gofr.f90:57-73)
            for (int t = threadIdx.x; t < P * P; t += kThreads) {
                const int i = t / P, j = t % P;
                if (j <= i) continue;
                const int itab = (i < nup && j < nup) ? 1 : ((i >= nup && j >= nup) ? 2 : 0);
                double r2 = 0.0;
                for (int c = 0; c < 3; ++c) {
                    double dx = xs[3 * i + c] - xs[3 * j + c];
                    dx = dx - o.el * single::fnint(dx / o.el);
                    r2 += dx * dx;
                }
                const double r = sqrt(r2);
                const int index = r < 0.5 * o.el ? (int)(o.scaleg * r) : o.ntabg;
                atomicAdd(&g[itab * (o.ntabg + 1) + index], 1);
            }
            // density profile about the origin (gofr.f90:75-90)
            for (int t = threadIdx.x; t < 3 * P; t += kThreads) {
                const int i = t / 3, is = t % 3;
                double dx = xs[t];
                dx = dx - o.el * single::fnint(dx / o.el);
                const int itab = i < nup ? is : is + 3;
                const int index = (int)(o.scaleg * dx);
                atomicAdd(&d[itab * (2 * o.ntabg + 1) + index + o.ntabg], 1);
            }
        }
        // S(q): rho_k of each species, k = ak(:,1..nqtot) (k = 0 first)
        for (int iq = threadIdx.x; iq < o.nqtot; iq += kThreads) {
            const double* a = o.akq + 3 * iq;
            double ur = 0.0, ui = 0.0, dr = 0.0, di = 0.0;
            for (int i = 0; i < P; ++i) {
                double s, c;
                sincos(a[0] * xs[3 * i] + a[1] * xs[3 * i + 1] + a[2] * xs[3 * i + 2], &s, &c);
                if (i < nup) {
                    ur += c;
                    ui -= s;
                } else {
                    dr += c;
                    di -= s;
                }
            }
            double* out = sv + ((size_t)w * o.nqtot + iq) * 4;
            out[0] = ur * ur + ui * ui;
            out[1] = dr * dr + di * di;
            out[2] = ur * dr + ui * di;   // rhokup * conjg(rhokdn)
            out[3] = ui * dr - ur * di;
        }
        __syncthreads();
        if (o.ntabg > 0) {
            for (int t = threadIdx.x; t < ng; t += kThreads) hg[(size_t)w * ng + t] = g[t];
            for (int t = threadIdx.x; t < ndh; t += kThreads) hd[(size_t)w * ndh + t] = d[t];
        }
        __syncthreads();
    }
}

// n(k) of one walker per CTA (momentum3d.f90:89-124); warp m % kWarps runs
// move m = i * nsamp + ii, whose three uniforms are draws 3m+1..3m+3 of the
// walker's stream
__global__ void __launch_bounds__(kThreads) ops_enk_kernel(const __grid_constant__ DevParams p,
                                                          const __grid_constant__ OpsDev o,
                                                          const KVecDev* __restrict__ kv,
                                                          const TabUD* __restrict__ tud,
                                                          const TabSS* __restrict__ tss,
                                                          const double* __restrict__ x,
                                                          const unsigned long long* __restrict__ irn,
                                                          const double* __restrict__ sinv, int n,
                                                          double* __restrict__ tk, int tab)
{
    extern __shared__ __align__(16) double osm[];
    const int P = p.npart, nd = p.nd, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nct = o.nnk + 1, nq = p.nk - 1;
    double* xs = osm;
    double* accv = xs + 3 * P;   // [kWarps][nkv]
    // with tab: (cos, sin) of every k vector at every particle, [nq][P], and
    // at each warp's moved particle, [kWarps][nq]
    // (16-byte aligned: the offset from the aligned start is rounded up to an even count)
    double2* cs = reinterpret_cast<double2*>(osm + ((3 * P + kWarps * o.nkv + 1) & ~1));
    double2* csn = cs + (size_t)nq * P + (size_t)warp * nq;
    // with tab: each particle's Jastrow sum at its current position, [P]
    double* uold = reinterpret_cast<double*>(cs + (size_t)nq * P + (size_t)kWarps * nq);
    for (int w = blockIdx.x; w < n; w += gridDim.x) {
        for (int t = threadIdx.x; t < 3 * P; t += kThreads) xs[t] = x[(size_t)w * 3 * P + t];
        for (int t = threadIdx.x; t < kWarps * o.nkv; t += kThreads) accv[t] = 0.0;
        __syncthreads();
        if (tab)
            for (int t = threadIdx.x; t < nq * P; t += kThreads) {
                const int k = t / P + 1, j = t - (k - 1) * P;
                double sn, c;
                sincos(kv[k].k[0] * xs[3 * j] + kv[k].k[1] * xs[3 * j + 1] + kv[k].k[2] * xs[3 * j + 2], &sn, &c);
                cs[t] = make_double2(c, sn);
            }
        if (tab)
            for (int i = warp; i < P; i += kWarps) {
                const double r[3] = {xs[3 * i], xs[3 * i + 1], xs[3 * i + 2]};
                const double u = single::warp_jastrow_sum(p, tud, tss, xs, i, r);
                if (lane == 0) uold[i] = u;
            }
        __syncthreads();
        const unsigned long long s0 = irn[w];
        const double* S = sinv + (size_t)w * nd * nd;
        double* mine = accv + warp * o.nkv;
        for (int m = warp; m < P * o.nsamp; m += kWarps) {
            const int i = m / o.nsamp;
            double dx[3], drr[3], xi[3];
            for (int c = 0; c < 3; ++c) {
                const unsigned long long st = walker::lcg_jump(s0, o.jA, o.jC, 3 * m + c + 1);
                dx[c] = (walker::lcg_uniform(st) - 0.5) * p.el;
                drr[c] = -dx[c];
                xi[c] = xs[3 * i + c] + dx[c];
            }
            double rat1, rat2;
            if (tab) {
                // getphione as exp(U(x_i') - U(x_i)) with U(x_i) computed once per walker
                rat1 = exp(single::warp_jastrow_sum(p, tud, tss, xs, i, xi) - uold[i]);
                for (int k = lane; k < nq; k += 32) {
                    double sn, c;
                    sincos(kv[k + 1].k[0] * xi[0] + kv[k + 1].k[1] * xi[1] + kv[k + 1].k[2] * xi[2], &sn, &c);
                    const double v = kv[k + 1].v;   // the shell amplitude 2 vorb, applied once per move
                    csn[k] = make_double2(v * c, v * sn);
                }
                __syncwarp();
                rat2 = single::warp_bcsone_tab(p, kv, tud, xs, S, i, xi, cs, csn);
                __syncwarp();
            } else {
                rat1 = single::warp_getphione(p, tud, tss, xs, i, drr);
                rat2 = single::warp_bcsone(p, kv, tud, xs, S, i, xi);
            }
            const double psirat = rat1 * rat2;
            // cos(dk m dx_c) for m = 0..nnk, c = 0..2, one per lane
            double ct = 1.0;
            if (lane < 3 * nct) {
                const int c = lane / nct, mm = lane % nct;
                ct = cos(o.dk * mm * dx[c]);
            }
            for (int v0 = 0; v0 < o.nkv; v0 += 32) {
                const int v = v0 + lane;
                const int* ikv = o.ik + 3 * (v < o.nkv ? v : 0);
                const double c0 = __shfl_sync(0xffffffffu, ct, ikv[0]);
                const double c1 = __shfl_sync(0xffffffffu, ct, nct + ikv[1]);
                const double c2 = __shfl_sync(0xffffffffu, ct, 2 * nct + ikv[2]);
                if (v < o.nkv) mine[v] += psirat * c0 * c1 * c2;
            }
        }
        __syncthreads();
        // per shell, warps then vectors in order
        for (int k = threadIdx.x; k <= o.ntabk; k += kThreads) {
            double s = 0.0;
            for (int ww = 0; ww < kWarps; ++ww)
                for (int j = 0; j < o.nkk[k]; ++j) s += accv[ww * o.nkv + o.indk[k] + j];
            tk[(size_t)w * (o.ntabk + 1) + k] = s;
        }
        __syncthreads();
    }
}

// Weight of each walker for the operator sums: weight * exp(psil - psigl) *
// is * wt0 (operators.f90:103), once per walker.
__global__ void ops_weight_kernel(DevStack s, int n, double* __restrict__ wt)
{
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < n; w += gridDim.x * blockDim.x)
        wt[w] = s.weight[w] * exp(s.psil[w] - s.psigl[w]) * s.is[w] * (double)s.wt0[w];
}

// The weighted sums (addgofr/addsofq/addenk accumulation), walkers in pop
// order (index n-1 first), one thread per running sum, with the walker
// weights of ops_weight_kernel.
__global__ void ops_reduce_kernel(const __grid_constant__ OpsDev o, int n, const double* __restrict__ wts,
                                  const int* __restrict__ hg, const int* __restrict__ hd,
                                  const double* __restrict__ sv, const double* __restrict__ tk,
                                  double* __restrict__ sums)
{
    const int ng = o.ntabg > 0 ? 3 * (o.ntabg + 1) : 0, ndh = o.ntabg > 0 ? 6 * (2 * o.ntabg + 1) : 0;
    const int nq = 3 * o.nqtot, nk = o.nkv > 0 ? o.ntabk + 1 : 0;
    const int total = 2 * (ng + ndh + nq + nk) + 3;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        double acc = sums[t];
        int u = t;
        for (int w = n - 1; w >= 0; --w) {
            const double wt = wts[w];
            double add;
            if (u < 2 * ng) {
                const int b = u % ng;
                const double cnt = (double)hg[(size_t)w * ng + b];
                add = (u < ng ? 2.0 : 4.0) * wt * cnt;
            } else if (u < 2 * (ng + ndh)) {
                const int v = u - 2 * ng, b = v % ndh;
                const double cnt = (double)hd[(size_t)w * ndh + b];
                const bool center = (b % (2 * o.ntabg + 1)) == o.ntabg;
                add = (v < ndh ? (center ? 0.5 : 1.0) : (center ? 0.25 : 1.0)) * wt * cnt;
            } else if (u < 2 * (ng + ndh + nq)) {
                const int v = u - 2 * (ng + ndh), b = v % nq, itab = b / o.nqtot, iq = b % o.nqtot;
                const double* e = sv + ((size_t)w * o.nqtot + iq) * 4;
                const double val = e[itab];
                const double sq = itab < 2 ? val * val : e[2] * e[2] - e[3] * e[3];
                add = (v < nq ? val : sq) * wt;
            } else if (u < total - 3) {
                const int v = u - 2 * (ng + ndh + nq), k = v % nk;
                const double e = tk[(size_t)w * nk + k] / o.nkk[k];
                add = (v < nk ? e : e * e) * wt;
            } else {
                add = (u == total - 1) ? wt * o.nsamp : wt;   // wsg = wsq, wsk
            }
            acc += add;
        }
        sums[t] = acc;
    }
}

}  // namespace

size_t ops_walker_smem(const DevParams& p, const OpsDev& o)
{
    return sizeof(double) * 3 * p.npart + sizeof(int) * (size_t)(3 * (o.ntabg + 1) + 6 * (2 * o.ntabg + 1)) + 16;
}

cudaError_t launch_ops_walker(const DevParams& p, const OpsDev& o, const double* x, int n, int* hg, int* hd,
                              double* sv, int grid, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const size_t smem = ops_walker_smem(p, o);
    cudaError_t e = cudaFuncSetAttribute(ops_walker_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    ops_walker_kernel<<<grid < n ? grid : n, kThreads, smem, st>>>(p, o, x, n, hg, hd, sv);
    return cudaGetLastError();
}

cudaError_t launch_ops_enk(const DevParams& p, const OpsDev& o, const KVecDev* kv, const TabUD* tud,
                           const TabSS* tss, const double* x, const unsigned long long* irn, const double* sinv,
                           int n, double* tk, int grid, cudaStream_t st)
{
    if (n <= 0 || o.nkv <= 0) return cudaSuccess;
    const size_t base = sizeof(double) * ((3 * (size_t)p.npart + (size_t)kWarps * o.nkv + 1) & ~(size_t)1);
    const size_t nq = p.nk > 1 ? p.nk - 1 : 1;
    const size_t with_tab = base + sizeof(double2) * nq * ((size_t)p.npart + kWarps) + sizeof(double) * p.npart;
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const int tab = with_tab <= (size_t)optin ? 1 : 0;   // plane-wave tables on chip when they fit
    const size_t smem = tab ? with_tab : base;
    cudaError_t e = cudaFuncSetAttribute(ops_enk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    ops_enk_kernel<<<grid < n ? grid : n, kThreads, smem, st>>>(p, o, kv, tud, tss, x, irn, sinv, n, tk, tab);
    return cudaGetLastError();
}

cudaError_t launch_ops_reduce(const OpsDev& o, int n, const DevStack& s, const int* hg, const int* hd,
                              const double* sv, const double* tk, double* sums, double* wts, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    ops_weight_kernel<<<(n + 255) / 256, 256, 0, st>>>(s, n, wts);
    ops_reduce_kernel<<<1, 1024, 0, st>>>(o, n, wts, hg, hd, sv, tk, sums);
    return cudaGetLastError();
}

}  // namespace dmc
