// Single-particle moves and parameter derivatives of the DMCBS walker path
// (sm_103a):
//  - bcsone   (psislaterbcs.f90:296-376): determinant ratio for one particle
//    moved, from the stored inverse of the pair matrix;
//  - getphione (coshpot.f90:207-264): Jastrow ratio exp(U' - U) for the same
//    move; move1 (wavefunction.f90:393-404) is their product;
//  - getderbcs (psislaterbcs.f90:449-524, optsw on, optbeta off):
//    d log|det| / d vorb(shell) = tr(S^-1 dS/dvorb);
//  - the sums that calder (optimizer.f90:90-116) accumulates over a walker
//    population for the stochastic-reconfiguration step.
// One warp per walker for the ratios (a few hundred flops each); one CTA per
// walker for the derivatives, which contract the whole inverse.
#include <cuda_runtime.h>
#include <math.h>

#include "dmc_device.cuh"
#include "dmc_kernels.h"
#include "dmc_walker.cuh"
#include "dmc_single.cuh"

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
__global__ void sr_sums_kernel(const double* __restrict__ der, const double* __restrict__ d2psi,
                               const double* __restrict__ v, int n, int np, double hbar, double eunit,
                               double npart, double* __restrict__ sums)
{
    const int nout = np * np + 2 * np + 2;
    for (int t = threadIdx.x; t < nout; t += blockDim.x) {
        double s = sums[t];
        for (int w = n - 1; w >= 0; --w) {
            // ene = (-hbar*d2psi + v)/eunit/npart (dmcbcs.f90:497)
            const double e = __ddiv_rn(__ddiv_rn(__dadd_rn(__dmul_rn(-hbar, d2psi[w]), v[w]), eunit), npart);
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

cudaError_t launch_jasder(const DevParams& p, const double* jq, const double* x, double* dpsi, int nw, int grid,
                          cudaStream_t st, int stride)
{
    if (nw <= 0) return cudaSuccess;
    const size_t smem = sizeof(double) * (size_t)(p.nql > 0 ? p.nql : 1);
    jasder_kernel<<<grid < nw ? grid : nw, kThreads, smem, st>>>(p, jq, x, dpsi, nw, stride);
    return cudaGetLastError();
}

cudaError_t launch_sr_sums(const double* der, const double* d2psi, const double* v, int n, int np, double hbar,
                           double eunit, int npart, double* sums, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    sr_sums_kernel<<<1, 1024, 0, st>>>(der, d2psi, v, n, np, hbar, eunit, (double)npart, sums);
    return cudaGetLastError();
}

}  // namespace dmc
