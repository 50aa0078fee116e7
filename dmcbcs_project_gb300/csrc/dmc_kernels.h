// Launchers of the GB300 DMCBS kernels (implemented in dmc_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "dmc_device.cuh"

namespace dmc {

// Bytes of dynamic shared memory of the walker kernel for these sizes; fills
// the on-chip layout.  limit_bytes is the per-CTA limit.
int walker_smem_bytes(const DevParams& p, int limit_bytes, SmemLayout* Lout, int nt = kThreads,
                      bool union_global = false);
// dynamic shared-memory opt-in of both walker kernels for layout L (once,
// before any graph capture); gf: the idmc = 10 instances (their moves) too
cudaError_t prepare_walker(const SmemLayout& L, bool gf = false);
// static shared memory of the walker kernels (the largest instance; gf: the
// idmc = 10 instances included), -1 on error
int walker_static_smem_bytes(bool gf = false);
// the idmc = 10 instances (dmc_walker_gf.cu): static shared memory, the
// shared-memory opt-in, and the move launch that launch_walker forwards to
int walker_gf_static_smem_bytes();
// the instances with the union region in global scratch (dmc_walker_big.cu),
// launch_walker forwards every launch with L.un_in_smem == 0 to them
int walker_big_static_smem_bytes();
cudaError_t walker_big_attrs(int smem);
cudaError_t launch_walker_big(const DevParams& p, const KernelArgs& a, const SmemLayout& L, int grid, cudaStream_t st,
                              bool mixed, bool gf);
cudaError_t walker_gf_attrs(int smem, int nt, bool both, bool mixed);
cudaError_t launch_walker_gf(const DevParams& p, const KernelArgs& a, const SmemLayout& L, int grid, cudaStream_t st,
                             bool mixed);

cudaError_t launch_walker(const DevParams& p, const KernelArgs& a, const SmemLayout& L, int grid, cudaStream_t st,
                          bool mixed = false);

// whether the batched inverse of one n x n matrix fits one CTA's shared
// memory (1), not (0), or the device query failed (-1); *two_buffers: the
// blocked form's second buffer fits as well
int matinv_fits(int n, bool* two_buffers = nullptr);

// estimator block sums with compensation (comp: their error terms,
// [3][DMC_NEST_MAX] for valblk, valblk2, wtblk); part: kEstBlocks x 3
// DMC_NEST_MAX doubles of partial sums, ticket: one counter, zero between
// launches (the kernel leaves it zero)
constexpr int kEstBlocks = 64;
cudaError_t launch_estimators(const double* est, int n, int nest, double* vb, double* vb2, double* wb, double* comp,
                              double* part, unsigned int* ticket, cudaStream_t st, const int* pn = nullptr,
                              unsigned long long* steps = nullptr);

cudaError_t launch_branch(const DevStack& in, const DevStack& out, int n, int n3, int cap, double factor,
                          int* counts, int* offs, unsigned long long* irn1, unsigned long long* wtisto,
                          cudaStream_t st);
// the same with the walker count on the device: *pn walkers in, the count
// out to *pn_out; with need != nullptr a population-control pass that
// branches with *dfactor only when *need is set and then copies the result
// back into `in` (the walkers stay in `in` either way); overflow sets bit 1
// of *flags
cudaError_t launch_branch_dev(const DevStack& in, const DevStack& out, const int* pn, int* pn_out, const int* need,
                              const double* dfactor, int* flags, int n3, int cap, int nsm, int* counts, int* offs,
                              unsigned long long* irn1, unsigned long long* wtisto, cudaStream_t st);
// population control decision (dmcbcs.f90): *need, *factor for the next pass
cudaError_t launch_popctl(const int* pn, double nwalk, double popup, double popdn, int* need, double* factor,
                          int* flags, cudaStream_t st);

// Single-particle ratios and parameter derivatives (dmc_single.cu)
cudaError_t launch_bcsone(const DevParams& p, const KVecDev* kv, const TabUD* tud, const double* x,
                          const double* smati, const int* ipart, const double* dr, double* ratio, int nw,
                          cudaStream_t st);
cudaError_t launch_getphione(const DevParams& p, const TabUD* tud, const TabSS* tss, const double* x,
                             const int* ipart, const double* drr, double* ratio, int nw, cudaStream_t st);
// walker arrays in host memory the device addresses directly (pinned and
// mapped, or managed), laid out as dmc_walkers
struct HostWalkers {
    double *x, *dpsi, *dpsig, *psil, *psigl, *d2psi, *d2psig, *v, *vext, *weight, *psil0, *psigl0, *wt0;
    int* is;
    long long* irn;
};
cudaError_t launch_walkers_put(const HostWalkers& h, const DevStack& d, int n, int n3, int* pn, int grid,
                               cudaStream_t st);
// with pn: the count is read on the device, at most cap walkers written
cudaError_t launch_walkers_get(const DevStack& d, const HostWalkers& h, int n, int n3, int grid, cudaStream_t st,
                               const int* pn = nullptr, int cap = 0);
size_t derbcs_smem_bytes(const DevParams& p);
// most parameters of the adjoint gradients: vorb (DMC_MAX_SHELLS), bfact,
// b, d and the 16 Jastrow knots
constexpr int kPgradMax = DMC_MAX_SHELLS + 3 + 16;
// {f, f', lap f} records of the b and d derivative tables of beta
struct PgTab {
    double f, df, d2f, pad;
};
// adjoint parameter gradients (dmc_single.cu): doubles of one CTA's core
// (on chip when it fits in smem_limit bytes, else in gscr: grid x that) and
// of its global slice (slices: grid x that, always); the grid that keeps
// every SM's resident CTAs busy (0 on a CUDA error); ktd the Jastrow knot
// basis on the table grid ([16][ntab+1], needed with nknot > 0)
size_t pgrad_doubles(const DevParams& p);
size_t pgrad_slice_doubles(const DevParams& p);
int pgrad_grid(const DevParams& p, int nw, int nsm, int smem_limit);
cudaError_t launch_pgrad(const DevParams& p, const KVecDev* kv, const TabUD* tud, const double* x, const double* sinv,
                         const double* dpsi, const double* dphi, double* dlog, double* deloc, int nw, int np,
                         double bfact, const PgTab* btd, const PgTab* ktd, int nbeta, int nknot, int grid,
                         double* gscr, double* slices, int smem_limit, cudaStream_t st);
// particle-by-particle sweeps with Sherman-Morrison updates (dmc_sweep.cu):
// nsweep sweeps of the n walkers of stack st (positions and random states
// updated in place); the inverse comes from inv64 (FP64, fresh) or, when
// inv64 is null, from inv32, and leaves in inv32; tab is cos/sin scratch
// [n][nk-1][npart]; accepted[w] counts the walker's accepted moves; prop
// is scratch for each sweep's proposals, [n][npart][4] doubles
size_t sweep_smem_bytes(const DevParams& p, int walkers_per_cta);
// jA/jC: ran1 jump-ahead tables for 0 .. 5 npart steps
cudaError_t launch_sweeps(const DevParams& p, const DevStack& st, int n, int nsweep, const double* inv64,
                          float* inv32, float2* tab, const KVecMP* kv, const TabUDmp* tud, const TabSSmp* tss,
                          const unsigned long long* jA, const unsigned long long* jC, unsigned long long* accepted,
                          double* prop, cudaStream_t stream);
// dpsi[w*stride + off + shell]; stride < 0 means norb
cudaError_t launch_derbcs(const DevParams& p, const KVecDev* kv, const double* x, const double* smati, double* dpsi,
                          int nw, int grid, cudaStream_t st, int stride = -1, int off = 0);
// getjasder: dpsi[w*stride + 0..1] = d U_long / d beta, d U_long / d gamma
cudaError_t launch_jasder(const DevParams& p, const double* jq, const double* x, double* dpsi, int nw, int grid,
                          cudaStream_t st, int stride);
// adds the calder sums of n walkers (pop order) to sums[np*np + 2*np + 2]:
// ovec, ovecw, pmat (column-major), esum, esum2; ene: scratch of n doubles
cudaError_t launch_sr_sums(const double* der, const double* d2psi, const double* v, int n, int np, double hbar,
                           double eunit, int npart, double* sums, double* ene, cudaStream_t st);

// Operators (dmc_ops.cu): per-walker histograms and S(q) values, n(k) per
// walker, and the weighted sums over the population in pop order.  sums:
// gnow, gerr [3(ntabg+1)], dnow, derr [6(2 ntabg+1)], snow, serr [3 nqtot],
// enknow, enkerr [ntabk+1], then wsg, wsq, wsk.
size_t ops_walker_smem(const DevParams& p, const OpsDev& o);
cudaError_t launch_ops_walker(const DevParams& p, const OpsDev& o, const double* x, int n, int* hg, int* hd,
                              double* sv, int grid, cudaStream_t st);
cudaError_t launch_ops_enk(const DevParams& p, const OpsDev& o, const KVecDev* kv, const TabUD* tud,
                           const TabSS* tss, const double* x, const unsigned long long* irn, const double* sinv,
                           int n, double* tk, int grid, cudaStream_t st);
// wts: scratch of n doubles for the walker weights
cudaError_t launch_ops_reduce(const OpsDev& o, int n, const DevStack& s, const int* hg, const int* hd,
                              const double* sv, const double* tk, double* sums, double* wts, cudaStream_t st);

// deferred step decision (idmc = 1, -2): weights and estimator records of
// the pushed walkers after a MODE_STEP walker launch with a.defer set
cudaError_t launch_step_decide(const DevParams& p, const KernelArgs& a, cudaStream_t st);

// FMA throughput of the FP64 (kind 0) or FP32 (kind 1) pipe, TFLOP/s
cudaError_t probe_fma_peak(int kind, int nsm, double* tflops);

// The mixed path's double-float elementary functions on device arrays:
// fn 0: sin(pi a), cos(pi a); fn 1: sin(2 pi u), cos(2 pi u) of u = m 2^-48
// (in holds the integers m); fn 2: log x.  out[2i], out[2i+1] (fn 2: out[i]).
cudaError_t launch_dfmath_eval(int fn, int n, const void* in, double* out, cudaStream_t st);

}  // namespace dmc
