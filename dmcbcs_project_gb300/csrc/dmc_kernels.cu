// Kernels of the GB300 DMCBS walker path (sm_103a): the walker kernel
// instances of every idmc but 10 (one DMC move plus the full wavefunction and
// local energy of a walker per CTA, in plain FP64 and in the mixed
// double-float / FP32 form; the kernel is in dmc_walker_kernel.cuh, its
// stages in dmc_walker.cuh), and the population kernels (estimator sums,
// branching, stack reversal, batched inverse).
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include "dmc_device.cuh"
#include "dmc_kernels.h"
#include "dmc_attr.h"
#include "dmc_walker_kernel.cuh"

namespace dmc {

constexpr unsigned long long kMask48 = walker::kMask48;

// ---------------------------------------------------------------------------
// Deferred step decision for idmc = 1, -2 (every proposal is kept): one
// thread per pushed walker k computes its weight, sign weight and estimator
// record from its new scalars (written by the walker kernel) and the popped
// walker's old ones.
// ---------------------------------------------------------------------------
__global__ void step_decide_kernel(const __grid_constant__ DevParams p, const __grid_constant__ KernelArgs a)
{
    const int nw = a.pn ? *a.pn : a.nw;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nw) return;
    const int src = nw - 1 - k;
    const StepScalars nn{a.out.psil[k], a.out.psigl[k], a.out.d2psi[k], a.out.d2psig[k], a.out.v[k], a.out.vext[k],
                         a.out.is[k]};
    const StepScalars ol{a.in.psil[src], a.in.psigl[src], a.in.d2psi[src], a.in.d2psig[src], a.in.v[src],
                         a.in.vext[src], a.in.is[src]};
    double wnew;
    float wt0new;
    const float wt0 = a.in_wt0d ? (float)a.in_wt0d[src] : a.in.wt0[src];
    step_decision(p, a.opcomp, nn, ol, a.in.weight[src], wt0, true, 0.0, a.est + (size_t)k * p.nest * 2, wnew, wt0new);
    a.out.weight[k] = wnew;
    a.out.wt0[k] = wt0new;
}

cudaError_t launch_step_decide(const DevParams& p, const KernelArgs& a, cudaStream_t st)
{
    if (a.nw <= 0) return cudaSuccess;   // with a.pn, a.nw is the capacity
    step_decide_kernel<<<(a.nw + 127) / 128, 128, 0, st>>>(p, a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Estimator block sums (estimator.f90:72-82): est[n][nest][2] -> valblk,
// valblk2, wtblk (accumulated), fixed-order tree per estimator.
// ---------------------------------------------------------------------------
// s + x with the rounding error of the addition collected in c (Neumaier's
// variant of Kahan summation: also exact when |x| > |s|)
__device__ __forceinline__ void comp_add(double& s, double& c, double x)
{
    const double t = s + x;
    c += fabs(s) >= fabs(x) ? (s - t) + x : (x - t) + s;
    s = t;
}

// The estimator sums of one generation (addval, estimator.f90:72-84) over
// kEstBlocks CTAs, each a contiguous share of the walkers: thread (e, sub)
// sums estimator e over every nsub-th walker of the share, so that a warp
// reads consecutive records and the FP64 work is spread over many SMs.  The
// CTA that finishes last combines the shares' partial sums in CTA order and
// adds them to the block sums with compensation: the block sums carried
// across a block's generations keep their error terms in
// comp[3][DMC_NEST_MAX], added back when the sums are read.  The partition
// and every order are fixed, so the sums are the same run to run.
__global__ void __launch_bounds__(256) estimator_kernel(const double* est, int n, const int* pn, int nest,
                                                        double* valblk, double* valblk2, double* wtblk, double* comp,
                                                        double* part, unsigned int* ticket, unsigned long long* steps)
{
    if (pn) n = *pn;
    if (steps && blockIdx.x == 0 && threadIdx.x == 0) *steps += (unsigned long long)n;   // walker-steps of the generation
    const int nsub = (int)blockDim.x / nest;   // threads per estimator
    const int e = (int)threadIdx.x % nest, sub = (int)threadIdx.x / nest;
    const int per = (n + (int)gridDim.x - 1) / (int)gridDim.x;
    const int k0 = (int)blockIdx.x * per, k1 = min(n, k0 + per);
    __shared__ double red[256 * 3];
    if (sub < nsub) {
        double s0 = 0.0, s1 = 0.0, s2 = 0.0;
        for (int k = k0 + sub; k < k1; k += nsub) {
            const double v = est[((size_t)k * nest + e) * 2], wt = est[((size_t)k * nest + e) * 2 + 1];
            s0 += v * wt;
            s1 += v * v * wt;
            s2 += wt;
        }
        red[threadIdx.x * 3] = s0;
        red[threadIdx.x * 3 + 1] = s1;
        red[threadIdx.x * 3 + 2] = s2;
    }
    __syncthreads();
    if ((int)threadIdx.x < 3 * nest) {
        const int ee = (int)threadIdx.x / 3, q = (int)threadIdx.x % 3;
        double t = 0.0;
        for (int u = 0; u < nsub; ++u) t += red[(u * nest + ee) * 3 + q];
        part[((size_t)blockIdx.x * DMC_NEST_MAX + ee) * 3 + q] = t;
    }
    // the last CTA to finish (threadFenceReduction pattern) combines them
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    if ((int)threadIdx.x < 3 * nest) {
        const int ee = (int)threadIdx.x / 3, q = (int)threadIdx.x % 3;
        double t = 0.0;
        for (int blk = 0; blk < (int)gridDim.x; ++blk) t += __ldcg(part + ((size_t)blk * DMC_NEST_MAX + ee) * 3 + q);
        double* dst = q == 0 ? valblk : (q == 1 ? valblk2 : wtblk);
        comp_add(dst[ee], comp[q * DMC_NEST_MAX + ee], t);
    }
    if (threadIdx.x == 0) *ticket = 0u;
}

// ---------------------------------------------------------------------------
// branch (step.f90:287-315), three passes: copy counts, scan, scatter.
// The input stack is popped from the top: pop index m = n-1-j.
// ---------------------------------------------------------------------------
// Device-count form (BranchDev): n from *pn; with a condition flag the pass
// branches only when *need is set (population control) and otherwise copies
// every walker unchanged in place.
struct BranchDev {
    const int* pn;          // walkers in the input stack
    int* pn_out;            // walkers in the output stack (written by the scan)
    const int* need;        // nullptr: always branch
    const double* factor;   // weight factor when need is set
    int* flags;             // bit 1: the output stack overflowed
};

__global__ void branch_count_kernel(DevStack in, int n, double factor, int* counts,
                                    unsigned long long* irn1, unsigned long long* wtisto, BranchDev bd, int cap)
{
    if (bd.pn) {
        n = *bd.pn;
        if (bd.need) {
            if (!*bd.need) return;   // plain copy pass
            factor = *bd.factor;
        }
    }
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
    const int j = n - 1 - m;
    const double wt = in.weight[j] * factor;
    // ran1 on the walker's own state
    const unsigned long long s = in.irn[j] & kMask48;
    const unsigned long long s1 = (44485709377909ull * s + 96309754297ull) & kMask48;
    const double rn = lcg_uniform(s1);
    // int(w + u) as the reference truncates it, for weights in range; a
    // non-finite or huge weight gives at most cap + 1 copies (the pass then
    // reports an overflow) so the prefix sums stay bounded, NaN gives none
    const double xw = wt + rn;
    const double lim = (double)cap + 1.0;
    const int iwt = xw != xw ? 0 : (xw >= lim ? (int)lim : (xw <= -lim ? -(int)lim : (int)xw));
    counts[m] = iwt > 0 ? iwt : 0;
    irn1[m] = s1;
    if (iwt >= 0 && iwt < DMC_WTISTO) atomicAdd(&wtisto[iwt], 1ull);
    }
}

// single-CTA exclusive scan of counts[0..n) -> offs, total in offs[n]
__global__ void scan_kernel(const int* counts, int n, int* offs, int cap, BranchDev bd)
{
    __shared__ long long part[1024];
    if (bd.pn) {
        n = *bd.pn;
        if (bd.need && !*bd.need) {
            if (threadIdx.x == 0) *bd.pn_out = n;   // plain copy pass
            return;
        }
    }
    const int t = threadIdx.x, T = blockDim.x;
    const int chunk = (n + T - 1) / T;
    const int b = t * chunk, e = min(n, b + chunk);
    // sums in 64 bits, offsets stored saturated at cap + 1: copies at or
    // beyond cap are dropped by the scatter, so no offset past cap is used
    const long long sat = (long long)cap + 1;
    long long s = 0;
    for (int i = b; i < e; ++i) s += counts[i];
    part[t] = s;
    __syncthreads();
    // Hillis-Steele on the partials
    for (int o = 1; o < T; o <<= 1) {
        const long long v = t >= o ? part[t - o] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    long long run = part[t] - s;
    for (int i = b; i < e; ++i) {
        offs[i] = (int)(run < sat ? run : sat);
        run += counts[i];
    }
    if (t == T - 1) {
        const long long tot = part[T - 1];
        offs[n] = (int)(tot < sat ? tot : sat);
        if (bd.pn_out) {
            *bd.pn_out = (int)(tot < cap ? tot : cap);
            if (tot > cap) atomicOr(bd.flags, 2);
        }
    }
}

// ran2 (ran.f90:29-48) applied k times: the affine map s -> a s + c mod 2^48
// raised to the k-th power by squaring
__device__ __forceinline__ unsigned long long ran2_jump(unsigned long long s, unsigned k)
{
    unsigned long long A = 1ull, C = 0ull, a = 34522712143931ull, c = 55789347517ull;
    while (k) {
        if (k & 1u) {
            A = (a * A) & kMask48;
            C = (a * C + c) & kMask48;
        }
        c = (a * c + c) & kMask48;
        a = (a * a) & kMask48;
        k >>= 1;
    }
    return (A * s + C) & kMask48;
}

// One warp per output slot d < min(total, cap), so that a walker with many
// copies is spread over many warps: its source is the pop index m with
// offs[m] <= d < offs[m + 1] (binary search over the non-decreasing offsets;
// walkers without copies have offs[m] == offs[m + 1] and are never found),
// and copy c = d - offs[m] carries the state c + 1 ran2 steps after irn1[m]
// (the reference's loop advances the stream once per copy before the push).
__global__ void branch_scatter_kernel(DevStack in, DevStack out, int n, int n3, int cap, const int* counts,
                                      const int* offs, const unsigned long long* irn1, BranchDev bd)
{
    (void)counts;
    const int lane = threadIdx.x & 31;
    if (bd.pn) {
        n = *bd.pn;
        if (bd.need && !*bd.need) return;   // no population control this generation
    }
    if (n <= 0) return;
    const int total = min(offs[n], cap);
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int d = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; d < total; d += nwarps) {
        int lo = 0, hi = n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (offs[mid] <= d)
                lo = mid;
            else
                hi = mid - 1;
        }
        const int m = lo, j = n - 1 - m;
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
            out.weight[d] = copysign(1.0, in.weight[j]);
            out.psil0[d] = in.psil0[j];
            out.psigl0[d] = in.psigl0[j];
            out.wt0[d] = in.wt0[j];
            out.is[d] = in.is[j];
            out.irn[d] = ran2_jump(irn1[m], (unsigned)(d - offs[m]) + 1u);
        }
    }
}

// Population-control pass, second half: the branched stack back into the
// input stack (same order), so the pass leaves the walkers where they were
// whether or not it branched
__global__ void stack_copy_kernel(DevStack from, DevStack to, const int* pn, const int* need, int n3)
{
    if (!*need) return;
    const int n = *pn;
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < n; j += nwarps) {
        for (int e = lane; e < n3; e += 32) {
            to.x[(size_t)j * n3 + e] = from.x[(size_t)j * n3 + e];
            to.dpsi[(size_t)j * n3 + e] = from.dpsi[(size_t)j * n3 + e];
            to.dpsig[(size_t)j * n3 + e] = from.dpsig[(size_t)j * n3 + e];
        }
        if (lane == 0) {
            to.psil[j] = from.psil[j];
            to.psigl[j] = from.psigl[j];
            to.d2psi[j] = from.d2psi[j];
            to.d2psig[j] = from.d2psig[j];
            to.v[j] = from.v[j];
            to.vext[j] = from.vext[j];
            to.weight[j] = from.weight[j];
            to.psil0[j] = from.psil0[j];
            to.psigl0[j] = from.psigl0[j];
            to.wt0[j] = from.wt0[j];
            to.is[j] = from.is[j];
            to.irn[j] = from.irn[j];
        }
    }
}

// Population control of dmcbcs.f90 (after the branch of a generation): a
// second branch with factor nwalk/n when n left [popdn, popup] * nwalk.
// One thread: sets *need and *factor for the conditional branch pass;
// flags bit 0 when the population died out.
__global__ void popctl_kernel(const int* pn, double nwalk, double popup, double popdn, int* need, double* factor,
                              int* flags)
{
    const int n = *pn;
    const bool out = n > popup * nwalk || n < popdn * nwalk;
    if (n == 0) atomicOr(flags, 1);
    *need = (out && n > 0) ? 1 : 0;
    *factor = n > 0 ? nwalk / n : 1.0;
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------

int walker_smem_bytes(const DevParams& p, int limit_bytes, SmemLayout* Lout, int nt, bool union_global)
{
    SmemLayout L = make_layout(p, limit_bytes, nt, union_global);
    if (Lout) *Lout = L;
    return L.total * 8;
}

int walker_static_smem_bytes(bool gf)
{
    cudaFuncAttributes a[3]{};
    if (cudaFuncGetAttributes(&a[0], walker_kernel<double, kThreads, false>) != cudaSuccess) return -1;
    if (cudaFuncGetAttributes(&a[1], walker_kernel<df, kThreads, false>) != cudaSuccess) return -1;
    if (cudaFuncGetAttributes(&a[2], walker_kernel<df, 2 * kThreads, false>) != cudaSuccess) return -1;
    size_t m = 0;
    for (const auto& x : a) m = x.sharedSizeBytes > m ? x.sharedSizeBytes : m;
    if (!gf) return (int)m;
    const int g = walker_gf_static_smem_bytes();
    if (g < 0) return -1;
    return (int)m > g ? (int)m : g;
}

// attribute kinds of the per-device record: the carveout, then the dynamic
// shared-memory opt-in of walker_kernel<df / double, 256 / 512 threads>
enum : int { kAttrCarveout = 0, kAttrSmemBase = 1 };
static AttrCache g_attr;

template <class R, int NT>
static int set_smem_attr(int v)
{
    return (int)cudaFuncSetAttribute(walker_kernel<R, NT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
}

static cudaError_t walker_attrs(int smem, int nt, bool both, bool mixed)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    // every launch asks for the largest shared-memory carveout, so CTAs of
    // launches with different layouts (systems of a batch) can share an SM
    int rc = g_attr.ensure(dev, kAttrCarveout, 1, [](int) {
        const int c = (int)cudaSharedmemCarveoutMaxShared;
        cudaError_t r = cudaFuncSetAttribute(walker_kernel<df, kThreads, false>, cudaFuncAttributePreferredSharedMemoryCarveout, c);
        if (r == cudaSuccess)
            r = cudaFuncSetAttribute(walker_kernel<double, kThreads, false>, cudaFuncAttributePreferredSharedMemoryCarveout, c);
        if (r == cudaSuccess)
            r = cudaFuncSetAttribute(walker_kernel<df, 2 * kThreads, false>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     c);
        return (int)r;
    });
    if (rc) return (cudaError_t)rc;
    // the mixed kernel runs with the layout's thread count, the FP64 kernel
    // always with 256 (it is FP64-pipe bound: 16 warps did not speed it up)
    const bool wide = nt != kThreads;
    if (both || mixed) {
        rc = g_attr.ensure(dev, kAttrSmemBase + (wide ? 2 : 0), smem,
                           wide ? set_smem_attr<df, 2 * kThreads> : set_smem_attr<df, kThreads>);
        if (rc) return (cudaError_t)rc;
    }
    if (both || !mixed) {
        rc = g_attr.ensure(dev, kAttrSmemBase + 1, smem, set_smem_attr<double, kThreads>);
        if (rc) return (cudaError_t)rc;
    }
    return cudaSuccess;
}

cudaError_t prepare_walker(const SmemLayout& L, bool gf)
{
    if (!L.un_in_smem) return walker_big_attrs(L.total * 8);
    return gf ? walker_gf_attrs(L.total * 8, L.nt, true, false) : walker_attrs(L.total * 8, L.nt, true, false);
}

cudaError_t launch_walker(const DevParams& p, const KernelArgs& a, const SmemLayout& L, int grid, cudaStream_t st,
                          bool mixed)
{
    if (!L.un_in_smem) return launch_walker_big(p, a, L, grid, st, mixed, a.mode == MODE_STEP && p.idmc == 10);
    if (a.mode == MODE_STEP && p.idmc == 10) return launch_walker_gf(p, a, L, grid, st, mixed);
    const size_t smem = (size_t)L.total * 8;
    // the shared-memory opt-in is recorded per device and size (prepare_walker
    // sets it before any graph capture; this finds it set)
    const cudaError_t e = walker_attrs((int)smem, L.nt, false, mixed);
    if (e != cudaSuccess) return e;
    if (!mixed)
        walker_kernel<double, kThreads, false><<<grid, kThreads, smem, st>>>(p, a, L);
    else if (L.nt == 2 * kThreads)
        walker_kernel<df, 2 * kThreads, false><<<grid, 2 * kThreads, smem, st>>>(p, a, L);
    else
        walker_kernel<df, kThreads, false><<<grid, kThreads, smem, st>>>(p, a, L);
    return cudaGetLastError();
}

cudaError_t launch_estimators(const double* est, int n, int nest, double* vb, double* vb2, double* wb, double* comp,
                              double* part, unsigned int* ticket, cudaStream_t st,
                              const int* pn, unsigned long long* steps)
{
    if (n <= 0 && !pn) return cudaSuccess;
    if (nest < 1 || nest > DMC_NEST_MAX) return cudaErrorInvalidValue;
    estimator_kernel<<<kEstBlocks, 256, 0, st>>>(est, n, pn, nest, vb, vb2, wb, comp, part, ticket, steps);
    return cudaGetLastError();
}

cudaError_t launch_branch(const DevStack& in, const DevStack& out, int n, int n3, int cap, double factor, int* counts,
                          int* offs, unsigned long long* irn1, unsigned long long* wtisto, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const BranchDev none{nullptr, nullptr, nullptr, nullptr, nullptr};
    branch_count_kernel<<<(n + 255) / 256, 256, 0, st>>>(in, n, factor, counts, irn1, wtisto, none, cap);
    scan_kernel<<<1, 1024, 0, st>>>(counts, n, offs, cap, none);
    const int warps = n;
    branch_scatter_kernel<<<(warps * 32 + 255) / 256, 256, 0, st>>>(in, out, n, n3, cap, counts, offs, irn1, none);
    return cudaGetLastError();
}

cudaError_t launch_branch_dev(const DevStack& in, const DevStack& out, const int* pn, int* pn_out, const int* need,
                              const double* dfactor, int* flags, int n3, int cap, int nsm, int* counts, int* offs,
                              unsigned long long* irn1, unsigned long long* wtisto, cudaStream_t st)
{
    const BranchDev bd{pn, pn_out, need, dfactor, flags};
    branch_count_kernel<<<nsm * 4, 256, 0, st>>>(in, 0, 1.0, counts, irn1, wtisto, bd, cap);
    scan_kernel<<<1, 1024, 0, st>>>(counts, 0, offs, cap, bd);
    branch_scatter_kernel<<<nsm * 16, 256, 0, st>>>(in, out, 0, n3, cap, counts, offs, irn1, bd);
    if (need) stack_copy_kernel<<<nsm * 16, 256, 0, st>>>(out, in, pn_out, need, n3);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Whole walker stacks to and from the caller's host arrays in one launch each
// (dmc_put_walkers / dmc_get_walkers), reading and writing mapped host memory
// directly; the reference's single-precision wt0 (stack.f90:12) is converted
// here.  put also leaves the walker count in the device count slot.
// ---------------------------------------------------------------------------
__global__ void walkers_put_kernel(HostWalkers h, DevStack d, int n, int n3, int* pn)
{
    const size_t t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x, nt = (size_t)gridDim.x * blockDim.x;
    const size_t nb = (size_t)n * n3;
    for (size_t e = t0; e < nb; e += nt) {
        d.x[e] = h.x[e];
        d.dpsi[e] = h.dpsi[e];
        d.dpsig[e] = h.dpsig[e];
    }
    for (size_t k = t0; k < (size_t)n; k += nt) {
        d.psil[k] = h.psil[k];
        d.psigl[k] = h.psigl[k];
        d.d2psi[k] = h.d2psi[k];
        d.d2psig[k] = h.d2psig[k];
        d.v[k] = h.v[k];
        d.vext[k] = h.vext[k];
        d.weight[k] = h.weight[k];
        d.psil0[k] = h.psil0[k];
        d.psigl0[k] = h.psigl0[k];
        d.wt0[k] = (float)h.wt0[k];
        d.is[k] = h.is[k];
        d.irn[k] = (unsigned long long)h.irn[k];
    }
    if (t0 == 0 && pn) *pn = n;
}

// absent (null) host fields are skipped; with pn the count is read on the
// device and at most cap walkers are written
__global__ void walkers_get_kernel(DevStack d, HostWalkers h, int n, const int* pn, int cap, int n3)
{
    if (pn) n = min(*pn, cap);
    const size_t t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x, nt = (size_t)gridDim.x * blockDim.x;
    const size_t nb = (size_t)n * n3;
    for (size_t e = t0; e < nb; e += nt) {
        if (h.x) h.x[e] = d.x[e];
        if (h.dpsi) h.dpsi[e] = d.dpsi[e];
        if (h.dpsig) h.dpsig[e] = d.dpsig[e];
    }
    for (size_t k = t0; k < (size_t)n; k += nt) {
        if (h.psil) h.psil[k] = d.psil[k];
        if (h.psigl) h.psigl[k] = d.psigl[k];
        if (h.d2psi) h.d2psi[k] = d.d2psi[k];
        if (h.d2psig) h.d2psig[k] = d.d2psig[k];
        if (h.v) h.v[k] = d.v[k];
        if (h.vext) h.vext[k] = d.vext[k];
        if (h.weight) h.weight[k] = d.weight[k];
        if (h.psil0) h.psil0[k] = d.psil0[k];
        if (h.psigl0) h.psigl0[k] = d.psigl0[k];
        if (h.wt0) h.wt0[k] = (double)d.wt0[k];
        if (h.is) h.is[k] = d.is[k];
        if (h.irn) h.irn[k] = (long long)d.irn[k];
    }
}

cudaError_t launch_walkers_put(const HostWalkers& h, const DevStack& d, int n, int n3, int* pn, int grid,
                               cudaStream_t st)
{
    walkers_put_kernel<<<grid, 256, 0, st>>>(h, d, n, n3, pn);
    return cudaGetLastError();
}

cudaError_t launch_walkers_get(const DevStack& d, const HostWalkers& h, int n, int n3, int grid, cudaStream_t st,
                               const int* pn, int cap)
{
    if (!pn && n <= 0) return cudaSuccess;
    walkers_get_kernel<<<grid, 256, 0, st>>>(d, h, n, pn, cap, n3);
    return cudaGetLastError();
}

cudaError_t launch_popctl(const int* pn, double nwalk, double popup, double popdn, int* need, double* factor,
                          int* flags, cudaStream_t st)
{
    popctl_kernel<<<1, 1, 0, st>>>(pn, nwalk, popup, popdn, need, factor, flags);
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
    Ctx<double> ctx{p, dummy, L, sm, nullptr};
    double logdet;
    int sg;
    const bool ok = walker::inverse_stage<double>(ctx, logdet, sg);
    for (int t = threadIdx.x; t < n * n; t += kThreads) {
        const int r = t % n, cc = t / n;
        inv[b * n2 + t] = sm[L.S + r * p.ldS + cc];
    }
    if (threadIdx.x == 0) {
        detl[b] = ok ? logdet : DMC_MINUSHUGE;
        is[b] = ok ? sg : 1;
    }
}

// doubles of one n x n matrix with the pivot column and reduction scratch of
// the batched inverse (the second buffer of the blocked form comes on top)
static int matinv_doubles(int n)
{
    const int ld = n | 1;
    return round_up(n * ld, 2) + round_up(2 * n + 2, 2) + kThreads * 8;
}

int matinv_fits(int n, bool* two_buffers)
{
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
        return -1;
    const size_t one = (size_t)matinv_doubles(n) * 8 + 1024;
    if (two_buffers) *two_buffers = one + (size_t)round_up(n * (n | 1), 2) * 8 <= (size_t)optin;
    return one <= (size_t)optin ? 1 : 0;
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
    L.red = L.colk + round_up(2 * n + 2, 2);
    L.total = L.red + kThreads * 8;
    // second buffer of the blocked inverse, when both copies fit on chip
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    L.S2 = -1;
    if ((size_t)(L.total + round_up(n * p.ldS, 2)) * 8 + 1024 <= (size_t)optin) {
        L.S2 = L.total;
        L.total += round_up(n * p.ldS, 2);
    }
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

// ---------------------------------------------------------------------------
// Peak probes: 8 independent FMA chains per thread, enough warps per SM to
// cover the pipe latency; the result is stored so nothing is optimised away.
// ---------------------------------------------------------------------------
template <class T>
__global__ void fma_probe_kernel(T* out, int iters, T a, T b)
{
    T v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = (T)(threadIdx.x + k) * (T)1e-3;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = fma(v[k], a, b);
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += v[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void dfmath_eval_kernel(int fn, int n, const void* in, double* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    df s, c;
    if (fn == 0) {
        dfm::sincospi_df(from_double(static_cast<const double*>(in)[i]), s, c);
    } else if (fn == 1) {
        dfm::sincos2pi_u48(static_cast<const unsigned long long*>(in)[i], s, c);
    } else {
        out[i] = to_double(dfm::log_df(from_double(static_cast<const double*>(in)[i])));
        return;
    }
    out[2 * i] = to_double(s);
    out[2 * i + 1] = to_double(c);
}

cudaError_t launch_dfmath_eval(int fn, int n, const void* in, double* out, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    dfmath_eval_kernel<<<(n + 127) / 128, 128, 0, st>>>(fn, n, in, out);
    return cudaGetLastError();
}

cudaError_t probe_fma_peak(int kind, int nsm, double* tflops)
{
    const int threads = 256, blocks = nsm * 8;
    const int iters = kind == 0 ? 256 : 8192;
    void* out = nullptr;
    cudaError_t e = cudaMalloc(&out, (size_t)blocks * threads * 8);
    if (e != cudaSuccess) return e;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        if (kind == 0)
            fma_probe_kernel<double><<<blocks, threads>>>((double*)out, iters, 0.999999, 1e-7);
        else
            fma_probe_kernel<float><<<blocks, threads>>>((float*)out, iters, 0.999999f, 1e-7f);
        cudaEventRecord(e1);
        e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
    *tflops = flops / (best * 1e-3) / 1e12;
    return e;
}

}  // namespace dmc
