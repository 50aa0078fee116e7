// Kernels of the GB300 DMCBS walker path (sm_103a): the walker kernel (one
// DMC move plus the full wavefunction and local energy of a walker per CTA),
// in plain FP64 and in the mixed double-float / FP32 form, and the
// population kernels (estimator sums, branching, stack reversal, batched
// inverse).  The walker stages are in dmc_walker.cuh.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include "dmc_device.cuh"
#include "dmc_kernels.h"
#include "dmc_attr.h"
#include "dmc_walker.cuh"

namespace dmc {

using walker::block_sum;
using walker::Ctx;
using walker::HRes;
using walker::lcg_jump;
using walker::lcg_uniform;
using walker::min_image;
using walker::warp_sum;

constexpr unsigned long long kMask48 = walker::kMask48;

// Scalar part of one DMC/VMC move (step.f90:76-226): the estimator record
// est[nest][2] of the pushed walker, its new weight and sign weight.  nn and
// ol are the proposed and the old walker; take_new is the Metropolis
// decision (always true for idmc = 1, -2); ejfd = sum |dpsi|^2/m of the
// pushed walker (idmc = -1, 0).
struct StepScalars {
    double psil, psigl, d2psi, d2psig, v, vext;
    int is;
};
__device__ inline void step_decision(const DevParams& p, int opcomp, const StepScalars& nn, const StepScalars& ol,
                                     double o_weight, float o_wt0, bool take_new, double ejfd, double* est,
                                     double& wnew_out, float& wt0_out)
{
    const double hb = p.hbar;
    // psi/psi_G: exactly 1 when the guide function is psi itself (a2 = 0)
    auto gratio = [](double l, double lg) { return l == lg ? 1.0 : exp(l - lg); };
    const double eo = -hb * ol.d2psi + ol.v;     // old and new local energies
    const double en = -hb * nn.d2psi + nn.v;
    for (int q = 0; q < 2 * p.nest; ++q) est[q] = 0.0;
    auto add = [&](int i1, double val, double wt) {
        est[2 * (i1 - 1)] = val;
        est[2 * (i1 - 1) + 1] = wt;
    };
    const double nfac = p.nfac;
    double wnew = o_weight;
    float wt0new = o_wt0;
    // A DMC walker whose local energies are not finite (NaN or infinite
    // inputs, flagged DMC_STATUS_NONFINITE by the walker kernel) gets weight 0
    // and adds nothing to the estimators, so branching drops it; the
    // reference has no such case (its int(w + u) of a NaN weight is
    // undefined).  Finite walkers are untouched.
    if (p.idmc >= 1 || p.idmc == -2) {
        const bool fin = p.idmc == 2 ? (isfinite(eo) && (!take_new || isfinite(en)))
                                     : (isfinite(eo) && isfinite(en) && isfinite(-hb * ol.d2psig + ol.v) &&
                                        isfinite(-hb * nn.d2psig + nn.v));
        if (!fin) {
            wnew_out = 0.0;
            wt0_out = o_wt0;
            return;
        }
    }
    if (p.idmc == -1 || p.idmc == 0) {
        if (take_new) {
            const double ejf = -0.5 * hb * (nn.d2psi - ejfd) + nn.v;
            add(1, en * nfac, o_weight);
            add(2, (en - nn.v) * nfac, o_weight);
            add(3, nn.v * nfac, o_weight);
            add(4, nn.vext * nfac, o_weight);
            add(5, ejf * nfac, o_weight);
            add(6, 1.0, 1.0);
            wt0new = (float)nn.is;
        } else {
            const double ejf = -0.5 * hb * (ol.d2psi - ejfd) + ol.v;
            add(1, eo * nfac, o_weight);
            add(2, (eo - ol.v) * nfac, o_weight);
            add(3, ol.v * nfac, o_weight);
            add(4, ol.vext * nfac, o_weight);
            add(5, ejf * nfac, o_weight);
            add(6, 0.0, 1.0);
        }
    } else if (p.idmc == 1 || p.idmc == -2) {
        const double ego = -hb * ol.d2psig + ol.v;
        const double egn = -hb * nn.d2psig + nn.v;
        double wt = exp(-(0.5 * (ego + egn) - p.etrial) * p.dt);
        wnew = fmin(p.wtcut, wt);
        if (nn.is != ol.is) {
            if (p.fn) {
                wnew = 0.0;
                wt = 0.0;
            }
            add(5, 1.0, 1.0);
        } else {
            add(5, 0.0, 1.0);
        }
        const double wtg = wt * gratio(nn.psil, nn.psigl) * nn.is * (double)o_wt0;
        if (opcomp) {
            add(1, en * nfac, wtg);
            add(2, (en - nn.v) * nfac, wtg);
            add(3, nn.v * nfac, wtg);
            add(4, nn.vext * nfac, wtg);
            add(6, 0.5 * (ego + egn) * nfac, 1.0);
            add(7, gratio(nn.psil, nn.psigl), 1.0);
            add(8, nn.is * exp(nn.psil), 1.0);
            add(9, exp(nn.psigl), 1.0);
            add(10, 1.0 * nn.is, 1.0);
            add(11, wt, 1.0);
            add(12, wtg, 1.0);
            add(13, copysign(1.0, wtg), 1.0);
            add(14, copysign(1.0, wtg), wtg);
        }
    } else {   // idmc == 2
        if (take_new) {
            double wt = exp(-(0.5 * (eo + en) - p.etrial) * p.dt);
            wnew = fmin(p.wtcut, wt);
            if (nn.is != ol.is) {
                if (p.fn) {
                    wnew = 0.0;
                    wt = 0.0;
                }
                add(4, 1.0, 1.0);
            } else {
                add(4, 0.0, 1.0);
            }
            const double wtg = wt * gratio(nn.psil, nn.psigl) * nn.is * (double)o_wt0;
            if (opcomp) {
                add(1, en * nfac, wtg);
                add(2, (en - nn.v) * nfac, wtg);
                add(3, nn.v * nfac, wtg);
                add(6, gratio(nn.psil, nn.psigl), 1.0);
                add(7, nn.is * exp(nn.psil), 1.0);
                add(8, exp(nn.psigl), 1.0);
                add(9, 1.0 * nn.is, 1.0);
                add(10, wt, 1.0);
                add(11, wtg, 1.0);
                add(12, copysign(1.0, wtg), 1.0);
                add(13, copysign(1.0, wtg), wtg);
            }
            add(5, 1.0, 1.0);
        } else {
            const double wt = exp(-(eo - p.etrial) * p.dt);
            const double wtg = wt * gratio(ol.psil, ol.psigl) * ol.is * (double)o_wt0;
            wnew = fmin(p.wtcut, wt * o_weight);
            if (opcomp) {
                add(1, eo * nfac, wtg);
                add(2, (eo - ol.v) * nfac, wtg);
                add(3, ol.v * nfac, wtg);
                add(6, gratio(ol.psil, ol.psigl), 1.0);
                add(7, ol.is * exp(ol.psil), 1.0);
                add(8, exp(ol.psigl), 1.0);
                add(9, 1.0 * ol.is, 1.0);
                add(10, wt, 1.0);
                add(11, wtg, 1.0);
                add(12, copysign(1.0, wtg), 1.0);
                add(13, copysign(1.0, wtg), wtg);
            }
            add(5, 0.0, 1.0);
        }
    }
    wnew_out = wnew;
    wt0_out = wt0new;
}

// ---------------------------------------------------------------------------
// The walker kernel: persistent CTAs, one walker per CTA per iteration.
// ---------------------------------------------------------------------------
template <class R, int NT>
__global__ void __launch_bounds__(NT, NT == kThreads ? 2 : 1)
walker_kernel(const __grid_constant__ DevParams p, const __grid_constant__ KernelArgs a, SmemLayout L)
{
    extern __shared__ __align__(16) double sm[];
    const int P = p.npart, n3 = 3 * P;
    const double* kvsrc = reinterpret_cast<const double*>(walker::Prec<R>::kv(a));
    for (int i = threadIdx.x; i < p.nk * 8; i += NT) sm[L.kq + i] = kvsrc[i];
    {
        using KV = typename walker::Prec<R>::KV;
        const KV* kg = walker::Prec<R>::kv(a);
        R* ks = walker::at<R>(sm, L.ksoa);
        for (int q = threadIdx.x; q < p.nk; q += NT) {
            ks[q] = kg[q].k[0];
            ks[p.nk + q] = kg[q].k[1];
            ks[2 * p.nk + q] = kg[q].k[2];
            ks[3 * p.nk + q] = kg[q].k2;
            ks[4 * p.nk + q] = kg[q].v;
            int* kn = reinterpret_cast<int*>(ks + 5 * p.nk);
            for (int cc = 0; cc < 3; ++cc) kn[cc * p.nk + q] = kg[q].n[cc];
        }
    }
    double* pb = L.pb_in_smem ? sm + L.pb : a.gscratch + (size_t)blockIdx.x * L.pb_size;
    Ctx<R, NT> c{p, a, L, sm, pb};
    __shared__ double s_old[9];
    __syncthreads();
    const int nw = a.pn ? *a.pn : a.nw;   // the population is counted on the device in a generation
    for (int w = blockIdx.x; w < nw; w += gridDim.x) {
        double* x = sm + L.x;
        double* xo = sm + L.xo;
        double* dxs = sm + L.dx;
        double* drift = sm + L.drift;
        const int src = nw - 1 - w;   // MODE_STEP pops from the top
        unsigned long long s0 = 0;
        if (a.mode == MODE_STEP) {
            // step.f90:59-74: wrap, gaussians, drift, proposal
            s0 = a.in.irn[src] & kMask48;
            if (threadIdx.x >= NT - 32 && threadIdx.x < NT - 32 + 9) {
                // the popped walker's scalars for the step decision (latency hidden behind the proposal)
                const int k = threadIdx.x - (NT - 32);
                double v;
                switch (k) {
                    case 0: v = a.in.psil[src]; break;
                    case 1: v = a.in.psigl[src]; break;
                    case 2: v = a.in.d2psi[src]; break;
                    case 3: v = a.in.d2psig[src]; break;
                    case 4: v = a.in.v[src]; break;
                    case 5: v = a.in.vext[src]; break;
                    case 6: v = a.in.weight[src]; break;
                    case 7: v = a.in_wt0d ? (double)(float)a.in_wt0d[src] : (double)a.in.wt0[src]; break;
                    default: v = (double)a.in.is[src]; break;
                }
                s_old[k] = v;
            }
            const double* x1 = a.in.x + (size_t)src * n3;
            const double* g1 = a.in.dpsig + (size_t)src * n3;
            for (int e = threadIdx.x; e < n3; e += NT) xo[e] = min_image(x1[e], p);
            // Box-Muller pairs (ran.f90:74-104): draws t = 1..nrand from the
            // walker's stream, pair i uses draws 2i-1, 2i
            const int npairs = (n3 + 1) / 2;
            for (int q = threadIdx.x; q < npairs; q += NT) {
                double gs, gc;   // r sin(2 pi u1), r cos(2 pi u1), r = sqrt(-2 log u2)
                if constexpr (walker::is_df<R>::value) {
                    // the same deviates in double-float on the FP32 pipe:
                    // u = (state | 1) 2^-48 is exact there
                    const unsigned long long m1 = lcg_jump(s0, a.jumpA, a.jumpC, 2 * q + 1) | 1ull;
                    const unsigned long long m2 = lcg_jump(s0, a.jumpA, a.jumpC, 2 * q + 2) | 1ull;
                    df sn, cs;
                    dfm::sincos2pi_u48(m1, sn, cs);
                    const df lg = dfm::log_df(dfm::u48(m2));
                    const df r = dsqrt(df{-2.0f * lg.hi, -2.0f * lg.lo});
                    gs = to_double(sn * r);
                    gc = to_double(cs * r);
                } else {
                    const double u1 = lcg_uniform(lcg_jump(s0, a.jumpA, a.jumpC, 2 * q + 1));
                    const double u2 = lcg_uniform(lcg_jump(s0, a.jumpA, a.jumpC, 2 * q + 2));
                    double sn, cs;
                    sincospi(2.0 * u1, &sn, &cs);
                    const double r = sqrt(-2.0 * log(u2));
                    gs = sn * r;
                    gc = cs * r;
                }
                if (2 * q + 1 < n3) {
                    dxs[2 * q] = gs;
                    dxs[2 * q + 1] = gc;
                } else {
                    dxs[2 * q] = gc;   // odd count: the last one uses cos (ran.f90:95-102)
                }
            }
            __syncthreads();
            for (int e = threadIdx.x; e < n3; e += NT) {
                const int sp = (e / 3) < p.nup ? 0 : 1;
                const double sig = p.sigma[sp];
                double d = g1[e] * (sig * sig) * p.sqm[sp];
                if (p.cutdrift) d = fmin(p.dcut[sp], fmax(-p.dcut[sp], d));
                drift[e] = d;
                const double dxe = d + sig * dxs[e];
                dxs[e] = dxe;
                x[e] = min_image(xo[e] + dxe, p);
            }
        } else {
            for (int e = threadIdx.x; e < n3; e += NT) x[e] = a.xin[(size_t)w * n3 + e];
        }
        __syncthreads();
        const int hmode = a.mode == MODE_STEP ? MODE_HPSI : a.mode;
        HRes h = walker::hpsi_eval<R>(c, a.mode == MODE_STEP ? MODE_STEP : hmode);
        double* dpsi = sm + L.acc;
        const double* dpsig = (p.a2 == 0.0) ? dpsi : sm + L.dg;
        // failure flags of this walker (DMC_STATUS_*): a singular pair matrix
        // (matrixlapack.f90:19-25, psislaterbcs.f90:210) and results that are
        // not finite (NaN or infinite positions, overflowing terms)
        {
            int bad = 0;
            for (int e = threadIdx.x; e < n3; e += NT) {
                const double val = a.mode == MODE_GETPHI ? sm[L.acc + 4 * P + e] : dpsi[e];
                if (!isfinite(val)) bad = 1;
            }
            bad = __syncthreads_or(bad);
            const double lap = a.mode == MODE_GETPHI ? h.d2u : (a.mode == MODE_BCS ? h.d2phi : h.d2psi);
            const double lg = a.mode == MODE_GETPHI ? h.u : h.psil;
            if (!isfinite(lap) || !isfinite(lg) || !isfinite(h.v)) bad = 1;
            const int flags = (h.singular ? DMC_STATUS_SINGULAR : 0) | (bad ? DMC_STATUS_NONFINITE : 0);
            if (threadIdx.x == 0) {
                if (flags && a.status) atomicOr(a.status, flags);
                if (a.wstatus && a.mode != MODE_STEP) a.wstatus[w] = flags;
            }
        }
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
                for (int e = threadIdx.x; e < n3; e += NT) {
                    double val = dpsi[e];
                    if (a.mode == MODE_GETPHI) val = sm[L.acc + 4 * P + e];
                    a.o_dpsi[(size_t)w * n3 + e] = val;
                }
            if (a.o_dpsig)
                for (int e = threadIdx.x; e < n3; e += NT) a.o_dpsig[(size_t)w * n3 + e] = dpsig[e];
            if (a.o_sinv) {
                const int nd = p.nd;
                // column-major nd x nd as the reference's smati(nd,nd)
                for (int t = threadIdx.x; t < nd * nd; t += NT) {
                    const int r = t % nd, cc = t / nd;
                    a.o_sinv[(size_t)w * nd * nd + t] =
                        h.singular ? 0.0 : to_double(walker::at<R>(sm, L.S)[r * p.ldS + cc]);
                }
            }
            __syncthreads();
            continue;
        }
        // ---- step1 decision (step.f90:76-226) ----
        __shared__ int s_take_new;
        // the popped walker's scalars, fetched into shared memory before hpsi
        const double o_psil = s_old[0], o_psigl = s_old[1], o_d2psi = s_old[2];
        const double o_d2psig = s_old[3], o_v = s_old[4], o_vext = s_old[5];
        const double o_weight = s_old[6];
        const float o_wt0 = (float)s_old[7];
        const int o_is = (int)s_old[8];
        const int nr = p.nrand;
        unsigned long long irn_out = lcg_jump(s0, a.jumpA, a.jumpC, nr);
        double* est = a.est + (size_t)w * p.nest * 2;
        const bool metro = (p.idmc == -1 || p.idmc == 0 || p.idmc == 2);
        if (metro) {
            // Metropolis with the drift Green's function ratio (step.f90:80-91)
            double acc1[2] = {0.0, 0.0};
            for (int e = threadIdx.x; e < n3; e += NT) {
                const int sp = (e / 3) < p.nup ? 0 : 1;
                const double sig = p.sigma[sp];
                double dn = dpsig[e] * (sig * sig) * p.sqm[sp];
                if (p.cutdrift) dn = fmin(p.dcut[sp], fmax(-p.dcut[sp], dn));
                const double d1 = drift[e] + dn;
                const double d2 = drift[e] - dn - 2.0 * dxs[e];
                acc1[0] += d1 * d2 / (2.0 * (sig * sig));
            }
            block_sum<2, NT>(acc1, sm + L.red);
            if (threadIdx.x == 0) {
                double prob = (p.idmc == 2 ? 2.0 * (h.psigl - o_psigl) : 2.0 * (h.psil - o_psil)) + acc1[0];
                prob = prob == prob ? exp(fmin(0.0, prob)) : 0.0;   // a NaN proposal is rejected
                const double rn = lcg_uniform(lcg_jump(s0, a.jumpA, a.jumpC, nr + 1));
                s_take_new = rn < prob;
            }
            irn_out = lcg_jump(s0, a.jumpA, a.jumpC, nr + 1);
            __syncthreads();
        }
        const bool take_new = metro ? s_take_new != 0 : true;
        // sum |dpsi|^2/m of the pushed walker for the Jackson-Feenberg energy
        double ejfd[1] = {0.0};
        if (p.idmc == -1 || p.idmc == 0) {
            const double* dsrc = take_new ? dpsi : a.in.dpsi + (size_t)src * n3;
            for (int e = threadIdx.x; e < n3; e += NT) {
                const int sp = (e / 3) < p.nup ? 0 : 1;
                ejfd[0] += dsrc[e] * dsrc[e] * p.imass[sp];
            }
            block_sum<1, NT>(ejfd, sm + L.red);
        }
        // scalars of the pushed walker
        const int k = w;   // push order = pop order
        if (threadIdx.x == 0) {
            const StepScalars nn{h.psil, h.psigl, h.d2psi, h.d2psig, h.v, h.vext, h.is};
            const StepScalars ol{o_psil, o_psigl, o_d2psi, o_d2psig, o_v, o_vext, o_is};
            double wnew = o_weight;
            float wt0new = o_wt0;
            // idmc = 1, -2: weights and estimators in step_decide_kernel, one
            // thread per walker after this kernel
            if (!a.defer)
                step_decision(p, a.opcomp, nn, ol, o_weight, o_wt0, take_new, ejfd[0], est, wnew, wt0new);
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
            if (!a.defer) {
                o.weight[k] = wnew;
                o.wt0[k] = wt0new;
            }
            o.irn[k] = irn_out;
            o.psil0[k] = a.in.psil0[src];
            o.psigl0[k] = a.in.psigl0[src];
        }
        if (take_new) {
            for (int e = threadIdx.x; e < n3; e += NT) {
                a.out.x[(size_t)k * n3 + e] = x[e];
                a.out.dpsi[(size_t)k * n3 + e] = dpsi[e];
                a.out.dpsig[(size_t)k * n3 + e] = dpsig[e];
            }
        } else {
            for (int e = threadIdx.x; e < n3; e += NT) {
                a.out.x[(size_t)k * n3 + e] = xo[e];
                a.out.dpsi[(size_t)k * n3 + e] = a.in.dpsi[(size_t)src * n3 + e];
                a.out.dpsig[(size_t)k * n3 + e] = a.in.dpsig[(size_t)src * n3 + e];
            }
        }
        __syncthreads();
    }
}

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
__global__ void estimator_kernel(const double* est, int n, const int* pn, int nest, double* valblk, double* valblk2,
                                 double* wtblk, unsigned long long* steps)
{
    if (pn) n = *pn;
    const int e = blockIdx.x;
    if (steps && e == 0 && threadIdx.x == 0) *steps += (unsigned long long)n;   // walker-steps of the generation
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

// one warp per source walker; copy c (1-based) advanced by c ran2 steps
__global__ void branch_scatter_kernel(DevStack in, DevStack out, int n, int n3, int cap, const int* counts,
                                      const int* offs, const unsigned long long* irn1, BranchDev bd)
{
    const int lane = threadIdx.x & 31;
    if (bd.pn) {
        n = *bd.pn;
        if (bd.need && !*bd.need) return;   // no population control this generation
    }
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int m = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; m < n; m += nwarps) {
    const int j = n - 1 - m;

    const int cnt = counts[m];
    const int o0 = offs[m];
    unsigned long long s = irn1[m];
    const double wsign = copysign(1.0, in.weight[j]);
    for (int cp = 0; cp < cnt; ++cp) {
        s = (34522712143931ull * s + 55789347517ull) & kMask48;   // ran2 (ran.f90:29-48)
        const int d = o0 + cp;
        if (d >= cap) break;
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

int walker_smem_bytes(const DevParams& p, int limit_bytes, SmemLayout* Lout, int nt)
{
    SmemLayout L = make_layout(p, limit_bytes, nt);
    if (Lout) *Lout = L;
    return L.total * 8;
}

int walker_static_smem_bytes()
{
    cudaFuncAttributes a[3]{};
    if (cudaFuncGetAttributes(&a[0], walker_kernel<double, kThreads>) != cudaSuccess) return -1;
    if (cudaFuncGetAttributes(&a[1], walker_kernel<df, kThreads>) != cudaSuccess) return -1;
    if (cudaFuncGetAttributes(&a[2], walker_kernel<df, 2 * kThreads>) != cudaSuccess) return -1;
    size_t m = 0;
    for (const auto& x : a) m = x.sharedSizeBytes > m ? x.sharedSizeBytes : m;
    return (int)m;
}

// attribute kinds of the per-device record: the carveout, then the dynamic
// shared-memory opt-in of walker_kernel<df / double, 256 / 512 threads>
enum : int { kAttrCarveout = 0, kAttrSmemBase = 1 };
static AttrCache g_attr;

template <class R, int NT>
static int set_smem_attr(int v)
{
    return (int)cudaFuncSetAttribute(walker_kernel<R, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
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
        cudaError_t r = cudaFuncSetAttribute(walker_kernel<df, kThreads>, cudaFuncAttributePreferredSharedMemoryCarveout, c);
        if (r == cudaSuccess)
            r = cudaFuncSetAttribute(walker_kernel<double, kThreads>, cudaFuncAttributePreferredSharedMemoryCarveout, c);
        if (r == cudaSuccess)
            r = cudaFuncSetAttribute(walker_kernel<df, 2 * kThreads>, cudaFuncAttributePreferredSharedMemoryCarveout,
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

cudaError_t prepare_walker(const SmemLayout& L) { return walker_attrs(L.total * 8, L.nt, true, false); }

cudaError_t launch_walker(const DevParams& p, const KernelArgs& a, const SmemLayout& L, int grid, cudaStream_t st,
                          bool mixed)
{
    const size_t smem = (size_t)L.total * 8;
    // the shared-memory opt-in is recorded per device and size (prepare_walker
    // sets it before any graph capture; this finds it set)
    const cudaError_t e = walker_attrs((int)smem, L.nt, false, mixed);
    if (e != cudaSuccess) return e;
    if (!mixed)
        walker_kernel<double, kThreads><<<grid, kThreads, smem, st>>>(p, a, L);
    else if (L.nt == 2 * kThreads)
        walker_kernel<df, 2 * kThreads><<<grid, 2 * kThreads, smem, st>>>(p, a, L);
    else
        walker_kernel<df, kThreads><<<grid, kThreads, smem, st>>>(p, a, L);
    return cudaGetLastError();
}

cudaError_t launch_estimators(const double* est, int n, int nest, double* vb, double* vb2, double* wb, cudaStream_t st,
                              const int* pn, unsigned long long* steps)
{
    if (n <= 0 && !pn) return cudaSuccess;
    estimator_kernel<<<nest, 256, 0, st>>>(est, n, pn, nest, vb, vb2, wb, steps);
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
