// The walker kernel of the GB300 DMCBS path (sm_103a): one DMC/VMC move plus
// the full wavefunction and local energy of a walker per CTA, persistent
// CTAs, and the scalar step decision (step.f90:59-279).  Included by
// dmc_kernels.cu (the kernels of every idmc but 10), dmc_walker_gf.cu
// (GF = true: idmc = 10, two wavefunction evaluations per move, so that the
// second evaluation costs the other kernels no registers) and
// dmc_walker_big.cu (BIG = true: the union region of the layout in the CTA's
// global scratch slice, for systems whose orbitals do not fit on chip).
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "dmc_device.cuh"
#include "dmc_walker.cuh"

namespace dmc {

using walker::block_sum;
using walker::Ctx;
using walker::HRes;
using walker::lcg_jump;
using walker::lcg_uniform;
using walker::min_image;
using walker::warp_sum;

// Scalar part of one DMC/VMC move (step.f90:76-226): the estimator record
// est[nest][2] of the pushed walker, its new weight and sign weight.  nn and
// ol are the proposed and the old walker; take_new is the Metropolis
// decision (always true for idmc = 1, -2, 10); ejfd = sum |dpsi|^2/m of the
// pushed walker (idmc = -1, 0) or the summed weight wt1 + wt2 of the two
// proposals (idmc = 10).
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
                                        isfinite(-hb * nn.d2psig + nn.v) && (p.idmc != 10 || isfinite(ejfd)));
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
    } else if (p.idmc == 10) {
        // step.f90:248-271; ejfd carries wt1 + wt2 of the two proposals.
        // Estimator 6 takes ego, egn as the old and the chosen walker's guide
        // local energies (the reference leaves them unset on this path).
        const double ego = -hb * ol.d2psig + ol.v;
        const double egn = -hb * nn.d2psig + nn.v;
        double wt = ejfd;
        if (nn.is != ol.is) {
            if (p.fn) wt = 0.0;
            add(5, 1.0, 1.0);
        } else {
            add(5, 0.0, 1.0);
        }
        wt = 0.5 * wt * exp(p.etrial * p.dt);
        wnew = wt;
        const double wtg = wt * gratio(nn.psil, nn.psigl) * nn.is * (double)o_wt0;
        if (opcomp) {
            add(1, en * nfac, wtg);
            add(2, (en - nn.v) * nfac, wtg);
            add(3, nn.v * nfac, wtg);
            add(4, nn.vext * nfac, wtg);
            add(6, 0.5 * (ego + egn) * nfac, 1.0);
        }
        add(7, gratio(nn.psil, nn.psigl), 1.0);
        add(8, nn.is * exp(nn.psil), 1.0);
        add(9, exp(nn.psigl), 1.0);
        add(10, 1.0 * nn.is, 1.0);
        add(11, wt, 1.0);
        add(12, wtg, 1.0);
        add(13, copysign(1.0, wtg), 1.0);
        add(14, copysign(1.0, wtg), wtg);
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
template <class R, int NT, bool GF, bool BIG = false>
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
    // the CTA's global scratch slice: the union region (BIG), then the beta
    // pair data when they are not on chip.  The on-chip instances compute
    // their pointer in the original form: the general one cost the mixed
    // kernel 1 % (measured), from code generation alone.
    double* gs = nullptr;
    double* pb;
    if constexpr (BIG) {
        gs = a.gscratch + (size_t)blockIdx.x * L.gstride;
        pb = gs + round_up(L.rsize, 2);
    } else {
        pb = L.pb_in_smem ? sm + L.pb : a.gscratch + (size_t)blockIdx.x * L.pb_size;
    }
    Ctx<R, NT, BIG> c{p, a, L, sm, pb, gs};
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
            s0 = a.in.irn[src] & walker::kMask48;
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
            if (GF && p.idmc == 10) {
                // step.f90:232-238: x + sigma g, no drift and no wrap
                for (int e = threadIdx.x; e < n3; e += NT) {
                    const double dxe = p.sigma[(e / 3) < p.nup ? 0 : 1] * dxs[e];
                    dxs[e] = dxe;
                    x[e] = xo[e] + dxe;
                }
            } else {
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
            }
        } else {
            for (int e = threadIdx.x; e < n3; e += NT) x[e] = a.xin[(size_t)w * n3 + e];
        }
        __syncthreads();
        double* dpsi = sm + L.acc;
        const double* dpsig = (p.a2 == 0.0) ? dpsi : sm + L.dg;
        // failure flags of this walker (DMC_STATUS_*): a singular pair matrix
        // (matrixlapack.f90:19-25, psislaterbcs.f90:210) and results that are
        // not finite (NaN or infinite positions, overflowing terms).  Ends
        // with a barrier, after which the evaluation's shared data may change.
        auto flag_walker = [&](const HRes& hh) {
            int bad = 0;
            for (int e = threadIdx.x; e < n3; e += NT) {
                const double val = a.mode == MODE_GETPHI ? sm[L.acc + 4 * P + e] : dpsi[e];
                if (!isfinite(val)) bad = 1;
            }
            bad = __syncthreads_or(bad);
            const double lap = a.mode == MODE_GETPHI ? hh.d2u : (a.mode == MODE_BCS ? hh.d2phi : hh.d2psi);
            const double lg = a.mode == MODE_GETPHI ? hh.u : hh.psil;
            if (!isfinite(lap) || !isfinite(lg) || !isfinite(hh.v)) bad = 1;
            const int flags = (hh.singular ? DMC_STATUS_SINGULAR : 0) | (bad ? DMC_STATUS_NONFINITE : 0);
            if (threadIdx.x == 0) {
                if (flags && a.status) atomicOr(a.status, flags);
                if (a.wstatus && a.mode != MODE_STEP) a.wstatus[w] = flags;
            }
        };
        // idmc = 10 (step.f90:237-250) evaluates two proposals: after the
        // first (x + dx) its vectors go to the output stack and its scalars
        // to shared memory (thread 0 holds the results), then x - dx is
        // evaluated by the same code (one copy of hpsi_eval in the kernel).
        const bool gf = GF && a.mode == MODE_STEP && p.idmc == 10;
        __shared__ double s_first[7];
        const int kout = w;   // push order = pop order
        HRes h;
        for (int pass = 0;; ++pass) {
            h = walker::hpsi_eval<R>(c, a.mode);
            flag_walker(h);
            if (!gf || pass == 1) break;
            for (int e = threadIdx.x; e < n3; e += NT) {
                a.out.x[(size_t)kout * n3 + e] = x[e];
                a.out.dpsi[(size_t)kout * n3 + e] = dpsi[e];
                a.out.dpsig[(size_t)kout * n3 + e] = dpsig[e];
                x[e] = xo[e] - dxs[e];
            }
            if (threadIdx.x == 0) {
                s_first[0] = h.psil;
                s_first[1] = h.psigl;
                s_first[2] = h.d2psi;
                s_first[3] = h.d2psig;
                s_first[4] = h.v;
                s_first[5] = h.vext;
                s_first[6] = (double)h.is;
            }
            __syncthreads();
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
            if (a.o_dphi && a.mode == MODE_HPSI)
                for (int e = threadIdx.x; e < n3; e += NT) a.o_dphi[(size_t)w * n3 + e] = sm[L.acc + 4 * P + e];
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
        __shared__ int s_pick_first;
        double gf_wsum = 0.0;
        if (gf) {
            // step.f90:243-247: weights exp(-v dt) Psi_G'/Psi_G of the two
            // proposals; the first is kept with its share of the sum, or
            // whenever the second crossed a node
            if (threadIdx.x == 0) {
                const double wt1 = exp(-s_first[4] * p.dt) * exp(s_first[1] - o_psigl);
                const double wt2 = exp(-h.v * p.dt) * exp(h.psigl - o_psigl);
                gf_wsum = wt1 + wt2;
                const double rn = lcg_uniform(lcg_jump(s0, a.jumpA, a.jumpC, nr + 1));
                s_pick_first = (rn < wt1 / gf_wsum || h.is != o_is) ? 1 : 0;
            }
            irn_out = lcg_jump(s0, a.jumpA, a.jumpC, nr + 1);
            __syncthreads();
        }
        const bool first = gf && s_pick_first != 0;
        if (first && threadIdx.x == 0) {
            h.psil = s_first[0];
            h.psigl = s_first[1];
            h.d2psi = s_first[2];
            h.d2psig = s_first[3];
            h.v = s_first[4];
            h.vext = s_first[5];
            h.is = (int)s_first[6];
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
        const int k = kout;
        if (threadIdx.x == 0) {
            const StepScalars nn{h.psil, h.psigl, h.d2psi, h.d2psig, h.v, h.vext, h.is};
            const StepScalars ol{o_psil, o_psigl, o_d2psi, o_d2psig, o_v, o_vext, o_is};
            double wnew = o_weight;
            float wt0new = o_wt0;
            // idmc = 1, -2: weights and estimators in step_decide_kernel, one
            // thread per walker after this kernel
            if (!a.defer)
                step_decision(p, a.opcomp, nn, ol, o_weight, o_wt0, take_new, gf ? gf_wsum : ejfd[0], est, wnew,
                              wt0new);
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
        if (first) {
            // the first proposal's vectors are already in the output stack
        } else if (take_new) {
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

}   // namespace dmc
