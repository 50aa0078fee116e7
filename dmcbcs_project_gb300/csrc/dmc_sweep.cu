// Particle-by-particle Metropolis sweeps with Sherman-Morrison updates of the
// inverse pair matrix, in FP32 (sm_103a).
//
// No counterpart in the reference's walker loop, whose moves are
// all-particle (step.f90:43-285); the single-particle ratio it builds on is
// bcsone / getphione / move1 (psislaterbcs.f90:296-376, coshpot.f90:207-264,
// wavefunction.f90:393-404), which the reference uses only for n(k).
//
// One warp per walker.  Per move of particle i (in order 0..npart-1, every
// sweep):
//   - five draws of the walker's ran1 stream (ran.f90:8-27): three Gaussian
//     deviates (gaussian(3), ran.f90:74-104) and one uniform, and the
//     proposal x_i' = x_i + sigma_i g (sigma of setstep, step.f90:29-30)
//     wrapped into the box, all in FP64 for the whole sweep ahead of its
//     moves, one move per lane (particle i has not moved before its own move
//     of the sweep);
//   - distances in FP32;
//   - the new row (up particle) or column (down particle) s' of the pair
//     matrix: phi(r_i' - r_j) = v_0 + sum_q 2 vorb(shell q) cos(k_q.(r_i'-r_j))
//     + beta(|r_i' - r_j|), and the unpaired plane waves at r_i', from a
//     cos/sin table of every k vector at every particle;
//   - determinant ratio R = s'.X(:,i) (row) or X(c,:).s' (column) and the
//     Jastrow ratio exp(U' - U) from the pair tables;
//   - accept when u < R^2 exp(2 (U' - U)); on acceptance the inverse X is
//     updated by Sherman-Morrison (rank one, FP32) and the table column of
//     particle i is replaced.
// The inverse X enters in FP64 (a fresh inverse of the pair matrix from the
// FP64 walker kernel: the periodic full recompute) or as the FP32 inverse
// carried from the previous call; it leaves in FP32.
#include <cuda_runtime.h>
#include <math.h>

#include "dmc_device.cuh"
#include "dmc_kernels.h"
#include "dmc_walker.cuh"

namespace dmc {
namespace {

constexpr int kSweepWarps = 4;   // most walkers per CTA, one warp each

// floats of one warp's shared memory: FP32 positions for the distances (3
// npart), X (nd x ldx), the new entries s' and the v / w vector (nd each),
// the moved particle's orbitals (v-scaled and plain, 2 (nk-1) float2).  The
// FP64 positions stay in the walker stack and the sweep's proposals in a
// global slice per walker, so that a warp's share is small enough for all
// walkers of a 4096-walker population at N = 66 to be resident at once.
__host__ __device__ inline int sweep_warp_floats(const DevParams& p)
{
    const int ldx = p.nd | 1;
    const int nq = p.nk > 1 ? p.nk - 1 : 1;
    return 3 * p.npart + 2 + p.nd * ldx + 2 * p.nd + 8 * nq + 8;
}

// FP32 4-point Lagrange grid position (index clamp of coshpot.f90:174)
__device__ __forceinline__ walker::Lagrange<float> lag_f(float r, float scale, int ntab)
{
    const float t = r * scale;
    int idx = (int)t;
    idx = max(1, min(idx, ntab - 2));
    return walker::lagrange_f(t - (float)idx, idx);
}

// u(r) of an up-down (or, with ss, a same-spin) pair, FP32; zero beyond L/2
__device__ __forceinline__ float jas_u(const DevParams& p, const TabUDmp* tud, const TabSSmp* tss, bool opposite,
                                       float r)
{
    if (!(r < (float)p.range)) return 0.0f;
    const walker::Lagrange<float> W = lag_f(r, (float)p.scale, p.ntab);
    if (opposite) {
        const TabUDmp* T = tud + (W.idx - 1);
        return W.c1 * T[0].u.hi + W.c2 * T[1].u.hi + W.c3 * T[2].u.hi + W.c4 * T[3].u.hi;
    }
    const TabSSmp* T = tss + (W.idx - 1);
    return W.c1 * T[0].u + W.c2 * T[1].u + W.c3 * T[2].u + W.c4 * T[3].u;
}

// beta(r) (radialfun, betafun.f90:173-194), FP32
__device__ __forceinline__ float beta_f(const DevParams& p, const TabUDmp* tud, float r)
{
    if (p.nobeta || r > (float)p.rangeb) return 0.0f;
    const walker::Lagrange<float> W = lag_f(r, (float)p.scaleb, p.ntab);
    const TabUDmp* T = tud + (W.idx - 1);
    return W.c1 * T[0].b.hi + W.c2 * T[1].b.hi + W.c3 * T[2].b.hi + W.c4 * T[3].b.hi;
}

__device__ __forceinline__ float warp_sum_f(float v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double ran1_step(unsigned long long& s)
{
    s = (44485709377909ull * s + 96309754297ull) & walker::kMask48;
    return walker::lcg_uniform(s);
}

// FP32 minimum image
__device__ __forceinline__ float min_image_f(float d, float el, float eli) { return d - el * rintf(d * eli); }

__global__ void __launch_bounds__(32 * kSweepWarps) sweep_kernel(const __grid_constant__ DevParams p, DevStack st,
                                                                 int n, int nsweep, const double* __restrict__ inv64,
                                                                 float* __restrict__ inv32, float2* __restrict__ tab,
                                                                 const KVecMP* __restrict__ kv,
                                                                 const TabUDmp* __restrict__ tud,
                                                                 const TabSSmp* __restrict__ tss,
                                                                 const unsigned long long* __restrict__ jA,
                                                                 const unsigned long long* __restrict__ jC,
                                                                 unsigned long long* __restrict__ accepted, int wpc,
                                                                 double* __restrict__ prop)
{
    extern __shared__ __align__(16) double smw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int P = p.npart, nd = p.nd, ldx = nd | 1, nq = p.nk - 1, nup = p.nup;
    float* xsf = reinterpret_cast<float*>(smw + (size_t)wib * (sweep_warp_floats(p) / 2 + 1));
    float* X = xsf + 3 * P + (P & 1);                  // X(r, c) = X[r + c ldx]: column-major as smati
    float* snew = X + nd * ldx;
    float* vw = snew + nd;
    float2* onew = reinterpret_cast<float2*>(vw + nd + (((nd * ldx + 2 * nd) & 1) ? 1 : 0));   // v-scaled
    float2* oraw = onew + (nq > 0 ? nq : 1);                                                 // plain
    const float v0 = kv[0].v.hi;
    const float elf = (float)p.el, elif = (float)p.eli;
    const int w = blockIdx.x * wpc + wib;
    if (w >= n) return;   // whole warps only: the warp is the unit below
    double* xs = st.x + (size_t)w * 3 * P;     // FP64 positions, wrapped in place
    double* drw = prop + (size_t)w * 4 * P;    // [P][4]: the proposal x_i + sigma g and u of move i
    // ---- load the walker: positions (wrapped), inverse, cos/sin table ----
    for (int e = lane; e < 3 * P; e += 32) {
        const double xv = walker::min_image(xs[e], p);
        xs[e] = xv;
        xsf[e] = (float)xv;
    }
    if (inv64) {
        for (int e = lane; e < nd * nd; e += 32) {
            const int r = e % nd, c = e / nd;
            X[r + c * ldx] = (float)inv64[(size_t)w * nd * nd + e];
        }
    } else {
        for (int e = lane; e < nd * nd; e += 32) {
            const int r = e % nd, c = e / nd;
            X[r + c * ldx] = inv32[(size_t)w * nd * nd + e];
        }
    }
    float2* T = tab + (size_t)w * nq * P;   // T[q P + j] = (cos, sin)(k_{q+1} . x_j)
    __syncwarp();
    for (int e = lane; e < nq * P; e += 32) {
        const int q = e / P, j = e % P;
        const KVecMP& K = kv[q + 1];
        float sn, cs;
        sincosf(K.k[0].hi * (float)xs[3 * j] + K.k[1].hi * (float)xs[3 * j + 1] + K.k[2].hi * (float)xs[3 * j + 2],
                &sn, &cs);
        T[e] = make_float2(cs, sn);
    }
    unsigned long long s = st.irn[w] & walker::kMask48;
    unsigned long long nacc = 0;
    __syncwarp();
    for (int sw = 0; sw < nsweep; ++sw) {
        // the sweep's draws, one move per lane: move i takes ran1 draws
        // 5i+1 .. 5i+5 of the stream -- gaussian(3) from four uniforms, then
        // the acceptance uniform -- reached by jump-ahead (one FP64
        // Box-Muller per lane instead of one per move on a single lane).
        // Particle i moves only at its own move, so its proposal
        // x_i + sigma g is fixed by the sweep's start and is made here too:
        // the moves themselves do no FP64 arithmetic
        for (int i = lane; i < P; i += 32) {
            unsigned long long t = (jA[5 * i] * s + jC[5 * i]) & walker::kMask48;
            const double u1 = ran1_step(t), u2 = ran1_step(t), u3 = ran1_step(t), u4 = ran1_step(t);
            const double rn = ran1_step(t);
            double sn, cs;
            sincospi(2.0 * u1, &sn, &cs);
            const double r12 = sqrt(-2.0 * log(u2));
            const double g[3] = {sn * r12, cs * r12, cospi(2.0 * u3) * sqrt(-2.0 * log(u4))};
            const double sig = p.sigma[i < nup ? 0 : 1];
            for (int c = 0; c < 3; ++c) drw[4 * i + c] = walker::min_image(xs[3 * i + c] + sig * g[c], p);
            drw[4 * i + 3] = rn;
        }
        s = (jA[5 * P] * s + jC[5 * P]) & walker::kMask48;
        __syncwarp();
        // lanes 0-3 hold move i's proposal and uniform, read one move ahead
        double pv = lane < 4 ? drw[lane] : 0.0;
        for (int i = 0; i < P; ++i) {
            const bool up = i < nup;
            const double xn[3] = {__shfl_sync(0xffffffffu, pv, 0), __shfl_sync(0xffffffffu, pv, 1),
                                  __shfl_sync(0xffffffffu, pv, 2)};   // the proposal, FP64
            const double rn = __shfl_sync(0xffffffffu, pv, 3);
            const double pcur = pv;
            if (lane < 4 && i + 1 < P) pv = drw[4 * (i + 1) + lane];
            const float xf[3] = {(float)xn[0], (float)xn[1], (float)xn[2]};
            // the moved particle's plane waves
            for (int q = lane; q < nq; q += 32) {
                const KVecMP& K = kv[q + 1];
                float sn, cs;
                sincosf(K.k[0].hi * xf[0] + K.k[1].hi * xf[1] + K.k[2].hi * xf[2], &sn, &cs);
                oraw[q] = make_float2(cs, sn);
                const float vq = K.v.hi;
                onew[q] = make_float2(vq * cs, vq * sn);
            }
            __syncwarp();
            // the new row (up) or column (down) of the pair matrix
            const int nloop = up ? p.npair + p.nexdn : p.npair + p.nexup;
            for (int e = lane; e < nd; e += 32) {
                float ph;
                if (e < nloop) {
                    const int jj = up ? e + p.npair + p.nexup : e;
                    // two chains, loads unrolled ahead of the multiply-adds
                    float acc = v0, acc2 = 0.0f;
                    int q = 0;
#pragma unroll 4
                    for (; q + 1 < nq; q += 2) {
                        const float2 a = onew[q], b = T[q * P + jj];
                        const float2 a2 = onew[q + 1], b2 = T[(q + 1) * P + jj];
                        acc = fmaf(a.x, b.x, fmaf(a.y, b.y, acc));
                        acc2 = fmaf(a2.x, b2.x, fmaf(a2.y, b2.y, acc2));
                    }
                    if (q < nq) {
                        const float2 a = onew[q], b = T[q * P + jj];
                        acc = fmaf(a.x, b.x, fmaf(a.y, b.y, acc));
                    }
                    acc += acc2;
                    float d2 = 0.0f;
                    for (int c = 0; c < 3; ++c) {
                        const float d = min_image_f(xf[c] - xsf[3 * jj + c], elf, elif);
                        d2 = fmaf(d, d, d2);
                    }
                    ph = acc + beta_f(p, tud, sqrtf(d2));
                } else {
                    const int u = e - nloop;
                    const double* a = up ? p.akup[u] : p.akdn[u];
                    const int sn = up ? p.sinup[u] : p.sindn[u];
                    const float arg = (float)a[0] * xf[0] + (float)a[1] * xf[1] + (float)a[2] * xf[2];
                    ph = sn ? sinf(arg) : cosf(arg);
                }
                snew[e] = ph;
            }
            __syncwarp();
            // v_k = sum_q s'_q X(q, k) (row i replaced) or w_k = sum_q X(k, q) s'_q
            // (column c replaced); the ratio is v_i or w_c
            const int cix = up ? i : i - nup;
            for (int k = lane; k < nd; k += 32) {
                // four partial sums: the chain is shared-memory latency bound
                float a[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                const int rs = up ? 1 : ldx, cs = up ? ldx : 1;   // X(q, k) or X(k, q)
                const float* xb = X + k * cs;
                int q = 0;
                for (; q + 3 < nd; q += 4) {
#pragma unroll
                    for (int u = 0; u < 4; ++u) a[u] = fmaf(snew[q + u], xb[(q + u) * rs], a[u]);
                }
                for (; q < nd; ++q) a[0] = fmaf(snew[q], xb[q * rs], a[0]);
                vw[k] = (a[0] + a[1]) + (a[2] + a[3]);
            }
            // Jastrow: U(r_i') - U(r_i) over the pairs getphione counts.  A
            // lane takes its partners j = lane + 32 u kJasLanes at a time, all
            // their table lookups in flight before any is used; the
            // differences are added in partner order (skipped pairs add 0).
            constexpr int kJasLanes = 3;
            float du = 0.0f;
            for (int j0 = lane; j0 < P; j0 += 32 * kJasLanes) {
                float dj[kJasLanes];
#pragma unroll
                for (int u = 0; u < kJasLanes; ++u) {
                    const int j = j0 + 32 * u;
                    dj[u] = 0.0f;
                    const bool opp = up != (j < nup);
                    if (j < P && j != i && (opp || p.ieq)) {
                        float dn = 0.0f, dold = 0.0f;
                        for (int c = 0; c < 3; ++c) {
                            const float a = min_image_f(xf[c] - xsf[3 * j + c], elf, elif);
                            const float b = min_image_f(xsf[3 * i + c] - xsf[3 * j + c], elf, elif);
                            dn = fmaf(a, a, dn);
                            dold = fmaf(b, b, dold);
                        }
                        dj[u] = jas_u(p, tud, tss, opp, fmaxf(sqrtf(dn), 1.0e-14f)) -
                                jas_u(p, tud, tss, opp, fmaxf(sqrtf(dold), 1.0e-14f));
                    }
                }
#pragma unroll
                for (int u = 0; u < kJasLanes; ++u)
                    if (j0 + 32 * u < P) du += dj[u];
            }
            du = warp_sum_f(du);
            __syncwarp();
            const float R = vw[cix];
            const float prob = R * R * expf(2.0f * du);
            const bool acc = rn < (double)prob;   // R = 0 or NaN: rejected
            if (acc) {
                const float iR = 1.0f / R;
                // Sherman-Morrison (rank one): every column (row) but cix first
                if (up) {
                    for (int k = lane; k < nd; k += 32) {
                        if (k == cix) continue;
                        const float f = vw[k] * iR;
                        for (int q = 0; q < nd; ++q) X[q + k * ldx] = fmaf(-X[q + cix * ldx], f, X[q + k * ldx]);
                    }
                    __syncwarp();
                    for (int q = lane; q < nd; q += 32) X[q + cix * ldx] *= iR;
                } else {
                    for (int k = lane; k < nd; k += 32) {
                        if (k == cix) continue;
                        const float f = vw[k] * iR;
                        for (int q = 0; q < nd; ++q) X[k + q * ldx] = fmaf(-X[cix + q * ldx], f, X[k + q * ldx]);
                    }
                    __syncwarp();
                    for (int q = lane; q < nd; q += 32) X[cix + q * ldx] *= iR;
                }
                for (int q = lane; q < nq; q += 32) T[q * P + i] = oraw[q];
                if (lane < 3) {
                    xs[3 * i + lane] = pcur;
                    xsf[3 * i + lane] = (float)pcur;
                }
                ++nacc;
            }
            __syncwarp();
        }
    }
    // ---- write back (the positions are already in the stack) ----
    for (int e = lane; e < nd * nd; e += 32) {
        const int r = e % nd, c = e / nd;
        inv32[(size_t)w * nd * nd + e] = X[r + c * ldx];
    }
    if (lane == 0) {
        st.irn[w] = s;
        accepted[w] += nacc;
    }
}

}  // namespace

size_t sweep_smem_bytes(const DevParams& p, int wpc) { return (size_t)wpc * (sweep_warp_floats(p) / 2 + 1) * 8; }

cudaError_t launch_sweeps(const DevParams& p, const DevStack& st, int n, int nsweep, const double* inv64,
                          float* inv32, float2* tab, const KVecMP* kv, const TabUDmp* tud, const TabSSmp* tss,
                          const unsigned long long* jA, const unsigned long long* jC, unsigned long long* accepted,
                          double* prop, cudaStream_t stream)
{
    if (n <= 0 || nsweep <= 0) return cudaSuccess;
    if (!prop) return cudaErrorInvalidValue;
    // walkers per CTA: four, or fewer where a walker's shared memory (its
    // inverse is nd^2 floats) would not fit four times
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return e;
    int wpc = kSweepWarps;
    while (wpc > 1 && sweep_smem_bytes(p, wpc) > (size_t)optin) wpc /= 2;
    const size_t smem = sweep_smem_bytes(p, wpc);
    if (smem > (size_t)optin) return cudaErrorInvalidValue;
    if (smem > 48 * 1024) {
        e = cudaFuncSetAttribute(sweep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    // the largest shared-memory share of the SM: eight 4-walker CTAs per SM
    // at N = 66, so that 4096 walkers are resident at once
    e = cudaFuncSetAttribute(sweep_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    const int grid = (n + wpc - 1) / wpc;
    sweep_kernel<<<grid, 32 * wpc, smem, stream>>>(p, st, n, nsweep, inv64, inv32, tab, kv, tud, tss, jA, jC,
                                                   accepted, wpc, prop);
    return cudaGetLastError();
}

}  // namespace dmc
