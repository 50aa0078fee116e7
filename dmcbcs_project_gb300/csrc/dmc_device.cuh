// Device-side data layout of the GB300 DMCBS walker path.
//
// HBM layout
//  - walker stacks: structure of arrays, one walker per row; coordinates and
//    gradients x/dpsi/dpsig as [cap][npart][3] doubles (the reference's
//    x(3,npart) per walker), scalars as [cap] arrays, the 48-bit random
//    state as uint64 [cap].
//  - tables: one 64-byte record per grid point for up-down pairs
//    {v, u, u'/., u''-part, beta, beta', lap beta, 0} so that the 4-point
//    Lagrange stencil of one pair touches 256 contiguous bytes, and a
//    32-byte record {0, u, u', u''} for same-spin pairs.
//  - k vectors: 64-byte records (k, |k|^2, 2 vorb(shell), integer n).
// On-chip layout (one walker per CTA) is described by SmemLayout below.
#pragma once

#include <cstdint>
#include "../../include/dmcbcs_gpu.h"
#include "dmc_df32.cuh"

namespace dmc {

constexpr int kThreads = 256;        // threads per walker CTA
constexpr int kWarps = kThreads / 32;
constexpr int kMaxNest = DMC_NEST_MAX;

// grid record for up-down pairs (coshpot.f90 tables + betafun.f90 tables)
struct __align__(16) TabUD {
    double v, u, du, d2u, b, db, d2b, pad;
};
// grid record for same-spin pairs (no potential, no beta)
struct __align__(16) TabSS {
    double v, u, du, d2u;
};

// mixed-precision records, all double-float: the beta values enter the pair
// matrix, and for close pairs the Jastrow kinetic term and the potential
// cancel to a few parts in 10^3
struct __align__(16) TabUDmp {
    df v, u, du, d2u, b, db, d2b, pad;
};
struct __align__(16) TabSSmp {
    float v, u, du, d2u;
};
struct __align__(16) KVecMP {
    df k[3];
    df k2;
    df v;
    int n[3];
    int pad;
};

struct __align__(16) KVecDev {
    double k[3];
    double k2;
    double v;       // 2 * vorb(shell) (psislaterbcs.f90:259)
    double pad;
    int n[3];
    int shell;      // 1-based shell index (1 for k = 0)
};

// the kernels stage k-vector records as 8 doubles each
static_assert(sizeof(KVecMP) == 64 && sizeof(KVecDev) == 64, "k-vector records must be 64 bytes");

enum Mode : int {
    MODE_HPSI = 0,     // x -> hpsi outputs (wavefunction.f90:161-201)
    MODE_BCS = 1,      // x -> determinant part only (psislaterbcs.f90:155-225)
    MODE_GETPHI = 2,   // x -> Jastrow + potential only (coshpot.f90:154-205)
    MODE_STEP = 3,     // one step1 move of every walker (step.f90:43-285)
};

struct DevParams {
    int npart, nup, ndn, npair, nexup, nexdn, nd, nk, ncol, norb, ntab, nmax;
    int ieq, nobeta, cutdrift, fn, idmc, onebody, nest, nrand;
    int ntab0;            // last non-zero Jastrow grid point (healing distance)
    int nql;              // long-range Jastrow q vectors (0: off)
    double jbeta, jgamma; // its parameters
    int ldS, ldU;
    double el, eli, range, scale, rangeb, scaleb;
    double mass[2], sqm[2], imass[2], isqm[2];
    double hbar, a2, dt, etrial, wtcut, nfac;
    double sigma[2], dcut[2];
    double qex[3], v0ex, v0exjas, vorb1;
    // double-float copies for the mixed-precision kernel
    df el_df, scaleb_df, rangeb_df, range_df;
    df eli2_df;           // 2 / L: orbital base angle over pi
    float eli_f;
    double akup[DMC_MAX_UNPAIRED][3], ak2up[DMC_MAX_UNPAIRED];
    double akdn[DMC_MAX_UNPAIRED][3], ak2dn[DMC_MAX_UNPAIRED];
    int sinup[DMC_MAX_UNPAIRED], sindn[DMC_MAX_UNPAIRED];
};

// Operators (g(r), density profile, S(q), n(k)) on the device
struct OpsDev {
    int ntabg, ntabq, ntabk, nsamp, nqtot, nkv, nnk;
    double scaleg, el, dk;
    const double* akq;                 // [nqtot][3], k = 0 first
    const int* ik;                     // [nkv][3], sorted by |ik|^2
    const int* indk;                   // [ntabk+1] first vector of each shell
    const int* nkk;                    // [ntabk+1] vectors per shell
    const unsigned long long *jA, *jC; // LCG jump-ahead, [3 npart nsamp + 1]
};

// SoA walker stack on the device
struct DevStack {
    double *x, *dpsi, *dpsig;
    double *psil, *psigl, *d2psi, *d2psig, *v, *vext, *weight, *psil0, *psigl0;
    float* wt0;
    int* is;
    unsigned long long* irn;
};

// Arguments of the walker kernel.  For MODE_STEP the input is stack `in`
// (n walkers, popped from the top) and the output stack `out`; otherwise
// positions come from `xin` and results go to the `o_*` arrays.
struct KernelArgs {
    int mode;
    int nw;
    int opcomp;
    int defer;                   // MODE_STEP: weights and estimators left to step_decide_kernel
    const int* pn;               // MODE_STEP: walker count on the device (nullptr: nw)
    const double* xin;
    double *o_psil, *o_dpsi, *o_d2psi, *o_v, *o_vext, *o_psigl, *o_dpsig, *o_d2psig, *o_sinv;
    double* o_dphi;              // MODE_HPSI: also the determinant's drift alone (as MODE_BCS gives it)
    int* o_is;
    DevStack in, out;
    double* est;                 // [nw][nest][2]: (val, wt) per estimator
    const KVecDev* kv;           // [nk]
    const TabUD* tud;            // [ntab+1]
    const TabSS* tss;            // [ntab+1]
    const KVecMP* kv_mp;         // mixed-precision copies of kv, tud, tss
    const TabUDmp* tud_mp;
    const TabSSmp* tss_mp;
    const unsigned long long* jumpA;   // LCG jump-ahead multipliers, [nrand+1]
    const unsigned long long* jumpC;   // LCG jump-ahead increments, [nrand+1]
    double* gscratch;            // per-CTA global scratch when the pair data do not fit on chip
    const double* jq;            // long-range Jastrow q records, [nql][8]
    int* status;                 // the context's status word, DMC_STATUS_* flags OR-ed over walkers
    int* wstatus;                // batched evaluations: DMC_STATUS_* flags of walker w (nullptr: none)
    const double* in_wt0d;       // MODE_STEP: the old wt0 in double precision (input stack in the
                                 // caller's host arrays), else nullptr: in.wt0
};

// On-chip layout of one walker CTA, offsets in doubles.
struct SmemLayout {
    int nt;               // threads of the walker CTA (256, or 512 at one CTA per SM)
    int x, xr, xo, dx, drift, dg, kq, S, pb, R, U, D, E, acc, colk, red, total;
    int ksoa;             // k-vector fields as arrays: kx, ky, kz, k^2, v [5][nk],
                          // then the integer components n [3][nk]
    int S2;               // second nd x ldS buffer of the blocked inverse (-1: none)
    int pb_in_smem;
    int pb_size;          // doubles of pair data per walker
    int rows_jas, rows_beta;   // rows of the up-down block per reduction chunk
    int rsize;            // doubles in the union region
    int un_in_smem;       // 0: the union region (U, D, E, S2, pair vectors) lives in
                          // the CTA's global scratch slice, at offset 0 of it
    int gstride;          // doubles of global scratch per CTA: the union region
                          // (when not on chip), then the beta pair data (idem)
};

__host__ __device__ inline int round_up(int a, int b) { return (a + b - 1) / b * b; }

// union_global: the union region goes to the CTA's global scratch slice
// (systems whose orbitals and second inverse buffer do not fit on chip); its
// offsets keep their values, above every on-chip offset.
__host__ __device__ inline SmemLayout make_layout(const DevParams& p, int smem_limit_bytes, int nt = kThreads,
                                                  bool union_global = false)
{
    SmemLayout L;
    L.nt = nt;
    const int n3 = p.npart * 3;
    int off = 0;
    auto take = [&](int nd) { int o = off; off += round_up(nd, 2); return o; };
    L.x = take(n3);               // positions being evaluated
    L.xr = take(n3);              // the same in the kernel's arithmetic type
    L.xo = take(n3);              // old positions (step)
    L.dx = take(n3);              // drift + gaussian displacement (step)
    L.drift = take(n3);           // old drift (step)
    L.dg = take(n3);              // guide-function gradient when a2 != 0
    L.kq = take(p.nk * 8);        // k vector records
    L.ksoa = take(p.nk * 7);      // the same fields as arrays (conflict-free reads across k)
    L.S = take(p.nd * p.ldS);     // pair matrix -> inverse
    L.colk = take(2 * p.nd + 2);  // pivot column of the unblocked Gauss-Jordan
    L.acc = take(p.npart * 8);    // per particle: drift(3), lap, du(3), spare
    L.red = take(nt * 8);        // reductions and per-thread partial sums
    // union region: Jastrow pair vectors, then orbitals U|D|E, then beta terms
    const int nE = p.npart * 3 * (p.nmax + 1) * 2;
    const int nUDE = p.nup * p.ldU + p.ndn * p.ldU + nE;
    L.R = off;
    L.U = L.R;
    L.D = L.R + p.nup * p.ldU;
    L.E = L.D + p.ndn * p.ldU;
    // the blocked inverse ping-pongs the pair matrix with a second buffer at
    // E (the orbital powers are dead once S is formed)
    const int nUDS = p.nup * p.ldU + p.ndn * p.ldU + p.nd * p.ldS;
    int rsize = nUDE > nUDS ? nUDE : nUDS;
    L.S2 = L.E;
    const int row_pairs = p.ndn > 0 ? p.ndn : 1;
    const int minrows = 1;
    // at least one row of pair data must fit
    if (rsize < row_pairs * 4) rsize = row_pairs * 4;
    L.un_in_smem = union_global ? 0 : 1;
    if (!union_global) off += round_up(rsize, 2);
    L.rsize = rsize;
    L.rows_jas = rsize / (row_pairs * 3);
    L.rows_beta = rsize / (row_pairs * 4);
    if (L.rows_jas < minrows) L.rows_jas = minrows;
    if (L.rows_beta < minrows) L.rows_beta = minrows;
    // beta pair data (f'/r, lap f) per up-down pair
    L.pb_size = p.nup * p.ndn * 2;
    const int with_pb = off + round_up(L.pb_size, 2);
    if (!union_global && with_pb * 8 <= smem_limit_bytes) {
        L.pb = off;
        off = with_pb;
        L.pb_in_smem = 1;
    } else {
        L.pb = -1;
        L.pb_in_smem = 0;
    }
    L.gstride = (union_global ? round_up(rsize, 2) : 0) + (L.pb_in_smem ? 0 : round_up(L.pb_size, 2));
    L.total = off;
    return L;
}

}  // namespace dmc
