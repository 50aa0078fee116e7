// C ABI of the GB300 DMCBS walker path: contexts, device buffers, walker
// stacks and the generation driver (dmcbcs.f90:426-449 for one process).
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "../../include/dmcbcs_gpu.h"
#include "dmc_device.cuh"
#include "dmc_kernels.h"
#include "dmc_setup.h"
#include "dmc_text.h"

namespace dmc {
cudaError_t launch_matinv(const double* a_colmajor, double* inv_colmajor, double* detl, int* is, int n, int nb,
                          cudaStream_t st);
cudaError_t launch_reverse(const DevStack& in, const DevStack& out, int n, int n3, cudaStream_t st);
}  // namespace dmc

using namespace dmc;

namespace {

constexpr unsigned long long kMask48 = (1ull << 48) - 1ull;
constexpr unsigned long long kMult1 = 44485709377909ull, kAdd1 = 96309754297ull;
constexpr unsigned long long kMult2 = 34522712143931ull, kAdd2 = 55789347517ull;

// Device array owned by its holder: freed by release() or on destruction.
template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    cudaError_t alloc(size_t cnt)
    {
        if (cnt <= n && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(cnt, 1) * sizeof(T));
        if (e == cudaSuccess) n = cnt;
        return e;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

struct StackBufs {
    DevBuf<double> x, dpsi, dpsig, psil, psigl, d2psi, d2psig, v, vext, weight, psil0, psigl0;
    DevBuf<float> wt0;
    DevBuf<int> is;
    DevBuf<unsigned long long> irn;
    cudaError_t alloc(int cap, int n3)
    {
        cudaError_t e = cudaSuccess;
        auto A = [&](cudaError_t r) {
            if (e == cudaSuccess) e = r;
        };
        A(x.alloc((size_t)cap * n3));
        A(dpsi.alloc((size_t)cap * n3));
        A(dpsig.alloc((size_t)cap * n3));
        A(psil.alloc(cap));
        A(psigl.alloc(cap));
        A(d2psi.alloc(cap));
        A(d2psig.alloc(cap));
        A(v.alloc(cap));
        A(vext.alloc(cap));
        A(weight.alloc(cap));
        A(psil0.alloc(cap));
        A(psigl0.alloc(cap));
        A(wt0.alloc(cap));
        A(is.alloc(cap));
        A(irn.alloc(cap));
        return e;
    }
    void release()
    {
        x.release(); dpsi.release(); dpsig.release(); psil.release(); psigl.release(); d2psi.release();
        d2psig.release(); v.release(); vext.release(); weight.release(); psil0.release(); psigl0.release();
        wt0.release(); is.release(); irn.release();
    }
    DevStack view()
    {
        DevStack s;
        s.x = x.p; s.dpsi = dpsi.p; s.dpsig = dpsig.p; s.psil = psil.p; s.psigl = psigl.p; s.d2psi = d2psi.p;
        s.d2psig = d2psig.p; s.v = v.p; s.vext = vext.p; s.weight = weight.p; s.psil0 = psil0.p;
        s.psigl0 = psigl0.p; s.wt0 = wt0.p; s.is = is.p; s.irn = irn.p;
        return s;
    }
};

}  // namespace

// CUDA events owned for the length of a call (destroyed on every return path)
struct EventVec {
    std::vector<cudaEvent_t> v;
    explicit EventVec(size_t n) : v(n, nullptr) {}
    ~EventVec()
    {
        for (cudaEvent_t e : v)
            if (e) cudaEventDestroy(e);
    }
    cudaEvent_t& operator[](size_t i) { return v[i]; }
};

struct dmc_ctx {
    Setup S;
    dmc_system_desc sd;
    dmc_run_desc rd;
    DevParams P;
    SmemLayout L;
    int device = 0, nsm = 0, grid = 0, cap = 0, n3 = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double last_ms = 0.0;
    // tables
    DevBuf<KVecDev> kv;
    DevBuf<TabUD> tud;
    DevBuf<TabSS> tss;
    DevBuf<KVecMP> kv_mp;
    DevBuf<TabUDmp> tud_mp;
    DevBuf<TabSSmp> tss_mp;
    int precision = DMC_PREC_FP64;
    DevBuf<unsigned long long> jumpA, jumpC;
    DevBuf<double> gscratch;
    DevBuf<double> jq;
    // population
    StackBufs st[2];
    int istin = 0;
    int n = 0;
    // walker count on the device during generations: pop = {n slot 0, n slot 1,
    // error flags (bit 0 died out, bit 1 overflow), population-control flag};
    // popf = {population-control factor}; psteps counts walker-steps
    DevBuf<int> pop;
    DevBuf<double> popf;
    DevBuf<unsigned long long> psteps;
    int pcur = 0;          // slot of the current count
    bool n_stale = false;  // the device count leads (host n out of date)
    // captured generations by (opcomp, stack parity, count-slot parity),
    // valid while the parameters, launch arguments and precision match the
    // capture
    cudaGraphExec_t gexec[2][2][2] = {};
    int gnl[2][2][2] = {};
    DevParams gP;
    KernelArgs gA;
    int gprec = -1;
    int layout_gen = 0;     // bumped by every change of the walker layout
    int glayout = -1;       // the layout_gen the captured generations saw
    DevBuf<double> est;
    DevBuf<int> counts, offs, status;
    DevBuf<int> wstat;      // per-walker flags of the last batched evaluation
    int wstat_n = 0;        // its walker count
    int hstatus = 0;        // DMC_STATUS_* flags met on the host (stack overflow)
    DevBuf<unsigned long long> irn1, wtisto;
    // estimator block sums valblk, valblk2, wtblk and their compensation
    // terms: one buffer of 6 DMC_NEST_MAX doubles (vb2, wb and vbc point
    // into it), read with one copy
    DevBuf<double> vb;
    double *vb2 = nullptr, *wb = nullptr, *vbc = nullptr;
    DevBuf<double> estpart;            // the estimator kernel's per-CTA partial sums
    DevBuf<unsigned int> estticket;    // its last-CTA counter (zero between launches)
    // batch staging
    DevBuf<double> bx, bpsil, bdpsi, bd2psi, bv, bvext, bpsigl, bdpsig, bd2psig, bsinv;
    DevBuf<int> bis;
    DevBuf<unsigned char> flush;
    // single-particle moves and parameter derivatives
    DevBuf<double> sx, sdr, sratio, sder, ssinv, srsum, srene;
    DevBuf<double> pg_dpsi, pg_dphi, pg_dlog, pg_del, pg_scr;   // adjoint parameter gradients
    DevBuf<PgTab> pg_btab;                                      // d beta / d b, d beta / d d tables
    DevBuf<PgTab> pg_ktab;                                      // Jastrow knot basis on the table grid
    DevBuf<double> pg_slice;                                    // per-CTA slices of the adjoint kernel
    // particle-by-particle sweeps: FP32 inverses carried between calls, the
    // cos/sin tables, accepted moves per walker
    DevBuf<float> sm_inv;
    DevBuf<float2> sm_tab;
    DevBuf<double> sm_prop;       // each sweep's proposals and acceptance uniforms, [n][npart][4]
    DevBuf<unsigned long long> sm_acc, sm_jA, sm_jC;   // accepted moves; ran1 jumps of 0..5 npart steps
    int sm_n = 0;                 // walkers whose FP32 inverse sm_inv holds (0: none)
    DevBuf<int> sip;
    int64_t sr_count = 0;
    bool sr_jas = false, sr_det = true;   // iopt(1), iopt(2) of the optimizer deck
    bool sr_adj = false;                  // SR over every parameter of dmc_param_grad
    // operators (g(r), density profile, S(q), n(k))
    struct Ops {
        bool on = false;
        OpsDev dev{};
        std::vector<double> akq;
        std::vector<int> ik, indk, nkk, numshq;
        DevBuf<double> akq_d, sv, tk, sums, wts;
        DevBuf<int> ik_d, indk_d, nkk_d, hg, hd;
        DevBuf<unsigned long long> jA, jC;
        std::vector<double> val[4], err[4];   // after the last update: g, density, S(q), n(k)
        double totw[3] = {0, 0, 0};
    } ops;
    int64_t launches = 0;
    std::string err;
};

namespace {

int fail(dmc_ctx* c, int code, const std::string& msg)
{
    if (c) c->err = msg;
    return code;
}

// Bring the host walker count up to date after generations that counted on
// the device; reports a population that died out or overflowed the stack.
int sync_n(dmc_ctx* c)
{
    if (!c->n_stale) return DMC_OK;
    int h[4] = {0, 0, 0, 0};
    if (cudaMemcpyAsync(h, c->pop.p, sizeof h, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)
        return fail(c, DMC_ERR_CUDA, "walker count");
    c->n = h[c->pcur];
    c->n_stale = false;
    if (h[2]) {
        cudaMemsetAsync(c->pop.p + 2, 0, sizeof(int), c->stream);
        if (h[2] & 2) {
            c->hstatus |= DMC_STATUS_OVERFLOW;
            return fail(c, DMC_ERR_OVERFLOW, "stack overflow in branch");
        }
        return fail(c, DMC_ERR_EMPTY, "population died out");
    }
    return DMC_OK;
}

int cuda_fail(dmc_ctx* c, cudaError_t e, const char* where)
{
    return fail(c, DMC_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(expr)                                              \
    do {                                                      \
        cudaError_t _e = (expr);                              \
        if (_e != cudaSuccess) return cuda_fail(c, _e, #expr); \
    } while (0)

int nest_for(int idmc)
{
    switch (idmc) {
    case -1: case 0: return 6;
    case -2: case 1: case 10: return 14;
    case 2: return 13;
    }
    return -1;
}

void fill_params(dmc_ctx* c)
{
    const Setup& S = c->S;
    DevParams& p = c->P;
    std::memset(&p, 0, sizeof p);
    p.npart = S.npart; p.nup = S.nup; p.ndn = S.ndn; p.npair = S.npair; p.nexup = S.nexup; p.nexdn = S.nexdn;
    p.nd = S.nd; p.nk = S.nk; p.ncol = S.ncol; p.norb = S.norb; p.ntab = S.ntab; p.nmax = S.nmax;
    p.ieq = S.ieq; p.nobeta = S.nobeta; p.cutdrift = S.cutdrift; p.fn = c->rd.fn; p.idmc = c->rd.idmc;
    p.onebody = (S.v0ex != 0.0 || S.v0exjas != 0.0);
    p.ntab0 = S.ntab0;
    p.nql = S.nql;
    p.jbeta = S.jbeta;
    p.jgamma = S.jgamma;
    p.nest = nest_for(c->rd.idmc);
    p.nrand = 2 * ((3 * S.npart + 1) / 2);
    p.ldS = S.nd | 1;
    // U/D row pitch: even (16-byte pairs) with an odd number of 16-byte
    // units, so rows read by neighbouring lanes fall in different banks
    {
        const int nq = S.nk - 1;
        int half = nq + 1;
        if (half % 2 == 0) ++half;
        p.ldU = 2 * half;
    }
    p.el = S.el; p.eli = S.eli; p.range = S.range; p.scale = S.scale; p.rangeb = S.rangeb; p.scaleb = S.scaleb;
    for (int s = 0; s < 2; ++s) {
        p.mass[s] = S.mass[s];
        p.sqm[s] = S.sqm[s];
        p.imass[s] = 1.0 / S.mass[s];
        p.isqm[s] = 1.0 / S.sqm[s];
        p.sigma[s] = S.sigma[s];
        p.dcut[s] = S.dcut[s];
    }
    p.hbar = S.hbar; p.a2 = S.a2; p.dt = c->rd.dt; p.etrial = S.etrial; p.wtcut = c->rd.wtcut; p.nfac = S.nfac;
    for (int k = 0; k < 3; ++k) p.qex[k] = S.qex[k];
    p.v0ex = S.v0ex; p.v0exjas = S.v0exjas; p.vorb1 = S.vorb[0];
    p.el_df = from_double(S.el);
    p.scaleb_df = from_double(S.scaleb);
    p.rangeb_df = from_double(S.rangeb);
    p.range_df = from_double(S.range);
    p.eli2_df = from_double(2.0 * S.eli);
    p.eli_f = (float)S.eli;
    for (int i = 0; i < DMC_MAX_UNPAIRED; ++i) {
        for (int k = 0; k < 3; ++k) {
            p.akup[i][k] = S.akup[i][k];
            p.akdn[i][k] = S.akdn[i][k];
        }
        p.ak2up[i] = S.ak2up[i]; p.ak2dn[i] = S.ak2dn[i]; p.sinup[i] = S.sinup[i]; p.sindn[i] = S.sindn[i];
    }
}

int upload_kv(dmc_ctx* c)
{
    std::vector<KVecDev> kv(c->S.nk);
    for (int q = 0; q < c->S.nk; ++q) {
        const KVec& K = c->S.kv[q];
        KVecDev& d = kv[q];
        std::memset(&d, 0, sizeof d);
        for (int k = 0; k < 3; ++k) {
            d.k[k] = K.k[k];
            d.n[k] = K.n[k];
        }
        d.k2 = K.k2;
        d.v = q == 0 ? c->S.vorb[0] : 2.0 * c->S.vorb[K.shell - 1];
        d.shell = q == 0 ? 1 : K.shell;
    }
    CK(c->kv.alloc(kv.size()));
    CK(cudaMemcpy(c->kv.p, kv.data(), kv.size() * sizeof(KVecDev), cudaMemcpyHostToDevice));
    std::vector<KVecMP> km(kv.size());
    for (size_t q = 0; q < kv.size(); ++q) {
        std::memset(&km[q], 0, sizeof(KVecMP));
        for (int k = 0; k < 3; ++k) {
            km[q].k[k] = from_double(kv[q].k[k]);
            km[q].n[k] = kv[q].n[k];
        }
        km[q].k2 = from_double(kv[q].k2);
        km[q].v = from_double(kv[q].v);
    }
    CK(c->kv_mp.alloc(km.size()));
    CK(cudaMemcpy(c->kv_mp.p, km.data(), km.size() * sizeof(KVecMP), cudaMemcpyHostToDevice));
    c->P.vorb1 = c->S.vorb[0];
    return DMC_OK;
}

int upload_tables(dmc_ctx* c)
{
    const Setup& S = c->S;
    const int nt = S.ntab + 1;
    std::vector<TabUD> ud(nt);
    std::vector<TabSS> ss(nt);
    for (int i = 0; i < nt; ++i) {
        ud[i] = TabUD{S.vtab[0][i], S.utab[0][i], S.dutab[0][i], S.d2utab[0][i], S.btab[i], S.dbtab[i], S.d2btab[i], 0.0};
        ss[i] = TabSS{S.vtab[1][i], S.utab[1][i], S.dutab[1][i], S.d2utab[1][i]};
    }
    CK(c->tud.alloc(nt));
    CK(c->tss.alloc(nt));
    CK(cudaMemcpy(c->tud.p, ud.data(), nt * sizeof(TabUD), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->tss.p, ss.data(), nt * sizeof(TabSS), cudaMemcpyHostToDevice));
    // mixed-precision copies in double-float
    std::vector<TabUDmp> udm(nt);
    std::vector<TabSSmp> ssm(nt);
    for (int i = 0; i < nt; ++i) {
        std::memset(&udm[i], 0, sizeof(TabUDmp));
        udm[i].v = from_double(S.vtab[0][i]);
        udm[i].u = from_double(S.utab[0][i]);
        udm[i].du = from_double(S.dutab[0][i]);
        udm[i].d2u = from_double(S.d2utab[0][i]);
        udm[i].b = from_double(S.btab[i]);
        udm[i].db = from_double(S.dbtab[i]);
        udm[i].d2b = from_double(S.d2btab[i]);
        ssm[i] = TabSSmp{(float)S.vtab[1][i], (float)S.utab[1][i], (float)S.dutab[1][i], (float)S.d2utab[1][i]};
    }
    CK(c->tud_mp.alloc(nt));
    CK(c->tss_mp.alloc(nt));
    CK(cudaMemcpy(c->tud_mp.p, udm.data(), nt * sizeof(TabUDmp), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->tss_mp.p, ssm.data(), nt * sizeof(TabSSmp), cudaMemcpyHostToDevice));
    if (S.nql > 0) {
        CK(c->jq.alloc(S.jq.size()));
        CK(cudaMemcpy(c->jq.p, S.jq.data(), S.jq.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    // LCG jump tables for t = 0..nrand+1 steps of ran1
    const int nj = c->P.nrand + 2;
    std::vector<unsigned long long> A(nj), C(nj);
    A[0] = 1;
    C[0] = 0;
    for (int t = 1; t < nj; ++t) {
        A[t] = (A[t - 1] * kMult1) & kMask48;
        C[t] = (C[t - 1] * kMult1 + kAdd1) & kMask48;
    }
    CK(c->jumpA.alloc(nj));
    CK(c->jumpC.alloc(nj));
    CK(cudaMemcpy(c->jumpA.p, A.data(), nj * sizeof(unsigned long long), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->jumpC.p, C.data(), nj * sizeof(unsigned long long), cudaMemcpyHostToDevice));
    return DMC_OK;
}

KernelArgs base_args(dmc_ctx* c)
{
    KernelArgs a;
    std::memset(&a, 0, sizeof a);
    a.kv = c->kv.p;
    a.tud = c->tud.p;
    a.tss = c->tss.p;
    a.kv_mp = c->kv_mp.p;
    a.tud_mp = c->tud_mp.p;
    a.tss_mp = c->tss_mp.p;
    a.jumpA = c->jumpA.p;
    a.jumpC = c->jumpC.p;
    a.gscratch = c->gscratch.p;
    a.jq = c->jq.p;
    a.status = c->status.p;
    return a;
}

int grid_for(dmc_ctx* c, int nw) { return std::max(1, std::min(nw, c->grid)); }

int run_eval(dmc_ctx* c, int mode, int nw, const double* dx, double* psil, int* is, double* dpsi, double* d2psi,
             double* v, double* vext, double* psigl, double* dpsig, double* d2psig, double* sinv, cudaStream_t st,
             double* dphi = nullptr)
{
    if (nw <= 0) return DMC_OK;
    KernelArgs a = base_args(c);
    a.mode = mode;
    a.nw = nw;
    a.xin = dx;
    a.o_psil = psil; a.o_is = is; a.o_dpsi = dpsi; a.o_d2psi = d2psi; a.o_v = v; a.o_vext = vext;
    a.o_psigl = psigl; a.o_dpsig = dpsig; a.o_d2psig = d2psig; a.o_sinv = sinv; a.o_dphi = dphi;
    CK(c->wstat.alloc(nw));
    a.wstatus = c->wstat.p;
    c->wstat_n = nw;
    CK(launch_walker(c->P, a, c->L, grid_for(c, nw), st, c->precision == DMC_PREC_MIXED));
    return DMC_OK;
}

// host-staged batch evaluation: copy x in, run, copy requested outputs out
int batch_eval(dmc_ctx* c, int mode, int nw, const double* x, double* psil, int* is, double* dpsi, double* d2psi,
               double* v, double* vext, double* psigl, double* dpsig, double* d2psig, double* sinv)
{
    if (!c) return DMC_ERR_INVALID;
    if (nw < 0 || (nw > 0 && !x)) return fail(c, DMC_ERR_INVALID, "bad batch arguments");
    if (nw == 0) return DMC_OK;
    const size_t n3 = (size_t)c->n3, nd2 = (size_t)c->S.nd * c->S.nd;
    CK(c->bx.alloc(nw * n3));
    if (psil) CK(c->bpsil.alloc(nw));
    if (is) CK(c->bis.alloc(nw));
    if (dpsi) CK(c->bdpsi.alloc(nw * n3));
    if (d2psi) CK(c->bd2psi.alloc(nw));
    if (v) CK(c->bv.alloc(nw));
    if (vext) CK(c->bvext.alloc(nw));
    if (psigl) CK(c->bpsigl.alloc(nw));
    if (dpsig) CK(c->bdpsig.alloc(nw * n3));
    if (d2psig) CK(c->bd2psig.alloc(nw));
    if (sinv) CK(c->bsinv.alloc(nw * nd2));
    CK(cudaMemcpyAsync(c->bx.p, x, nw * n3 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    int rc = run_eval(c, mode, nw, c->bx.p, psil ? c->bpsil.p : nullptr, is ? c->bis.p : nullptr,
                      dpsi ? c->bdpsi.p : nullptr, d2psi ? c->bd2psi.p : nullptr, v ? c->bv.p : nullptr,
                      vext ? c->bvext.p : nullptr, psigl ? c->bpsigl.p : nullptr, dpsig ? c->bdpsig.p : nullptr,
                      d2psig ? c->bd2psig.p : nullptr, sinv ? c->bsinv.p : nullptr, c->stream);
    if (rc) return rc;
    auto D2H = [&](void* h, const void* d, size_t bytes) {
        return cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, c->stream);
    };
    if (psil) CK(D2H(psil, c->bpsil.p, nw * sizeof(double)));
    if (is) CK(D2H(is, c->bis.p, nw * sizeof(int)));
    if (dpsi) CK(D2H(dpsi, c->bdpsi.p, nw * n3 * sizeof(double)));
    if (d2psi) CK(D2H(d2psi, c->bd2psi.p, nw * sizeof(double)));
    if (v) CK(D2H(v, c->bv.p, nw * sizeof(double)));
    if (vext) CK(D2H(vext, c->bvext.p, nw * sizeof(double)));
    if (psigl) CK(D2H(psigl, c->bpsigl.p, nw * sizeof(double)));
    if (dpsig) CK(D2H(dpsig, c->bdpsig.p, nw * n3 * sizeof(double)));
    if (d2psig) CK(D2H(d2psig, c->bd2psig.p, nw * sizeof(double)));
    if (sinv) CK(D2H(sinv, c->bsinv.p, nw * nd2 * sizeof(double)));
    CK(cudaStreamSynchronize(c->stream));
    return DMC_OK;
}

}  // namespace

extern "C" {

int dmc_abi_version(void) { return DMC_ABI_VERSION; }

const char* dmc_status_string(int s)
{
    switch (s) {
    case DMC_OK: return "ok";
    case DMC_ERR_INVALID: return "invalid argument";
    case DMC_ERR_CUDA: return "CUDA error";
    case DMC_ERR_UNSUPPORTED: return "unsupported";
    case DMC_ERR_OVERFLOW: return "walker stack overflow";
    case DMC_ERR_SETUP: return "table set-up failed";
    case DMC_ERR_EMPTY: return "population died out";
    case DMC_ERR_NOMEM: return "out of memory";
    case DMC_ERR_NOALLOC_LIMIT: return "size above the no-allocation scratch maximum";
    }
    return "unknown status";
}

// Walker layouts a context can run (threads per CTA, CTAs per SM, what stays
// on chip).  LAYOUT_HEURISTIC: on chip, two CTAs per SM when they fit (with
// the beta pair data moved to global scratch if that makes them fit), else
// one CTA with 16 warps for the mixed kernel; the union region off chip only
// when nothing else fits.  The others are the alternatives the layout tuner
// times: on chip with 256 threads throughout, and the union region in global
// scratch at the CTAs per SM its smaller on-chip part allows.
enum { LAYOUT_HEURISTIC = 0, LAYOUT_ONCHIP_256 = 1, LAYOUT_UNION_GLOBAL = 2, LAYOUT_KINDS = 3 };

static int plan_layout(dmc_ctx* c, int optin, int kind, SmemLayout* Lout, int* per_sm_out)
{
    int smem_sm = 0;
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c->device);
    const int regs_ok = 2;   // launch bounds give <= 128 registers at 256 threads
    if (kind != LAYOUT_UNION_GLOBAL) {
        // dynamic + static shared memory + the 1 KB the runtime reserves per block
        const int static_smem = std::max(0, walker_static_smem_bytes(c->rd.idmc == 10));
        const int limit = std::min(optin, 227 * 1024) - 64 - static_smem;
        SmemLayout L;
        walker_smem_bytes(c->P, limit, &L);
        const int need = L.total * 8 + static_smem + 1024;
        int per_sm = std::max(1, std::min(regs_ok, smem_sm / need));
        if (per_sm < regs_ok) {
            // two CTAs per SM when the beta pair data move to global scratch
            // (L2-resident, written by the pair stage and read once by the
            // beta drift terms) and the rest of the layout fits twice
            SmemLayout L2;
            walker_smem_bytes(c->P, smem_sm / regs_ok - static_smem - 1024, &L2);
            if (L2.total * 8 + static_smem + 1024 <= smem_sm / regs_ok) {
                L = L2;
                per_sm = regs_ok;
            }
        }
        if (per_sm == 1 && kind == LAYOUT_HEURISTIC) {
            // one CTA per SM: twice the threads (16 warps) on the same walker
            // in the mixed kernel, with the larger reduction buffer they need,
            // when that still fits (N = 132: 578k -> 719k walker-steps/s; the
            // FP64 kernel keeps 256 threads, the buffer is simply larger than
            // it needs)
            SmemLayout L512;
            walker_smem_bytes(c->P, limit, &L512, 2 * kThreads);
            if (L512.total * 8 <= limit && L512.total * 8 + static_smem + 1024 <= smem_sm) L = L512;
        }
        if ((long long)L.total * 8 <= (long long)limit) {
            *Lout = L;
            *per_sm_out = per_sm;
            return DMC_OK;
        }
        if (kind != LAYOUT_HEURISTIC) return DMC_ERR_UNSUPPORTED;
        // the orbitals, their powers and the second inverse buffer do not fit
        // on chip (above about N = 144 at seven shells, N = 120 at ten)
    }
    // the union region in an L2-resident global slice per CTA; the pair
    // matrix, positions and accumulators stay in shared memory
    const int static_big = std::max(0, walker_big_static_smem_bytes());
    const int limit_big = std::min(optin, 227 * 1024) - 64 - static_big;
    SmemLayout LB;
    walker_smem_bytes(c->P, limit_big, &LB, kThreads, true);
    if ((long long)LB.total * 8 > (long long)limit_big) return DMC_ERR_UNSUPPORTED;
    *Lout = LB;
    *per_sm_out = std::max(1, std::min(regs_ok, smem_sm / (LB.total * 8 + static_big + 1024)));
    return DMC_OK;
}

// Make L the context's layout: grid, global scratch, kernel attributes; the
// captured generations of the old layout are dropped at their next use.
static int apply_layout(dmc_ctx* c, const SmemLayout& L, int per_sm)
{
    const int grid = c->nsm * per_sm;
    if (L.gstride > 0 && c->gscratch.alloc((size_t)grid * L.gstride) != cudaSuccess)
        return fail(c, DMC_ERR_NOMEM, "walker scratch");
    cudaError_t e = prepare_walker(L);
    if (e == cudaSuccess && c->rd.idmc == 10) e = prepare_walker(L, true);
    if (e != cudaSuccess) return fail(c, DMC_ERR_CUDA, std::string("walker layout: ") + cudaGetErrorString(e));
    c->L = L;
    c->grid = grid;
    ++c->layout_gen;
    return DMC_OK;
}

const char* dmc_last_error(const dmc_ctx* c) { return c ? c->err.c_str() : "no context"; }

int dmc_create(const dmc_system_desc* sd, const dmc_run_desc* rd, dmc_ctx** out)
{
    if (!sd || !rd || !out) return DMC_ERR_INVALID;
    *out = nullptr;
    dmc_ctx* c = new (std::nothrow) dmc_ctx();
    if (!c) return DMC_ERR_NOMEM;
    c->sd = *sd;
    c->rd = *rd;
    if (nest_for(rd->idmc) < 0) {
        delete c;
        return DMC_ERR_INVALID;
    }
    if (rd->nwalk < 1 || !(rd->dt > 0.0)) {
        delete c;
        return DMC_ERR_INVALID;
    }
    int rc = c->S.build(*sd, *rd, c->err);
    if (rc != DMC_OK) {
        delete c;
        return rc;
    }
    fill_params(c);
    c->n3 = 3 * c->S.npart;
    cudaError_t e = cudaGetDevice(&c->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, c->device);
    int optin = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
    if (e != cudaSuccess) {
        dmc_destroy(c);
        return DMC_ERR_CUDA;
    }
    {
        SmemLayout L;
        int per_sm = 1;
        int rc2 = plan_layout(c, optin, LAYOUT_HEURISTIC, &L, &per_sm);
        if (rc2 == DMC_OK) rc2 = apply_layout(c, L, per_sm);
        if (rc2 != DMC_OK) {
            dmc_destroy(c);
            return rc2;
        }
    }
    const double stmax = rd->stmax > 0.0 ? rd->stmax : 10.0;
    c->cap = std::max(1, (int)(rd->nwalk * stmax));
    if (upload_kv(c) || upload_tables(c)) {
        dmc_destroy(c);
        return DMC_ERR_CUDA;
    }
    const int nest = c->P.nest;
    if (c->st[0].alloc(c->cap, c->n3) || c->st[1].alloc(c->cap, c->n3) || c->est.alloc((size_t)c->cap * nest * 2) ||
        c->counts.alloc(c->cap) || c->offs.alloc(c->cap + 1) || c->irn1.alloc(c->cap) ||
        c->wtisto.alloc(DMC_WTISTO) || c->vb.alloc(6 * DMC_NEST_MAX) || c->estpart.alloc(kEstBlocks * 3 * DMC_NEST_MAX) ||
        c->estticket.alloc(1) || c->status.alloc(1) ||
        c->pop.alloc(4) || c->popf.alloc(1) ||
        c->psteps.alloc(1)) {
        dmc_destroy(c);
        return DMC_ERR_NOMEM;
    }
    cudaMemset(c->wtisto.p, 0, DMC_WTISTO * sizeof(unsigned long long));
    c->vb2 = c->vb.p + DMC_NEST_MAX;
    c->wb = c->vb.p + 2 * DMC_NEST_MAX;
    c->vbc = c->vb.p + 3 * DMC_NEST_MAX;
    cudaMemset(c->vb.p, 0, 6 * DMC_NEST_MAX * sizeof(double));
    cudaMemset(c->estticket.p, 0, sizeof(unsigned int));
    cudaMemset(c->status.p, 0, sizeof(int));
    cudaMemset(c->pop.p, 0, 4 * sizeof(int));
    cudaMemset(c->psteps.p, 0, sizeof(unsigned long long));
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        dmc_destroy(c);
        return DMC_ERR_CUDA;
    }
    *out = c;
    return DMC_OK;
}

int dmc_destroy(dmc_ctx* c)
{
    if (!c) return DMC_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    c->kv.release(); c->tud.release(); c->tss.release(); c->kv_mp.release(); c->tud_mp.release();
    c->tss_mp.release(); c->jumpA.release(); c->jumpC.release(); c->jq.release();
    c->gscratch.release(); c->st[0].release(); c->st[1].release(); c->est.release(); c->counts.release();
    c->offs.release(); c->status.release(); c->wstat.release(); c->irn1.release(); c->wtisto.release(); c->vb.release();
    c->bx.release(); c->bpsil.release(); c->bdpsi.release();
    c->bd2psi.release(); c->bv.release(); c->bvext.release(); c->bpsigl.release(); c->bdpsig.release();
    c->bd2psig.release(); c->bsinv.release(); c->bis.release(); c->flush.release();
    for (auto& a : c->gexec)
        for (auto& b : a)
            for (auto& g : b)
                if (g) cudaGraphExecDestroy(g);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return DMC_OK;
}

int dmc_get_info(const dmc_ctx* c, dmc_info* o)
{
    if (!c || !o) return DMC_ERR_INVALID;
    std::memset(o, 0, sizeof *o);
    const Setup& S = c->S;
    o->npart = S.npart; o->nup = S.nup; o->ndn = S.ndn; o->npair = S.npair; o->nexup = S.nexup;
    o->nexdn = S.nexdn; o->nd = S.nd; o->nk = S.nk; o->ncol = S.ncol; o->ntab = S.ntab; o->capacity = c->cap;
    o->nest = c->P.nest; o->el = S.el; o->eunit = S.eunit; o->nfac = S.nfac; o->etrial = S.etrial;
    o->sigma[0] = S.sigma[0]; o->sigma[1] = S.sigma[1];
    size_t bytes = 0;
    bytes += 2 * ((size_t)c->cap * (3 * c->n3 + 12) * 8 + (size_t)c->cap * 16);
    bytes += (size_t)(S.ntab + 1) * (sizeof(TabUD) + sizeof(TabSS));
    bytes += c->gscratch.n * 8 + c->est.n * 8;
    o->device_bytes = (int64_t)bytes;
    return DMC_OK;
}

int dmc_get_table(const dmc_ctx* c, int which, double* out, int n)
{
    if (!c || !out) return DMC_ERR_INVALID;
    const Setup& S = c->S;
    const int nt = S.ntab + 1;
    auto two = [&](const std::vector<double>* t) {
        if (n < 2 * nt) return DMC_ERR_INVALID;
        for (int ic = 0; ic < 2; ++ic) std::memcpy(out + ic * nt, t[ic].data(), nt * sizeof(double));
        return DMC_OK;
    };
    auto one = [&](const std::vector<double>& t) {
        if (n < nt) return DMC_ERR_INVALID;
        std::memcpy(out, t.data(), nt * sizeof(double));
        return DMC_OK;
    };
    switch (which) {
    case 0: return two(S.utab);
    case 1: return two(S.dutab);
    case 2: return two(S.d2utab);
    case 3: return two(S.vtab);
    case 4: return one(S.btab);
    case 5: return one(S.dbtab);
    case 6: return one(S.d2btab);
    case 7:
        if (n < 3 * S.nk) return DMC_ERR_INVALID;
        for (int q = 0; q < S.nk; ++q)
            for (int k = 0; k < 3; ++k) out[3 * q + k] = S.kv[q].k[k];
        return DMC_OK;
    case 8:
        if (n < S.nk) return DMC_ERR_INVALID;
        for (int q = 0; q < S.nk; ++q) out[q] = S.kv[q].k2;
        return DMC_OK;
    case 9:
        if (n < S.norb) return DMC_ERR_INVALID;
        for (int q = 0; q < S.norb; ++q) out[q] = S.numsh[q];
        return DMC_OK;
    case 10:
        if (n < S.norb) return DMC_ERR_INVALID;
        for (int q = 0; q < S.norb; ++q) out[q] = S.vorb[q];
        return DMC_OK;
    case 11:
        if (n < 2) return DMC_ERR_INVALID;
        out[0] = S.jbeta;
        out[1] = S.jgamma;
        return DMC_OK;
    case 12:
        if (n < 3) return DMC_ERR_INVALID;
        out[0] = S.bfact;
        out[1] = S.bbeta;
        out[2] = S.dbeta;
        return DMC_OK;
    }
    return DMC_ERR_INVALID;
}

int dmc_set_jastrow_spline(dmc_ctx* c, const double* knots, int nknots)
{
    if (!c) return DMC_ERR_INVALID;
    int rc = c->S.set_jastrow_spline(knots, nknots, c->err);
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->stream));
    // the spline reaches L/2: the mixed path keeps the whole up-down Jastrow
    // in double-float (no zero tail beyond the healing distance)
    c->P.ntab0 = nknots > 0 ? c->S.ntab : c->S.ntab0;
    return upload_tables(c);
}

int dmc_get_jastrow_spline(const dmc_ctx* c, double* knots, int cap, int* nknots)
{
    if (!c || !nknots) return DMC_ERR_INVALID;
    const int n = (int)c->S.jknots.size();
    *nknots = n;
    if (n > 0 && (!knots || cap < n)) return DMC_ERR_INVALID;
    for (int k = 0; k < n; ++k) knots[k] = c->S.jknots[k];
    return DMC_OK;
}

int dmc_set_vorb(dmc_ctx* c, const double* vorb, int norb)
{
    if (!c || !vorb) return DMC_ERR_INVALID;
    int rc = c->S.set_vorb(vorb, norb, c->err);
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->stream));
    return upload_kv(c);
}

int dmc_hpsi_batch(dmc_ctx* c, int nw, const double* x, double* psil, int* is, double* dpsi, double* d2psi,
                   double* v, double* vext, double* psigl, double* dpsig, double* d2psig)
{
    return batch_eval(c, MODE_HPSI, nw, x, psil, is, dpsi, d2psi, v, vext, psigl, dpsig, d2psig, nullptr);
}

int dmc_hpsi_device(dmc_ctx* c, int nw, const double* x, double* psil, int* is, double* dpsi, double* d2psi,
                    double* v, double* vext, double* psigl, double* dpsig, double* d2psig, void* stream)
{
    if (!c || nw < 0 || (nw > 0 && !x)) return DMC_ERR_INVALID;
    return run_eval(c, MODE_HPSI, nw, x, psil, is, dpsi, d2psi, v, vext, psigl, dpsig, d2psig, nullptr,
                    (cudaStream_t)stream);
}

int dmc_bcs_batch(dmc_ctx* c, int nw, const double* x, double* phil, int* is, double* dphi, double* d2phi,
                  double* smati)
{
    return batch_eval(c, MODE_BCS, nw, x, phil, is, dphi, d2phi, nullptr, nullptr, nullptr, nullptr, nullptr,
                      smati);
}

int dmc_getphi_batch(dmc_ctx* c, int nw, const double* x, double* u, double* du, double* d2u, double* v)
{
    return batch_eval(c, MODE_GETPHI, nw, x, u, nullptr, du, d2u, v, nullptr, nullptr, nullptr, nullptr, nullptr);
}

int dmc_matinv_batch(dmc_ctx* c, int n, int nb, double* a, double* detl, int* is)
{
    if (!c || n < 1 || n > 2 * DMC_MAX_PART || nb < 0 || (nb > 0 && (!a || !detl || !is)))
        return fail(c, DMC_ERR_INVALID, "bad matinv arguments");
    if (nb == 0) return DMC_OK;
    const int fits = matinv_fits(n);
    if (fits < 0) return fail(c, DMC_ERR_CUDA, "matinv: device query");
    if (!fits) return fail(c, DMC_ERR_UNSUPPORTED, "matinv: the matrix does not fit one CTA's shared memory");
    const size_t n2 = (size_t)n * n;
    DevBuf<double> da, dd;
    DevBuf<int> di;
    CK(da.alloc(nb * n2));
    CK(dd.alloc(nb));
    CK(di.alloc(nb));
    CK(cudaMemcpyAsync(da.p, a, nb * n2 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    cudaError_t e = launch_matinv(da.p, da.p, dd.p, di.p, n, nb, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(a, da.p, nb * n2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(detl, dd.p, nb * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(is, di.p, nb * sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    da.release();
    dd.release();
    di.release();
    if (e != cudaSuccess) return cuda_fail(c, e, "matinv");
    return DMC_OK;
}

// ---- walker population ----------------------------------------------------

int dmc_init_walkers(dmc_ctx* c)
{
    if (!c) return DMC_ERR_INVALID;
    const int np = c->S.npart, n3 = c->n3, nw = c->rd.nwalk;
    if (nw > c->cap) return fail(c, DMC_ERR_OVERFLOW, "nwalk exceeds the stack capacity");
    // dmcbcs.f90:238-282: one random configuration, then each walker is the
    // previous one with npart random transpositions; the walker stream seeds
    // follow one ran2 chain from the input seed.
    unsigned long long gs = (unsigned long long)c->rd.seed & kMask48;
    unsigned long long chain = (unsigned long long)c->rd.seed;
    auto ran1 = [&](unsigned long long& s) {
        s = (kMult1 * (s & kMask48) + kAdd1) & kMask48;
        return (double)(s | 1ull) * (1.0 / 281474976710656.0);
    };
    std::vector<double> x(n3), X((size_t)nw * n3), W(nw, 1.0), Z(nw, 0.0);
    std::vector<unsigned long long> irn(nw);
    for (int k = 0; k < n3; ++k) x[k] = c->S.el * (ran1(gs) - 0.5);
    for (int w = 0; w < nw; ++w) {
        for (int i = 0; i < np; ++i) {
            const double r = ran1(gs);
            const int j = (int)(np * r + 1) - 1;
            for (int k = 0; k < 3; ++k) std::swap(x[3 * i + k], x[3 * j + k]);
        }
        std::memcpy(&X[(size_t)w * n3], x.data(), n3 * sizeof(double));
        chain = (kMult2 * (chain & kMask48) + kAdd2) & kMask48;   // ran2 on the walker seed
        irn[w] = chain;
    }
    StackBufs& s = c->st[c->istin];
    CK(cudaMemcpy(s.x.p, X.data(), X.size() * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s.weight.p, W.data(), nw * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s.psil0.p, Z.data(), nw * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s.psigl0.p, Z.data(), nw * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s.irn.p, irn.data(), nw * sizeof(unsigned long long), cudaMemcpyHostToDevice));
    c->n = nw;
    c->n_stale = false;
    return DMC_OK;
}

int dmc_load_walkers(dmc_ctx* c, const dmc_walkers* w)
{
    if (!c || !w || w->n < 0 || (w->n > 0 && (!w->x || !w->irn))) return DMC_ERR_INVALID;
    const int n = w->n;
    if (n > c->cap) return fail(c, DMC_ERR_OVERFLOW, "more walkers than the stack capacity");
    StackBufs& s = c->st[c->istin];
    std::vector<double> ones(n, 1.0), zeros(n, 0.0);
    CK(cudaMemcpy(s.x.p, w->x, (size_t)n * c->n3 * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s.weight.p, w->weight ? w->weight : ones.data(), n * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s.psil0.p, w->psil0 ? w->psil0 : zeros.data(), n * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s.psigl0.p, w->psigl0 ? w->psigl0 : zeros.data(), n * sizeof(double), cudaMemcpyHostToDevice));
    std::vector<unsigned long long> irn(n);
    for (int k = 0; k < n; ++k) irn[k] = (unsigned long long)w->irn[k];
    CK(cudaMemcpy(s.irn.p, irn.data(), n * sizeof(unsigned long long), cudaMemcpyHostToDevice));
    c->n = n;
    c->n_stale = false;
    return DMC_OK;
}

int dmc_save_walkers(dmc_ctx* c, const char* path, double tau)
{
    if (!c || !path) return DMC_ERR_INVALID;
    if (c) {
        const int rs = sync_n(c);
        if (rs) return rs;
    }
    const int n = c->n;
    const size_t n3 = (size_t)c->n3;
    std::vector<double> x(std::max<size_t>(1, n * n3)), w(n + 1), pl(n + 1), pg(n + 1);
    std::vector<int64_t> irn(n + 1);
    dmc_walkers h;
    std::memset(&h, 0, sizeof h);
    h.n = n;
    h.x = x.data();
    h.weight = w.data();
    h.psil = pl.data();
    h.psigl = pg.data();
    h.irn = irn.data();
    int rc = dmc_get_walkers(c, &h);
    if (rc) return rc;
    // pop order: the top of the stack (last index) first
    std::vector<double> xr(x.size()), wr(n + 1), plr(n + 1), pgr(n + 1);
    std::vector<int64_t> ir(n + 1);
    for (int k = 0; k < n; ++k) {
        const int j = n - 1 - k;
        std::copy(x.begin() + (size_t)j * n3, x.begin() + (size_t)(j + 1) * n3, xr.begin() + (size_t)k * n3);
        wr[k] = w[j];
        plr[k] = pl[j];
        pgr[k] = pg[j];
        ir[k] = irn[j];
    }
    rc = dmc_fort9_write(path, c->S.npart, n, xr.data(), wr.data(), plr.data(), pgr.data(), ir.data(), tau);
    if (rc) return fail(c, rc, std::string("cannot write ") + path);
    return DMC_OK;
}

int dmc_restore_walkers(dmc_ctx* c, const char* path, double* tau)
{
    if (!c || !path) return DMC_ERR_INVALID;
    const size_t n3 = (size_t)c->n3;
    int n = 0;
    double t = 0.0;
    int rc = dmc_fort9_read(path, c->S.npart, 0, nullptr, nullptr, nullptr, nullptr, nullptr, &n, &t);
    if (rc != DMC_OK && rc != DMC_ERR_OVERFLOW) return fail(c, DMC_ERR_INVALID, std::string("cannot read ") + path);
    if (n > c->cap) return fail(c, DMC_ERR_OVERFLOW, "more walkers in the file than the stack capacity");
    std::vector<double> x(std::max<size_t>(1, n * n3)), w(n + 1), p0(n + 1), pg0(n + 1);
    std::vector<int64_t> irn(n + 1);
    rc = dmc_fort9_read(path, c->S.npart, n, x.data(), w.data(), p0.data(), pg0.data(), irn.data(), &n, &t);
    if (rc) return fail(c, DMC_ERR_INVALID, std::string("malformed walker file ") + path);
    dmc_walkers h;
    std::memset(&h, 0, sizeof h);
    h.n = n;
    h.x = x.data();
    h.weight = w.data();
    h.psil0 = p0.data();
    h.psigl0 = pg0.data();
    h.irn = irn.data();
    rc = dmc_load_walkers(c, &h);
    if (rc) return rc;
    if (tau) *tau = t;
    return DMC_OK;
}

int dmc_get_status(dmc_ctx* c, int* flags, int clear)
{
    if (!c || !flags) return DMC_ERR_INVALID;
    int d = 0;
    CK(cudaMemcpyAsync(&d, c->status.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    *flags = d | c->hstatus;
    if (clear) {
        CK(cudaMemsetAsync(c->status.p, 0, sizeof(int), c->stream));
        CK(cudaStreamSynchronize(c->stream));
        c->hstatus = 0;
    }
    return DMC_OK;
}

int dmc_walker_status(dmc_ctx* c, int nw, int* status)
{
    if (!c || nw < 0 || (nw > 0 && !status)) return DMC_ERR_INVALID;
    if (nw > c->wstat_n) return fail(c, DMC_ERR_INVALID, "more walkers than the last batched evaluation");
    if (nw == 0) return DMC_OK;
    CK(cudaMemcpyAsync(status, c->wstat.p, nw * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return DMC_OK;
}

int dmc_num_walkers(dmc_ctx* c, int* n)
{
    if (!c || !n) return DMC_ERR_INVALID;
    if (c) {
        const int rs = sync_n(c);
        if (rs) return rs;
    }
    *n = c->n;
    return DMC_OK;
}

// The address under which the context's device reads a caller's array:
// pinned memory (mapped into the device's address space), managed memory,
// or device memory of this same device.  nullptr otherwise -- pageable
// memory, and device memory of another GPU (which the walker kernel cannot
// read without peer access) -- so the caller's arrays then go through
// copies.
static void* device_view(const void* p, int device)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost) {
        // the mapped address is the one of the current device (the
        // context's device is current during every call)
        int cur = -1;
        if (cudaGetDevice(&cur) != cudaSuccess || cur != device) return nullptr;
        return a.devicePointer;
    }
    if (a.type == cudaMemoryTypeManaged) return const_cast<void*>(p);
    if (a.type == cudaMemoryTypeDevice && a.device == device) return const_cast<void*>(p);
    return nullptr;
}

// Device views of every non-null field of w; false when one of them is not
// addressable from the device.  Looked up on every call: memory freed and
// allocated again at the same address may be of another kind.
static bool host_views(dmc_ctx* c, const dmc_walkers* w, HostWalkers* h)
{
    void* key[15] = {w->x, w->dpsi, w->dpsig, w->psil, w->psigl, w->d2psi, w->d2psig, w->v, w->vext, w->weight,
                     w->psil0, w->psigl0, w->wt0, w->is, w->irn};
    void* view[15];
    for (int k = 0; k < 15; ++k) {
        view[k] = key[k] ? device_view(key[k], c->device) : nullptr;
        if (key[k] && !view[k]) return false;
    }
    double** d[13] = {&h->x, &h->dpsi, &h->dpsig, &h->psil, &h->psigl, &h->d2psi, &h->d2psig, &h->v, &h->vext,
                      &h->weight, &h->psil0, &h->psigl0, &h->wt0};
    for (int k = 0; k < 13; ++k) *d[k] = static_cast<double*>(view[k]);
    h->is = static_cast<int*>(view[13]);
    h->irn = static_cast<long long*>(view[14]);
    return true;
}

int dmc_get_walkers(dmc_ctx* c, dmc_walkers* w)
{
    if (!c || !w) return DMC_ERR_INVALID;
    if (c) {
        const int rs = sync_n(c);
        if (rs) return rs;
    }
    if (w->n < c->n) {
        w->n = c->n;
        return fail(c, DMC_ERR_INVALID, "walker arrays too small");
    }
    const int n = c->n;
    const size_t n3 = (size_t)c->n3;
    StackBufs& s = c->st[c->istin];
    HostWalkers hv;
    if (n > 0 && host_views(c, w, &hv)) {
        // one launch writes every field into the caller's mapped arrays
        CK(launch_walkers_get(s.view(), hv, n, (int)n3, 8 * c->nsm, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        w->n = n;
        return DMC_OK;
    }
    CK(cudaStreamSynchronize(c->stream));
    auto D = [&](void* h, const void* d, size_t bytes) {
        return h ? cudaMemcpy(h, d, bytes, cudaMemcpyDeviceToHost) : cudaSuccess;
    };
    CK(D(w->x, s.x.p, n * n3 * 8));
    CK(D(w->dpsi, s.dpsi.p, n * n3 * 8));
    CK(D(w->dpsig, s.dpsig.p, n * n3 * 8));
    CK(D(w->psil, s.psil.p, n * 8));
    CK(D(w->psigl, s.psigl.p, n * 8));
    CK(D(w->d2psi, s.d2psi.p, n * 8));
    CK(D(w->d2psig, s.d2psig.p, n * 8));
    CK(D(w->v, s.v.p, n * 8));
    CK(D(w->vext, s.vext.p, n * 8));
    CK(D(w->weight, s.weight.p, n * 8));
    CK(D(w->psil0, s.psil0.p, n * 8));
    CK(D(w->psigl0, s.psigl0.p, n * 8));
    CK(D(w->is, s.is.p, n * sizeof(int)));
    if (w->irn) {
        std::vector<unsigned long long> t(n);
        CK(cudaMemcpy(t.data(), s.irn.p, n * 8, cudaMemcpyDeviceToHost));
        for (int k = 0; k < n; ++k) w->irn[k] = (int64_t)t[k];
    }
    if (w->wt0) {
        std::vector<float> t(n);
        CK(cudaMemcpy(t.data(), s.wt0.p, n * sizeof(float), cudaMemcpyDeviceToHost));
        for (int k = 0; k < n; ++k) w->wt0[k] = t[k];
    }
    w->n = n;
    return DMC_OK;
}

static int reverse_stacks(dmc_ctx* c)
{
    CK(launch_reverse(c->st[c->istin].view(), c->st[1 - c->istin].view(), c->n, c->n3, c->stream));
    c->istin = 1 - c->istin;
    return DMC_OK;
}

int dmc_initial_eval(dmc_ctx* c, double* sums)
{
    if (!c) return DMC_ERR_INVALID;
    if (c) {
        const int rs = sync_n(c);
        if (rs) return rs;
    }
    const int n = c->n;
    StackBufs& s = c->st[c->istin];
    int rc = run_eval(c, MODE_HPSI, n, s.x.p, s.psil.p, s.is.p, s.dpsi.p, s.d2psi.p, s.v.p, s.vext.p, s.psigl.p,
                      s.dpsig.p, s.d2psig.p, nullptr, c->stream);
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->stream));
    std::vector<double> psil(n), psigl(n), d2psi(n), d2psig(n), v(n), w(n, 1.0);
    std::vector<int> is(n);
    std::vector<float> wt0(n);
    CK(cudaMemcpy(psil.data(), s.psil.p, n * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(psigl.data(), s.psigl.p, n * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(d2psi.data(), s.d2psi.p, n * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(d2psig.data(), s.d2psig.p, n * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(v.data(), s.v.p, n * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(is.data(), s.is.p, n * sizeof(int), cudaMemcpyDeviceToHost));
    // dmcbcs.f90:316-345 in pop order (top of the stack first)
    const double hb = c->S.hbar, eu = c->S.eunit, np = c->S.npart;
    double a[9] = {0, 0, 0, 0, 0, 0, 0, (double)n, 0};
    double e1[3] = {0, 0, 0};
    const bool dmc = c->rd.idmc != -1 && c->rd.idmc != 0;
    for (int k = 0; k < n; ++k) {
        const int j = n - 1 - k;
        const double el = (-hb * d2psi[j] + v[j]) / eu / np;
        a[0] += el;
        a[1] += el * el;
        a[2] += std::exp(2.0 * psil[j]);
        a[3] += std::exp(4.0 * psil[j]);
        a[4] += std::exp(2.0 * psigl[j]);
        a[5] += std::exp(4.0 * psigl[j]);
        a[6] += 1.0 * is[j];
        a[8] += 1.0;
        wt0[j] = (float)is[j];
        if (dmc) {
            const double wt = std::exp(-(-hb * d2psig[j] + v[j] - c->S.etrial) * c->rd.dt);
            e1[0] += el * wt;
            e1[1] += el * el * wt;
            e1[2] += wt;
        }
    }
    CK(cudaMemcpy(s.weight.p, w.data(), n * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s.wt0.p, wt0.data(), n * sizeof(float), cudaMemcpyHostToDevice));
    if (sums) {
        std::memcpy(sums, a, sizeof a);
        if (dmc && e1[2] != 0.0) {
            const double vn = e1[0] / e1[2], v2 = e1[1] / e1[2];
            sums[9] = vn;
            sums[10] = std::sqrt(std::fabs(v2 - vn * vn) / e1[2]);
        } else {
            sums[9] = sums[10] = 0.0;
        }
    }
    // the initial pass pops every walker once; at tau = 0 a DMC run pops
    // them once more for the operators (dmcbcs.f90:385-392)
    rc = reverse_stacks(c);
    if (rc) return rc;
    if (dmc) {
        rc = reverse_stacks(c);
        if (rc) return rc;
    }
    CK(cudaMemsetAsync(c->vb.p, 0, 6 * DMC_NEST_MAX * 8, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return DMC_OK;
}

int dmc_step(dmc_ctx* c, int opcomp)
{
    if (!c) return DMC_ERR_INVALID;
    if (c) {
        const int rs = sync_n(c);
        if (rs) return rs;
    }
    const int n = c->n;
    if (n == 0) return fail(c, DMC_ERR_EMPTY, "no walkers");
    KernelArgs a = base_args(c);
    a.mode = MODE_STEP;
    a.nw = n;
    a.opcomp = opcomp ? 1 : 0;
    a.in = c->st[c->istin].view();
    a.out = c->st[1 - c->istin].view();
    a.est = c->est.p;
    // DMC without Metropolis keeps every proposal: the weights and estimator
    // records are computed one thread per walker after the walker kernel
    a.defer = (c->P.idmc == 1 || c->P.idmc == -2) ? 1 : 0;
    CK(cudaEventRecord(c->ev0, c->stream));
    CK(launch_walker(c->P, a, c->L, grid_for(c, n), c->stream, c->precision == DMC_PREC_MIXED));
    if (a.defer) CK(launch_step_decide(c->P, a, c->stream));
    CK(cudaEventRecord(c->ev1, c->stream));
    CK(launch_estimators(c->est.p, n, c->P.nest, c->vb.p, c->vb2, c->wb, c->vbc, c->estpart.p, c->estticket.p,
                         c->stream));
    c->launches += a.defer ? 3 : 2;
    c->istin = 1 - c->istin;
    return DMC_OK;
}

int dmc_last_step_ms(dmc_ctx* c, double* ms)
{
    if (!c || !ms) return DMC_ERR_INVALID;
    CK(cudaEventSynchronize(c->ev1));
    float f = 0.f;
    CK(cudaEventElapsedTime(&f, c->ev0, c->ev1));
    *ms = f;
    return DMC_OK;
}

int dmc_branch(dmc_ctx* c, double factor)
{
    if (!c) return DMC_ERR_INVALID;
    if (c) {
        const int rs = sync_n(c);
        if (rs) return rs;
    }
    const int n = c->n;
    StackBufs& in = c->st[c->istin];
    StackBufs& out = c->st[1 - c->istin];
    CK(launch_branch(in.view(), out.view(), n, c->n3, c->cap, factor, c->counts.p, c->offs.p, c->irn1.p,
                     c->wtisto.p, c->stream));
    if (n > 0) c->launches += 3;
    int total = 0;
    if (n > 0) {
        CK(cudaMemcpyAsync(&total, c->offs.p + n, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    c->istin = 1 - c->istin;
    if (total > c->cap) {
        c->n = c->cap;
        c->n_stale = false;
        c->hstatus |= DMC_STATUS_OVERFLOW;
        return fail(c, DMC_ERR_OVERFLOW, "stack overflow in branch");
    }
    c->n = total;
    c->n_stale = false;
    return DMC_OK;
}

// One generation enqueued with the walker count on the device (no host
// round trip): the move of every walker, its weights and estimator sums,
// the branch (DMC) and the population control of dmcbcs.f90 as a
// conditional second pass.  The stack and count slots swap a fixed number
// of times, so the same launch sequence can be captured as a graph.
// The parity changes of one generation, as gen_async makes them: the move
// and the DMC branch swap the stacks, both branch passes swap the count slots.
static void advance_parities(dmc_ctx* c)
{
    const int idmc = c->rd.idmc;
    const int nbr = (idmc > 0 || idmc == -2) ? 1 : 0;
    c->istin = (c->istin + 1 + nbr) & 1;
    c->pcur = (c->pcur + nbr + 1) & 1;
}

static int gen_async(dmc_ctx* c, int opcomp, int* nlaunch, const DevStack* in_host = nullptr,
                     const double* wt0_host = nullptr)
{
    if (!c->n_stale) {   // the host count is current: hand it to the device
        CK(cudaMemcpyAsync(c->pop.p + c->pcur, &c->n, sizeof(int), cudaMemcpyHostToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        c->n_stale = true;
    }
    int nl = 0;
    KernelArgs a = base_args(c);
    a.mode = MODE_STEP;
    a.nw = c->cap;                    // bound; the count is read from a.pn
    a.pn = c->pop.p + c->pcur;
    a.opcomp = opcomp ? 1 : 0;
    a.in = in_host ? *in_host : c->st[c->istin].view();
    a.in_wt0d = wt0_host;
    a.out = c->st[1 - c->istin].view();
    a.est = c->est.p;
    a.defer = (c->P.idmc == 1 || c->P.idmc == -2) ? 1 : 0;
    // the move itself, for dmc_last_step_ms (in a capture the records become
    // external event nodes of the graph)
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(c->stream, &cap));
    const unsigned evflags = cap == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
    CK(cudaEventRecordWithFlags(c->ev0, c->stream, evflags));
    CK(launch_walker(c->P, a, c->L, c->grid, c->stream, c->precision == DMC_PREC_MIXED));
    ++nl;
    if (a.defer) {
        CK(launch_step_decide(c->P, a, c->stream));
        ++nl;
    }
    CK(cudaEventRecordWithFlags(c->ev1, c->stream, evflags));
    CK(launch_estimators(c->est.p, 0, c->P.nest, c->vb.p, c->vb2, c->wb, c->vbc, c->estpart.p, c->estticket.p,
                         c->stream, a.pn, c->psteps.p));
    ++nl;
    c->istin = 1 - c->istin;
    int* pop = c->pop.p;
    auto branch = [&](const int* need, const double* fac) -> int {
        CK(launch_branch_dev(c->st[c->istin].view(), c->st[1 - c->istin].view(), pop + c->pcur, pop + (1 - c->pcur),
                             need, fac, pop + 2, c->n3, c->cap, c->nsm, c->counts.p, c->offs.p, c->irn1.p,
                             c->wtisto.p, c->stream));
        nl += need ? 4 : 3;
        if (!need) c->istin = 1 - c->istin;   // the conditional pass leaves the walkers in place
        c->pcur = 1 - c->pcur;
        return DMC_OK;
    };
    const int idmc = c->rd.idmc;
    if (idmc > 0 || idmc == -2) {
        const int rc = branch(nullptr, nullptr);
        if (rc) return rc;
    }
    CK(launch_popctl(pop + c->pcur, (double)c->rd.nwalk, c->rd.popup, c->rd.popdn, pop + 3, c->popf.p, pop + 2,
                     c->stream));
    ++nl;
    const int rc = branch(pop + 3, c->popf.p);
    if (rc) return rc;
    c->launches += nl;
    if (nlaunch) *nlaunch = nl;
    return DMC_OK;
}

// Drop the captured generations when anything they baked in changed.
static void check_graphs(dmc_ctx* c)
{
    const KernelArgs A = base_args(c);
    if (c->gprec == c->precision && c->glayout == c->layout_gen && std::memcmp(&c->gP, &c->P, sizeof c->P) == 0 &&
        std::memcmp(&c->gA, &A, sizeof A) == 0)
        return;
    for (auto& a : c->gexec)
        for (auto& b : a)
            for (auto& g : b)
                if (g) {
                    cudaGraphExecDestroy(g);
                    g = nullptr;
                }
    std::memcpy(&c->gP, &c->P, sizeof c->P);
    std::memcpy(&c->gA, &A, sizeof A);
    c->gprec = c->precision;
    c->glayout = c->layout_gen;
}

// One generation as a captured graph, one per (opcomp, stack parity,
// count-slot parity) at its start, captured on first use.
static int gen_graph(dmc_ctx* c, int opcomp, int* nlaunch)
{
    if (!c->n_stale) {   // the host count is current: hand it to the device
        CK(cudaMemcpyAsync(c->pop.p + c->pcur, &c->n, sizeof(int), cudaMemcpyHostToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        c->n_stale = true;
    }
    check_graphs(c);
    const int op = opcomp ? 1 : 0, pi = c->istin, pc = c->pcur;
    cudaGraphExec_t& ex = c->gexec[op][pi][pc];
    if (!ex) {
        cudaGraph_t graph = nullptr;
        const int64_t l0 = c->launches;
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        int nl = 0;
        int rc = gen_async(c, op, &nl);
        const cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
        if (rc == DMC_OK && ce != cudaSuccess) rc = cuda_fail(c, ce, "generation capture");
        if (rc == DMC_OK) {
            const cudaError_t ie = cudaGraphInstantiate(&ex, graph, 0);
            if (ie != cudaSuccess) rc = cuda_fail(c, ie, "generation graph");
        }
        if (graph) cudaGraphDestroy(graph);
        // the capture only recorded the launches: restore the parities
        c->istin = pi;
        c->pcur = pc;
        c->launches = l0;
        c->gnl[op][pi][pc] = nl;
        if (rc) return rc;
    }
    CK(cudaGraphLaunch(ex, c->stream));
    advance_parities(c);
    c->launches += c->gnl[op][pi][pc];
    if (nlaunch) *nlaunch = c->gnl[op][pi][pc];
    return DMC_OK;
}

int dmc_tune_layout(dmc_ctx* c, int passes, int* kind_out, double* ms_out)
{
    if (!c || passes < 1) return DMC_ERR_INVALID;
    int rc = sync_n(c);
    if (rc) return rc;
    if (c->n == 0) return fail(c, DMC_ERR_EMPTY, "no walkers to time the layouts on");
    int optin = 0;
    CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
    CK(cudaStreamSynchronize(c->stream));
    double best = 0.0;
    int best_kind = -1, best_psm = 1;
    SmemLayout bestL{};
    std::vector<std::array<int, 4>> seen;   // (threads, CTAs per SM, union on chip, beta data on chip)
    for (int kind = 0; kind < LAYOUT_KINDS; ++kind) {
        SmemLayout L;
        int psm = 1;
        if (plan_layout(c, optin, kind, &L, &psm) != DMC_OK) continue;
        const std::array<int, 4> key{L.nt, psm, L.un_in_smem, L.pb_in_smem};
        if (std::find(seen.begin(), seen.end(), key) != seen.end()) continue;
        seen.push_back(key);
        rc = apply_layout(c, L, psm);
        if (rc) return rc;
        // one wavefunction evaluation of the current walkers per pass (the
        // walker state does not change), after one untimed pass
        KernelArgs a = base_args(c);
        a.mode = MODE_HPSI;
        a.nw = c->n;
        a.xin = c->st[c->istin].x.p;
        a.status = nullptr;
        const bool mixed = c->precision == DMC_PREC_MIXED;
        CK(launch_walker(c->P, a, c->L, c->grid, c->stream, mixed));
        CK(cudaEventRecord(c->ev0, c->stream));
        for (int i = 0; i < passes; ++i) CK(launch_walker(c->P, a, c->L, c->grid, c->stream, mixed));
        CK(cudaEventRecord(c->ev1, c->stream));
        CK(cudaEventSynchronize(c->ev1));
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
        const double per = ms / passes;
        if (best_kind < 0 || per < best) {
            best = per;
            best_kind = kind;
            bestL = L;
            best_psm = psm;
        }
    }
    if (best_kind < 0) return fail(c, DMC_ERR_UNSUPPORTED, "no walker layout fits");
    rc = apply_layout(c, bestL, best_psm);
    if (rc) return rc;
    if (kind_out) *kind_out = best_kind;
    if (ms_out) *ms_out = best;
    return DMC_OK;
}

int dmc_generation(dmc_ctx* c, int opcomp, int* nt)
{
    if (!c) return DMC_ERR_INVALID;
    int rc = gen_graph(c, opcomp, nullptr);
    if (rc) return rc;
    // the count (and any error of the generation) comes back only on request
    if (nt) {
        rc = sync_n(c);
        *nt = c->n;
    }
    return rc;
}

int dmc_generation_host(dmc_ctx* c, const dmc_walkers* in, dmc_walkers* out, int opcomp)
{
    if (!c || !in || !out || in->n < 0 || out->n < 0) return DMC_ERR_INVALID;
    const int n = in->n;
    if (n == 0) return fail(c, DMC_ERR_EMPTY, "no walkers");
    if (n > c->cap) return fail(c, DMC_ERR_OVERFLOW, "more walkers than the stack capacity");
    if (!in->x || !in->dpsi || !in->dpsig || !in->psil || !in->psigl || !in->d2psi || !in->d2psig || !in->v ||
        !in->vext || !in->weight || !in->psil0 || !in->psigl0 || !in->wt0 || !in->is || !in->irn)
        return fail(c, DMC_ERR_INVALID, "dmc_generation_host needs every input field");
    HostWalkers hi, ho;
    if (!host_views(c, in, &hi) || !host_views(c, out, &ho)) {
        // arrays the device cannot address: hand the population over by copies
        int rc = dmc_put_walkers(c, in);
        if (rc == DMC_OK) rc = dmc_generation(c, opcomp, nullptr);
        if (rc == DMC_OK) rc = dmc_get_walkers(c, out);
        return rc;
    }
    // the walker kernel pops the caller's population directly (device views
    // of the host arrays; wt0 converted to single precision on the device)
    const DevStack hs{hi.x, hi.dpsi, hi.dpsig, hi.psil, hi.psigl, hi.d2psi, hi.d2psig, hi.v, hi.vext, hi.weight,
                      hi.psil0, hi.psigl0, nullptr, hi.is, reinterpret_cast<unsigned long long*>(hi.irn)};
    c->n = n;   // staged by the copy below before it returns (pageable source)
    CK(cudaMemcpyAsync(c->pop.p + c->pcur, &c->n, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    c->n_stale = true;
    int rc = gen_async(c, opcomp, nullptr, &hs, hi.wt0);
    if (rc) return rc;
    // the new population into the caller's arrays, its count read on the device
    CK(launch_walkers_get(c->st[c->istin].view(), ho, 0, c->n3, 8 * c->nsm, c->stream, c->pop.p + c->pcur, out->n));
    ++c->launches;
    rc = sync_n(c);
    if (rc) return rc;
    if (c->n > out->n) {
        out->n = c->n;
        return fail(c, DMC_ERR_INVALID, "walker arrays too small");
    }
    out->n = c->n;
    return DMC_OK;
}

int dmc_zero_estimators(dmc_ctx* c)
{
    if (!c) return DMC_ERR_INVALID;
    CK(cudaMemsetAsync(c->vb.p, 0, 6 * DMC_NEST_MAX * 8, c->stream));
    return DMC_OK;
}

int dmc_get_estimators(dmc_ctx* c, double* valblk, double* valblk2, double* wtblk)
{
    if (!c || !valblk || !valblk2 || !wtblk) return DMC_ERR_INVALID;
    const int ne = c->P.nest;
    double h[6 * DMC_NEST_MAX];
    CK(cudaMemcpyAsync(h, c->vb.p, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    // the compensated sums: each block sum plus its error term
    for (int e = 0; e < ne; ++e) {
        valblk[e] = h[e] + h[3 * DMC_NEST_MAX + e];
        valblk2[e] = h[DMC_NEST_MAX + e] + h[4 * DMC_NEST_MAX + e];
        wtblk[e] = h[2 * DMC_NEST_MAX + e] + h[5 * DMC_NEST_MAX + e];
    }
    return DMC_OK;
}

int dmc_block_update(dmc_ctx* c, double* valnow, double* errnow)
{
    if (!c || !valnow || !errnow) return DMC_ERR_INVALID;
    double a[DMC_NEST_MAX], b[DMC_NEST_MAX], w[DMC_NEST_MAX];
    int rc = dmc_get_estimators(c, a, b, w);
    if (rc) return rc;
    for (int i = 0; i < c->P.nest; ++i) {
        valnow[i] = a[i] / w[i];
        const double v2 = b[i] / w[i];
        errnow[i] = std::sqrt(std::fabs(v2 - valnow[i] * valnow[i]) / w[i]);
    }
    return dmc_zero_estimators(c);
}

int dmc_get_wtisto(dmc_ctx* c, int64_t* hist)
{
    if (!c || !hist) return DMC_ERR_INVALID;
    CK(cudaStreamSynchronize(c->stream));
    std::vector<unsigned long long> h(DMC_WTISTO);
    CK(cudaMemcpy(h.data(), c->wtisto.p, DMC_WTISTO * 8, cudaMemcpyDeviceToHost));
    for (int i = 0; i < DMC_WTISTO; ++i) hist[i] = (int64_t)h[i];
    return DMC_OK;
}

// ---- single-particle moves and parameter derivatives ---------------------

static int check_moves(dmc_ctx* c, int nw, const double* x, const int* ipart, const double* d, const double* ratio)
{
    if (nw < 0 || (nw > 0 && (!x || !ipart || !d || !ratio))) return fail(c, DMC_ERR_INVALID, "bad move arguments");
    for (int w = 0; w < nw; ++w)
        if (ipart[w] < 1 || ipart[w] > c->S.npart) return fail(c, DMC_ERR_INVALID, "particle index out of range");
    return DMC_OK;
}

static int stage_moves(dmc_ctx* c, int nw, const double* x, const int* ipart, const double* d)
{
    const size_t n3 = (size_t)c->n3;
    CK(c->sx.alloc(nw * n3));
    CK(c->sip.alloc(nw));
    CK(c->sdr.alloc(3 * (size_t)nw));
    CK(c->sratio.alloc(nw));
    CK(cudaMemcpyAsync(c->sx.p, x, nw * n3 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->sip.p, ipart, nw * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->sdr.p, d, 3 * nw * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    return DMC_OK;
}

int dmc_bcsone_batch(dmc_ctx* c, int nw, const double* x, const double* smati, const int* ipart, const double* dr,
                     double* ratio)
{
    if (!c) return DMC_ERR_INVALID;
    int rc = check_moves(c, nw, x, ipart, dr, ratio);
    if (rc || nw == 0) return rc;
    if (!smati) return fail(c, DMC_ERR_INVALID, "bcsone needs the stored inverse");
    const size_t nd2 = (size_t)c->S.nd * c->S.nd;
    if ((rc = stage_moves(c, nw, x, ipart, dr))) return rc;
    CK(c->ssinv.alloc(nw * nd2));
    CK(cudaMemcpyAsync(c->ssinv.p, smati, nw * nd2 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(launch_bcsone(c->P, c->kv.p, c->tud.p, c->sx.p, c->ssinv.p, c->sip.p, c->sdr.p, c->sratio.p, nw, c->stream));
    ++c->launches;
    CK(cudaMemcpyAsync(ratio, c->sratio.p, nw * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return DMC_OK;
}

int dmc_getphione_batch(dmc_ctx* c, int nw, const double* x, const int* ipart, const double* drr, double* ratio)
{
    if (!c) return DMC_ERR_INVALID;
    int rc = check_moves(c, nw, x, ipart, drr, ratio);
    if (rc || nw == 0) return rc;
    if ((rc = stage_moves(c, nw, x, ipart, drr))) return rc;
    CK(launch_getphione(c->P, c->tud.p, c->tss.p, c->sx.p, c->sip.p, c->sdr.p, c->sratio.p, nw, c->stream));
    ++c->launches;
    CK(cudaMemcpyAsync(ratio, c->sratio.p, nw * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return DMC_OK;
}

// d log|det| / d vorb for nw device-resident configurations (FP64 inverse)
static int derbcs_device(dmc_ctx* c, int nw, const double* dx, double* dder, int stride = -1, int off = 0)
{
    const size_t nd2 = (size_t)c->S.nd * c->S.nd;
    CK(c->ssinv.alloc(nw * nd2));
    const int prec = c->precision;
    c->precision = DMC_PREC_FP64;
    int rc = run_eval(c, MODE_BCS, nw, dx, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                      nullptr, c->ssinv.p, c->stream);
    c->precision = prec;
    if (rc) return rc;
    ++c->launches;
    CK(launch_derbcs(c->P, c->kv.p, dx, c->ssinv.p, dder, nw, c->grid, c->stream, stride, off));
    ++c->launches;
    return DMC_OK;
}

int dmc_getjasder_batch(dmc_ctx* c, int nw, const double* x, double* dpsi)
{
    if (!c) return DMC_ERR_INVALID;
    if (nw < 0 || (nw > 0 && (!x || !dpsi))) return fail(c, DMC_ERR_INVALID, "bad getjasder arguments");
    if (c->S.nql == 0) return fail(c, DMC_ERR_INVALID, "the long-range Jastrow is off (numq = 0)");
    if (nw == 0) return DMC_OK;
    const size_t n3 = (size_t)c->n3;
    CK(c->sx.alloc(nw * n3));
    CK(c->sder.alloc(2 * (size_t)nw));
    CK(cudaMemcpyAsync(c->sx.p, x, nw * n3 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(launch_jasder(c->P, c->jq.p, c->sx.p, c->sder.p, nw, c->grid, c->stream, 2));
    ++c->launches;
    CK(cudaMemcpyAsync(dpsi, c->sder.p, 2 * nw * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return DMC_OK;
}

static int pgrad_nbeta(const dmc_ctx* c) { return c->P.nobeta ? 0 : 3; }
static int pgrad_nknot(const dmc_ctx* c) { return (int)c->S.jknots.size(); }
static int pgrad_np(const dmc_ctx* c) { return c->S.norb + pgrad_nbeta(c) + pgrad_nknot(c); }

// the b and d derivative tables of beta on the device (built once: b and d
// do not change during a context's life)
static int pgrad_btab(dmc_ctx* c)
{
    if (c->P.nobeta || c->pg_btab.p) return DMC_OK;
    std::vector<double> t[2][3];
    c->S.beta_param_tables(t);
    const size_t nt = (size_t)c->S.ntabb + 1;
    std::vector<PgTab> h(2 * nt);
    for (int w = 0; w < 2; ++w)
        for (size_t i = 0; i < nt; ++i) h[w * nt + i] = PgTab{t[w][0][i], t[w][1][i], t[w][2][i], 0.0};
    CK(c->pg_btab.alloc(2 * nt));
    CK(cudaMemcpy(c->pg_btab.p, h.data(), 2 * nt * sizeof(PgTab), cudaMemcpyHostToDevice));
    return DMC_OK;
}

// the Jastrow knot basis on the up-down table grid (built once: the grid
// and the knot spacing do not change during a context's life)
static int pgrad_ktab(dmc_ctx* c)
{
    if (c->S.jknots.empty() || c->pg_ktab.p) return DMC_OK;
    std::vector<double> t[3];
    c->S.knot_basis_tables(t);
    std::vector<PgTab> h(t[0].size());
    for (size_t i = 0; i < h.size(); ++i) h[i] = PgTab{t[0][i], t[1][i], t[2][i], 0.0};
    CK(c->pg_ktab.alloc(h.size()));
    CK(cudaMemcpy(c->pg_ktab.p, h.data(), h.size() * sizeof(PgTab), cudaMemcpyHostToDevice));
    return DMC_OK;
}

int dmc_param_count(const dmc_ctx* c, int* np)
{
    if (!c || !np) return DMC_ERR_INVALID;
    *np = pgrad_np(c);
    return DMC_OK;
}

// the adjoint gradients of nw walkers at device positions dx into device
// arrays dlog[nw][np], del[nw][np] (stream-ordered)
static int pgrad_device(dmc_ctx* c, int nw, const double* dx, double* dlog, double* del)
{
    const size_t n3 = (size_t)c->n3, nd2 = (size_t)c->S.nd * c->S.nd;
    const int np = pgrad_np(c);
    CK(c->pg_dpsi.alloc(nw * n3));
    CK(c->pg_dphi.alloc(nw * n3));
    CK(c->ssinv.alloc(nw * nd2));
    // the total drift, the determinant's drift and the inverse, in FP64, from
    // one evaluation
    const int prec = c->precision;
    c->precision = DMC_PREC_FP64;
    int rc = run_eval(c, MODE_HPSI, nw, dx, nullptr, nullptr, c->pg_dpsi.p, nullptr, nullptr, nullptr, nullptr,
                      nullptr, nullptr, c->ssinv.p, c->stream, c->pg_dphi.p);
    c->precision = prec;
    if (rc) return rc;
    ++c->launches;
    rc = pgrad_btab(c);
    if (rc == DMC_OK) rc = pgrad_ktab(c);
    if (rc) return rc;
    int optin = 0;
    CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
    const size_t need = pgrad_doubles(c->P);
    const int grid = pgrad_grid(c->P, nw, c->nsm, optin);
    if (grid < 1) return fail(c, DMC_ERR_CUDA, "adjoint kernel occupancy");
    double* scr = nullptr;
    if (need * 8 > (size_t)optin) {
        CK(c->pg_scr.alloc((size_t)grid * need));
        scr = c->pg_scr.p;
    }
    CK(c->pg_slice.alloc((size_t)grid * pgrad_slice_doubles(c->P)));
    CK(launch_pgrad(c->P, c->kv.p, c->tud.p, dx, c->ssinv.p, c->pg_dpsi.p, c->pg_dphi.p, dlog, del, nw, np,
                    c->S.bfact, c->pg_btab.p, c->pg_ktab.p, pgrad_nbeta(c), pgrad_nknot(c), grid, scr,
                    c->pg_slice.p, optin, c->stream));
    ++c->launches;
    return DMC_OK;
}

int dmc_param_grad(dmc_ctx* c, int nw, const double* x, double* dlogpsi, double* deloc)
{
    if (!c) return DMC_ERR_INVALID;
    if (nw < 0 || (nw > 0 && (!x || !dlogpsi || !deloc))) return fail(c, DMC_ERR_INVALID, "bad param_grad arguments");
    if (nw == 0) return DMC_OK;
    const size_t n3 = (size_t)c->n3;
    const int np = pgrad_np(c);
    CK(c->sx.alloc(nw * n3));
    CK(c->pg_dlog.alloc((size_t)nw * np));
    CK(c->pg_del.alloc((size_t)nw * np));
    CK(cudaMemcpyAsync(c->sx.p, x, nw * n3 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    int rc = pgrad_device(c, nw, c->sx.p, c->pg_dlog.p, c->pg_del.p);
    if (rc) return rc;
    CK(cudaMemcpyAsync(dlogpsi, c->pg_dlog.p, (size_t)nw * np * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(deloc, c->pg_del.p, (size_t)nw * np * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return DMC_OK;
}

int dmc_set_beta(dmc_ctx* c, double b, double d, double bfact)
{
    if (!c) return DMC_ERR_INVALID;
    if (c->P.nobeta || !(bfact > 0.0) || !(b > 0.0) || !(d > 0.0) || !std::isfinite(b * d * bfact))
        return fail(c, DMC_ERR_INVALID, "dmc_set_beta needs the beta function on and b, d, bfact > 0");
    CK(cudaStreamSynchronize(c->stream));
    c->S.set_beta(b, d, bfact);
    c->sd.bbeta = b;
    c->sd.dbeta = d;
    c->sd.bfact = bfact;
    c->pg_btab.release();   // the b and d derivative tables follow on the next gradient
    return upload_tables(c);
}

int dmc_sm_sweeps(dmc_ctx* c, int nsweeps, int recompute_every, int64_t* accepted, int64_t* moves)
{
    if (!c || nsweeps < 0 || recompute_every < 0) return DMC_ERR_INVALID;
    if (c->P.onebody || c->P.nql > 0 || c->S.a2 != 0.0)
        return fail(c, DMC_ERR_UNSUPPORTED,
                    "particle-by-particle sweeps need no one-body or long-range Jastrow and a2 = 0");
    int rc = sync_n(c);
    if (rc) return rc;
    const int n = c->n;
    if (n == 0) return fail(c, DMC_ERR_EMPTY, "no walkers");
    if (accepted) *accepted = 0;
    if (moves) *moves = 0;
    if (nsweeps == 0) return DMC_OK;   // nothing moves; the walkers keep their values
    const size_t nd2 = (size_t)c->S.nd * c->S.nd, n3 = (size_t)c->n3;
    const int nq = std::max(1, c->S.nk - 1);
    c->sm_n = 0;                       // no carried inverse until these sweeps end
    CK(c->sm_inv.alloc((size_t)n * nd2));
    CK(c->sm_tab.alloc((size_t)n * nq * c->S.npart));
    CK(c->sm_prop.alloc((size_t)n * 4 * c->S.npart));
    CK(c->sm_acc.alloc((size_t)n));
    CK(cudaMemsetAsync(c->sm_acc.p, 0, (size_t)n * sizeof(unsigned long long), c->stream));
    if (!c->sm_jA.p) {
        const int nj = 5 * c->S.npart + 1;
        std::vector<unsigned long long> A(nj), Cc(nj);
        A[0] = 1;
        Cc[0] = 0;
        for (int t = 1; t < nj; ++t) {
            A[t] = (A[t - 1] * kMult1) & kMask48;
            Cc[t] = (Cc[t - 1] * kMult1 + kAdd1) & kMask48;
        }
        CK(c->sm_jA.alloc(nj));
        CK(c->sm_jC.alloc(nj));
        CK(cudaMemcpy(c->sm_jA.p, A.data(), nj * sizeof(unsigned long long), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(c->sm_jC.p, Cc.data(), nj * sizeof(unsigned long long), cudaMemcpyHostToDevice));
    }
    StackBufs& s = c->st[c->istin];
    const DevStack view = s.view();
    // chunks of recompute_every sweeps, each starting from a fresh FP64
    // inverse of the pair matrix (the walker kernel, FP64, MODE_BCS); with
    // recompute_every = 0 only the first chunk starts from one
    const int chunk = recompute_every > 0 ? recompute_every : std::max(nsweeps, 1);
    for (int done = 0; done < nsweeps; done += chunk) {
        const int ns = std::min(chunk, nsweeps - done);
        const bool fresh = done == 0 || recompute_every > 0;
        if (fresh) {
            CK(c->ssinv.alloc((size_t)n * nd2));
            CK(c->pg_dphi.alloc((size_t)n * n3));
            const int prec = c->precision;
            c->precision = DMC_PREC_FP64;
            rc = run_eval(c, MODE_BCS, n, s.x.p, nullptr, nullptr, c->pg_dphi.p, nullptr, nullptr, nullptr, nullptr,
                          nullptr, nullptr, c->ssinv.p, c->stream);
            c->precision = prec;
            if (rc) return rc;
            ++c->launches;
        }
        CK(launch_sweeps(c->P, view, n, ns, fresh ? c->ssinv.p : nullptr, c->sm_inv.p, c->sm_tab.p, c->kv_mp.p,
                         c->tud_mp.p, c->tss_mp.p, c->sm_jA.p, c->sm_jC.p, c->sm_acc.p, c->sm_prop.p, c->stream));
        ++c->launches;
    }
    c->sm_n = n;
    // the walkers' stored evaluation at their new positions (hpsi in the
    // context's precision), so step1 and the estimators continue from them
    rc = run_eval(c, MODE_HPSI, n, s.x.p, s.psil.p, s.is.p, s.dpsi.p, s.d2psi.p, s.v.p, s.vext.p, s.psigl.p,
                  s.dpsig.p, s.d2psig.p, nullptr, c->stream);
    if (rc) return rc;
    ++c->launches;
    std::vector<unsigned long long> acc(n);
    CK(cudaMemcpyAsync(acc.data(), c->sm_acc.p, n * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    int64_t a = 0;
    for (unsigned long long v : acc) a += (int64_t)v;
    if (accepted) *accepted = a;
    if (moves) *moves = (int64_t)n * nsweeps * c->S.npart;
    return DMC_OK;
}

int dmc_sm_inverse(dmc_ctx* c, int nw, double* sinv)
{
    if (!c || nw < 0 || (nw > 0 && !sinv)) return DMC_ERR_INVALID;
    if (nw > c->sm_n) return fail(c, DMC_ERR_INVALID, "more walkers than the last sweeps carried");
    const size_t nd2 = (size_t)c->S.nd * c->S.nd;
    std::vector<float> h((size_t)nw * nd2);
    CK(cudaMemcpyAsync(h.data(), c->sm_inv.p, h.size() * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (size_t e = 0; e < h.size(); ++e) sinv[e] = h[e];
    return DMC_OK;
}

int dmc_getderbcs_batch(dmc_ctx* c, int nw, const double* x, double* dpsi)
{
    if (!c) return DMC_ERR_INVALID;
    if (nw < 0 || (nw > 0 && (!x || !dpsi))) return fail(c, DMC_ERR_INVALID, "bad getderbcs arguments");
    if (nw == 0) return DMC_OK;
    const size_t n3 = (size_t)c->n3, np = (size_t)c->S.norb;
    CK(c->sx.alloc(nw * n3));
    CK(c->sder.alloc(nw * np));
    CK(cudaMemcpyAsync(c->sx.p, x, nw * n3 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    int rc = derbcs_device(c, nw, c->sx.p, c->sder.p);
    if (rc) return rc;
    CK(cudaMemcpyAsync(dpsi, c->sder.p, nw * np * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return DMC_OK;
}

// ---- operators: operators.f90 with gofr.f90, sofq.f90, momentum3d.f90 ------

namespace {
int ops_counts(const dmc_ctx* c, int which)
{
    const OpsDev& o = c->ops.dev;
    switch (which) {
    case 0: return o.ntabg > 0 ? 3 * (o.ntabg + 1) : 0;
    case 1: return o.ntabg > 0 ? 6 * (2 * o.ntabg + 1) : 0;
    case 2: return 3 * o.nqtot;
    case 3: return o.nkv > 0 ? o.ntabk + 1 : 0;
    }
    return 0;
}
int ops_nsums(const dmc_ctx* c) { return 2 * (ops_counts(c, 0) + ops_counts(c, 1) + ops_counts(c, 2) + ops_counts(c, 3)) + 3; }
}  // namespace

int dmc_set_operators(dmc_ctx* c, int ntabg, int ntabq, int ntabk)
{
    if (!c) return DMC_ERR_INVALID;
    if (ntabg < 0 || ntabq < 0 || ntabk < 0 || ntabg > 100000) return fail(c, DMC_ERR_INVALID, "bad operator table sizes");
    if (ntabk > 80) return fail(c, DMC_ERR_UNSUPPORTED, "n(k) is built for |ik|^2 <= 80");
    auto& O = c->ops;
    // a fresh operator state; the old one's device buffers are freed
    O.~Ops();
    new (&O) dmc_ctx::Ops();
    OpsDev& o = O.dev;
    std::memset(&o, 0, sizeof o);
    const Setup& S = c->S;
    o.el = S.el;
    o.ntabg = ntabg;
    if (ntabg > 0) o.scaleg = 1.0 / (0.5 * S.el / ntabg);   // dr = el/(2 ntab), gofr.f90:33-34
    if (ntabq > 0) {
        // setupsofq (sofq.f90:17-33): kstates3d half shells, k = 0 first
        std::vector<KVec> kq;
        std::string err;
        if (ntabq > DMC_MAX_SHELLS) return fail(c, DMC_ERR_UNSUPPORTED, "too many S(q) shells");
        int rc = k_shells(S.el, ntabq, kq, O.numshq, err);
        if (rc) return fail(c, rc, err);
        o.ntabq = ntabq;
        o.nqtot = 0;
        for (int i = 0; i < ntabq; ++i) o.nqtot += O.numshq[i];
        if (o.nqtot > (int)kq.size()) return fail(c, DMC_ERR_SETUP, "S(q) k vectors");
        O.akq.resize(3 * (size_t)o.nqtot);
        for (int q = 0; q < o.nqtot; ++q)
            for (int k = 0; k < 3; ++k) O.akq[3 * q + k] = kq[q].k[k];
    }
    if (ntabk > 0) {
        // setupenk (momentum3d.f90:14-71): ik in [0, nnk]^3 with |ik|^2 <= ntab,
        // exchange-sorted by |ik|^2, grouped into shells
        o.nsamp = 10;
        o.dk = 2.0 * (4.0 * std::atan(1.0)) / S.el;
        o.nnk = (int)(std::sqrt((double)ntabk) + 1.0);
        std::vector<int> ik2;
        for (int ix = 0; ix <= o.nnk; ++ix)
            for (int iy = 0; iy <= o.nnk; ++iy)
                for (int iz = 0; iz <= o.nnk; ++iz)
                    if (ix * ix + iy * iy + iz * iz <= ntabk) {
                        ik2.push_back(ix * ix + iy * iy + iz * iz);
                        O.ik.push_back(ix);
                        O.ik.push_back(iy);
                        O.ik.push_back(iz);
                    }
        const int ntot = (int)ik2.size();
        for (int i = 1; i < ntot; ++i)
            for (int j = 0; j < i; ++j)
                if (ik2[i] < ik2[j]) {
                    std::swap(ik2[i], ik2[j]);
                    for (int k = 0; k < 3; ++k) std::swap(O.ik[3 * i + k], O.ik[3 * j + k]);
                }
        O.indk.assign(1, 0);
        O.nkk.assign(1, 1);
        for (int i = 1; i < ntot; ++i) {
            if (ik2[i] != ik2[i - 1]) {
                O.indk.push_back(i);
                O.nkk.push_back(0);
            }
            O.nkk.back()++;
        }
        o.nkv = ntot;
        o.ntabk = (int)O.nkk.size() - 1;
        if (3 * (o.nnk + 1) > 32) return fail(c, DMC_ERR_UNSUPPORTED, "n(k) table too large");
        // ran1 jump-ahead for the 3 N nsamp draws of a walker
        const int nj = 3 * S.npart * o.nsamp + 1;
        std::vector<unsigned long long> A(nj), C(nj);
        A[0] = 1;
        C[0] = 0;
        for (int t = 1; t < nj; ++t) {
            A[t] = (A[t - 1] * 44485709377909ull) & ((1ull << 48) - 1);
            C[t] = (C[t - 1] * 44485709377909ull + 96309754297ull) & ((1ull << 48) - 1);
        }
        CK(O.jA.alloc(nj));
        CK(O.jC.alloc(nj));
        CK(cudaMemcpy(O.jA.p, A.data(), nj * 8, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(O.jC.p, C.data(), nj * 8, cudaMemcpyHostToDevice));
        CK(O.ik_d.alloc(O.ik.size()));
        CK(O.indk_d.alloc(O.indk.size()));
        CK(O.nkk_d.alloc(O.nkk.size()));
        CK(cudaMemcpy(O.ik_d.p, O.ik.data(), O.ik.size() * sizeof(int), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(O.indk_d.p, O.indk.data(), O.indk.size() * sizeof(int), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(O.nkk_d.p, O.nkk.data(), O.nkk.size() * sizeof(int), cudaMemcpyHostToDevice));
        o.ik = O.ik_d.p;
        o.indk = O.indk_d.p;
        o.nkk = O.nkk_d.p;
        o.jA = O.jA.p;
        o.jC = O.jC.p;
    }
    if (o.nqtot > 0) {
        CK(O.akq_d.alloc(O.akq.size()));
        CK(cudaMemcpy(O.akq_d.p, O.akq.data(), O.akq.size() * 8, cudaMemcpyHostToDevice));
        o.akq = O.akq_d.p;
    }
    const int ns = ops_nsums(c);
    CK(O.sums.alloc(ns));
    CK(cudaMemset(O.sums.p, 0, ns * sizeof(double)));
    O.on = ntabg > 0 || ntabq > 0 || ntabk > 0;
    for (int w = 0; w < 4; ++w) {
        O.val[w].assign(ops_counts(c, w), 0.0);
        O.err[w].assign(ops_counts(c, w), 0.0);
    }
    return DMC_OK;
}

int dmc_zero_operators(dmc_ctx* c)
{
    if (!c) return DMC_ERR_INVALID;
    if (!c->ops.on) return DMC_OK;
    CK(cudaMemsetAsync(c->ops.sums.p, 0, ops_nsums(c) * sizeof(double), c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int w = 0; w < 4; ++w) {
        std::fill(c->ops.val[w].begin(), c->ops.val[w].end(), 0.0);
        std::fill(c->ops.err[w].begin(), c->ops.err[w].end(), 0.0);
    }
    return DMC_OK;
}

int dmc_add_operators(dmc_ctx* c)
{
    if (!c) return DMC_ERR_INVALID;
    if (c) {
        const int rs = sync_n(c);
        if (rs) return rs;
    }
    auto& O = c->ops;
    if (!O.on) return fail(c, DMC_ERR_INVALID, "operators are not set up");
    const int n = c->n;
    if (n > 0) {
        StackBufs& s = c->st[c->istin];
        const OpsDev& o = O.dev;
        const int ng = ops_counts(c, 0), ndh = ops_counts(c, 1), nk = ops_counts(c, 3);
        CK(O.hg.alloc((size_t)n * ng));
        CK(O.hd.alloc((size_t)n * ndh));
        CK(O.sv.alloc((size_t)n * o.nqtot * 4));
        CK(O.tk.alloc((size_t)n * nk));
        if (o.ntabg > 0 || o.nqtot > 0) {
            CK(launch_ops_walker(c->P, o, s.x.p, n, O.hg.p, O.hd.p, O.sv.p, c->grid, c->stream));
            ++c->launches;
        }
        if (o.nkv > 0) {
            // hpsi(w) of addenk leaves the walker's inverse in smatisave
            const size_t nd2 = (size_t)c->S.nd * c->S.nd;
            CK(c->ssinv.alloc(n * nd2));
            const int prec = c->precision;
            c->precision = DMC_PREC_FP64;
            int rc = run_eval(c, MODE_BCS, n, s.x.p, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                              nullptr, nullptr, c->ssinv.p, c->stream);
            c->precision = prec;
            if (rc) return rc;
            ++c->launches;
            CK(launch_ops_enk(c->P, o, c->kv.p, c->tud.p, c->tss.p, s.x.p, s.irn.p, c->ssinv.p, n, O.tk.p, c->grid,
                              c->stream));
            ++c->launches;
        }
        CK(O.wts.alloc((size_t)n));
        CK(launch_ops_reduce(o, n, s.view(), O.hg.p, O.hd.p, O.sv.p, O.tk.p, O.sums.p, O.wts.p, c->stream));
        c->launches += 2;
        int rc = reverse_stacks(c);   // the pop/push pass of dmcbcs.f90:465-473
        if (rc) return rc;
        ++c->launches;
    }
    CK(cudaStreamSynchronize(c->stream));
    return DMC_OK;
}

int dmc_update_operators(dmc_ctx* c)
{
    if (!c) return DMC_ERR_INVALID;
    auto& O = c->ops;
    if (!O.on) return fail(c, DMC_ERR_INVALID, "operators are not set up");
    const int ns = ops_nsums(c);
    std::vector<double> h(ns);
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(h.data(), O.sums.p, ns * sizeof(double), cudaMemcpyDeviceToHost));
    const double ws[4] = {h[ns - 3], h[ns - 3], h[ns - 2], h[ns - 1]};
    size_t off = 0;
    for (int w = 0; w < 4; ++w) {
        const int m = ops_counts(c, w);
        const double* now = h.data() + off;
        const double* er = now + m;
        off += 2 * (size_t)m;
        if (m == 0 || ws[w] == 0.0) continue;
        // updategofr / updatesofq / updateenk: block average and error
        const double norm = 1.0 / ws[w];
        for (int k = 0; k < m; ++k) {
            const double v = now[k] * norm;
            O.val[w][k] = v;
            O.err[w][k] = std::sqrt(std::fabs(er[k] * norm - v * v) / ws[w]);
        }
    }
    if (ws[0] != 0.0) O.totw[0] = ws[0];
    if (ws[2] != 0.0) O.totw[1] = ws[2];
    if (ws[3] != 0.0) O.totw[2] = ws[3];
    CK(cudaMemset(O.sums.p, 0, ns * sizeof(double)));
    return DMC_OK;
}

int dmc_get_operators(dmc_ctx* c, int which, double* values, double* errors, int cap, int* n, double* wsum)
{
    if (!c || which < 0 || which > 7) return DMC_ERR_INVALID;
    auto& O = c->ops;
    const int w = which & 3;
    const int m = O.on ? ops_counts(c, w) : 0;
    if (n) *n = m;
    if (m == 0 || (!values && !errors && !wsum)) return DMC_OK;
    if ((values || errors) && cap < m) return fail(c, DMC_ERR_INVALID, "operator arrays too small");
    if (which < 4) {
        if (values) std::copy(O.val[w].begin(), O.val[w].end(), values);
        if (errors) std::copy(O.err[w].begin(), O.err[w].end(), errors);
        if (wsum) *wsum = O.totw[w == 0 || w == 1 ? 0 : (w == 2 ? 1 : 2)];
        return DMC_OK;
    }
    // running sums before the block update
    const int ns = ops_nsums(c);
    std::vector<double> h(ns);
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(h.data(), O.sums.p, ns * sizeof(double), cudaMemcpyDeviceToHost));
    size_t off = 0;
    for (int k = 0; k < w; ++k) off += 2 * (size_t)ops_counts(c, k);
    if (values) std::copy(h.begin() + off, h.begin() + off + m, values);
    if (errors) std::copy(h.begin() + off + m, h.begin() + off + 2 * m, errors);
    if (wsum) *wsum = h[ns - 3 + (w == 0 || w == 1 ? 0 : (w == 2 ? 1 : 2))];
    return DMC_OK;
}

int dmc_write_operators(dmc_ctx* c, const char* dir, double tau)
{
    if (!c || !dir) return DMC_ERR_INVALID;
    auto& O = c->ops;
    if (!O.on) return fail(c, DMC_ERR_INVALID, "operators are not set up");
    const Setup& S = c->S;
    const std::string d(dir);
    auto E = [](double v) { return fortran_e(v, 15, 7); };
    const double pi = 4.0 * std::atan(1.0);
    const int npart = S.npart;
    if (O.dev.ntabg > 0) {
        // writegofr, gofr.f90:132-176 (gofr.out, rho.out)
        const int ntab = O.dev.ntabg;
        const double dr = 0.5 * S.el / ntab, rho = npart / (S.el * S.el * S.el);
        FILE* f = std::fopen((d + "/gofr.out").c_str(), "a");
        if (!f) return fail(c, DMC_ERR_INVALID, "cannot open gofr.out");
        std::fprintf(f, "# r*kF, g(r), err\n# total weight = %s\n# tau = %s\n", E(O.totw[0]).c_str(), E(tau).c_str());
        for (int i = 0; i < ntab; ++i) {
            const double r0 = i * dr, r1 = (i + 1) * dr, r = (i + 0.5) * dr;
            const double vol = 4.0 * pi * (r1 * r1 * r1 - r0 * r0 * r0) / 3.0;
            const double facl = 1.0 / (rho * npart * vol);
            std::string line = E(r);
            for (int t = 0; t < 3; ++t)
                line += E(O.val[0][t * (ntab + 1) + i] * facl) + E(O.err[0][t * (ntab + 1) + i] * facl);
            std::fprintf(f, "%s\n", line.c_str());
        }
        std::fprintf(f, " \n \n");
        std::fclose(f);
        f = std::fopen((d + "/rho.out").c_str(), "a");
        if (!f) return fail(c, DMC_ERR_INVALID, "cannot open rho.out");
        std::fprintf(f, "# r, xrhoup, err, xrhodn, err, yrhoup, err, yrhodn, err, zrhoup, err, zrhodn, err\n");
        std::fprintf(f, "# total weight = %s\n# tau = %s\n", E(O.totw[0]).c_str(), E(tau).c_str());
        const int order[6] = {0, 3, 1, 4, 2, 5};
        for (int i = -ntab; i <= ntab; ++i) {
            std::string line = E(i * dr);
            for (int t : order) {
                const size_t at = (size_t)t * (2 * ntab + 1) + (i + ntab);
                line += E(O.val[1][at] / npart) + E(O.err[1][at] / npart);
            }
            std::fprintf(f, "%s\n", line.c_str());
        }
        std::fprintf(f, " \n \n");
        std::fclose(f);
    }
    if (O.dev.ntabq > 0) {
        // writesofq, sofq.f90:90-117
        FILE* f = std::fopen((d + "/sofq.out").c_str(), "a");
        if (!f) return fail(c, DMC_ERR_INVALID, "cannot open sofq.out");
        std::fprintf(f, "# q/kF, s(q), err\n# total weight = %s\n# tau = %s\n", E(O.totw[1]).c_str(), E(tau).c_str());
        const int nq = O.dev.nqtot;
        int k = 0;
        for (int iq = 0; iq < O.dev.ntabq; ++iq) {
            double ave[3] = {0, 0, 0}, err[3] = {0, 0, 0};
            for (int j = 0; j < O.numshq[iq]; ++j, ++k)
                for (int t = 0; t < 3; ++t) {
                    ave[t] += O.val[2][t * nq + k];
                    err[t] += O.err[2][t * nq + k];
                }
            const double* a = &O.akq[3 * (k - 1)];
            const double q = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
            std::string line = E(q / S.kunit);
            for (int t = 0; t < 3; ++t)
                line += E(ave[t] / O.numshq[iq] / npart) + E(err[t] / O.numshq[iq] / npart);
            std::fprintf(f, "%s\n", line.c_str());
        }
        std::fprintf(f, "  \n  \n");
        std::fclose(f);
    }
    if (O.dev.nkv > 0) {
        // writeenk, momentum3d.f90:172-190
        FILE* f = std::fopen((d + "/nofk.out").c_str(), "a");
        if (!f) return fail(c, DMC_ERR_INVALID, "cannot open nofk.out");
        std::fprintf(f, "# k/kF, n(k), err\n# total weight = %s\n# tau = %s\n", E(O.totw[2]).c_str(), E(tau).c_str());
        for (int ir = 0; ir <= O.dev.ntabk; ++ir) {
            const int* v = &O.ik[3 * O.indk[ir]];
            const double kk = std::sqrt(O.dev.dk * O.dev.dk * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]));
            std::fprintf(f, "%s%s%s\n", E(kk).c_str(), E(O.val[3][ir]).c_str(), E(O.err[3][ir]).c_str());
        }
        std::fprintf(f, " \n \n");
        std::fclose(f);
    }
    return DMC_OK;
}

// ---- stochastic reconfiguration ---------------------------------------------

// SR parameters: (beta, gamma) of the long-range Jastrow when iopt(1), then
// vorb when iopt(2) (calder, optimizer.f90:100-104); or, in the adjoint
// mode, every parameter of dmc_param_grad
static int sr_nparm(const dmc_ctx* c)
{
    if (c->sr_adj) return pgrad_np(c);
    return (c->sr_jas ? 2 : 0) + (c->sr_det ? c->S.norb : 0);
}

static int sr_buffers(dmc_ctx* c)
{
    const size_t np = (size_t)sr_nparm(c), nout = np * np + 2 * np + 2;
    if (c->srsum.n < nout) {
        CK(c->srsum.alloc(nout));
        CK(cudaMemset(c->srsum.p, 0, nout * sizeof(double)));
        c->sr_count = 0;
    }
    return DMC_OK;
}

int dmc_sr_configure(dmc_ctx* c, int opt_jastrow, int opt_det)
{
    if (!c) return DMC_ERR_INVALID;
    if (!opt_jastrow && !opt_det) return fail(c, DMC_ERR_INVALID, "no parameters to optimise");
    if (opt_jastrow && c->S.nql == 0) return fail(c, DMC_ERR_INVALID, "the long-range Jastrow is off (numq = 0)");
    c->sr_jas = opt_jastrow != 0;
    c->sr_det = opt_det != 0;
    c->sr_adj = false;
    c->srsum.release();
    c->sr_count = 0;
    return sr_buffers(c);
}

int dmc_sr_configure_adjoint(dmc_ctx* c)
{
    if (!c) return DMC_ERR_INVALID;
    c->sr_adj = true;
    c->srsum.release();
    c->sr_count = 0;
    return sr_buffers(c);
}

int dmc_sr_accumulate(dmc_ctx* c, int64_t* nsamples)
{
    if (!c) return DMC_ERR_INVALID;
    if (c) {
        const int rs = sync_n(c);
        if (rs) return rs;
    }
    int rc = sr_buffers(c);
    if (rc) return rc;
    const int n = c->n, np = sr_nparm(c);
    if (n > 0) {
        StackBufs& s = c->st[c->istin];
        CK(c->sder.alloc((size_t)n * np));
        if (c->sr_adj) {
            // O_k = d log Psi / d theta_k of every adjoint parameter
            CK(c->pg_del.alloc((size_t)n * np));
            if ((rc = pgrad_device(c, n, s.x.p, c->sder.p, c->pg_del.p))) return rc;
        } else {
            if (c->sr_jas) {
                CK(launch_jasder(c->P, c->jq.p, s.x.p, c->sder.p, n, c->grid, c->stream, np));
                ++c->launches;
            }
            if (c->sr_det && (rc = derbcs_device(c, n, s.x.p, c->sder.p, np, c->sr_jas ? 2 : 0))) return rc;
        }
        CK(c->srene.alloc((size_t)n));   // the walkers' local energies
        CK(launch_sr_sums(c->sder.p, s.d2psi.p, s.v.p, n, np, c->S.hbar, c->S.eunit, c->S.npart, c->srsum.p,
                          c->srene.p, c->stream));
        c->launches += 2;
        if ((rc = reverse_stacks(c))) return rc;
        ++c->launches;
        c->sr_count += n;
    }
    CK(cudaStreamSynchronize(c->stream));
    if (nsamples) *nsamples = c->sr_count;
    return DMC_OK;
}

int dmc_sr_get_sums(dmc_ctx* c, double* ovec, double* ovecw, double* pmat, double* e, int64_t* nsamples)
{
    if (!c) return DMC_ERR_INVALID;
    int rc = sr_buffers(c);
    if (rc) return rc;
    const size_t np = (size_t)sr_nparm(c), nout = np * np + 2 * np + 2;
    std::vector<double> h(nout);
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(h.data(), c->srsum.p, nout * sizeof(double), cudaMemcpyDeviceToHost));
    if (ovec) std::copy(h.begin(), h.begin() + np, ovec);
    if (ovecw) std::copy(h.begin() + np, h.begin() + 2 * np, ovecw);
    if (pmat) std::copy(h.begin() + 2 * np, h.begin() + 2 * np + np * np, pmat);
    if (e) {
        e[0] = h[nout - 2];
        e[1] = h[nout - 1];
    }
    if (nsamples) *nsamples = c->sr_count;
    return DMC_OK;
}

int dmc_sr_zero(dmc_ctx* c)
{
    if (!c) return DMC_ERR_INVALID;
    int rc = sr_buffers(c);
    if (rc) return rc;
    const size_t np = (size_t)sr_nparm(c), nout = np * np + 2 * np + 2;
    CK(cudaMemsetAsync(c->srsum.p, 0, nout * sizeof(double), c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->sr_count = 0;
    return DMC_OK;
}

// In-place inverse of a column-major n x n matrix by Gauss-Jordan elimination
// with partial pivoting (the SR matrix: n = norb, at most a few dozen).
// Returns false for an exactly singular matrix.
static bool host_inverse(int n, double* a)
{
    std::vector<int> piv(n);
    auto A = [&](int i, int j) -> double& { return a[i + (size_t)j * n]; };
    for (int k = 0; k < n; ++k) {
        int p = k;
        for (int i = k + 1; i < n; ++i)
            if (std::fabs(A(i, k)) > std::fabs(A(p, k))) p = i;
        if (A(p, k) == 0.0) return false;
        piv[k] = p;
        if (p != k)
            for (int j = 0; j < n; ++j) std::swap(A(k, j), A(p, j));
        const double pinv = 1.0 / A(k, k);
        A(k, k) = 1.0;
        for (int j = 0; j < n; ++j) A(k, j) *= pinv;
        for (int i = 0; i < n; ++i) {
            if (i == k) continue;
            const double m = A(i, k);
            A(i, k) = 0.0;
            for (int j = 0; j < n; ++j) A(i, j) -= m * A(k, j);
        }
    }
    for (int k = n - 1; k >= 0; --k)
        if (piv[k] != k)
            for (int i = 0; i < n; ++i) std::swap(A(i, k), A(i, piv[k]));
    return true;
}

int dmc_sr_update(dmc_ctx* c, double delta0, double eps, double* newpars, double* eave, double* eerr)
{
    if (!c) return DMC_ERR_INVALID;
    const int np = sr_nparm(c);
    if (c->sr_count <= 0) return fail(c, DMC_ERR_INVALID, "no samples accumulated for the SR step");
    std::vector<double> ovec(np), ovecw(np), pmat((size_t)np * np), e(2);
    int64_t ns = 0;
    int rc = dmc_sr_get_sums(c, ovec.data(), ovecw.data(), pmat.data(), e.data(), &ns);
    if (rc) return rc;
    const double cnt = (double)ns;
    for (int i = 0; i < np; ++i) {
        ovec[i] /= cnt;
        ovecw[i] /= cnt;
    }
    for (auto& q : pmat) q /= cnt;
    const double esum = e[0] / cnt, esum2 = e[1] / cnt;
    const double err = std::sqrt(std::fabs(esum * esum - esum2) / cnt);
    std::vector<double> f(np), dpar(np);
    for (int i = 0; i < np; ++i) f[i] = -2.0 * ovecw[i] + 2.0 * ovec[i] * esum;
    for (int i = 0; i < np; ++i) {
        for (int j = 0; j < np; ++j) pmat[i + (size_t)j * np] -= ovec[i] * ovec[j];
        pmat[i + (size_t)i * np] += eps;
    }
    if (!host_inverse(np, pmat.data())) return fail(c, DMC_ERR_INVALID, "singular SR matrix");
    for (int i = 0; i < np; ++i) {
        double sm = 0.0;
        for (int j = 0; j < np; ++j) sm += pmat[i + (size_t)j * np] * f[j];
        dpar[i] = delta0 * sm;
    }
    // params = params + newpars; setjasparam / setdetparam (optimizer.f90:163, 72-88)
    if (c->sr_adj) {
        // vorb, then bfact, b, d, then the Jastrow knots (dmc_param_grad's order)
        std::vector<double> vorb(c->S.vorb);
        for (int i = 0; i < c->S.norb; ++i) vorb[i] += dpar[i];
        if ((rc = dmc_set_vorb(c, vorb.data(), c->S.norb))) return rc;
        int off = c->S.norb;
        if (pgrad_nbeta(c)) {
            if ((rc = dmc_set_beta(c, c->S.bbeta + dpar[off + 1], c->S.dbeta + dpar[off + 2],
                                   c->S.bfact + dpar[off])))
                return rc;
            off += 3;
        }
        if (pgrad_nknot(c)) {
            std::vector<double> kn(c->S.jknots);
            for (size_t k = 0; k < kn.size(); ++k) kn[k] += dpar[off + k];
            if ((rc = dmc_set_jastrow_spline(c, kn.data(), (int)kn.size()))) return rc;
        }
    } else if (c->sr_jas) {
        c->S.set_jaslong(c->S.jbeta + dpar[0], c->S.jgamma + dpar[1]);
        c->P.jbeta = c->S.jbeta;
        c->P.jgamma = c->S.jgamma;
        CK(cudaStreamSynchronize(c->stream));
        CK(cudaMemcpy(c->jq.p, c->S.jq.data(), c->S.jq.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    if (c->sr_det && !c->sr_adj) {
        const int off = c->sr_jas ? 2 : 0;
        std::vector<double> vorb(c->S.vorb);
        for (int i = 0; i < c->S.norb; ++i) vorb[i] += dpar[off + i];
        if ((rc = dmc_set_vorb(c, vorb.data(), c->S.norb))) return rc;
    }
    if ((rc = dmc_sr_zero(c))) return rc;
    if (newpars) std::copy(dpar.begin(), dpar.end(), newpars);
    if (eave) *eave = esum;
    if (eerr) *eerr = err;
    return DMC_OK;
}

int dmc_timed_generations(dmc_ctx* c, int ngen, int opcomp_last, int flush_l2, int64_t* walker_steps,
                          double* device_ms, int64_t* launches)
{
    if (!c || ngen < 0) return DMC_ERR_INVALID;
    int rc = sync_n(c);
    if (rc) return rc;
    if (c->n == 0) return fail(c, DMC_ERR_EMPTY, "no walkers");
    if (flush_l2) {
        int l2 = 0;
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, c->device);
        const size_t fb = std::max<size_t>((size_t)2 * l2, 64u << 20);
        CK(c->flush.alloc(fb));
    }
    CK(cudaMemsetAsync(c->psteps.p, 0, sizeof(unsigned long long), c->stream));
    // Each generation is a captured graph, one per (stack, count-slot)
    // parity at its start; the timed region of generation g lies between
    // events ev[2g] and ev[2g+1] (the L2 flush before it is not timed).
    EventVec ev(2 * (size_t)ngen);
    for (auto& e : ev.v) CK(cudaEventCreate(&e));
    int64_t lsum = 0;
    // the host count goes to the device once, before any capture
    CK(cudaMemcpyAsync(c->pop.p + c->pcur, &c->n, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->n_stale = true;
    for (int g = 0; g < ngen && rc == DMC_OK; ++g) {
        if (flush_l2) CK(cudaMemsetAsync(c->flush.p, g & 0xff, c->flush.n, c->stream));
        const bool last = (g == ngen - 1) && opcomp_last;
        CK(cudaEventRecord(ev[2 * g], c->stream));
        int nl = 0;
        rc = gen_graph(c, last ? 1 : 0, &nl);
        if (rc) break;
        lsum += nl;
        CK(cudaEventRecord(ev[2 * g + 1], c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    double total = 0.0;
    for (int g = 0; g < ngen && rc == DMC_OK; ++g) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, ev[2 * g], ev[2 * g + 1]));
        total += ms;
    }
    unsigned long long steps = 0;
    CK(cudaMemcpy(&steps, c->psteps.p, sizeof steps, cudaMemcpyDeviceToHost));
    const int rs = sync_n(c);
    if (rc == DMC_OK) rc = rs;
    if (walker_steps) *walker_steps = (int64_t)steps;
    if (device_ms) *device_ms = total;
    if (launches) *launches = lsum;
    return rc;
}

int dmc_put_walkers(dmc_ctx* c, const dmc_walkers* w)
{
    if (!c || !w || w->n < 0) return DMC_ERR_INVALID;
    const int n = w->n;
    if (n > c->cap) return fail(c, DMC_ERR_OVERFLOW, "more walkers than the stack capacity");
    if (n > 0 && (!w->x || !w->dpsi || !w->dpsig || !w->psil || !w->psigl || !w->d2psi || !w->d2psig || !w->v ||
                  !w->vext || !w->weight || !w->psil0 || !w->psigl0 || !w->wt0 || !w->is || !w->irn))
        return fail(c, DMC_ERR_INVALID, "dmc_put_walkers needs every field");
    StackBufs& s = c->st[c->istin];
    const size_t n3 = (size_t)c->n3;
    HostWalkers hv;
    if (n > 0 && host_views(c, w, &hv)) {
        // one launch reads every field from the caller's mapped arrays and
        // leaves the count in the device count slot for the next generation
        CK(cudaStreamSynchronize(c->stream));
        CK(launch_walkers_put(hv, s.view(), n, (int)n3, c->pop.p + c->pcur, 8 * c->nsm, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        c->n = n;
        c->n_stale = true;
        return DMC_OK;
    }
    auto H = [&](void* d, const void* h, size_t bytes) {
        return cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, c->stream);
    };
    CK(H(s.x.p, w->x, n * n3 * 8));
    CK(H(s.dpsi.p, w->dpsi, n * n3 * 8));
    CK(H(s.dpsig.p, w->dpsig, n * n3 * 8));
    CK(H(s.psil.p, w->psil, n * 8));
    CK(H(s.psigl.p, w->psigl, n * 8));
    CK(H(s.d2psi.p, w->d2psi, n * 8));
    CK(H(s.d2psig.p, w->d2psig, n * 8));
    CK(H(s.v.p, w->v, n * 8));
    CK(H(s.vext.p, w->vext, n * 8));
    CK(H(s.weight.p, w->weight, n * 8));
    CK(H(s.psil0.p, w->psil0, n * 8));
    CK(H(s.psigl0.p, w->psigl0, n * 8));
    CK(H(s.is.p, w->is, n * sizeof(int)));
    CK(H(s.irn.p, w->irn, n * 8));
    std::vector<float> t(n);
    for (int k = 0; k < n; ++k) t[k] = (float)w->wt0[k];
    CK(H(s.wt0.p, t.data(), n * sizeof(float)));
    CK(cudaStreamSynchronize(c->stream));
    c->n = n;
    c->n_stale = false;
    return DMC_OK;
}

int dmc_set_precision(dmc_ctx* c, int precision)
{
    if (!c) return DMC_ERR_INVALID;
    if (precision != DMC_PREC_FP64 && precision != DMC_PREC_MIXED)
        return fail(c, DMC_ERR_INVALID, "precision must be DMC_PREC_FP64 or DMC_PREC_MIXED");
    CK(cudaStreamSynchronize(c->stream));
    c->precision = precision;
    return DMC_OK;
}

int dmc_get_precision(const dmc_ctx* c, int* precision)
{
    if (!c || !precision) return DMC_ERR_INVALID;
    *precision = c->precision;
    return DMC_OK;
}

int dmc_dfmath_eval(int fn, int n, const void* in, double* out)
{
    if (fn < 0 || fn > 2 || n < 0 || (n > 0 && (!in || !out))) return DMC_ERR_INVALID;
    if (n == 0) return DMC_OK;
    const size_t nin = (size_t)n * 8, nout = (size_t)n * 8 * (fn == 2 ? 1 : 2);
    void* din = nullptr;
    double* dout = nullptr;
    cudaError_t e = cudaMalloc(&din, nin);
    if (e == cudaSuccess) e = cudaMalloc((void**)&dout, nout);
    if (e == cudaSuccess) e = cudaMemcpy(din, in, nin, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = launch_dfmath_eval(fn, n, din, dout, 0);
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, nout, cudaMemcpyDeviceToHost);
    cudaFree(din);
    cudaFree(dout);
    return e == cudaSuccess ? DMC_OK : DMC_ERR_CUDA;
}

int dmc_probe_peak(int kind, double* tflops)
{
    if (!tflops || (kind != 0 && kind != 1)) return DMC_ERR_INVALID;
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return DMC_ERR_CUDA;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return DMC_ERR_CUDA;
    return probe_fma_peak(kind, nsm, tflops) == cudaSuccess ? DMC_OK : DMC_ERR_CUDA;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batches of systems of uneven size: one graph per generation, each system's
// generation on its own stream (fork/join through events on the batch stream)
// ---------------------------------------------------------------------------
struct dmc_batch {
    std::vector<dmc_ctx*> sys;
    std::vector<int> grid;            // walker-kernel CTAs per system
    std::vector<int> order;           // launch order: longest walker first
    cudaStream_t stream = nullptr;    // fork/join stream
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join, done;
    // captured generations keyed by opcomp and every system's (stack, count
    // slot) parities; valid while each system's parameters, launch arguments,
    // precision and grid match the snapshot taken at capture
    struct Graph {
        cudaGraphExec_t exec = nullptr;
        int nl = 0;                 // kernels in the graph
        std::vector<int> nls;       // of which per system
    };
    std::map<uint64_t, Graph> graphs;
    std::vector<DevParams> gP;
    std::vector<KernelArgs> gA;
    std::vector<int> gprec, ggrid, glayout;
    DevBuf<unsigned char> flush;
    std::string err;
};

namespace {

int bfail(dmc_batch* b, int code, const std::string& msg)
{
    b->err = msg;
    return code;
}

#define CKB(expr)                                                                            \
    do {                                                                                     \
        cudaError_t _e = (expr);                                                             \
        if (_e != cudaSuccess) return bfail(b, DMC_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
    } while (0)

// algorithmic flops of one walker-step (pair-matrix products, inverse,
// contractions, pair loop, beta lookups, move): the tuner's first cost guess
double flops_per_walker(const dmc_ctx* c)
{
    const double nu = c->S.nup, nd_ = c->S.ndn, nd = c->S.nd, K = 2.0 * c->S.nk - 1.0, N = c->S.npart;
    return 10.0 * nu * nd_ * K + 2.0 * nd * nd * nd + 8.0 * nd * (nu + nd_) + 30.0 * N * (N - 1) + 40.0 * nu * nd_ +
           30.0 * N;
}

int per_sm_of(const dmc_ctx* c) { return std::max(1, c->grid / std::max(1, c->nsm)); }

// launch order of the systems: decreasing time per walker, so that systems
// with short walkers fill the tail of the long ones
void set_order(dmc_batch* b, const std::vector<double>& tau)
{
    b->order.resize(b->sys.size());
    for (size_t s = 0; s < b->order.size(); ++s) b->order[s] = (int)s;
    std::stable_sort(b->order.begin(), b->order.end(), [&](int x, int y) { return tau[x] > tau[y]; });
}

void drop_graphs(dmc_batch* b)
{
    for (auto& kv : b->graphs)
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    b->graphs.clear();
}

// hand each system's host count to the device (outside any capture)
int push_counts(dmc_batch* b)
{
    for (dmc_ctx* c : b->sys) {
        int rc = sync_n(c);
        if (rc) return bfail(b, rc, c->err);
        if (c->n == 0) return bfail(b, DMC_ERR_EMPTY, "a system of the batch has no walkers");
        CKB(cudaMemcpyAsync(c->pop.p + c->pcur, &c->n, sizeof(int), cudaMemcpyHostToDevice, c->stream));
        CKB(cudaStreamSynchronize(c->stream));
        c->n_stale = true;
    }
    return DMC_OK;
}

// one generation of every system, forked from and joined to the batch stream
int batch_gen_async(dmc_batch* b, int opcomp, int* nlaunch, std::vector<int>& nls)
{
    CKB(cudaEventRecord(b->fork, b->stream));
    int nl = 0;
    nls.assign(b->sys.size(), 0);
    for (const int s : b->order) {
        dmc_ctx* c = b->sys[s];
        CKB(cudaStreamWaitEvent(c->stream, b->fork, 0));
        const int g0 = c->grid;
        c->grid = b->grid[s];
        int k = 0;
        const int rc = gen_async(c, opcomp, &k);
        c->grid = g0;
        if (rc) return bfail(b, rc, c->err);
        nl += k;
        nls[s] = k;
        CKB(cudaEventRecord(b->join[s], c->stream));
        CKB(cudaStreamWaitEvent(b->stream, b->join[s], 0));
    }
    if (nlaunch) *nlaunch = nl;
    return DMC_OK;
}

// one wavefunction evaluation of every system's current walkers, each on its
// own stream with grids[s] CTAs (no walker state changes); ms[s] = time from
// the fork to the end of system s, returns the time to the join in *total
int batch_eval_pass(dmc_batch* b, const std::vector<int>& grids, bool concurrent, std::vector<double>& ms,
                    double* total)
{
    const size_t ns = b->sys.size();
    ms.assign(ns, 0.0);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CKB(cudaEventCreate(&e0));
    CKB(cudaEventCreate(&e1));
    int rc = DMC_OK;
    double tsum = 0.0;
    for (size_t i = 0; i < ns && rc == DMC_OK; ++i) {
        const int s = b->order[i];
        if (!concurrent || i == 0) {
            if (cudaEventRecord(e0, b->stream) != cudaSuccess) rc = DMC_ERR_CUDA;
        }
        dmc_ctx* c = b->sys[s];
        if (rc == DMC_OK && cudaStreamWaitEvent(c->stream, e0, 0) != cudaSuccess) rc = DMC_ERR_CUDA;
        if (rc == DMC_OK) {
            KernelArgs a = base_args(c);
            a.mode = MODE_HPSI;
            a.nw = c->n;
            a.xin = c->st[c->istin].x.p;
            a.status = nullptr;
            if (launch_walker(c->P, a, c->L, std::max(1, std::min(grids[s], c->n)), c->stream,
                              c->precision == DMC_PREC_MIXED) != cudaSuccess)
                rc = DMC_ERR_CUDA;
        }
        if (rc == DMC_OK && cudaEventRecord(b->done[s], c->stream) != cudaSuccess) rc = DMC_ERR_CUDA;
        if (rc == DMC_OK && cudaStreamWaitEvent(b->stream, b->done[s], 0) != cudaSuccess) rc = DMC_ERR_CUDA;
        if (rc == DMC_OK && !concurrent) {
            float t = 0.f;
            // (in order: e0 was recorded after the previous system ended)
            if (cudaEventSynchronize(b->done[s]) != cudaSuccess ||
                cudaEventElapsedTime(&t, e0, b->done[s]) != cudaSuccess)
                rc = DMC_ERR_CUDA;
            ms[s] = t;
            tsum += t;
        }
    }
    if (rc == DMC_OK && concurrent) {
        if (cudaEventRecord(e1, b->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) rc = DMC_ERR_CUDA;
        for (size_t s = 0; s < ns && rc == DMC_OK; ++s) {
            float t = 0.f;
            if (cudaEventElapsedTime(&t, e0, b->done[s]) != cudaSuccess) rc = DMC_ERR_CUDA;
            ms[s] = t;
        }
        float t = 0.f;
        if (rc == DMC_OK && cudaEventElapsedTime(&t, e0, e1) != cudaSuccess) rc = DMC_ERR_CUDA;
        tsum = t;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return bfail(b, rc, "tuning pass");
    if (total) *total = tsum;
    return DMC_OK;
}

}  // namespace

extern "C" {

int dmc_batch_plan(int nsys, const double* tau, const int* nw, const int* per_sm, const int* maxgrid, int nsm,
                   int* grids)
{
    if (nsys < 1 || nsys > DMC_BATCH_MAX || !tau || !nw || !per_sm || !maxgrid || !grids || nsm < 1)
        return DMC_ERR_INVALID;
    int units = 2 * nsm;   // half-SM slots
    std::vector<int> unit(nsys);
    for (int s = 0; s < nsys; ++s) {
        if (!(tau[s] > 0.0) || nw[s] < 1 || (per_sm[s] != 1 && per_sm[s] != 2) || maxgrid[s] < 1)
            return DMC_ERR_INVALID;
        unit[s] = 2 / per_sm[s];
        grids[s] = 1;
        units -= unit[s];
    }
    if (units < 0) return DMC_ERR_INVALID;
    auto waves = [&](int s, int g) { return (nw[s] + g - 1) / g; };
    // the smallest grid that takes one wave of walkers off system s (0: none)
    auto next_grid = [&](int s) {
        const int w = waves(s, grids[s]);
        if (w <= 1) return 0;
        const int g = (nw[s] + w - 2) / (w - 1);
        return g <= maxgrid[s] && (g - grids[s]) * unit[s] <= units ? g : 0;
    };
    for (;;) {
        int best = -1;
        double tb = -1.0;
        for (int s = 0; s < nsys; ++s) {
            if (!next_grid(s)) continue;
            const double t = waves(s, grids[s]) * tau[s];
            if (t > tb) {
                tb = t;
                best = s;
            }
        }
        if (best < 0) break;
        const int g = next_grid(best);
        units -= (g - grids[best]) * unit[best];
        grids[best] = g;
    }
    return DMC_OK;
}

int dmc_batch_create(dmc_ctx* const* ctxs, int nsys, dmc_batch** out)
{
    if (!ctxs || !out || nsys < 1 || nsys > DMC_BATCH_MAX) return DMC_ERR_INVALID;
    *out = nullptr;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return DMC_ERR_CUDA;
    for (int s = 0; s < nsys; ++s) {
        if (!ctxs[s] || ctxs[s]->device != dev) return DMC_ERR_INVALID;
        for (int t = 0; t < s; ++t)
            if (ctxs[t] == ctxs[s]) return DMC_ERR_INVALID;
    }
    dmc_batch* b = new (std::nothrow) dmc_batch();
    if (!b) return DMC_ERR_NOMEM;
    b->sys.assign(ctxs, ctxs + nsys);
    b->join.assign(nsys, nullptr);
    b->done.assign(nsys, nullptr);
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    for (int s = 0; s < nsys && e == cudaSuccess; ++s) {
        e = cudaEventCreateWithFlags(&b->join[s], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreate(&b->done[s]);
    }
    if (e != cudaSuccess) {
        dmc_batch_destroy(b);
        return DMC_ERR_CUDA;
    }
    // first split: every system on its whole persistent grid, launched in
    // decreasing order of algorithmic flops per walker-step
    std::vector<double> tau(nsys);
    b->grid.resize(nsys);
    for (int s = 0; s < nsys; ++s) {
        tau[s] = flops_per_walker(ctxs[s]);
        b->grid[s] = ctxs[s]->grid;
    }
    set_order(b, tau);
    *out = b;
    return DMC_OK;
}

int dmc_batch_destroy(dmc_batch* b)
{
    if (!b) return DMC_ERR_INVALID;
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_graphs(b);
    for (cudaEvent_t e : b->join)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : b->done)
        if (e) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return DMC_OK;
}

const char* dmc_batch_last_error(const dmc_batch* b) { return b ? b->err.c_str() : "null batch"; }

int dmc_batch_set_grids(dmc_batch* b, const int* grids)
{
    if (!b || !grids) return DMC_ERR_INVALID;
    for (size_t s = 0; s < b->sys.size(); ++s)
        if (grids[s] < 1 || grids[s] > b->sys[s]->grid) return bfail(b, DMC_ERR_INVALID, "grid out of range");
    b->grid.assign(grids, grids + b->sys.size());
    return DMC_OK;
}

int dmc_batch_get_grids(const dmc_batch* b, int* grids)
{
    if (!b || !grids) return DMC_ERR_INVALID;
    std::copy(b->grid.begin(), b->grid.end(), grids);
    return DMC_OK;
}

int dmc_batch_tune(dmc_batch* b, int rounds, int* grids, double* ms)
{
    if (!b || rounds < 0) return DMC_ERR_INVALID;
    const int ns = (int)b->sys.size();
    for (dmc_ctx* c : b->sys) {
        const int rc = sync_n(c);
        if (rc) return bfail(b, rc, c->err);
        if (c->n == 0) return bfail(b, DMC_ERR_EMPTY, "a system of the batch has no walkers");
        CKB(cudaStreamSynchronize(c->stream));
    }
    std::vector<int> nw(ns), psm(ns), mg(ns), full(ns);
    for (int s = 0; s < ns; ++s) b->grid[s] = std::max(1, std::min(b->grid[s], b->sys[s]->grid));
    for (int s = 0; s < ns; ++s) {
        const dmc_ctx* c = b->sys[s];
        nw[s] = c->n;
        psm[s] = std::min(2, per_sm_of(c));
        mg[s] = c->grid;
        full[s] = c->grid;
    }
    // each system alone on the whole GPU (after one warm-up pass)
    std::vector<double> t;
    double tot = 0.0;
    int rc = batch_eval_pass(b, full, false, t, &tot);
    if (!rc) rc = batch_eval_pass(b, full, false, t, &tot);
    if (rc) return rc;
    std::vector<double> tau(ns);
    for (int s = 0; s < ns; ++s) {
        const int g = std::min(full[s], nw[s]);
        tau[s] = std::max(1e-6, t[s]) / ((nw[s] + g - 1) / g);
    }
    const std::vector<int> order0 = b->order;
    set_order(b, tau);
    std::vector<int> cur(ns), best = b->grid;
    double best_ms = 0.0;
    {
        // the split in use, as the reference point
        std::vector<double> tt;
        rc = batch_eval_pass(b, best, true, tt, &best_ms);
        if (rc) return rc;
        // every system on its whole persistent grid: the CTA scheduler then
        // starts each system's CTAs as the previous system's CTAs retire
        double pass = 0.0;
        rc = batch_eval_pass(b, full, true, tt, &pass);
        if (rc) return rc;
        if (pass < best_ms) {
            best_ms = pass;
            best = full;
        }
    }
    for (int r = 0; r <= rounds; ++r) {
        rc = dmc_batch_plan(ns, tau.data(), nw.data(), psm.data(), mg.data(), b->sys[0]->nsm, cur.data());
        if (rc) return bfail(b, rc, "plan");
        std::vector<double> ts;
        double pass = 0.0;
        rc = batch_eval_pass(b, cur, true, ts, &pass);
        if (rc) return rc;
        if (pass < best_ms) {
            best_ms = pass;
            best = cur;
        }
        // per-walker times seen with the other systems resident
        for (int s = 0; s < ns; ++s) {
            const int g = std::min(cur[s], nw[s]);
            tau[s] = std::max(1e-6, ts[s]) / ((nw[s] + g - 1) / g);
        }
    }
    if (best != b->grid || b->order != order0) drop_graphs(b);
    b->grid = best;
    if (grids) std::copy(best.begin(), best.end(), grids);
    if (ms) *ms = best_ms;
    return DMC_OK;
}

int dmc_batch_generations(dmc_batch* b, int ngen, int opcomp_last, int flush_l2, int64_t* walker_steps,
                          double* device_ms, int64_t* launches)
{
    if (!b || ngen < 0) return DMC_ERR_INVALID;
    const int ns = (int)b->sys.size();
    int rc = DMC_OK;
    for (dmc_ctx* c : b->sys) {
        rc = sync_n(c);
        if (rc) return bfail(b, rc, c->err);
        if (c->n == 0) return bfail(b, DMC_ERR_EMPTY, "a system of the batch has no walkers");
    }
    if (flush_l2) {
        int l2 = 0;
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, b->sys[0]->device);
        const size_t fb = std::max<size_t>((size_t)2 * l2, 64u << 20);
        CKB(b->flush.alloc(fb));
    }
    // a system's own layout may have changed (dmc_tune_layout): never more
    // CTAs than its grid, whose global scratch slices exist
    for (int s = 0; s < ns; ++s) b->grid[s] = std::max(1, std::min(b->grid[s], b->sys[s]->grid));
    // drop the captured generations when anything they baked in changed
    {
        bool same = (int)b->gP.size() == ns && b->ggrid == b->grid;
        for (int s = 0; s < ns && same; ++s) {
            dmc_ctx* c = b->sys[s];
            const KernelArgs A = base_args(c);
            same = b->gprec[s] == c->precision && b->glayout[s] == c->layout_gen &&
                   std::memcmp(&b->gP[s], &c->P, sizeof c->P) == 0 && std::memcmp(&b->gA[s], &A, sizeof A) == 0;
        }
        if (!same) {
            drop_graphs(b);
            b->gP.resize(ns);
            b->gA.resize(ns);
            b->gprec.resize(ns);
            b->glayout.resize(ns);
            for (int s = 0; s < ns; ++s) {
                dmc_ctx* c = b->sys[s];
                const KernelArgs A = base_args(c);
                std::memcpy(&b->gP[s], &c->P, sizeof c->P);
                std::memcpy(&b->gA[s], &A, sizeof A);
                b->gprec[s] = c->precision;
                b->glayout[s] = c->layout_gen;
            }
            b->ggrid = b->grid;
        }
    }
    for (dmc_ctx* c : b->sys) CKB(cudaMemsetAsync(c->psteps.p, 0, sizeof(unsigned long long), c->stream));
    rc = push_counts(b);
    if (rc) return rc;
    EventVec ev(2 * (size_t)ngen);
    for (auto& e : ev.v) CKB(cudaEventCreate(&e));
    int64_t lsum = 0;
    for (int g = 0; g < ngen && rc == DMC_OK; ++g) {
        if (flush_l2) CKB(cudaMemsetAsync(b->flush.p, g & 0xff, b->flush.n, b->stream));
        const int op = (g == ngen - 1) && opcomp_last ? 1 : 0;
        uint64_t key = (uint64_t)op;
        for (int s = 0; s < ns; ++s)
            key |= (uint64_t)(b->sys[s]->istin | (b->sys[s]->pcur << 1)) << (1 + 2 * s);
        auto it = b->graphs.find(key);
        if (it == b->graphs.end()) {
            std::vector<int> pi(ns), pc(ns);
            std::vector<int64_t> l0(ns);
            for (int s = 0; s < ns; ++s) {
                pi[s] = b->sys[s]->istin;
                pc[s] = b->sys[s]->pcur;
                l0[s] = b->sys[s]->launches;
            }
            cudaGraph_t graph = nullptr;
            dmc_batch::Graph G;
            CKB(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            rc = batch_gen_async(b, op, &G.nl, G.nls);
            const cudaError_t ce = cudaStreamEndCapture(b->stream, &graph);
            if (rc == DMC_OK && ce != cudaSuccess) rc = bfail(b, DMC_ERR_CUDA, "batch capture");
            if (rc == DMC_OK && cudaGraphInstantiate(&G.exec, graph, 0) != cudaSuccess)
                rc = bfail(b, DMC_ERR_CUDA, "batch graph instantiate");
            if (graph) cudaGraphDestroy(graph);
            // the capture only recorded the launches: restore the parities
            for (int s = 0; s < ns; ++s) {
                b->sys[s]->istin = pi[s];
                b->sys[s]->pcur = pc[s];
                b->sys[s]->launches = l0[s];
            }
            if (rc) break;
            it = b->graphs.emplace(key, G).first;
        }
        CKB(cudaEventRecord(ev[2 * g], b->stream));
        CKB(cudaGraphLaunch(it->second.exec, b->stream));
        CKB(cudaEventRecord(ev[2 * g + 1], b->stream));
        for (int s = 0; s < ns; ++s) {
            advance_parities(b->sys[s]);
            b->sys[s]->launches += it->second.nls[s];
        }
        lsum += it->second.nl;
    }
    if (rc == DMC_OK) CKB(cudaStreamSynchronize(b->stream));
    double total = 0.0;
    for (int g = 0; g < ngen && rc == DMC_OK; ++g) {
        float ms = 0.f;
        CKB(cudaEventElapsedTime(&ms, ev[2 * g], ev[2 * g + 1]));
        total += ms;
    }
    int64_t steps = 0;
    for (dmc_ctx* c : b->sys) {
        unsigned long long st = 0;
        CKB(cudaMemcpy(&st, c->psteps.p, sizeof st, cudaMemcpyDeviceToHost));
        steps += (int64_t)st;
        const int rs = sync_n(c);
        if (rc == DMC_OK && rs) rc = bfail(b, rs, c->err);
    }
    if (walker_steps) *walker_steps = steps;
    if (device_ms) *device_ms = total;
    if (launches) *launches = lsum;
    return rc;
}

}  // extern "C"
