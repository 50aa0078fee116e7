// Host-side set-up tables for the GB300 DMCBS path.  Each function follows
// the reference routine cited beside it; the algorithms (k-shell
// enumeration and order, image-summed beta table, RK4 zero-energy Jastrow
// with energy bisection, 4-point Lagrange grids) have to be the same for the
// tables to agree with the reference's.
#include "dmc_setup.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstring>

#include "dmc_spline.h"

namespace dmc {
namespace {

const double kPi = 3.14159265358979323846;

}  // namespace

// kstates3d (kshell.f90:20-156): integer vectors of the half set of each
// |n|^2 shell, in the order the reference's exchange sort leaves them.
int k_shells(double el, int nsh0, std::vector<KVec>& out, std::vector<int>& numsh0, std::string& err)
{
    const int i2max = 2 * nsh0;
    const int imax = (int)std::lround(std::sqrt((float)i2max));  // nint(sqrt(real(i2max)))
    std::vector<std::array<int, 3>> v;
    auto add = [&](int a, int b, int c) { v.push_back({a, b, c}); };
    for (int ix = 0; ix <= imax; ++ix)
        for (int iy = 0; iy <= imax; ++iy)
            for (int iz = 0; iz <= imax; ++iz) {
                if (ix * ix + iy * iy + iz * iz > i2max) continue;
                add(ix, iy, iz);
                if (ix == 0 && iy != 0 && iz != 0) add(ix, iy, -iz);
                if (iy == 0 && ix != 0 && iz != 0) add(ix, iy, -iz);
                if (iz == 0 && ix != 0 && iy != 0) add(ix, -iy, iz);
                if (ix != 0 && iy != 0 && iz != 0) {
                    add(ix, iy, -iz);
                    add(ix, -iy, iz);
                    add(ix, -iy, -iz);
                }
            }
    auto n2 = [](const std::array<int, 3>& a) { return a[0] * a[0] + a[1] * a[1] + a[2] * a[2]; };
    // the reference's exchange sort (swap whenever |n_i|^2 >= |n_j|^2, i<j)
    const size_t nk = v.size();
    for (size_t i = 0; i + 1 < nk; ++i)
        for (size_t j = i + 1; j < nk; ++j)
            if (n2(v[i]) >= n2(v[j])) std::swap(v[i], v[j]);
    std::vector<int> numsh(nk + 2, 0);
    int i2m = 0, nsh = 1;
    for (size_t i = 0; i < nk; ++i) {
        if (n2(v[i]) > i2m) {
            ++nsh;
            i2m = n2(v[i]);
        }
        numsh[nsh] += 2;   // counted twice, as the reference does after its loop
    }
    if (nsh0 >= nsh) {
        err = "too many k shells requested";
        return DMC_ERR_SETUP;
    }
    const double piel = 2.0 * kPi / el;
    out.clear();
    numsh0.assign(nsh0, 0);
    size_t k = 0;
    for (int sh = 1; sh <= nsh0; ++sh) {
        numsh0[sh - 1] = numsh[sh] / 2;
        const int m = std::max(1, numsh[sh] / 2);
        for (int j = 0; j < m; ++j, ++k) {
            KVec q;
            for (int c = 0; c < 3; ++c) {
                q.n[c] = v[k][c];
                q.k[c] = piel * v[k][c];
            }
            q.k2 = q.k[0] * q.k[0] + q.k[1] * q.k[1] + q.k[2] * q.k[2];
            q.shell = sh;
            out.push_back(q);
        }
    }
    return DMC_OK;
}

namespace {

// ---- beta function (betafun.f90) ----------------------------------------
//
// The construction is templated on its scalar type: double builds the
// tables, std::complex<double> with b or d given a tiny imaginary part
// builds their exact derivatives with respect to b or d (complex-step
// differentiation: Im f(p + i h) / h = f'(p) to rounding, with no
// cancellation).  Branches and the image count follow the real parts, so the
// derivative is that of the same piecewise construction.

inline double re(double v) { return v; }
inline double re(const std::complex<double>& v) { return v.real(); }

template <class T>
struct Beta {
    T b, c, d, small, c0, c1, c2, c3, c4;
    double el;

    // beta0, betafun.f90:127-149
    void beta0(double r, T& b1, T& b1p, T& b1pp) const
    {
        const T x = b * r;
        if (r < re(small)) {
            b1 = c0 + x * (c1 + x * (c2 + x * (c3 + x * c4)));
            b1p = c1 + x * (2.0 * c2 + x * (3.0 * c3 + 4.0 * c4 * x));
            b1pp = 2.0 * c2 + x * (6.0 * c3 + 12.0 * c4 * x);
        } else {
            const T ex = std::exp(-x), ex10 = std::exp(-d * x);
            b1 = (1.0 + c * x) * (1.0 - ex10) * ex / x;
            b1p = ex * (-1.0 - x * (1.0 + c * x) + ex10 * (1.0 + x * (1.0 + d) * (1.0 + c * x))) / (x * x);
            b1pp = ex * (2.0 + x * (2.0 + x * (1.0 + c * x))
                         - ex10 * (2.0 + x * (1.0 + d) * (2.0 + x * (1.0 + d) * (1.0 + x * c)))) / (x * x * x);
        }
        b1p = b * b1p;
        b1pp = (b * b) * b1pp;
        b1 /= d;
        b1p /= d;
        b1pp /= d;
    }

    // beta, betafun.f90:151-171: symmetric about L/2, zero at L/2
    void beta(double r, T& b1, T& b1p, T& b1pp) const
    {
        if (r > el * 0.5) {
            b1 = b1p = b1pp = T(0.0);
            return;
        }
        T bet0, t1, t2, bet1, bet1p, bet1pp, bet2, bet2p, bet2pp;
        beta0(el * 0.5, bet0, t1, t2);
        beta0(r, bet1, bet1p, bet1pp);
        beta0(el - r, bet2, bet2p, bet2pp);
        b1 = bet1 + bet2 - 2.0 * bet0;
        b1p = (r < 1.0e-14) ? T(0.0) : bet1p - bet2p;
        b1pp = bet1pp + bet2pp;
    }
};

// initbeta, betafun.f90:74-125, then the bfact scaling of setbeta (:62-64),
// on n + 1 points of [0, L/2]
template <class T>
void beta_tables_t(double el, int n, T bb, T dd, double bfact, std::vector<T>& bt, std::vector<T>& dbt,
                   std::vector<T>& d2bt)
{
    Beta<T> B;
    B.el = el;
    B.b = bb;
    B.d = dd;
    const T e1 = std::exp(bb * el * (1.0 + dd)), e2 = std::exp(dd * bb * el);
    B.c = 0.5 * (2.0 + 2.0 * dd * bb * el + (dd * bb * el) * (dd * bb * el) * e1 + 2.0 * dd * bb * bb * el * el * e1
                 + 2.0 * bb * el - 2.0 * e2 * bb * el - 2.0 * e2)
          / (el * el * (e2 - 1.0 - dd + dd * e1) * (bb * bb));
    const T c = B.c, d = dd;
    B.c0 = d;
    B.small = 1.0e-3 / bb;
    B.c1 = -d + c * d - d * d / 2.0;
    B.c2 = d / 2.0 + d * d / 2.0 + d * d * d / 6.0 + c * (-d - d * d / 2.0);
    B.c3 = -d / 6.0 - d * d / 4.0 - d * d * d / 6.0 - d * d * d * d / 24.0 + c * (d / 2.0 + d * d / 2.0 + d * d * d / 6.0);
    B.c4 = d / 24.0 + d * d / 12.0 + d * d * d / 12.0 + d * d * d * d / 24.0 + d * d * d * d * d / 120.0
           - c * (d / 6.0 + d * d / 4.0 + d * d * d / 6.0 + d * d * d * d / 24.0);
    const double dr = 0.5 * el / n;
    // number of periodic images whose beta is still above 1e-10
    int nj = 0;
    T betan = 10.0, t1, t2;
    while (std::fabs(re(betan)) > 1.0e-10) {
        ++nj;
        B.beta(el * nj, betan, t1, t2);
    }
    bt.assign(n + 1, T(0.0));
    dbt.assign(n + 1, T(0.0));
    d2bt.assign(n + 1, T(0.0));
    for (int i = 0; i <= n; ++i) {
        const double r = i * dr;
        T f, fp, fpp;
        B.beta(r, f, fp, fpp);
        for (int j = 1; j <= nj; ++j) {
            T b2, b2p, b2pp, b3, b3p, b3pp;
            B.beta(j * el - r, b2, b2p, b2pp);
            B.beta(j * el + r, b3, b3p, b3pp);
            f = f + b2 + b3;
            fp = fp - b2p + b3p;
            fpp = fpp + b2pp + b3pp;
        }
        bt[i] = f;
        dbt[i] = fp;
        d2bt[i] = fpp;
    }
    const T shift = bt[n];
    for (int i = 0; i <= n; ++i) {
        bt[i] -= shift;
        if (i != 0)
            d2bt[i] = d2bt[i] + 2.0 * dbt[i] / (i * dr);   // + (ndim-1) f'/r
        else
            d2bt[i] = 3.0 * d2bt[i];                       // quadratic at the origin
    }
    const double af = std::fabs(bfact);
    for (int i = 0; i <= n; ++i) {
        bt[i] *= af;
        dbt[i] *= af;
        d2bt[i] *= af;
    }
}

void beta_tables(Setup& s, double bb, double dd, double bfact)
{
    beta_tables_t<double>(s.el, s.ntabb, bb, dd, bfact, s.btab, s.dbtab, s.d2btab);
}

// ---- Jastrow from the two-body zero-energy equation (rungekutta.f90) ----

struct Cosh {
    double amu, hbarp;
    // vpot, coshpot.f90:145-152
    double v(double v0, double r) const
    {
        const double ch = std::cosh(amu * r);
        return -2.0 * v0 * (amu * amu) * hbarp / (ch * ch);
    }
};

// rk3d, rungekutta.f90:127-150: u'' = -(E - V) u / hb from u(0)=0, u'(0)=1;
// returns the number of sign changes of u.
int rk3d(const Cosh& P, double v0, std::vector<double>& psi, std::vector<double>& dpsi, double ene, double hb,
         double dr, int n)
{
    psi[0] = 0.0;
    dpsi[0] = 1.0;
    int ncross = 0;
    for (int i = 1; i <= n; ++i) {
        const double r = (i - 1) * dr;
        const double vh = P.v(v0, r + 0.5 * dr);
        const double k1a = -(ene - P.v(v0, r)) * psi[i - 1] / hb;
        const double k1b = dpsi[i - 1];
        const double k2a = -(ene - vh) * (psi[i - 1] + 0.5 * dr * k1b) / hb;
        const double k2b = dpsi[i - 1] + 0.5 * dr * k1a;
        const double k3a = -(ene - vh) * (psi[i - 1] + 0.5 * dr * k2b) / hb;
        const double k3b = dpsi[i - 1] + 0.5 * dr * k2a;
        const double k4a = -(ene - P.v(v0, r + dr)) * (psi[i - 1] + dr * k3b) / hb;
        const double k4b = dpsi[i - 1] + dr * k3a;
        dpsi[i] = dpsi[i - 1] + (k1a + 2.0 * k2a + 2.0 * k3a + k4a) * dr / 6.0;
        psi[i] = psi[i - 1] + (k1b + 2.0 * k2b + 2.0 * k3b + k4b) * dr / 6.0;
        if (psi[i] != std::copysign(std::fabs(psi[i]), psi[i - 1])) ++ncross;
    }
    return ncross;
}

// orbital, 3-D branch (rungekutta.f90:57-99): nodeless solution whose
// logarithmic derivative vanishes at the healing distance, by bisection on E.
bool jastrow_orbital(const Cosh& P, double v0, std::vector<double>& f, std::vector<double>& df,
                     std::vector<double>& d2f, double hb, int n, double dr)
{
    double emin = P.v(v0, 0.0);
    for (int i = 1; i <= n; ++i) emin = std::min(emin, P.v(v0, i * dr));
    double emax = 0.001;
    while (rk3d(P, v0, f, df, emax, hb, dr, n) <= 0) emax *= 2.0;
    double ene = 0.5 * (emin + emax);
    for (int iter = 0;; ++iter) {
        rk3d(P, v0, f, df, ene, hb, dr, n);
        const double r = dr * n;
        const double der = (df[n] - f[n] / r) / r / f[n];
        if (der < 0.0)
            emax = ene;
        else
            emin = ene;
        if (std::fabs(der) < 1.0e-8) break;
        ene = 0.5 * (emin + emax);
        if (iter + 1 > 100) return false;
    }
    // u(r) = r f(r): convert to f, f', f''
    f[0] = df[0];
    d2f[0] = (P.v(v0, 0.0) - ene) * df[0] / (3.0 * hb);
    df[0] = 0.0;
    for (int i = 1; i <= n; ++i) {
        const double r = i * dr;
        df[i] = (df[i] - f[i] / r) / r;
        f[i] = f[i] / r;
        d2f[i] = (P.v(v0, r) - ene) * f[i] / hb - 2.0 * df[i] / r;
    }
    return true;
}

}  // namespace

int Setup::build(const dmc_system_desc& sd, const dmc_run_desc& rd, std::string& err)
{
    if (sd.ndim != 3) {
        err = "only ndim = 3 is on this path";
        return DMC_ERR_UNSUPPORTED;
    }
    if (sd.nbin[0] < 0 || sd.nbin[1] < 0 || sd.nbin[0] + sd.nbin[1] < 2 || sd.nbin[0] + sd.nbin[1] > DMC_MAX_PART) {
        err = "particle numbers out of range";
        return DMC_ERR_INVALID;
    }
    if (sd.norb < 1 || sd.norb > DMC_MAX_SHELLS || sd.nexup < 0 || sd.nexup > DMC_MAX_UNPAIRED || sd.nexdn < 0 ||
        sd.nexdn > DMC_MAX_UNPAIRED || sd.ntab < 8 || !(sd.rho > 0.0)) {
        err = "bad pairing or table parameters";
        return DMC_ERR_INVALID;
    }
    if (sd.bfact < 0.0) {
        err = "bfact < 0 (beta table read from unit 80) is not supported";
        return DMC_ERR_UNSUPPORTED;
    }
    if (sd.numq < 0 || sd.numq > DMC_MAX_SHELLS) {
        err = "numq out of range";
        return DMC_ERR_INVALID;
    }
    npart = sd.nbin[0] + sd.nbin[1];
    ntab = sd.ntab;
    hbar = sd.hbar;
    a2 = sd.a2;
    for (int s = 0; s < 2; ++s) {
        mass[s] = sd.mass[s];
        sqm[s] = std::sqrt(mass[s]);
    }
    // setupbcs, psislaterbcs.f90:35-153
    rho = sd.rho;
    el = std::pow(npart / rho, 1.0 / 3.0);
    eli = 1.0 / el;
    nexup = sd.nexup;
    nexdn = sd.nexdn;
    norb = sd.norb;
    vorb.assign(sd.vorb, sd.vorb + norb);
    for (int i = 0; i < nexup; ++i) {
        sinup[i] = 0;
        for (int c = 0; c < 3; ++c) {
            akup[i][c] = sd.ikup[i][c] * 2.0 * kPi / el;
            if (sd.ikup[i][c] != 0) sinup[i] = sd.ikup[i][c] < 0;   // sin if the last non-zero entry < 0
        }
        ak2up[i] = akup[i][0] * akup[i][0] + akup[i][1] * akup[i][1] + akup[i][2] * akup[i][2];
    }
    for (int i = 0; i < nexdn; ++i) {
        sindn[i] = 0;
        for (int c = 0; c < 3; ++c) {
            akdn[i][c] = sd.ikdn[i][c] * 2.0 * kPi / el;
            if (sd.ikdn[i][c] != 0) sindn[i] = sd.ikdn[i][c] < 0;
        }
        ak2dn[i] = akdn[i][0] * akdn[i][0] + akdn[i][1] * akdn[i][1] + akdn[i][2] * akdn[i][2];
    }
    int rc = k_shells(el, norb, kv, numsh, err);
    if (rc != DMC_OK) return rc;
    nk = (int)kv.size();
    ncol = 2 * nk - 1;
    nmax = 0;
    for (const KVec& q : kv)
        for (int c = 0; c < 3; ++c) nmax = std::max(nmax, std::abs(q.n[c]));
    const int np2 = npart - nexup - nexdn;
    if (np2 < 0 || np2 % 2 != 0) {
        err = "inconsistent pairing number";
        return DMC_ERR_INVALID;
    }
    npair = np2 / 2;
    nup = npair + nexup;
    ndn = npair + nexdn;
    nd = npair + nexup + nexdn;
    if (nup != sd.nbin[0] || ndn != sd.nbin[1]) {
        err = "unpaired states do not match the spin populations";
        return DMC_ERR_INVALID;
    }
    // setbeta, betafun.f90:12-72
    nobeta = (sd.bfact == 0.0);
    ntabb = ntab;
    rangeb = 0.5 * el;
    scaleb = ntabb / rangeb;
    if (!nobeta) beta_tables(*this, sd.bbeta, sd.dbeta, sd.bfact);
    else {
        btab.assign(ntabb + 1, 0.0);
        dbtab.assign(ntabb + 1, 0.0);
        d2btab.assign(ntabb + 1, 0.0);
    }
    for (int c = 0; c < 3; ++c) qex[c] = sd.nqex[c] * 2.0 * kPi / el;
    v0ex = sd.v0ex * 0.5;
    v0exjas = sd.v0exjas * v0ex;
    numq = sd.numq;
    jbeta = sd.jbeta;
    jgamma = sd.jgamma;
    // setjaslong (jastrowlongrange.f90:10-20): the q vectors of numq shells
    // (kstates3d, q = 0 excluded as getjaslong does) and their weights
    // gamma exp(-beta |q|) / |q|
    jq.clear();
    nql = 0;
    if (numq > 0) {
        std::vector<KVec> kq;
        std::vector<int> nsh;
        int rc = k_shells(el, numq, kq, nsh, err);
        if (rc) return rc;
        for (size_t q = 1; q < kq.size(); ++q) {
            const double qmod = std::sqrt(kq[q].k2);
            const double rec[8] = {kq[q].k[0], kq[q].k[1], kq[q].k[2], kq[q].k2,
                                   sd.jgamma * std::exp(-sd.jbeta * qmod) / qmod, 0.0, 0.0, 0.0};
            jq.insert(jq.end(), rec, rec + 8);
            ++nql;
        }
    }
    // setphi, coshpot.f90:14-143
    const double mu = mass[0] * mass[1] / (mass[0] + mass[1]);
    hbarp = 2.0 * (hbar / (2.0 * mu));
    range = 0.5 * el;
    const double dr = range / ntab;
    scale = 1.0 / dr;
    cjas[0] = sd.cjas[0];
    cjas[1] = sd.cjas[1];
    const double v0op = sd.v0op == 0.0 ? sd.v0 : sd.v0op;
    const double v0eq = sd.v0eq == 0.0 ? sd.v0 : sd.v0eq;
    Cosh P{sd.amu, hbarp};
    for (int ic = 0; ic < 2; ++ic) {
        vtab[ic].assign(ntab + 1, 0.0);
        utab[ic].assign(ntab + 1, 0.0);
        dutab[ic].assign(ntab + 1, 0.0);
        d2utab[ic].assign(ntab + 1, 0.0);
    }
    for (int i = 0; i <= ntab; ++i) vtab[0][i] = P.v(sd.v0, i * dr);   // opposite spins only
    ntab0 = (int)(ntab * sd.djas / (0.5 * el));
    if (ntab0 < 1 || ntab0 > ntab) {
        err = "Jastrow healing distance outside (0, L/2]";
        return DMC_ERR_INVALID;
    }
    std::vector<double> f(ntab0 + 1), df(ntab0 + 1), d2f(ntab0 + 1);
    for (int ic = 0; ic < 2; ++ic) {
        if (cjas[ic] != 0.0) {
            if (!jastrow_orbital(P, ic == 0 ? v0op : v0eq, f, df, d2f, hbarp, ntab0, dr)) {
                err = "Jastrow orbital: no convergence";
                return DMC_ERR_SETUP;
            }
            for (int i = 0; i <= ntab0; ++i) {
                utab[ic][i] = f[i] / f[ntab0];
                dutab[ic][i] = df[i] / f[ntab0];
                d2utab[ic][i] = d2f[i] / f[ntab0];
            }
        }
        for (int i = ntab0 + 1; i <= ntab; ++i) {
            utab[ic][i] = 1.0;
            dutab[ic][i] = 0.0;
            d2utab[ic][i] = 0.0;
        }
        // log f, f'/f and f''/f - (f'/f)^2, times the Jastrow strength
        for (int i = 0; i <= ntab; ++i) {
            double& u = utab[ic][i];
            double& du = dutab[ic][i];
            double& d2u = d2utab[ic][i];
            if (cjas[ic] != 0.0) {
                du = du / u;
                d2u = d2u / u - du * du;
                u = std::log(u);
            }
            u *= cjas[ic];
            du *= cjas[ic];
            d2u *= cjas[ic];
        }
    }
    iop = true;   // the potential table switches opposite-spin pairs on (coshpot.f90:88)
    ieq = cjas[1] != 0.0;
    // the reference's up-down Jastrow, kept for the opt-in spline on top of it
    uref = utab[0];
    duref = dutab[0];
    d2uref = d2utab[0];
    jknots.clear();
    bbeta = sd.bbeta;
    dbeta = sd.dbeta;
    bfact = sd.bfact;
    // units, dmcbcs.f90:146-170
    if (rd.units) {
        kunit = std::pow(3.0 * (kPi * kPi) * (npart / (el * el * el)), 1.0 / 3.0);
        eunit = 3.0 / 5.0 * hbar / (2.0 * mu) * (kunit * kunit);
    } else {
        kunit = 1.0;
        eunit = 1.0;
    }
    etrial = rd.etrial * eunit * npart;
    // setstep, step.f90:11-41
    nfac = 1.0 / eunit / npart;
    const double sig = std::sqrt(2.0 * hbar * rd.dt);
    cutdrift = rd.dcut >= 0.0;
    for (int s = 0; s < 2; ++s) {
        sigma[s] = sig / std::sqrt(mass[s]);
        dcut[s] = cutdrift ? sigma[s] * rd.dcut : 0.0;
    }
    return DMC_OK;
}

void Setup::set_jaslong(double beta, double gamma)
{
    jbeta = beta;
    jgamma = gamma;
    for (int q = 0; q < nql; ++q) {
        double* rec = &jq[8 * (size_t)q];
        const double qmod = std::sqrt(rec[3]);
        rec[4] = gamma * std::exp(-beta * qmod) / qmod;
    }
}

int Setup::set_jastrow_spline(const double* knots, int n, std::string& err)
{
    if (n != 0 && n != kJastrowKnots) {
        err = "the Jastrow spline has 16 knots (0 switches it off)";
        return DMC_ERR_INVALID;
    }
    if (n > 0 && !knots) {
        err = "no knot values";
        return DMC_ERR_INVALID;
    }
    for (int k = 0; k < n; ++k)
        if (!std::isfinite(knots[k])) {
            err = "knot values must be finite";
            return DMC_ERR_INVALID;
        }
    jknots.assign(knots, knots + n);
    utab[0] = uref;
    dutab[0] = duref;
    d2utab[0] = d2uref;
    if (n == 0) return DMC_OK;
    const double h = el / kJastrowCells, dr = range / ntab;
    for (int i = 0; i <= ntab; ++i) {
        const double r = i * dr;
        double u = 0.0, du = 0.0, d2u = 0.0;
        for (int k = 0; k < n; ++k) {
            double f, fp, fpp;
            jastrow_knot_basis(k, r, h, f, fp, fpp);
            u += jknots[k] * f;
            du += jknots[k] * fp;
            d2u += jknots[k] * fpp;
        }
        utab[0][i] += u;
        dutab[0][i] += du;
        d2utab[0][i] += d2u;
    }
    return DMC_OK;
}

void Setup::set_beta(double b, double d, double bf)
{
    bbeta = b;
    dbeta = d;
    bfact = bf;
    beta_tables(*this, b, d, bf);
}

void Setup::knot_basis_tables(std::vector<double> (&out)[3]) const
{
    const double h = el / kJastrowCells, dr = range / ntab;
    const size_t nt = (size_t)ntab + 1;
    for (auto& o : out) o.assign((size_t)kJastrowKnots * nt, 0.0);
    for (int k = 0; k < kJastrowKnots; ++k)
        for (int i = 0; i <= ntab; ++i) {
            double f, fp, fpp;
            jastrow_knot_basis(k, i * dr, h, f, fp, fpp);
            out[0][k * nt + i] = f;
            out[1][k * nt + i] = fp;
            out[2][k * nt + i] = fpp;
        }
}

void Setup::beta_param_tables(std::vector<double> (&out)[2][3]) const
{
    using C = std::complex<double>;
    const double h = 1.0e-20;
    for (int which = 0; which < 2; ++which) {
        std::vector<C> t[3];
        const C bb(bbeta, which == 0 ? h * std::max(1.0, std::fabs(bbeta)) : 0.0);
        const C dd(dbeta, which == 1 ? h * std::max(1.0, std::fabs(dbeta)) : 0.0);
        const double step = which == 0 ? bb.imag() : dd.imag();
        beta_tables_t<C>(el, ntabb, bb, dd, bfact, t[0], t[1], t[2]);
        for (int m = 0; m < 3; ++m) {
            out[which][m].resize(t[m].size());
            for (size_t i = 0; i < t[m].size(); ++i) out[which][m][i] = t[m][i].imag() / step;
        }
    }
}

int Setup::set_vorb(const double* v, int n, std::string& err)
{
    if (n != norb) {
        err = "set_vorb: norb mismatch";
        return DMC_ERR_INVALID;
    }
    vorb.assign(v, v + n);
    return DMC_OK;
}

}  // namespace dmc
