// Host-side set-up of one DMCBS system: the module state that the reference
// builds once in setpsi/setupbcs/setbeta/setphi/setstep before the walker
// loop.  Everything here runs once per context on the CPU; the tables are
// then uploaded to the GPU.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/dmcbcs_gpu.h"

namespace dmc {

// One k vector of the s-wave pairing basis: integer lattice vector n and
// k = 2*pi*n/L (kshell.f90:141-155).
struct KVec {
    int n[3];
    double k[3];
    double k2;
    int shell;   // 1-based shell index of the reference's vorb(shell)
};

// kstates3d (kshell.f90:20-156): the half set of k vectors of shells
// 1..nsh0 (k = 0 first) and the half-shell sizes numsh0[nsh0].
int k_shells(double el, int nsh0, std::vector<KVec>& out, std::vector<int>& numsh0, std::string& err);

struct Setup {
    // sizes
    int npart = 0, nup = 0, ndn = 0, npair = 0, nexup = 0, nexdn = 0, nd = 0;
    int norb = 0, nk = 0, ncol = 0, ntab = 0, nmax = 0;
    // box and species
    double el = 0, eli = 0, rho = 0;
    double mass[2] = {1, 1}, sqm[2] = {1, 1};
    double hbar = 0.5;
    double a2 = 0;
    // s-wave pairing (psislaterbcs.f90:5-21)
    std::vector<KVec> kv;          // nk entries, kv[0] = 0
    std::vector<int> numsh;        // half-shell sizes per shell (norb)
    std::vector<double> vorb;      // norb
    double akup[DMC_MAX_UNPAIRED][3], ak2up[DMC_MAX_UNPAIRED];
    double akdn[DMC_MAX_UNPAIRED][3], ak2dn[DMC_MAX_UNPAIRED];
    int sinup[DMC_MAX_UNPAIRED], sindn[DMC_MAX_UNPAIRED];
    // one-body and long-range Jastrow
    double qex[3] = {0, 0, 0}, v0ex = 0, v0exjas = 0;
    int numq = 0;
    // long-range Jastrow: nql q vectors, 8 doubles each (qx, qy, qz, q^2,
    // gamma exp(-beta |q|)/|q|, 0, 0, 0)
    int nql = 0;
    std::vector<double> jq;
    double jbeta = 0, jgamma = 0;
    // beta table (betafun.f90): swbtab, swdbtab, swd2btab on [0, L/2]
    bool nobeta = true;
    int ntabb = 0;
    double rangeb = 0, scaleb = 0;
    std::vector<double> btab, dbtab, d2btab;
    // Jastrow + potential tables (coshpot.f90), [ic][0..ntab]
    double range = 0, scale = 0, hbarp = 1;
    int ntab0 = 0;   // grid index of the healing distance
    double cjas[2] = {0, 0};
    bool iop = false, ieq = false;
    std::vector<double> utab[2], dutab[2], d2utab[2], vtab[2];
    // units (dmcbcs.f90:146-170) and step (step.f90:11-41)
    double eunit = 1, nfac = 1, etrial = 0;
    double kunit = 1;              // k_F of the unit system (dmcbcs.f90:150,158)
    double sigma[2] = {0, 0}, dcut[2] = {0, 0};
    bool cutdrift = false;

    // Returns DMC_OK or an error code with a message in err.
    // beta parameters as read (setbeta, betafun.f90:19-21)
    double bbeta = 0, dbeta = 0, bfact = 0;
    // the reference's up-down Jastrow tables and the opt-in spline on top
    // (dmc_spline.h): jknots empty = off
    std::vector<double> uref, duref, d2uref;
    std::vector<double> jknots;

    int build(const dmc_system_desc& sd, const dmc_run_desc& rd, std::string& err);
    // the up-down Jastrow = reference + sum_k knots[k] phi_k (n = 16), or the
    // reference alone (n = 0); rebuilds utab/dutab/d2utab[0]
    int set_jastrow_spline(const double* knots, int n, std::string& err);
    // phi_k, phi_k', phi_k'' of every knot k < 16 at every point of the
    // up-down table grid (the values set_jastrow_spline adds to the table):
    // out[m][k * (ntab + 1) + i]
    void knot_basis_tables(std::vector<double> (&out)[3]) const;
    // d/db and d/dd of the beta tables (btab, dbtab, d2btab, bfact-scaled):
    // out[0][*] for b, out[1][*] for d, each ntabb + 1 values
    void beta_param_tables(std::vector<double> (&out)[2][3]) const;
    // new b, d and bfact of the beta function (on): rebuilds its tables
    void set_beta(double b, double d, double bf);
    int set_vorb(const double* v, int n, std::string& err);
    // setjasparam (jastrowlongrange.f90:57-61): new beta, gamma; recomputes
    // the q-vector weights
    void set_jaslong(double beta, double gamma);
};

}  // namespace dmc
