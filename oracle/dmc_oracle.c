/*
 * dmc_oracle.c -- CPU oracle for the DMCBS walker hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a plain-C restatement of the
 * reference Fortran (CalebRHicks/DMCBS_Project) for the walker hot path.
 * The tests hold the CUDA product library against it: only the tests, the
 * smoke check and the CPU-baseline leg of the benchmark load it.  The
 * product never links, loads or calls it.
 *
 * Parity status.  The reference is Fortran + MPI + MKL and cannot be built
 * on these machines (no Fortran compiler, no MPI, no MKL/LAPACK), and it
 * ships no tests or golden outputs.  Parity with the reference's own outputs
 * is therefore UNPINNED.  Pieces are pinned independently:
 *   - ran1/ran2 against an integer restatement of the recurrence,
 *   - orc_matinv (restated dgetrf+dgetri) against LAPACK dgetrf/dgetri,
 *   - hpsi against analytic known answers (free Fermi gas, one pair) and
 *     against central finite differences (the reference's own chkder /
 *     chkone / chkderp self-checks, restated as tests),
 *   - the setup tables against their defining equations.
 *
 * Every routine follows one reference routine (file:line), keeping its
 * operation and summation order.  Arrays keep the Fortran column-major
 * layout: a(i,j) of an n x m array is a[(i-1) + (j-1)*n].
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/dmcbcs_gpu.h"

#define R8 double
#define MAXP DMC_MAX_PART

/* ------------------------------------------------------------------------ */
/* random numbers: ran.f90                                                  */
/* ------------------------------------------------------------------------ */

static const int64_t MASK24 = (((int64_t)1) << 24) - 1;
static const int64_t MASK48 = (((int64_t)1) << 48) - 1;
#define TWOM48 (1.0 / 281474976710656.0)

/* ran1, ran.f90:8-27: 48-bit LCG in two 24-bit limbs. */
double orc_ran1(int64_t* irn)
{
    const int64_t mult1 = 44485709377909LL;
    const int64_t m11 = mult1 & MASK24, m12 = (mult1 >> 24) & MASK24;
    const int64_t iadd1 = 96309754297LL;
    int64_t is2 = ((*irn) >> 24) & MASK24;
    int64_t is1 = (*irn) & MASK24;
    *irn = ((((is1 * m12 + is2 * m11) & MASK24) << 24) + is1 * m11 + iadd1) & MASK48;
    return (double)((*irn) | 1) * TWOM48;
}

/* ran2, ran.f90:29-48. */
double orc_ran2(int64_t* irn)
{
    const int64_t mult2 = 34522712143931LL;
    const int64_t m21 = mult2 & MASK24, m22 = (mult2 >> 24) & MASK24;
    const int64_t iadd2 = 55789347517LL;
    int64_t is2 = ((*irn) >> 24) & MASK24;
    int64_t is1 = (*irn) & MASK24;
    *irn = ((((is1 * m22 + is2 * m21) & MASK24) << 24) + is1 * m21 + iadd2) & MASK48;
    return (double)((*irn) | 1) * TWOM48;
}

/* randn, ran.f90:60-72 (the module stream is passed explicitly). */
static void randn(int64_t* irn, int n, double* out)
{
    for (int i = 0; i < n; i++) out[i] = orc_ran1(irn);
}

/* gaussian, ran.f90:74-104: Box-Muller over pairs. */
static void gaussian(int64_t* irn, int n, double* g)
{
    double rn[3 * MAXP + 2];
    int nr = 2 * ((n + 1) / 2);
    double pi = 4.0 * atan(1.0);
    randn(irn, nr, rn);
    for (int i = 1; i <= n / 2; i++) {
        double rn1 = rn[2 * i - 2], rn2 = rn[2 * i - 1];
        double arg = 2.0 * pi * rn1;
        double x1 = sin(arg), x2 = cos(arg), x3 = sqrt(-2.0 * log(rn2));
        g[2 * i - 2] = x1 * x3;
        g[2 * i - 1] = x2 * x3;
    }
    if (n % 2 != 0) {
        double rn1 = rn[n - 1], rn2 = rn[n];
        double arg = 2.0 * pi * rn1;
        g[n - 1] = cos(arg) * sqrt(-2.0 * log(rn2));
    }
}

void orc_gaussian(int64_t* irn, int n, double* g) { gaussian(irn, n, g); }

/* Fortran nint: round half away from zero. */
static inline double fnint(double a) { return round(a); }
static inline double fsign(double a, double b) { return copysign(fabs(a), b); }

/* ------------------------------------------------------------------------ */
/* state                                                                    */
/* ------------------------------------------------------------------------ */

typedef struct {
    double *x, *dpsi, *dpsig;                 /* [cap][npart][3] */
    double *psil, *d2psi, *v, *weight, *psigl, *d2psig, *psil0, *psigl0, *vext;
    float* wt0;                               /* real(kind=i4): single precision */
    int* is;
    int64_t* irn;
    int n;
} wstack;

typedef struct orc_state {
    /* system */
    int ndim, npart, nbin[2], ntab;
    double mass[2], hbar, a2;
    double pmass[MAXP], sqm[MAXP];
    /* slaterbcs, psislaterbcs.f90:5-21 */
    double el, rho;
    int npair, nup, ndn, nexup, nexdn, norb, nk, nd;
    double akup[DMC_MAX_UNPAIRED][3], akdn[DMC_MAX_UNPAIRED][3];
    double ak2up[DMC_MAX_UNPAIRED], ak2dn[DMC_MAX_UNPAIRED];
    int sinup[DMC_MAX_UNPAIRED], sindn[DMC_MAX_UNPAIRED];
    double vorb[DMC_MAX_SHELLS];
    int numsh[DMC_MAX_SHELLS];
    double *ak, *ak2;                         /* ak(3,nk), ak2(nk) */
    double qex[3], v0ex, v0exjas;
    /* jaslong, jastrowlongrange.f90:5-8 */
    int numq, nkq;
    double *akq, *ak2q, jbeta, jgamma;
    /* betafun, betafun.f90:5-10 */
    int nobeta, ntabb;
    double rangeb, scaleb, b, c, d, small, c0, c1, c2, c3, c4;
    double *swbtab, *swdbtab, *swd2btab;      /* (0:ntabb) */
    /* potential, coshpot.f90:5-12 */
    double hbarp, v0, amu, range, scale, eli, cjas[2], djas, v0op, v0eq;
    int iop, ieq;
    double *utab, *dutab, *d2utab, *vtab;     /* (2,0:ntab): [ic + 2*i] */
    /* opt-in up-down Jastrow spline on top of the reference's table (no
       counterpart in the reference): the reference's ic = 0 columns and
       the knot values, njk = 0 or 16 */
    double *uref0, *duref0, *d2uref0;
    double jknots[16];
    int njk;
    /* step, step.f90:5-9 */
    int idmc, cutdrift, fn;
    double dt, etrial, nfac, wtcut, eunit;
    double sigma[MAXP], dcut[MAXP];
    int64_t wtisto[DMC_WTISTO];
    /* run */
    int nwalk, cap;
    double popup, popdn;
    int64_t seed;
    wstack st[2];
    int istin;                                /* 0 or 1 */
    /* estimator.f90 */
    int nest;
    double valblk[DMC_NEST_MAX], valblk2[DMC_NEST_MAX], wtblk[DMC_NEST_MAX];
    int nthreads;
    /* operators.f90 (g(r), S(q), n(k)); NULL until orc_set_operators */
    struct orc_ops* ops;
} orc_state;
static void free_ops(struct orc_ops* o);

/* ------------------------------------------------------------------------ */
/* k shells: kshell.f90:20-156                                              */
/* ------------------------------------------------------------------------ */

static int kstates3d(double elbox, int nsh0, int* numsh0, double** akout, double** ak2out, int* nkout)
{
    int i2max = 2 * nsh0;
    int imax = (int)lroundf(sqrtf((float)i2max));    /* nint(sqrt(real(i2max))) */
    int nk = 0;
    for (int ix = 0; ix <= imax; ix++)
        for (int iy = 0; iy <= imax; iy++)
            for (int iz = 0; iz <= imax; iz++) {
                int i2 = ix * ix + iy * iy + iz * iz;
                if (i2 <= i2max) {
                    nk++;
                    if (ix == 0 && iy != 0 && iz != 0) nk++;
                    if (iy == 0 && ix != 0 && iz != 0) nk++;
                    if (iz == 0 && ix != 0 && iy != 0) nk++;
                    if (ix != 0 && iy != 0 && iz != 0) nk += 3;
                }
            }
    int* ik = (int*)calloc((size_t)nk * 3, sizeof(int));   /* iktmp(nk,3): [i][c] */
    nk = 0;
#define SETK(a, b, c) do { ik[nk * 3 + 0] = (a); ik[nk * 3 + 1] = (b); ik[nk * 3 + 2] = (c); nk++; } while (0)
    for (int ix = 0; ix <= imax; ix++)
        for (int iy = 0; iy <= imax; iy++)
            for (int iz = 0; iz <= imax; iz++) {
                int i2 = ix * ix + iy * iy + iz * iz;
                if (i2 <= i2max) {
                    SETK(ix, iy, iz);
                    if (ix == 0 && iy != 0 && iz != 0) SETK(ix, iy, -iz);
                    if (iy == 0 && ix != 0 && iz != 0) SETK(ix, iy, -iz);
                    if (iz == 0 && ix != 0 && iy != 0) SETK(ix, -iy, iz);
                    if (ix != 0 && iy != 0 && iz != 0) {
                        SETK(ix, iy, -iz);
                        SETK(ix, -iy, iz);
                        SETK(ix, -iy, -iz);
                    }
                }
            }
#undef SETK
    /* exchange sort, kshell.f90:110-118 (swaps on >=) */
    for (int i = 0; i < nk - 1; i++)
        for (int j = i + 1; j < nk; j++) {
            int si = ik[i * 3] * ik[i * 3] + ik[i * 3 + 1] * ik[i * 3 + 1] + ik[i * 3 + 2] * ik[i * 3 + 2];
            int sj = ik[j * 3] * ik[j * 3] + ik[j * 3 + 1] * ik[j * 3 + 1] + ik[j * 3 + 2] * ik[j * 3 + 2];
            if (si >= sj) {
                for (int c = 0; c < 3; c++) { int t = ik[i * 3 + c]; ik[i * 3 + c] = ik[j * 3 + c]; ik[j * 3 + c] = t; }
            }
        }
    int* numsh = (int*)calloc((size_t)nk + 1, sizeof(int));    /* 1-based */
    int i2m = 0, nsh = 1;
    for (int i = 0; i < nk; i++) {
        int i2 = ik[i * 3] * ik[i * 3] + ik[i * 3 + 1] * ik[i * 3 + 1] + ik[i * 3 + 2] * ik[i * 3 + 2];
        if (i2 > i2m) { nsh++; i2m = i2; }
        numsh[nsh]++;
    }
    for (int i = 1; i <= nsh; i++) numsh[i] *= 2;
    double pi = 4.0 * atan(1.0);
    double piel = 2.0 * pi / elbox;
    if (nsh0 >= nsh) { free(ik); free(numsh); return -1; }   /* "Too many states" */
    int nkk = 1;
    for (int i = 2; i <= nsh0; i++) nkk += numsh[i] / 2;
    double* ak = (double*)calloc((size_t)3 * (nkk > 0 ? nkk : 1), sizeof(double));
    double* ak2 = (double*)calloc((size_t)(nkk > 0 ? nkk : 1), sizeof(double));
    int k = 0;
    for (int i = 1; i <= nsh0; i++) {
        numsh0[i - 1] = numsh[i] / 2;
        int m = numsh[i] / 2 > 1 ? numsh[i] / 2 : 1;
        for (int j = 0; j < m; j++) {
            ak[3 * k + 0] = piel * ik[k * 3 + 0];
            ak[3 * k + 1] = piel * ik[k * 3 + 1];
            ak[3 * k + 2] = piel * ik[k * 3 + 2];
            ak2[k] = ak[3 * k] * ak[3 * k] + ak[3 * k + 1] * ak[3 * k + 1] + ak[3 * k + 2] * ak[3 * k + 2];
            k++;
        }
    }
    free(ik);
    free(numsh);
    *akout = ak;
    *ak2out = ak2;
    *nkout = nkk;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* beta function: betafun.f90                                               */
/* ------------------------------------------------------------------------ */

/* beta0, betafun.f90:127-149 */
static void beta0(const orc_state* s, double r, double* b1, double* b1p, double* b1pp)
{
    double b = s->b, c = s->c, d = s->d;
    double x;
    if (r < s->small) {
        x = b * r;
        *b1 = s->c0 + x * (s->c1 + x * (s->c2 + x * (s->c3 + x * s->c4)));
        *b1p = s->c1 + x * (2.0 * s->c2 + x * (3.0 * s->c3 + 4.0 * s->c4 * x));
        *b1pp = 2.0 * s->c2 + x * (6.0 * s->c3 + 12.0 * s->c4 * x);
    } else {
        x = b * r;
        double ex = exp(-x);
        double ex10 = exp(-d * x);
        *b1 = (1.0 + c * x) * (1.0 - ex10) * ex / x;
        *b1p = ex * (-1.0 - x * (1.0 + c * x) + ex10 * (1.0 + x * (1.0 + d) * (1.0 + c * x))) / (x * x);
        *b1pp = ex * (2.0 + x * (2.0 + x * (1.0 + c * x))
                      - ex10 * (2.0 + x * (1.0 + d) * (2.0 + x * (1.0 + d) * (1.0 + x * c)))) / (x * x * x);
    }
    *b1p = b * (*b1p);
    *b1pp = (b * b) * (*b1pp);
    *b1 = *b1 / d;
    *b1p = *b1p / d;
    *b1pp = *b1pp / d;
}

/* beta, betafun.f90:151-171 */
static void betaf(const orc_state* s, double r, double* b1, double* b1p, double* b1pp)
{
    const double tiny = 1.0e-14;
    double el = s->el;
    if (r > el * 0.5) { *b1 = 0.0; *b1p = 0.0; *b1pp = 0.0; return; }
    double bet0, d1, d2, bet1, bet1p, bet1pp, bet2, bet2p, bet2pp;
    beta0(s, el * 0.5, &bet0, &d1, &d2);
    beta0(s, r, &bet1, &bet1p, &bet1pp);
    beta0(s, el - r, &bet2, &bet2p, &bet2pp);
    *b1 = bet1 + bet2 - 2.0 * bet0;
    *b1p = (r < tiny) ? 0.0 : bet1p - bet2p;
    *b1pp = bet1pp + bet2pp;
}

/* initbeta, betafun.f90:74-125 */
static void initbeta(orc_state* s, double bbeta, double dbeta)
{
    double el = s->el;
    double b = bbeta, d = dbeta;
    s->b = b;
    s->d = d;
    s->c = 0.5 * (2.0 + 2.0 * d * b * el + (d * b * el) * (d * b * el) * exp(b * el * (1.0 + d))
                  + 2.0 * d * b * b * el * el * exp(b * el * (1.0 + d)) + 2.0 * b * el
                  - 2.0 * exp(d * b * el) * b * el - 2.0 * exp(d * b * el))
           / (el * el * (exp(d * b * el) - 1.0 - d + d * exp(b * el * (1.0 + d))) * (b * b));
    double c = s->c;
    s->c0 = d;
    s->small = 1.0e-3 / b;
    s->c1 = -d + c * d - d * d / 2.0;
    s->c2 = d / 2.0 + d * d / 2.0 + d * d * d / 6.0 + c * (-d - d * d / 2.0);
    s->c3 = -d / 6.0 - d * d / 4.0 - d * d * d / 6.0 - d * d * d * d / 24.0
            + c * (d / 2.0 + d * d / 2.0 + d * d * d / 6.0);
    s->c4 = d / 24.0 + d * d / 12.0 + d * d * d / 12.0 + d * d * d * d / 24.0 + d * d * d * d * d / 120.0
            - c * (d / 6.0 + d * d / 4.0 + d * d * d / 6.0 + d * d * d * d / 24.0);
    int ntabb = s->ntabb;
    double dr = 0.5 * el / ntabb;
    int nj = 0;
    double betan = 10.0, dum1, dum2;
    while (fabs(betan) > 1.0e-10) {
        nj++;
        betaf(s, el * nj, &betan, &dum1, &dum2);
    }
    for (int i = 0; i <= ntabb; i++) {
        double r = i * dr, b1, b1p, b1pp;
        betaf(s, r, &b1, &b1p, &b1pp);
        s->swbtab[i] = b1;
        s->swdbtab[i] = b1p;
        s->swd2btab[i] = b1pp;
        for (int j = 1; j <= nj; j++) {
            double b2, b2p, b2pp, b3, b3p, b3pp;
            betaf(s, j * el - r, &b2, &b2p, &b2pp);
            betaf(s, j * el + r, &b3, &b3p, &b3pp);
            s->swbtab[i] = s->swbtab[i] + b2 + b3;
            s->swdbtab[i] = s->swdbtab[i] - b2p + b3p;
            s->swd2btab[i] = s->swd2btab[i] + b2pp + b3pp;
        }
    }
    for (int i = 0; i <= ntabb; i++) {
        double r = i * dr;
        s->swbtab[i] = s->swbtab[i] - s->swbtab[ntabb];
        if (i != 0)
            s->swd2btab[i] = s->swd2btab[i] + (s->ndim - 1.0) * s->swdbtab[i] / r;
        else
            s->swd2btab[i] = 3.0 * s->swd2btab[i];
    }
}

/* radialfun, betafun.f90:173-194 */
static void radialfun(const orc_state* s, double r, double* f, double* df, double* d2f)
{
    if (s->nobeta || r > s->rangeb) { *f = 0.0; *df = 0.0; *d2f = 0.0; return; }
    double ddr = s->scaleb * r;
    int index = (int)ddr;
    if (index > s->ntabb - 2) index = s->ntabb - 2;
    if (index < 1) index = 1;
    ddr = ddr - index;
    double a1 = -ddr * (ddr - 1.0) * (ddr - 2.0) / 6.0;
    double a2 = (ddr + 1.0) * (ddr - 1.0) * (ddr - 2.0) / 2.0;
    double a3 = -(ddr + 1.0) * ddr * (ddr - 2.0) / 2.0;
    double a4 = (ddr + 1.0) * ddr * (ddr - 1.0) / 6.0;
    const double *t = s->swbtab, *dt = s->swdbtab, *d2t = s->swd2btab;
    *f = a1 * t[index - 1] + a2 * t[index] + a3 * t[index + 1] + a4 * t[index + 2];
    *df = a1 * dt[index - 1] + a2 * dt[index] + a3 * dt[index + 1] + a4 * dt[index + 2];
    *d2f = a1 * d2t[index - 1] + a2 * d2t[index] + a3 * d2t[index + 1] + a4 * d2t[index + 2];
}

void orc_radialfun(const orc_state* s, double r, double* f3)
{
    radialfun(s, r, &f3[0], &f3[1], &f3[2]);
}

/* ------------------------------------------------------------------------ */
/* Jastrow and potential tables: coshpot.f90, rungekutta.f90                */
/* ------------------------------------------------------------------------ */

/* vpot, coshpot.f90:145-152 */
static double vpot(const orc_state* s, double v0, double r)
{
    double ch = cosh(s->amu * r);
    return -2.0 * v0 * (s->amu * s->amu) * s->hbarp / (ch * ch);
}

/* rk3d, rungekutta.f90:127-150 */
static void rk3d(const orc_state* s, double v0, double* psi, double* dpsi, double ene, double hb,
                 double dr, int ntab, int* ncross)
{
    psi[0] = 0.0;
    dpsi[0] = 1.0;
    *ncross = 0;
    for (int i = 1; i <= ntab; i++) {
        double r = (i - 1) * dr;
        double k1a = -(ene - vpot(s, v0, r)) * psi[i - 1] / hb;
        double k1b = dpsi[i - 1];
        double k2a = -(ene - vpot(s, v0, r + 0.5 * dr)) * (psi[i - 1] + 0.5 * dr * k1b) / hb;
        double k2b = dpsi[i - 1] + 0.5 * dr * k1a;
        double k3a = -(ene - vpot(s, v0, r + 0.5 * dr)) * (psi[i - 1] + 0.5 * dr * k2b) / hb;
        double k3b = dpsi[i - 1] + 0.5 * dr * k2a;
        double k4a = -(ene - vpot(s, v0, r + dr)) * (psi[i - 1] + dr * k3b) / hb;
        double k4b = dpsi[i - 1] + dr * k3a;
        dpsi[i] = dpsi[i - 1] + (k1a + 2.0 * k2a + 2.0 * k3a + k4a) * dr / 6.0;
        psi[i] = psi[i - 1] + (k1b + 2.0 * k2b + 2.0 * k3b + k4b) * dr / 6.0;
        if (psi[i] != fsign(psi[i], psi[i - 1])) (*ncross)++;
    }
}

/* orbital (3-D branch), rungekutta.f90:8-17,57-99 */
static int orbital3d(const orc_state* s, double v0, double* psi, double* dpsi, double* d2psi,
                     double hb, int ntab, double dr, int nodes)
{
    const double convergence = 1.0e-8;
    const int itmax = 100;
    double emax = vpot(s, v0, 0.0), emin = emax;
    for (int i = 1; i <= ntab; i++) {
        double vv = vpot(s, v0, i * dr);
        emax = emax > vv ? emax : vv;
        emin = emin < vv ? emin : vv;
    }
    emax = 0.001;
    int ncross;
    rk3d(s, v0, psi, dpsi, emax, hb, dr, ntab, &ncross);
    while (ncross <= nodes) {
        emax = 2.0 * emax;
        rk3d(s, v0, psi, dpsi, emax, hb, dr, ntab, &ncross);
    }
    double ene = 0.5 * (emin + emax);
    int iter = 0;
    for (;;) {
        rk3d(s, v0, psi, dpsi, ene, hb, dr, ntab, &ncross);
        double r = dr * ntab;
        double der = (dpsi[ntab] - psi[ntab] / r) / r;
        der = der / psi[ntab];
        if (der < 0.0) emax = ene; else emin = ene;
        if (fabs(der) < convergence) break;
        ene = 0.5 * (emin + emax);
        iter++;
        if (iter > itmax) return -1;   /* "orbital: no convergence" */
    }
    psi[0] = dpsi[0];
    d2psi[0] = (vpot(s, v0, 0.0) - ene) * dpsi[0] / (3.0 * hb);
    dpsi[0] = 0.0;
    for (int i = 1; i <= ntab; i++) {
        double r = i * dr;
        dpsi[i] = (dpsi[i] - psi[i] / r) / r;
        psi[i] = psi[i] / r;
        d2psi[i] = (vpot(s, v0, r) - ene) * psi[i] / hb - 2.0 * dpsi[i] / r;
    }
    return 0;
}

/* setphi, coshpot.f90:14-143 (hbin = hbar/(2 mu), dmcbcs.f90:143) */
static int setphi(orc_state* s, double hbin)
{
    int ntab = s->ntab;
    double el = s->el;
    s->eli = (el != 0.0) ? 1.0 / el : 0.0;
    s->hbarp = 2.0 * hbin;
    double el2 = 0.5 * el;
    s->range = (el != 0.0) ? 0.5 * el : s->djas;
    double dr = s->range / ntab;
    s->scale = 1.0 / dr;
    s->iop = 0;
    s->ieq = 0;
    s->vtab = (double*)calloc((size_t)2 * (ntab + 1), sizeof(double));
    for (int i = 0; i <= ntab; i++) {
        double r = i * dr;
        s->vtab[0 + 2 * i] = vpot(s, s->v0, r);
        s->vtab[1 + 2 * i] = 0.0;
        s->iop = 1;
    }
    int ntab0 = (int)(ntab * s->djas / el2);
    if (el == 0.0) ntab0 = (int)(ntab * s->djas / s->range);
    s->utab = (double*)calloc((size_t)2 * (ntab + 1), sizeof(double));
    s->dutab = (double*)calloc((size_t)2 * (ntab + 1), sizeof(double));
    s->d2utab = (double*)calloc((size_t)2 * (ntab + 1), sizeof(double));
    double* f = (double*)calloc((size_t)ntab0 + 1, sizeof(double));
    double* df = (double*)calloc((size_t)ntab0 + 1, sizeof(double));
    double* d2f = (double*)calloc((size_t)ntab0 + 1, sizeof(double));
    int rc = 0;
    for (int ic = 0; ic < 2; ic++) {
        if (s->cjas[ic] != 0.0) {
            double v0use = (ic == 0) ? s->v0op : s->v0eq;
            if (orbital3d(s, v0use, f, df, d2f, s->hbarp, ntab0, dr, 0) != 0) { rc = -1; break; }
            for (int i = 0; i <= ntab0; i++) {
                s->utab[ic + 2 * i] = f[i] / f[ntab0];
                s->dutab[ic + 2 * i] = df[i] / f[ntab0];
                s->d2utab[ic + 2 * i] = d2f[i] / f[ntab0];
            }
        }
    }
    free(f); free(df); free(d2f);
    if (rc) return rc;
    if (ntab0 < ntab) {
        for (int i = ntab0 + 1; i <= ntab; i++)
            for (int ic = 0; ic < 2; ic++) {
                s->utab[ic + 2 * i] = 1.0;
                s->dutab[ic + 2 * i] = 0.0;
                s->d2utab[ic + 2 * i] = 0.0;
            }
    }
    for (int ic = 0; ic < 2; ic++) {
        for (int i = 0; i <= ntab; i++) {
            double* u = &s->utab[ic + 2 * i];
            double* du = &s->dutab[ic + 2 * i];
            double* d2u = &s->d2utab[ic + 2 * i];
            if (s->cjas[ic] != 0.0) {
                *du = *du / *u;
                *d2u = *d2u / *u - (*du) * (*du);
                *u = log(*u);
            }
            *u = s->cjas[ic] * (*u);
            *du = s->cjas[ic] * (*du);
            *d2u = s->cjas[ic] * (*d2u);
        }
    }
    if (s->cjas[0] != 0.0) s->iop = 1;
    if (s->cjas[1] != 0.0) s->ieq = 1;
    s->uref0 = (double*)calloc((size_t)ntab + 1, sizeof(double));
    s->duref0 = (double*)calloc((size_t)ntab + 1, sizeof(double));
    s->d2uref0 = (double*)calloc((size_t)ntab + 1, sizeof(double));
    for (int i = 0; i <= ntab; i++) {
        s->uref0[i] = s->utab[2 * i];
        s->duref0[i] = s->dutab[2 * i];
        s->d2uref0[i] = s->d2utab[2 * i];
    }
    s->njk = 0;
    return 0;
}

/* The opt-in up-down Jastrow spline (the library's own addition, restated
 * here from its definition): u_s(r) = sum_k t_k phi_k(r) with knot spacing
 * h = L/34, phi_0(r) = B(r/h), phi_k(r) = B(r/h - k) + B(r/h + k), B the
 * centred cubic B-spline on [-2, 2].  Returns phi_k and its first two
 * r-derivatives. */
static void cubic_bspline(double t, double* f, double* fp, double* fpp)
{
    double a = fabs(t), sg = t < 0.0 ? -1.0 : 1.0;
    if (a >= 2.0) { *f = 0.0; *fp = 0.0; *fpp = 0.0; return; }
    if (a < 1.0) {
        *f = 2.0 / 3.0 - a * a + 0.5 * a * a * a;
        *fp = sg * (-2.0 * a + 1.5 * a * a);
        *fpp = -2.0 + 3.0 * a;
    } else {
        double q = 2.0 - a;
        *f = q * q * q / 6.0;
        *fp = -sg * 0.5 * q * q;
        *fpp = q;
    }
}

void orc_knot_basis(int k, double r, double h, double* out3)
{
    double f, fp, fpp;
    cubic_bspline(r / h - k, &f, &fp, &fpp);
    if (k > 0) {
        double f2, p2, q2;
        cubic_bspline(r / h + k, &f2, &p2, &q2);
        f += f2; fp += p2; fpp += q2;
    }
    out3[0] = f;
    out3[1] = fp / h;
    out3[2] = fpp / (h * h);
}

/* Sets the spline (n = 16 knots) or removes it (n = 0): the up-down
 * Jastrow table becomes the reference's plus u_s at every grid point. */
int orc_set_jastrow_spline(orc_state* s, const double* knots, int n)
{
    if (n != 0 && n != 16) return -1;
    s->njk = n;
    for (int k = 0; k < n; k++) s->jknots[k] = knots[k];
    double h = s->el / 34.0, dr = s->range / s->ntab;
    for (int i = 0; i <= s->ntab; i++) {
        double u = s->uref0[i], du = s->duref0[i], d2u = s->d2uref0[i];
        for (int k = 0; k < n; k++) {
            double b[3];
            orc_knot_basis(k, i * dr, h, b);
            u += s->jknots[k] * b[0];
            du += s->jknots[k] * b[1];
            d2u += s->jknots[k] * b[2];
        }
        s->utab[2 * i] = u;
        s->dutab[2 * i] = du;
        s->d2utab[2 * i] = d2u;
    }
    if (n > 0) s->iop = 1;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* set-up                                                                   */
/* ------------------------------------------------------------------------ */

static int alloc_stack(wstack* w, int cap, int npart)
{
    size_t v3 = (size_t)cap * npart * 3;
    w->x = (double*)calloc(v3, sizeof(double));
    w->dpsi = (double*)calloc(v3, sizeof(double));
    w->dpsig = (double*)calloc(v3, sizeof(double));
    w->psil = (double*)calloc(cap, sizeof(double));
    w->d2psi = (double*)calloc(cap, sizeof(double));
    w->v = (double*)calloc(cap, sizeof(double));
    w->weight = (double*)calloc(cap, sizeof(double));
    w->psigl = (double*)calloc(cap, sizeof(double));
    w->d2psig = (double*)calloc(cap, sizeof(double));
    w->psil0 = (double*)calloc(cap, sizeof(double));
    w->psigl0 = (double*)calloc(cap, sizeof(double));
    w->vext = (double*)calloc(cap, sizeof(double));
    w->wt0 = (float*)calloc(cap, sizeof(float));
    w->is = (int*)calloc(cap, sizeof(int));
    w->irn = (int64_t*)calloc(cap, sizeof(int64_t));
    w->n = 0;
    return (w->x && w->dpsi && w->dpsig && w->irn) ? 0 : -1;
}

static void free_stack(wstack* w)
{
    free(w->x); free(w->dpsi); free(w->dpsig); free(w->psil); free(w->d2psi); free(w->v);
    free(w->weight); free(w->psigl); free(w->d2psig); free(w->psil0); free(w->psigl0);
    free(w->vext); free(w->wt0); free(w->is); free(w->irn);
}

void orc_destroy(orc_state* s)
{
    if (!s) return;
    free(s->ak); free(s->ak2); free(s->akq); free(s->ak2q);
    free(s->swbtab); free(s->swdbtab); free(s->swd2btab);
    free(s->utab); free(s->dutab); free(s->d2utab); free(s->vtab);
    free(s->uref0); free(s->duref0); free(s->d2uref0);
    free_stack(&s->st[0]);
    free_stack(&s->st[1]);
    free_ops(s->ops);
    free(s);
}

/* Set-up of the modules in the order of dmcbcs.f90:142-177:
 * setpsi -> setupbcs (psislaterbcs.f90:23-153) -> setbeta (betafun.f90:12-72),
 * setjaslong; setphi; units (dmcbcs.f90:146-170); setstep (step.f90:11-41);
 * create (stack.f90:51-80).  Returns NULL on a set-up failure. */
orc_state* orc_create(const dmc_system_desc* sd, const dmc_run_desc* rd, int* status)
{
    orc_state* s = (orc_state*)calloc(1, sizeof(orc_state));
    *status = DMC_ERR_INVALID;
    if (!s) return NULL;
    if (sd->ndim != 3 || sd->nbin[0] < 0 || sd->nbin[1] < 0 || sd->nbin[0] + sd->nbin[1] > MAXP ||
        sd->nbin[0] + sd->nbin[1] < 1 || sd->norb < 0 || sd->norb > DMC_MAX_SHELLS ||
        sd->nexup < 0 || sd->nexup > DMC_MAX_UNPAIRED || sd->nexdn < 0 || sd->nexdn > DMC_MAX_UNPAIRED ||
        sd->ntab < 4 || sd->bfact < 0.0 || sd->rho <= 0.0) {
        free(s);
        return NULL;
    }
    s->ndim = 3;
    s->nbin[0] = sd->nbin[0];
    s->nbin[1] = sd->nbin[1];
    s->npart = sd->nbin[0] + sd->nbin[1];
    s->mass[0] = sd->mass[0];
    s->mass[1] = sd->mass[1];
    s->hbar = sd->hbar;
    s->ntab = sd->ntab;
    s->a2 = sd->a2;
    for (int i = 0; i < s->npart; i++) {
        s->pmass[i] = (i < s->nbin[0]) ? s->mass[0] : s->mass[1];
        s->sqm[i] = sqrt(s->pmass[i]);
    }
    /* setupbcs */
    s->rho = sd->rho;
    s->nexup = sd->nexup;
    s->nexdn = sd->nexdn;
    s->norb = sd->norb;
    for (int i = 0; i < s->norb; i++) s->vorb[i] = sd->vorb[i];
    s->el = pow(s->npart / s->rho, 1.0 / s->ndim);
    s->v0ex = sd->v0ex * 0.5;
    s->v0exjas = sd->v0exjas * s->v0ex;
    double pi = 4.0 * atan(1.0);
    for (int i = 0; i < s->nexup; i++) {
        s->sinup[i] = 0;
        for (int c = 0; c < 3; c++) {
            s->akup[i][c] = sd->ikup[i][c] * 2.0 * pi / s->el;
            if (sd->ikup[i][c] != 0) s->sinup[i] = (sd->ikup[i][c] < 0);
        }
        s->ak2up[i] = s->akup[i][0] * s->akup[i][0] + s->akup[i][1] * s->akup[i][1] + s->akup[i][2] * s->akup[i][2];
    }
    for (int i = 0; i < s->nexdn; i++) {
        s->sindn[i] = 0;
        for (int c = 0; c < 3; c++) {
            s->akdn[i][c] = sd->ikdn[i][c] * 2.0 * pi / s->el;
            if (sd->ikdn[i][c] != 0) s->sindn[i] = (sd->ikdn[i][c] < 0);
        }
        s->ak2dn[i] = s->akdn[i][0] * s->akdn[i][0] + s->akdn[i][1] * s->akdn[i][1] + s->akdn[i][2] * s->akdn[i][2];
    }
    if (kstates3d(s->el, s->norb, s->numsh, &s->ak, &s->ak2, &s->nk) != 0) {
        *status = DMC_ERR_SETUP;
        orc_destroy(s);
        return NULL;
    }
    int npair = s->npart - s->nexup - s->nexdn;
    if (npair % 2 != 0 || npair < 0) { orc_destroy(s); return NULL; }
    s->npair = npair / 2;
    s->nup = s->npair + s->nexup;
    s->ndn = s->npair + s->nexdn;
    s->nd = s->npair + s->nexup + s->nexdn;
    if (s->nup != s->nbin[0] || s->ndn != s->nbin[1]) { orc_destroy(s); return NULL; }
    /* setbeta */
    if (sd->bfact == 0.0) {
        s->nobeta = 1;
    } else {
        s->nobeta = 0;
        s->ntabb = s->ntab;
        s->swbtab = (double*)calloc((size_t)s->ntabb + 1, sizeof(double));
        s->swdbtab = (double*)calloc((size_t)s->ntabb + 1, sizeof(double));
        s->swd2btab = (double*)calloc((size_t)s->ntabb + 1, sizeof(double));
        s->rangeb = 0.5 * s->el;
        s->scaleb = s->ntabb / s->rangeb;
        initbeta(s, sd->bbeta, sd->dbeta);
        for (int i = 0; i <= s->ntabb; i++) {
            s->swbtab[i] = fabs(sd->bfact) * s->swbtab[i];
            s->swdbtab[i] = fabs(sd->bfact) * s->swdbtab[i];
            s->swd2btab[i] = fabs(sd->bfact) * s->swd2btab[i];
        }
    }
    for (int c = 0; c < 3; c++) s->qex[c] = sd->nqex[c] * 2.0 * pi / s->el;
    /* setjaslong, jastrowlongrange.f90:10-20 */
    s->numq = sd->numq;
    s->jbeta = sd->jbeta;
    s->jgamma = sd->jgamma;
    {
        int numshq[DMC_MAX_SHELLS + 1];
        if (s->numq < 0 || s->numq > DMC_MAX_SHELLS ||
            kstates3d(s->el, s->numq, numshq, &s->akq, &s->ak2q, &s->nkq) != 0) {
            *status = DMC_ERR_SETUP;
            orc_destroy(s);
            return NULL;
        }
    }
    /* setphi */
    s->v0 = sd->v0;
    s->amu = sd->amu;
    s->cjas[0] = sd->cjas[0];
    s->cjas[1] = sd->cjas[1];
    s->djas = sd->djas;
    s->v0op = (sd->v0op == 0.0) ? sd->v0 : sd->v0op;
    s->v0eq = (sd->v0eq == 0.0) ? sd->v0 : sd->v0eq;
    double mu = s->mass[0] * s->mass[1] / (s->mass[0] + s->mass[1]);
    if (setphi(s, s->hbar / (2.0 * mu)) != 0) {
        *status = DMC_ERR_SETUP;
        orc_destroy(s);
        return NULL;
    }
    /* units, dmcbcs.f90:146-170 */
    if (s->el != 0.0 && rd->units) {
        double rho = s->npart / pow(s->el, s->ndim);
        double kunit = pow(3.0 * (pi * pi) * rho, 1.0 / 3.0);
        s->eunit = 3.0 / (8.0 - s->ndim) * s->hbar / (2.0 * mu) * (kunit * kunit);
    } else {
        s->eunit = 1.0;
    }
    double etrial = rd->etrial * s->eunit;
    if (s->el != 0.0) etrial = etrial * s->npart;
    /* setstep, step.f90:11-41 */
    s->idmc = rd->idmc;
    s->dt = rd->dt;
    s->etrial = etrial;
    s->nfac = 1.0 / s->eunit;
    if (s->el != 0.0) s->nfac = s->nfac / s->npart;
    double sig = sqrt(2.0 * s->hbar * s->dt);
    s->wtcut = rd->wtcut;
    s->cutdrift = rd->dcut >= 0.0;
    for (int i = 0; i < s->npart; i++) {
        s->sigma[i] = sig / sqrt(s->pmass[i]);
        s->dcut[i] = s->cutdrift ? s->sigma[i] * rd->dcut : 0.0;
    }
    s->fn = rd->fn;
    s->nwalk = rd->nwalk;
    s->popup = rd->popup;
    s->popdn = rd->popdn;
    s->seed = rd->seed;
    double stmax = rd->stmax > 0.0 ? rd->stmax : 10.0;
    s->cap = (int)(rd->nwalk * stmax);
    if (s->cap < 1) s->cap = 1;
    if (alloc_stack(&s->st[0], s->cap, s->npart) || alloc_stack(&s->st[1], s->cap, s->npart)) {
        *status = DMC_ERR_NOMEM;
        orc_destroy(s);
        return NULL;
    }
    s->istin = 0;
    switch (s->idmc) {
    case -1: case 0: s->nest = 6; break;
    case -2: case 1: case 10: s->nest = 14; break;
    case 2: s->nest = 13; break;
    default: orc_destroy(s); return NULL;
    }
    s->nthreads = 1;
    *status = DMC_OK;
    return s;
}

void orc_set_threads(orc_state* s, int n) { s->nthreads = n > 0 ? n : 1; }

int orc_info(const orc_state* s, dmc_info* o)
{
    memset(o, 0, sizeof(*o));
    o->npart = s->npart; o->nup = s->nup; o->ndn = s->ndn; o->npair = s->npair;
    o->nexup = s->nexup; o->nexdn = s->nexdn; o->nd = s->nd; o->nk = s->nk;
    o->ncol = 2 * s->nk - 1; o->ntab = s->ntab; o->capacity = s->cap; o->nest = s->nest;
    o->el = s->el; o->eunit = s->eunit; o->nfac = s->nfac; o->etrial = s->etrial;
    o->sigma[0] = s->nbin[0] > 0 ? s->sigma[0] : 0.0;
    o->sigma[1] = s->nbin[1] > 0 ? s->sigma[s->nbin[0]] : 0.0;
    return 0;
}

int orc_get_table(const orc_state* s, int which, double* out, int n)
{
    int nt = s->ntab + 1;
    switch (which) {
    case 0: case 1: case 2: case 3: {
        const double* t = which == 0 ? s->utab : which == 1 ? s->dutab : which == 2 ? s->d2utab : s->vtab;
        if (n < 2 * nt) return -1;
        for (int ic = 0; ic < 2; ic++)
            for (int i = 0; i < nt; i++) out[ic * nt + i] = t[ic + 2 * i];
        return 0;
    }
    case 4: case 5: case 6: {
        if (n < nt) return -1;
        const double* t = which == 4 ? s->swbtab : which == 5 ? s->swdbtab : s->swd2btab;
        for (int i = 0; i < nt; i++) out[i] = s->nobeta ? 0.0 : t[i];
        return 0;
    }
    case 7:
        if (n < 3 * s->nk) return -1;
        memcpy(out, s->ak, sizeof(double) * 3 * s->nk);
        return 0;
    case 8:
        if (n < s->nk) return -1;
        memcpy(out, s->ak2, sizeof(double) * s->nk);
        return 0;
    case 9:
        if (n < s->norb) return -1;
        for (int i = 0; i < s->norb; i++) out[i] = s->numsh[i];
        return 0;
    }
    return -1;
}

/* setbcspar, psislaterbcs.f90:401-406 (optsw, no beta) */
int orc_set_vorb(orc_state* s, const double* vorb, int norb)
{
    if (norb != s->norb) return -1;
    for (int i = 0; i < norb; i++) s->vorb[i] = vorb[i];
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Jastrow + potential: getphi, coshpot.f90:154-205                         */
/* ------------------------------------------------------------------------ */

void orc_getphi(const orc_state* s, const double* x, double* u_, int* is_, double* du, double* d2u_, double* v_)
{
    const double tiny = 1.0e-14;
    int npart = s->npart, ntab = s->ntab;
    double u = 0.0, d2u = 0.0, v = 0.0;
    for (int k = 0; k < 3 * npart; k++) du[k] = 0.0;
    for (int i = 0; i < npart - 1; i++) {
        int spi = i < s->nbin[0] ? 1 : -1;
        for (int j = i + 1; j < npart; j++) {
            int spj = j < s->nbin[0] ? 1 : -1;
            if ((s->ieq && spi == spj) || (s->iop && spi != spj)) {
                double dx[3];
                for (int c = 0; c < 3; c++) {
                    dx[c] = x[3 * i + c] - x[3 * j + c];
                    dx[c] = dx[c] - s->el * fnint(dx[c] * s->eli);
                }
                double r = sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
                if (r < tiny) r = tiny;
                if (r < s->range) {
                    double dr = s->scale * r;
                    int index = (int)dr;
                    if (index > ntab - 2) index = ntab - 2;
                    if (index < 1) index = 1;
                    dr = dr - index;
                    double c1 = -dr * (dr - 1.0) * (dr - 2.0) / 6.0;
                    double c2 = (dr + 1.0) * (dr - 1.0) * (dr - 2.0) / 2.0;
                    double c3 = -(dr + 1.0) * dr * (dr - 2.0) / 2.0;
                    double c4 = (dr + 1.0) * dr * (dr - 1.0) / 6.0;
                    int it = (spi != spj) ? 0 : 1;
#define TB(t, k) (t)[it + 2 * (k)]
                    double vp = c1 * TB(s->vtab, index - 1) + c2 * TB(s->vtab, index)
                                + c3 * TB(s->vtab, index + 1) + c4 * TB(s->vtab, index + 2);
                    double uj = c1 * TB(s->utab, index - 1) + c2 * TB(s->utab, index)
                                + c3 * TB(s->utab, index + 1) + c4 * TB(s->utab, index + 2);
                    double duj = c1 * TB(s->dutab, index - 1) + c2 * TB(s->dutab, index)
                                 + c3 * TB(s->dutab, index + 1) + c4 * TB(s->dutab, index + 2);
                    double d2uj = c1 * TB(s->d2utab, index - 1) + c2 * TB(s->d2utab, index)
                                  + c3 * TB(s->d2utab, index + 1) + c4 * TB(s->d2utab, index + 2);
#undef TB
                    v = v + vp;
                    u = u + uj;
                    for (int c = 0; c < 3; c++) {
                        du[3 * i + c] = du[3 * i + c] + dx[c] * duj / (r * s->sqm[i]);
                        du[3 * j + c] = du[3 * j + c] - dx[c] * duj / (r * s->sqm[j]);
                    }
                    double mu = s->pmass[i] * s->pmass[j] / (s->pmass[i] + s->pmass[j]);
                    d2u = d2u + (d2uj + (s->ndim - 1.0) * duj / r) / mu;
                }
            }
        }
    }
    double ss = 0.0;
    for (int k = 0; k < 3 * npart; k++) ss += du[k] * du[k];
    d2u = d2u + ss;
    *u_ = u; *d2u_ = d2u; *v_ = v; *is_ = 1;
}

/* getphione, coshpot.f90:207-264 (drr = xold - xnew; i is 1-based) */
double orc_getphione(const orc_state* s, const double* x, const double* drr, int i1)
{
    const double tiny = 1.0e-14;
    int i = i1 - 1, ntab = s->ntab;
    double u = 0.0;
    int spi = i < s->nbin[0] ? 1 : -1;
    for (int j = 0; j < s->npart; j++) {
        if (j == i) continue;
        int spj = j < s->nbin[0] ? 1 : -1;
        if (!((s->ieq && spi == spj) || (s->iop && spi != spj))) continue;
        int it = (spi != spj) ? 0 : 1;
        for (int pass = 0; pass < 2; pass++) {
            double dx[3];
            for (int c = 0; c < 3; c++) {
                dx[c] = pass == 0 ? x[3 * i + c] - x[3 * j + c] : x[3 * i + c] - x[3 * j + c] - drr[c];
                dx[c] = dx[c] - s->el * fnint(dx[c] * s->eli);
            }
            double r = sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
            if (r < tiny) r = tiny;
            if (r < s->range) {
                double dr = s->scale * r;
                int index = (int)dr;
                if (index > ntab - 2) index = ntab - 2;
                if (index < 1) index = 1;
                dr = dr - index;
                double c1 = -dr * (dr - 1.0) * (dr - 2.0) / 6.0;
                double c2 = (dr + 1.0) * (dr - 1.0) * (dr - 2.0) / 2.0;
                double c3 = -(dr + 1.0) * dr * (dr - 2.0) / 2.0;
                double c4 = (dr + 1.0) * dr * (dr - 1.0) / 6.0;
                double uj = c1 * s->utab[it + 2 * (index - 1)] + c2 * s->utab[it + 2 * index]
                            + c3 * s->utab[it + 2 * (index + 1)] + c4 * s->utab[it + 2 * (index + 2)];
                u = pass == 0 ? u - uj : u + uj;
            }
        }
    }
    return exp(u);
}

/* bcsonebody, psislaterbcs.f90:378-395 */
static void bcsonebody(const orc_state* s, const double* x, double* g_, double* dg, double* d2g_, double* vext_)
{
    double vext = 0.0, g = 0.0, d2g = 0.0;
    double q2 = s->qex[0] * s->qex[0] + s->qex[1] * s->qex[1] + s->qex[2] * s->qex[2];
    for (int i = 0; i < s->npart; i++) {
        double arg = s->qex[0] * x[3 * i] + s->qex[1] * x[3 * i + 1] + s->qex[2] * x[3 * i + 2];
        double c = cos(arg), sn = sin(arg);
        vext = vext - s->v0ex * c;
        g = g - s->v0exjas * c;
        for (int k = 0; k < 3; k++) dg[3 * i + k] = s->v0exjas * s->qex[k] * sn;
        d2g = d2g + s->v0exjas * q2 * (s->v0exjas * sn * sn + c);
    }
    *g_ = g; *d2g_ = d2g; *vext_ = vext;
}

/* getjaslong, jastrowlongrange.f90:22-46 */
static void getjaslong(const orc_state* s, const double* x, double* u_, double* du, double* d2u_)
{
    double u = 0.0, d2u = 0.0;
    int npart = s->npart;
    for (int k = 0; k < 3 * npart; k++) du[k] = 0.0;
    for (int i = 0; i < npart - 1; i++)
        for (int j = i + 1; j < npart; j++) {
            double dx[3];
            for (int c = 0; c < 3; c++) dx[c] = x[3 * i + c] - x[3 * j + c];
            for (int iq = 1; iq < s->nkq; iq++) {
                const double* q = &s->akq[3 * iq];
                double qmod = sqrt(s->ak2q[iq]);
                double fact = s->jgamma * exp(-s->jbeta * qmod) / qmod;
                double arg = q[0] * dx[0] + q[1] * dx[1] + q[2] * dx[2];
                double c = 2.0 * cos(arg), sn = 2.0 * sin(arg);
                u = u + fact * c;
                for (int k = 0; k < 3; k++) {
                    du[3 * i + k] = du[3 * i + k] - fact * q[k] * sn;
                    du[3 * j + k] = du[3 * j + k] + fact * q[k] * sn;
                }
                d2u = d2u - 2.0 * fact * s->ak2q[iq] * c;
            }
        }
    double ss = 0.0;
    for (int k = 0; k < 3 * npart; k++) ss += du[k] * du[k];
    *u_ = u;
    *d2u_ = d2u + ss;
}

/* getjasder, jastrowlongrange.f90:63-78: d U / d beta by central
 * differences with dp = 1e-4 (beta moved up, down, then back), d U / d gamma
 * = U / gamma */
void orc_getjasder(orc_state* s, const double* x, double* dpsi)
{
    const double dp = 0.0001;
    double u, d2u, psi1, psi2;
    double* du = (double*)malloc(sizeof(double) * 3 * s->npart);
    dpsi[0] = dpsi[1] = 0.0;
    s->jbeta = s->jbeta + dp;
    getjaslong(s, x, &u, du, &d2u);
    psi1 = u;
    s->jbeta = s->jbeta - 2.0 * dp;
    getjaslong(s, x, &u, du, &d2u);
    psi2 = u;
    s->jbeta = s->jbeta + dp;
    getjaslong(s, x, &u, du, &d2u);
    dpsi[0] = (psi1 - psi2) / (2.0 * dp);
    dpsi[1] = u / s->jgamma;
    free(du);
}

/* ------------------------------------------------------------------------ */
/* dense inverse: rmatinv, matrixlapack.f90:13-41                           */
/* ------------------------------------------------------------------------ */

/* Restatement of LAPACK dgetrf: unblocked right-looking LU with partial
 * pivoting, the first maximum winning as in idamax (dgetf2).  Returns info
 * (0, or k>0 when U(k,k) is exactly zero). */
static int dgetrf(int n, double* a, int* ipiv)
{
#define A(i, j) a[(i) + (size_t)(j) * n]
    int info = 0;
    for (int j = 0; j < n; j++) {
        int jp = j;
        double amax = fabs(A(j, j));
        for (int i = j + 1; i < n; i++)
            if (fabs(A(i, j)) > amax) { amax = fabs(A(i, j)); jp = i; }
        ipiv[j] = jp;
        if (A(jp, j) != 0.0) {
            if (jp != j)
                for (int k = 0; k < n; k++) { double t = A(j, k); A(j, k) = A(jp, k); A(jp, k) = t; }
            double rp = 1.0 / A(j, j);
            for (int i = j + 1; i < n; i++) A(i, j) *= rp;
        } else if (info == 0) {
            info = j + 1;
        }
        for (int k = j + 1; k < n; k++) {
            double t = A(j, k);
            if (t != 0.0)
                for (int i = j + 1; i < n; i++) A(i, k) -= A(i, j) * t;
        }
    }
    return info;
#undef A
}

/* Restatement of LAPACK dgetri on the factors: inverse of U (dtrti2), then
 * solve inv(A)*L = inv(U), then undo the column interchanges. */
static void dgetri(int n, double* a, const int* ipiv, double* work)
{
#define A(i, j) a[(i) + (size_t)(j) * n]
    for (int j = 0; j < n; j++) {
        A(j, j) = 1.0 / A(j, j);
        double ajj = -A(j, j);
        /* x := U(0:j-1,0:j-1) * x with x = A(0:j-1,j)  (dtrmv upper, no-trans) */
        for (int jj = 0; jj < j; jj++) {
            double t = A(jj, j);
            if (t != 0.0) {
                for (int i = 0; i < jj; i++) A(i, j) += t * A(i, jj);
                A(jj, j) *= A(jj, jj);
            }
        }
        for (int i = 0; i < j; i++) A(i, j) *= ajj;
    }
    for (int j = n - 1; j >= 0; j--) {
        for (int i = j + 1; i < n; i++) { work[i] = A(i, j); A(i, j) = 0.0; }
        for (int jj = j + 1; jj < n; jj++) {
            double t = work[jj];
            if (t != 0.0)
                for (int i = 0; i < n; i++) A(i, j) -= A(i, jj) * t;
        }
    }
    for (int j = n - 2; j >= 0; j--) {
        int jp = ipiv[j];
        if (jp != j)
            for (int i = 0; i < n; i++) { double t = A(i, j); A(i, j) = A(i, jp); A(i, jp) = t; }
    }
#undef A
}

/* rmatinv, matrixlapack.f90:13-41: log|det| and sign from the LU diagonal
 * and pivots, then the inverse in place.  Returns the dgetrf info. */
int orc_matinv(int n, double* a, double* detl, int* is)
{
    int ipiv[2 * MAXP];
    double work[2 * MAXP];
    int info = dgetrf(n, a, ipiv);
    if (info != 0) {
        *detl = DMC_MINUSHUGE;
        return info;
    }
    int sgn = 1;
    double d = 0.0;
    for (int i = 0; i < n; i++) {
        d = d + log(fabs(a[i + (size_t)i * n]));
        sgn = sgn * (int)fsign(1.0, a[i + (size_t)i * n]);
        if (ipiv[i] != i) sgn = -sgn;
    }
    dgetri(n, a, ipiv, work);
    *detl = d;
    *is = sgn;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* BCS determinant: allpair + bcs, psislaterbcs.f90:155-294                 */
/* ------------------------------------------------------------------------ */

/* allpair, psislaterbcs.f90:227-294; smati, dph, d2ph are slices of the
 * caller's nd x nd arrays (leading dimension nd). */
static void allpair(const orc_state* s, const double* x, double* smati, double* dph, double* d2ph,
                    double* work)
{
    int nup = s->nup, ndn = s->ndn, nd = s->nd, K = 2 * s->nk - 1;
    double el = s->el;
    if (s->norb != 0) {
        double* up = work;                       /* uporbs(nup,K) */
        double* dn = up + (size_t)nup * K;       /* dnorbs(K,ndn) */
        double* dup = dn + (size_t)K * ndn;      /* duporbs(3,nup,K) */
        double* d2up = dup + (size_t)3 * nup * K;/* d2uporbs(nup,K) */
#define UP(i, k) up[(i) + (size_t)(k) * nup]
#define DN(k, j) dn[(k) + (size_t)(j) * K]
#define DUP(c, i, k) dup[(c) + 3 * ((i) + (size_t)(k) * nup)]
#define D2UP(i, k) d2up[(i) + (size_t)(k) * nup]
        for (int i = 0; i < nup; i++) {
            UP(i, 0) = s->vorb[0];
            for (int c = 0; c < 3; c++) DUP(c, i, 0) = 0.0;
            D2UP(i, 0) = 0.0;
        }
        for (int j = 0; j < ndn; j++) DN(0, j) = 1.0;
        int k = 0, kk = -1;
        for (int ksh = 2; ksh <= s->norb; ksh++) {
            for (int jj = 0; jj < s->numsh[ksh - 1]; jj++) {
                k++;
                kk += 2;
                double v = s->vorb[ksh - 1] * 2.0;
                const double* akk = &s->ak[3 * k];
                for (int i = 0; i < nup; i++) {
                    double arg = akk[0] * x[3 * i] + akk[1] * x[3 * i + 1] + akk[2] * x[3 * i + 2];
                    double c = cos(arg), sn = sin(arg);
                    UP(i, kk) = v * c;
                    for (int cc = 0; cc < 3; cc++) DUP(cc, i, kk) = -akk[cc] * v * sn;
                    D2UP(i, kk) = -s->ak2[k] * v * c;
                    UP(i, kk + 1) = v * sn;
                    for (int cc = 0; cc < 3; cc++) DUP(cc, i, kk + 1) = akk[cc] * v * c;
                    D2UP(i, kk + 1) = -s->ak2[k] * v * sn;
                }
                for (int i = 0; i < ndn; i++) {
                    const double* xd = &x[3 * (i + nup)];
                    double arg = akk[0] * xd[0] + akk[1] * xd[1] + akk[2] * xd[2];
                    DN(kk, i) = cos(arg);
                    DN(kk + 1, i) = sin(arg);
                }
            }
        }
        /* smati = matmul(uporbs,dnorbs); dph = duporbs*dnorbs; d2ph = d2uporbs*dnorbs */
        for (int j = 0; j < ndn; j++)
            for (int i = 0; i < nup; i++) {
                double a = 0.0, d2 = 0.0, g0 = 0.0, g1 = 0.0, g2 = 0.0;
                for (int q = 0; q < K; q++) {
                    double dq = DN(q, j);
                    a += UP(i, q) * dq;
                    g0 += DUP(0, i, q) * dq;
                    g1 += DUP(1, i, q) * dq;
                    g2 += DUP(2, i, q) * dq;
                    d2 += D2UP(i, q) * dq;
                }
                smati[i + (size_t)j * nd] = a;
                dph[0 + 3 * (i + (size_t)j * nd)] = g0;
                dph[1 + 3 * (i + (size_t)j * nd)] = g1;
                dph[2 + 3 * (i + (size_t)j * nd)] = g2;
                d2ph[i + (size_t)j * nd] = d2;
            }
#undef UP
#undef DN
#undef DUP
#undef D2UP
    }
    for (int i = 0; i < nup; i++)
        for (int j = 0; j < ndn; j++) {
            double dx[3];
            for (int c = 0; c < 3; c++) {
                dx[c] = x[3 * i + c] - x[3 * (j + nup) + c];
                dx[c] = dx[c] - el * fnint(dx[c] / el);
            }
            double r = sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
            double f, df, d2f;
            radialfun(s, r, &f, &df, &d2f);
            smati[i + (size_t)j * nd] += f;
            for (int c = 0; c < 3; c++) dph[c + 3 * (i + (size_t)j * nd)] += df * dx[c] / r;
            d2ph[i + (size_t)j * nd] += d2f;
        }
}

/* bcs, psislaterbcs.f90:155-225.  Returns smati (the inverse) in sinv when
 * non-NULL. */
void orc_bcs(const orc_state* s, const double* x, double* phil_, int* is_, double* dphi, double* d2phi_,
             double* sinv)
{
    int nd = s->nd, npair = s->npair, nexup = s->nexup, nexdn = s->nexdn, K = 2 * s->nk - 1;
    size_t nd2 = (size_t)nd * nd;
    double* smati = (double*)calloc(nd2 + 1, sizeof(double));
    double* d2ph = (double*)calloc(nd2 + 1, sizeof(double));
    double* dph = (double*)calloc(3 * nd2 + 1, sizeof(double));
    double* work = (double*)malloc(sizeof(double) * ((size_t)6 * (nd + 1) * K + 16));
    double phil = 0.0;
    int is = 1;
    allpair(s, x, smati, dph, d2ph, work);
    for (int i = 0; i < npair + nexup; i++)
        for (int j = 0; j < nexup; j++) {
            int jj = j + npair + nexdn;
            double arg = s->akup[j][0] * x[3 * i] + s->akup[j][1] * x[3 * i + 1] + s->akup[j][2] * x[3 * i + 2];
            double c = cos(arg), sn = sin(arg);
            size_t e = i + (size_t)jj * nd;
            if (s->sinup[j]) {
                smati[e] = sn;
                for (int q = 0; q < 3; q++) dph[q + 3 * e] = s->akup[j][q] * c;
                d2ph[e] = -s->ak2up[j] * sn;
            } else {
                smati[e] = c;
                for (int q = 0; q < 3; q++) dph[q + 3 * e] = -s->akup[j][q] * sn;
                d2ph[e] = -s->ak2up[j] * c;
            }
        }
    for (int i = 0; i < npair + nexdn; i++) {
        int ii = i + npair + nexup;
        for (int j = 0; j < nexdn; j++) {
            int jj = j + npair + nexup;
            const double* xd = &x[3 * ii];
            double arg = s->akdn[j][0] * xd[0] + s->akdn[j][1] * xd[1] + s->akdn[j][2] * xd[2];
            double c = cos(arg), sn = sin(arg);
            size_t e = jj + (size_t)i * nd;
            if (s->sindn[j]) {
                smati[e] = sn;
                for (int q = 0; q < 3; q++) dph[q + 3 * e] = -s->akdn[j][q] * c;
                d2ph[e] = -s->ak2dn[j] * sn;
            } else {
                smati[e] = c;
                for (int q = 0; q < 3; q++) dph[q + 3 * e] = s->akdn[j][q] * sn;
                d2ph[e] = -s->ak2dn[j] * c;
            }
        }
    }
    orc_matinv(nd, smati, &phil, &is);
    for (int k = 0; k < 3 * s->npart; k++) dphi[k] = 0.0;
    double d2phi = 0.0;
    if (!(phil < -1.e29)) {
        for (int i = 0; i < npair + nexup; i++) {
            for (int c = 0; c < 3; c++) {
                double sm = 0.0;
                for (int j = 0; j < nd; j++) sm += smati[j + (size_t)i * nd] * dph[c + 3 * (i + (size_t)j * nd)];
                dphi[3 * i + c] = sm / s->sqm[i];
            }
            double sm = 0.0;
            for (int j = 0; j < nd; j++) sm += smati[j + (size_t)i * nd] * d2ph[i + (size_t)j * nd];
            d2phi = d2phi + sm / s->pmass[i];
        }
        for (int i = 0; i < npair + nexdn; i++) {
            int j = npair + nexup + i;
            for (int c = 0; c < 3; c++) {
                double sm = 0.0;
                for (int q = 0; q < nd; q++) sm += smati[i + (size_t)q * nd] * dph[c + 3 * (q + (size_t)i * nd)];
                dphi[3 * j + c] = -sm / s->sqm[j];
            }
            double sm = 0.0;
            for (int q = 0; q < nd; q++) sm += smati[i + (size_t)q * nd] * d2ph[q + (size_t)i * nd];
            d2phi = d2phi + sm / s->pmass[j];
        }
        if (sinv) memcpy(sinv, smati, sizeof(double) * nd2);
    } else if (sinv) {
        memset(sinv, 0, sizeof(double) * nd2);
    }
    *phil_ = phil;
    *is_ = is;
    *d2phi_ = d2phi;
    free(smati); free(d2ph); free(dph); free(work);
}

/* bcsone, psislaterbcs.f90:296-376 (dr = xold - xnew, i 1-based, smatisave
 * passed in) */
double orc_bcsone(const orc_state* s, const double* x0, const double* dr, int i1, const double* smatisave)
{
    int npart = s->npart, nd = s->nd, npair = s->npair, nexup = s->nexup, nexdn = s->nexdn;
    double x[3 * MAXP];
    memcpy(x, x0, sizeof(double) * 3 * npart);
    int i = i1 - 1;
    double ph[2 * MAXP];
    for (int c = 0; c < 3; c++) x[3 * i + c] -= dr[c];
    int isup = (i1 <= s->nbin[0]);
    int nloop = isup ? npair + nexdn : npair + nexup;
    for (int j = 0; j < nloop; j++) {
        int jj = isup ? j + npair + nexup : j;
        double dx[3];
        for (int c = 0; c < 3; c++) {
            dx[c] = x[3 * i + c] - x[3 * jj + c];
            dx[c] = dx[c] - s->el * fnint(dx[c] / s->el);
        }
        ph[j] = s->vorb[0];
        int k = 0;
        for (int ish = 2; ish <= s->norb; ish++)
            for (int kk = 0; kk < s->numsh[ish - 1]; kk++) {
                k++;
                const double* a = &s->ak[3 * k];
                double arg = a[0] * dx[0] + a[1] * dx[1] + a[2] * dx[2];
                double c = cos(arg);
                double v = s->vorb[ish - 1] * 2.0;
                ph[j] = ph[j] + v * c;
            }
        double r = sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
        double f, d1, d2;
        radialfun(s, r, &f, &d1, &d2);
        ph[j] = ph[j] + f;
    }
    int jj = nloop;
    int nex = isup ? nexup : nexdn;
    for (int j = 0; j < nex; j++) {
        const double* a = isup ? s->akup[j] : s->akdn[j];
        int sn = isup ? s->sinup[j] : s->sindn[j];
        double arg = a[0] * x[3 * i] + a[1] * x[3 * i + 1] + a[2] * x[3 * i + 2];
        ph[jj] = sn ? sin(arg) : cos(arg);
        jj++;
    }
    double ratio = 0.0;
    if (isup) {
        for (int q = 0; q < nd; q++) ratio += smatisave[q + (size_t)i * nd] * ph[q];
    } else {
        int row = i - s->nbin[0];
        for (int q = 0; q < nd; q++) ratio += smatisave[row + (size_t)q * nd] * ph[q];
    }
    return ratio;
}

/* getderbcs, psislaterbcs.f90:449-524 (optsw=.true., optbeta=.false.) */
void orc_getderbcs(const orc_state* s, const double* x, double* dpsi)
{
    int nd = s->nd, npair = s->npair, nexup = s->nexup, nexdn = s->nexdn, npdet = s->norb;
    size_t nd2 = (size_t)nd * nd;
    double* smati = (double*)calloc(nd2 + 1, sizeof(double));
    double* d2ph = (double*)calloc(nd2 + 1, sizeof(double));
    double* dph = (double*)calloc(3 * nd2 + 1, sizeof(double));
    double* work = (double*)malloc(sizeof(double) * ((size_t)6 * (nd + 1) * (2 * s->nk - 1) + 16));
    double* dphi = (double*)calloc(nd2 * (npdet > 0 ? npdet : 1), sizeof(double));
    for (int p = 0; p < npdet; p++) dpsi[p] = 0.0;
    allpair(s, x, smati, dph, d2ph, work);
    for (int i = 0; i < npair + nexup; i++)
        for (int j = 0; j < nexup; j++) {
            int jj = j + npair + nexdn;
            double arg = s->akup[j][0] * x[3 * i] + s->akup[j][1] * x[3 * i + 1] + s->akup[j][2] * x[3 * i + 2];
            smati[i + (size_t)jj * nd] = s->sinup[j] ? sin(arg) : cos(arg);
        }
    for (int i = 0; i < npair + nexdn; i++) {
        int ii = i + npair + nexup;
        for (int j = 0; j < nexdn; j++) {
            int jj = j + npair + nexup;
            const double* xd = &x[3 * ii];
            double arg = s->akdn[j][0] * xd[0] + s->akdn[j][1] * xd[1] + s->akdn[j][2] * xd[2];
            smati[jj + (size_t)i * nd] = s->sindn[j] ? sin(arg) : cos(arg);
        }
    }
    double phil;
    int is = 1;
    orc_matinv(nd, smati, &phil, &is);
    for (int i = 0; i < npair + nexup; i++)
        for (int j = 0; j < npair + nexdn; j++) {
            int jj = j + npair + nexup;
            double dx[3];
            for (int c = 0; c < 3; c++) {
                dx[c] = x[3 * i + c] - x[3 * jj + c];
                dx[c] = dx[c] - s->el * fnint(dx[c] / s->el);
            }
            int np = 0;
            dphi[i + (size_t)j * nd + nd2 * np] = 1.0;
            np++;
            int k = 0;
            for (int ish = 2; ish <= s->norb; ish++) {
                for (int kk = 0; kk < s->numsh[ish - 1]; kk++) {
                    k++;
                    const double* a = &s->ak[3 * k];
                    double arg = a[0] * dx[0] + a[1] * dx[1] + a[2] * dx[2];
                    dphi[i + (size_t)j * nd + nd2 * np] += 2.0 * cos(arg);
                }
                np++;
            }
        }
    for (int p = 0; p < npdet; p++)
        for (int i = 0; i < nd; i++) {
            double sm = 0.0;
            for (int q = 0; q < nd; q++) sm += smati[q + (size_t)i * nd] * dphi[i + (size_t)q * nd + nd2 * p];
            dpsi[p] = dpsi[p] + sm;
        }
    free(smati); free(d2ph); free(dph); free(work); free(dphi);
}

/* ------------------------------------------------------------------------ */
/* hpsi, wavefunction.f90:161-201                                           */
/* ------------------------------------------------------------------------ */

typedef struct {
    double psil, d2psi, v, vext, psigl, d2psig;
    int is;
} hres;

static void hpsi(const orc_state* s, const double* x, hres* o, double* dpsi, double* dpsig)
{
    int n3 = 3 * s->npart;
    double du[3 * MAXP], du1[3 * MAXP], dulong[3 * MAXP], dphi[3 * MAXP];
    double u, d2u, v, u1, d2u1, v1, ulong, d2ulong, philog, d2phi;
    int isj, is;
    orc_getphi(s, x, &u, &isj, du, &d2u, &v);
    bcsonebody(s, x, &u1, du1, &d2u1, &v1);
    getjaslong(s, x, &ulong, dulong, &d2ulong);
    orc_bcs(s, x, &philog, &is, dphi, &d2phi, NULL);
    o->vext = v1;
    o->v = v + v1;
    o->is = isj * is;
    u = u + u1 + ulong;
    double d12 = 0.0, d13 = 0.0, d23 = 0.0;
    for (int k = 0; k < n3; k++) d12 += du[k] * du1[k];
    for (int k = 0; k < n3; k++) d13 += du[k] * dulong[k];
    for (int k = 0; k < n3; k++) d23 += du1[k] * dulong[k];
    d2u = d2u + d2u1 + d2ulong + 2.0 * (d12 + d13 + d23);
    for (int k = 0; k < n3; k++) du[k] = du[k] + du1[k] + dulong[k];
    o->psil = philog + u;
    for (int k = 0; k < n3; k++) dpsi[k] = dphi[k] + du[k];
    double dd = 0.0;
    for (int k = 0; k < n3; k++) dd += du[k] * dphi[k];
    o->d2psi = d2phi + d2u + 2.0 * dd;
    if (s->a2 == 0.0) {
        for (int k = 0; k < n3; k++) dpsig[k] = dpsi[k];
        o->d2psig = o->d2psi;
        o->psigl = o->psil;
    } else {
        double psi = exp(o->psil);
        double psig = sqrt(psi * psi + s->a2);
        double sdp = 0.0;
        for (int k = 0; k < n3; k++) dpsig[k] = psi * psi * dpsi[k] / (psig * psig);
        for (int k = 0; k < n3; k++) sdp += dpsi[k] * dpsi[k];
        o->d2psig = (sdp + o->d2psi) * psi * psi / (psig * psig) - psi * psi * psi * psi * sdp / (psig * psig * psig * psig);
        o->psigl = log(psig);
    }
}

/* Batched hpsi over nw walkers (OpenMP over walkers; each walker is the
 * sequential reference computation). */
void orc_hpsi_batch(orc_state* s, int nw, const double* x, double* psil, int* is, double* dpsi,
                    double* d2psi, double* v, double* vext, double* psigl, double* dpsig, double* d2psig)
{
    int n3 = 3 * s->npart;
#pragma omp parallel for schedule(dynamic, 1) num_threads(s->nthreads)
    for (int w = 0; w < nw; w++) {
        hres o;
        double dp[3 * MAXP], dg[3 * MAXP];
        hpsi(s, x + (size_t)w * n3, &o, dp, dg);
        if (psil) psil[w] = o.psil;
        if (is) is[w] = o.is;
        if (dpsi) memcpy(dpsi + (size_t)w * n3, dp, sizeof(double) * n3);
        if (d2psi) d2psi[w] = o.d2psi;
        if (v) v[w] = o.v;
        if (vext) vext[w] = o.vext;
        if (psigl) psigl[w] = o.psigl;
        if (dpsig) memcpy(dpsig + (size_t)w * n3, dg, sizeof(double) * n3);
        if (d2psig) d2psig[w] = o.d2psig;
    }
}

void orc_bcs_batch(orc_state* s, int nw, const double* x, double* phil, int* is, double* dphi, double* d2phi,
                   double* sinv)
{
    int n3 = 3 * s->npart;
    size_t nd2 = (size_t)s->nd * s->nd;
#pragma omp parallel for schedule(dynamic, 1) num_threads(s->nthreads)
    for (int w = 0; w < nw; w++)
        orc_bcs(s, x + (size_t)w * n3, &phil[w], &is[w], dphi + (size_t)w * n3, &d2phi[w],
                sinv ? sinv + nd2 * w : NULL);
}

/* ------------------------------------------------------------------------ */
/* walker stacks: stack.f90                                                 */
/* ------------------------------------------------------------------------ */

typedef struct {
    double x[3 * MAXP], dpsi[3 * MAXP], dpsig[3 * MAXP];
    double psil, d2psi, v, weight, psigl, d2psig, psil0, psigl0, vext;
    float wt0;
    int is;
    int64_t irn;
} walker;

static void wget(const orc_state* s, const wstack* st, int i, walker* w)
{
    int n3 = 3 * s->npart;
    memcpy(w->x, st->x + (size_t)i * n3, sizeof(double) * n3);
    memcpy(w->dpsi, st->dpsi + (size_t)i * n3, sizeof(double) * n3);
    memcpy(w->dpsig, st->dpsig + (size_t)i * n3, sizeof(double) * n3);
    w->psil = st->psil[i]; w->d2psi = st->d2psi[i]; w->v = st->v[i]; w->weight = st->weight[i];
    w->psigl = st->psigl[i]; w->d2psig = st->d2psig[i]; w->psil0 = st->psil0[i];
    w->psigl0 = st->psigl0[i]; w->vext = st->vext[i]; w->wt0 = st->wt0[i]; w->is = st->is[i];
    w->irn = st->irn[i];
}

static void wput(const orc_state* s, wstack* st, int i, const walker* w)
{
    int n3 = 3 * s->npart;
    memcpy(st->x + (size_t)i * n3, w->x, sizeof(double) * n3);
    memcpy(st->dpsi + (size_t)i * n3, w->dpsi, sizeof(double) * n3);
    memcpy(st->dpsig + (size_t)i * n3, w->dpsig, sizeof(double) * n3);
    st->psil[i] = w->psil; st->d2psi[i] = w->d2psi; st->v[i] = w->v; st->weight[i] = w->weight;
    st->psigl[i] = w->psigl; st->d2psig[i] = w->d2psig; st->psil0[i] = w->psil0;
    st->psigl0[i] = w->psigl0; st->vext[i] = w->vext; st->wt0[i] = w->wt0; st->is[i] = w->is;
    st->irn[i] = w->irn;
}

/* ------------------------------------------------------------------------ */
/* estimators: estimator.f90:72-113                                         */
/* ------------------------------------------------------------------------ */

typedef struct {
    double val[DMC_NEST_MAX], wt[DMC_NEST_MAX];
    unsigned char on[DMC_NEST_MAX];
} ecan;

static inline void addv(ecan* e, int i1, double val, double wt)
{
    e->val[i1 - 1] = val;
    e->wt[i1 - 1] = wt;
    e->on[i1 - 1] = 1;
}

static void flush_est(orc_state* s, const ecan* e)
{
    for (int i = 0; i < s->nest; i++)
        if (e->on[i]) {
            s->valblk[i] = s->valblk[i] + e->val[i] * e->wt[i];
            s->valblk2[i] = s->valblk2[i] + e->val[i] * e->val[i] * e->wt[i];
            s->wtblk[i] = s->wtblk[i] + e->wt[i];
        }
}

void orc_zero_estimators(orc_state* s)
{
    memset(s->valblk, 0, sizeof(s->valblk));
    memset(s->valblk2, 0, sizeof(s->valblk2));
    memset(s->wtblk, 0, sizeof(s->wtblk));
}

void orc_get_estimators(const orc_state* s, double* valblk, double* valblk2, double* wtblk)
{
    memcpy(valblk, s->valblk, sizeof(double) * s->nest);
    memcpy(valblk2, s->valblk2, sizeof(double) * s->nest);
    memcpy(wtblk, s->wtblk, sizeof(double) * s->nest);
}

/* update, estimator.f90:84-113 (one process) */
void orc_block_update(orc_state* s, double* valnow, double* errnow)
{
    for (int i = 0; i < s->nest; i++) {
        double vn = s->valblk[i] / s->wtblk[i];
        double v2 = s->valblk2[i] / s->wtblk[i];
        valnow[i] = vn;
        errnow[i] = sqrt(fabs(v2 - vn * vn) / s->wtblk[i]);
    }
    orc_zero_estimators(s);
}

/* ------------------------------------------------------------------------ */
/* step1, step.f90:43-285                                                   */
/* ------------------------------------------------------------------------ */

/* idmc = 10, step.f90:231-279: direct sampling of the Green's function with
 * importance sampling.  The two proposals x + sigma g and x - sigma g (no
 * drift, not wrapped), each weighted by exp(-v dt) Psi_G'/Psi_G; one more
 * uniform picks the first with its share of the summed weight, or always
 * when the second crossed a node; fixed node, weight 0.5 wt exp(etrial dt).
 * Estimator 6 is 0.5 (ego + egn) with ego, egn the old and the chosen
 * walker's guide local energies: the reference reads ego and egn there
 * without setting them on this path (step.f90:265). */
static const walker* step_gf(const orc_state* s, walker* w1, walker* w2, const double* g, int64_t* irn, int opcomp,
                             ecan* e)
{
    static __thread walker wb;   /* the second proposal */
    int npart = s->npart, n3 = 3 * npart;
    double hbar = s->hbar, nfac = s->nfac;
    double dx[3 * MAXP];
    for (int i = 0; i < npart; i++)
        for (int c = 0; c < 3; c++) dx[3 * i + c] = s->sigma[i] * g[3 * i + c];
    hres h;
    for (int k = 0; k < n3; k++) w2->x[k] = w1->x[k] + dx[k];
    hpsi(s, w2->x, &h, w2->dpsi, w2->dpsig);
    w2->psil = h.psil; w2->d2psi = h.d2psi; w2->v = h.v; w2->vext = h.vext;
    w2->psigl = h.psigl; w2->d2psig = h.d2psig; w2->is = h.is;
    double wt1 = exp(-w2->v * s->dt) * exp(w2->psigl - w1->psigl);
    for (int k = 0; k < n3; k++) wb.x[k] = w1->x[k] - dx[k];
    hpsi(s, wb.x, &h, wb.dpsi, wb.dpsig);
    wb.psil = h.psil; wb.d2psi = h.d2psi; wb.v = h.v; wb.vext = h.vext;
    wb.psigl = h.psigl; wb.d2psig = h.d2psig; wb.is = h.is;
    double wt2 = exp(-wb.v * s->dt) * exp(wb.psigl - w1->psigl);
    double wt = wt1 + wt2;
    wt1 = wt1 / wt;
    double rn = orc_ran1(irn);
    walker* w = (rn < wt1 || wb.is != w1->is) ? w2 : &wb;
    if (w->is != w1->is) {
        if (s->fn) wt = 0.0;
        addv(e, 5, 1.0, 1.0);
    } else {
        addv(e, 5, 0.0, 1.0);
    }
    wt = 0.5 * wt * exp(s->etrial * s->dt);
    w->weight = wt;
    double en = -hbar * w->d2psi + w->v;
    double wtg = wt * exp(w->psil - w->psigl) * w->is * (double)w1->wt0;
    double ego = -hbar * w1->d2psig + w1->v, egn = -hbar * w->d2psig + w->v;
    if (opcomp) {
        addv(e, 1, en * nfac, wtg);
        addv(e, 2, (en - w->v) * nfac, wtg);
        addv(e, 3, w->v * nfac, wtg);
        addv(e, 4, w->vext * nfac, wtg);
        addv(e, 6, 0.5 * (ego + egn) * nfac, 1.0);
    }
    addv(e, 7, exp(w->psil - w->psigl), 1.0);
    addv(e, 8, w->is * exp(w->psil), 1.0);
    addv(e, 9, exp(w->psigl), 1.0);
    addv(e, 10, 1.0 * w->is, 1.0);
    addv(e, 11, wt, 1.0);
    addv(e, 12, wtg, 1.0);
    addv(e, 13, fsign(1.0, wtg), 1.0);
    addv(e, 14, fsign(1.0, wtg), wtg);
    if (w == &wb) {
        /* the second proposal goes out through w2 */
        memcpy(w2->x, wb.x, sizeof(double) * n3);
        memcpy(w2->dpsi, wb.dpsi, sizeof(double) * n3);
        memcpy(w2->dpsig, wb.dpsig, sizeof(double) * n3);
        w2->psil = wb.psil; w2->d2psi = wb.d2psi; w2->v = wb.v; w2->vext = wb.vext;
        w2->psigl = wb.psigl; w2->d2psig = wb.d2psig; w2->is = wb.is; w2->weight = wb.weight;
    }
    w2->irn = *irn;
    w2->wt0 = w1->wt0;
    w2->psil0 = w1->psil0;
    w2->psigl0 = w1->psigl0;
    return w2;
}

/* One walker through step1's loop body.  w1 is the popped walker (modified
 * in place as the reference modifies it), w2 the proposal; returns the
 * walker that step1 pushes. */
static const walker* step_one(const orc_state* s, walker* w1, walker* w2, int opcomp, ecan* e)
{
    int npart = s->npart, n3 = 3 * npart;
    double el = s->el, hbar = s->hbar;
    double gauss[3 * MAXP], dx[3 * MAXP], drifto[3 * MAXP], driftn[3 * MAXP];
    double mass_i, sig, sq;
    int64_t irn;
    if (el != 0.0)
        for (int k = 0; k < n3; k++) w1->x[k] = w1->x[k] - el * fnint(w1->x[k] / el);
    irn = w1->irn & MASK48;                                      /* setrn */
    double eo = -hbar * w1->d2psi + w1->v;
    gaussian(&irn, n3, gauss);
    if (s->idmc == 10) return step_gf(s, w1, w2, gauss, &irn, opcomp, e);
    for (int i = 0; i < npart; i++) {
        mass_i = s->pmass[i];
        sig = s->sigma[i];
        sq = sqrt(mass_i);
        for (int c = 0; c < 3; c++) {
            gauss[3 * i + c] = sig * gauss[3 * i + c];
            double d = w1->dpsig[3 * i + c] * (sig * sig) * sq;
            if (s->cutdrift) d = fmin(s->dcut[i], fmax(-s->dcut[i], d));
            drifto[3 * i + c] = d;
        }
    }
    for (int k = 0; k < n3; k++) dx[k] = drifto[k] + gauss[k];
    for (int k = 0; k < n3; k++) w2->x[k] = w1->x[k] + dx[k];
    if (el != 0.0)
        for (int k = 0; k < n3; k++) w2->x[k] = w2->x[k] - el * fnint(w2->x[k] / el);
    hres h;
    hpsi(s, w2->x, &h, w2->dpsi, w2->dpsig);
    w2->psil = h.psil; w2->d2psi = h.d2psi; w2->v = h.v; w2->vext = h.vext;
    w2->psigl = h.psigl; w2->d2psig = h.d2psig; w2->is = h.is;
    w2->psil0 = w1->psil0; w2->psigl0 = w1->psigl0;
    double en = -hbar * w2->d2psi + w2->v;
    double nfac = s->nfac;
    switch (s->idmc) {
    case -1: case 0: {
        w2->weight = w1->weight;
        double prob = 2.0 * (w2->psil - w1->psil);
        for (int i = 0; i < npart; i++) {
            sig = s->sigma[i];
            sq = sqrt(s->pmass[i]);
            double dx1[3], dx2[3];
            for (int c = 0; c < 3; c++) {
                double d = w2->dpsig[3 * i + c] * (sig * sig) * sq;
                if (s->cutdrift) d = fmin(s->dcut[i], fmax(-s->dcut[i], d));
                driftn[3 * i + c] = d;
                dx1[c] = drifto[3 * i + c] + driftn[3 * i + c];
                dx2[c] = drifto[3 * i + c] - driftn[3 * i + c] - 2.0 * dx[3 * i + c];
            }
            prob = prob + (dx1[0] * dx2[0] + dx1[1] * dx2[1] + dx1[2] * dx2[2]) / (2.0 * (sig * sig));
        }
        prob = exp(fmin(0.0, prob));
        double rn = orc_ran1(&irn);
        if (rn < prob) {
            double dot = 0.0;
            for (int i = 0; i < npart; i++) {
                const double* d1 = &w2->dpsi[3 * i];
                dot = dot + (d1[0] * d1[0] + d1[1] * d1[1] + d1[2] * d1[2]) / s->pmass[i];
            }
            double ejf = -0.5 * hbar * (w2->d2psi - dot) + w2->v;
            addv(e, 1, en * nfac, w2->weight);
            addv(e, 2, (en - w2->v) * nfac, w2->weight);
            addv(e, 3, w2->v * nfac, w2->weight);
            addv(e, 4, w2->vext * nfac, w2->weight);
            addv(e, 5, ejf * nfac, w2->weight);
            addv(e, 6, 1.0, 1.0);
            w2->irn = irn;
            w2->wt0 = (float)w2->is;
            return w2;
        } else {
            double dot = 0.0;
            for (int i = 0; i < npart; i++) {
                const double* d1 = &w1->dpsi[3 * i];
                dot = dot + (d1[0] * d1[0] + d1[1] * d1[1] + d1[2] * d1[2]) / s->pmass[i];
            }
            double ejf = -0.5 * hbar * (w1->d2psi - dot) + w1->v;
            addv(e, 1, eo * nfac, w1->weight);
            addv(e, 2, (eo - w1->v) * nfac, w1->weight);
            addv(e, 3, w1->v * nfac, w1->weight);
            addv(e, 4, w1->vext * nfac, w1->weight);
            addv(e, 5, ejf * nfac, w1->weight);
            addv(e, 6, 0.0, 1.0);
            w1->irn = irn;
            return w1;
        }
    }
    case -2: case 1: {
        double ego = -hbar * w1->d2psig + w1->v;
        double egn = -hbar * w2->d2psig + w2->v;
        double wt = exp(-(0.5 * (ego + egn) - s->etrial) * s->dt);
        w2->weight = fmin(s->wtcut, wt);
        if (w2->is != w1->is) {
            if (s->fn) { w2->weight = 0.0; wt = 0.0; }
            addv(e, 5, 1.0, 1.0);
        } else {
            addv(e, 5, 0.0, 1.0);
        }
        double wtg = wt * exp(w2->psil - w2->psigl) * w2->is * (double)w1->wt0;
        if (opcomp) {
            addv(e, 1, en * nfac, wtg);
            addv(e, 2, (en - w2->v) * nfac, wtg);
            addv(e, 3, w2->v * nfac, wtg);
            addv(e, 4, w2->vext * nfac, wtg);
            addv(e, 6, 0.5 * (ego + egn) * nfac, 1.0);
            addv(e, 7, exp(w2->psil - w2->psigl), 1.0);
            addv(e, 8, w2->is * exp(w2->psil), 1.0);
            addv(e, 9, exp(w2->psigl), 1.0);
            addv(e, 10, 1.0 * w2->is, 1.0);
            addv(e, 11, wt, 1.0);
            addv(e, 12, wtg, 1.0);
            addv(e, 13, fsign(1.0, wtg), 1.0);
            addv(e, 14, fsign(1.0, wtg), wtg);
        }
        w2->irn = irn;
        w2->wt0 = w1->wt0;
        return w2;
    }
    case 2: {
        double prob = 2.0 * (w2->psigl - w1->psigl);
        for (int i = 0; i < npart; i++) {
            sig = s->sigma[i];
            sq = sqrt(s->pmass[i]);
            double dx1[3], dx2[3];
            for (int c = 0; c < 3; c++) {
                double d = w2->dpsig[3 * i + c] * (sig * sig) * sq;
                if (s->cutdrift) d = fmin(s->dcut[i], fmax(-s->dcut[i], d));
                driftn[3 * i + c] = d;
                dx1[c] = drifto[3 * i + c] + driftn[3 * i + c];
                dx2[c] = drifto[3 * i + c] - driftn[3 * i + c] - 2.0 * dx[3 * i + c];
            }
            prob = prob + (dx1[0] * dx2[0] + dx1[1] * dx2[1] + dx1[2] * dx2[2]) / (2.0 * (sig * sig));
        }
        prob = exp(fmin(0.0, prob));
        double rn = orc_ran1(&irn);
        if (rn < prob) {
            double wt = exp(-(0.5 * (eo + en) - s->etrial) * s->dt);
            w2->weight = fmin(s->wtcut, wt);
            if (w2->is != w1->is) {
                if (s->fn) { w2->weight = 0.0; wt = 0.0; }
                addv(e, 4, 1.0, 1.0);
            } else {
                addv(e, 4, 0.0, 1.0);
            }
            double wtg = wt * exp(w2->psil - w2->psigl) * w2->is * (double)w1->wt0;
            if (opcomp) {
                addv(e, 1, en * nfac, wtg);
                addv(e, 2, (en - w2->v) * nfac, wtg);
                addv(e, 3, w2->v * nfac, wtg);
                addv(e, 6, exp(w2->psil - w2->psigl), 1.0);
                addv(e, 7, w2->is * exp(w2->psil), 1.0);
                addv(e, 8, exp(w2->psigl), 1.0);
                addv(e, 9, 1.0 * w2->is, 1.0);
                addv(e, 10, wt, 1.0);
                addv(e, 11, wtg, 1.0);
                addv(e, 12, fsign(1.0, wtg), 1.0);
                addv(e, 13, fsign(1.0, wtg), wtg);
            }
            w2->irn = irn;
            w2->wt0 = w1->wt0;
            addv(e, 5, 1.0, 1.0);
            return w2;
        } else {
            double wt = exp(-(eo - s->etrial) * s->dt);
            double wtg = wt * exp(w1->psil - w1->psigl) * w1->is * (double)w1->wt0;
            w1->weight = fmin(s->wtcut, wt * w1->weight);
            if (opcomp) {
                addv(e, 1, eo * nfac, wtg);
                addv(e, 2, (eo - w1->v) * nfac, wtg);
                addv(e, 3, w1->v * nfac, wtg);
                addv(e, 6, exp(w1->psil - w1->psigl), 1.0);
                addv(e, 7, w1->is * exp(w1->psil), 1.0);
                addv(e, 8, exp(w1->psigl), 1.0);
                addv(e, 9, 1.0 * w1->is, 1.0);
                addv(e, 10, wt, 1.0);
                addv(e, 11, wtg, 1.0);
                addv(e, 12, fsign(1.0, wtg), 1.0);
                addv(e, 13, fsign(1.0, wtg), wtg);
            }
            w1->irn = irn;
            addv(e, 5, 0.0, 1.0);
            return w1;
        }
    }
    }
    return w1;
}

/* step1 over the whole input stack: pop order (top first) into the output
 * stack.  Walkers are independent, so they run in parallel; the estimator
 * contributions are added afterwards in the reference's pop order.
 * Returns 0, or -1 for idmc values not handled here. */
int orc_step(orc_state* s, int opcomp)
{
    if (s->idmc != -2 && s->idmc != -1 && s->idmc != 0 && s->idmc != 1 && s->idmc != 2 && s->idmc != 10) return -1;
    wstack* in = &s->st[s->istin];
    wstack* out = &s->st[1 - s->istin];
    int n = in->n;
    ecan* es = (ecan*)calloc((size_t)(n > 0 ? n : 1), sizeof(ecan));
#pragma omp parallel num_threads(s->nthreads)
    {
        walker* w1 = (walker*)malloc(sizeof(walker));
        walker* w2 = (walker*)malloc(sizeof(walker));
#pragma omp for schedule(dynamic, 1)
        for (int k = 0; k < n; k++) {
            int src = n - 1 - k;
            wget(s, in, src, w1);
            memset(w2, 0, sizeof(walker));
            const walker* r = step_one(s, w1, w2, opcomp, &es[k]);
            wput(s, out, k, r);
        }
        free(w1);
        free(w2);
    }
    for (int k = 0; k < n; k++) flush_est(s, &es[k]);
    free(es);
    out->n = n;
    in->n = 0;
    s->istin = 1 - s->istin;
    return 0;
}

/* branch, step.f90:287-315.  Returns 0 or DMC_ERR_OVERFLOW. */
int orc_branch(orc_state* s, double factor)
{
    wstack* in = &s->st[s->istin];
    wstack* out = &s->st[1 - s->istin];
    walker* w1 = (walker*)malloc(sizeof(walker));
    int no = 0, rc = 0;
    for (int k = in->n - 1; k >= 0; k--) {
        wget(s, in, k, w1);
        double wt = w1->weight * factor;
        w1->weight = fsign(1.0, w1->weight);
        double rn = orc_ran1(&w1->irn);
        int iwt = (int)(wt + rn);
        for (int i = 0; i < iwt; i++) {
            orc_ran2(&w1->irn);
            if (no >= s->cap) { rc = DMC_ERR_OVERFLOW; break; }
            wput(s, out, no++, w1);
        }
        if (iwt < DMC_WTISTO && iwt >= 0) s->wtisto[iwt]++;
        if (rc) break;
    }
    free(w1);
    out->n = no;
    in->n = 0;
    s->istin = 1 - s->istin;
    return rc;
}

/* One generation, dmcbcs.f90:436-448 (single process: checkpop moves
 * nothing). */
int orc_generation(orc_state* s, int opcomp, int* nt)
{
    int rc = orc_step(s, opcomp);
    if (rc) return rc;
    if (s->idmc > 0 || s->idmc == -2) {
        rc = orc_branch(s, 1.0);
        if (rc) return rc;
    }
    int n = s->st[s->istin].n;
    if (n > s->popup * s->nwalk || n < s->popdn * s->nwalk) {
        if (n == 0) return DMC_ERR_EMPTY;
        rc = orc_branch(s, 1.0 * s->nwalk / n);
        if (rc) return rc;
    }
    *nt = s->st[s->istin].n;
    return 0;
}

int orc_num_walkers(const orc_state* s) { return s->st[s->istin].n; }

/* Random initial walkers, dmcbcs.f90:238-300 (isite, first iteration,
 * single process). */
int orc_init_walkers(orc_state* s)
{
    int npart = s->npart, n3 = 3 * npart;
    int64_t irn = s->seed;
    int64_t gs = irn & MASK48;           /* setrn(irn) */
    walker* w1 = (walker*)calloc(1, sizeof(walker));
    double rn[3 * MAXP];
    randn(&gs, n3, rn);
    for (int k = 0; k < n3; k++) w1->x[k] = s->el * (rn[k] - 0.5);
    wstack* st = &s->st[s->istin];
    st->n = 0;
    if (s->nwalk > s->cap) { free(w1); return DMC_ERR_OVERFLOW; }
    for (int k = 0; k < s->nwalk; k++) {
        for (int i = 0; i < npart; i++) {
            double r1 = orc_ran1(&gs);
            int j = (int)(npart * r1 + 1) - 1;
            double t[3];
            memcpy(t, &w1->x[3 * i], sizeof t);
            memcpy(&w1->x[3 * i], &w1->x[3 * j], sizeof t);
            memcpy(&w1->x[3 * j], t, sizeof t);
        }
        w1->weight = 1.0;
        w1->irn = irn;
        orc_ran2(&w1->irn);
        irn = w1->irn;
        wput(s, st, st->n++, w1);
    }
    free(w1);
    return 0;
}

/* Walkers from the caller (fort.9 read, dmcbcs.f90:283-294). */
int orc_load_walkers(orc_state* s, int n, const double* x, const double* weight, const double* psil0,
                     const double* psigl0, const int64_t* irn)
{
    if (n > s->cap) return DMC_ERR_OVERFLOW;
    wstack* st = &s->st[s->istin];
    walker* w1 = (walker*)calloc(1, sizeof(walker));
    int n3 = 3 * s->npart;
    st->n = 0;
    for (int k = 0; k < n; k++) {
        memcpy(w1->x, x + (size_t)k * n3, sizeof(double) * n3);
        w1->weight = weight ? weight[k] : 1.0;
        w1->psil0 = psil0 ? psil0[k] : 0.0;
        w1->psigl0 = psigl0 ? psigl0[k] : 0.0;
        w1->irn = irn[k];
        wput(s, st, st->n++, w1);
    }
    free(w1);
    return 0;
}

/* Initial evaluation, dmcbcs.f90:314-395 for the first iteration (tau as
 * given; single process).  sums[9] = ene, ene2, psi, psi2, psig, psig2, sgn,
 * n, wtsum.  When tau==0 and DMC, the estimator-1 line and the operator pass
 * (one more pop/push) follow as in the reference; est[2] receives
 * valnow(1), errnow(1) of that line. */
int orc_initial_eval(orc_state* s, double tau, double* sums, double* est)
{
    wstack* in = &s->st[s->istin];
    wstack* out = &s->st[1 - s->istin];
    int n = in->n, n3 = 3 * s->npart;
    double hbar = s->hbar, eunit = s->eunit;
    int npart = s->npart;
    double* xs = (double*)malloc(sizeof(double) * (size_t)n * n3 + 8);
    hres* hr = (hres*)malloc(sizeof(hres) * (size_t)(n > 0 ? n : 1));
    double* dp = (double*)malloc(sizeof(double) * (size_t)n * n3 + 8);
    double* dg = (double*)malloc(sizeof(double) * (size_t)n * n3 + 8);
    for (int k = 0; k < n; k++) memcpy(xs + (size_t)k * n3, in->x + (size_t)(n - 1 - k) * n3, sizeof(double) * n3);
#pragma omp parallel for schedule(dynamic, 1) num_threads(s->nthreads)
    for (int k = 0; k < n; k++) hpsi(s, xs + (size_t)k * n3, &hr[k], dp + (size_t)k * n3, dg + (size_t)k * n3);
    double ene = 0, ene2 = 0, psi = 0, psi2 = 0, psig = 0, psig2 = 0, sgn = 0, wtsum = 0;
    int dmc = (tau == 0.0 && s->idmc != -1 && s->idmc != 0);
    orc_zero_estimators(s);
    walker* w1 = (walker*)malloc(sizeof(walker));
    for (int k = 0; k < n; k++) {
        wget(s, in, n - 1 - k, w1);
        memcpy(w1->dpsi, dp + (size_t)k * n3, sizeof(double) * n3);
        memcpy(w1->dpsig, dg + (size_t)k * n3, sizeof(double) * n3);
        w1->psil = hr[k].psil; w1->d2psi = hr[k].d2psi; w1->v = hr[k].v; w1->vext = hr[k].vext;
        w1->psigl = hr[k].psigl; w1->d2psig = hr[k].d2psig; w1->is = hr[k].is;
        double el = (-hbar * w1->d2psi + w1->v) / eunit / npart;
        ene = ene + el;
        ene2 = ene2 + el * el;
        psi = psi + exp(2.0 * w1->psil);
        psi2 = psi2 + exp(4.0 * w1->psil);
        psig = psig + exp(2.0 * w1->psigl);
        psig2 = psig2 + exp(4.0 * w1->psigl);
        sgn = sgn + 1.0 * w1->is;
        w1->wt0 = (float)w1->is;
        w1->weight = exp(w1->psigl - w1->psil0);
        w1->weight = 1.0;
        wtsum = wtsum + w1->weight;
        if (s->idmc == -1 || s->idmc == 0) w1->wt0 = (float)(1.0 * w1->is);
        if (dmc) {
            double wt = exp(-(-hbar * w1->d2psig + w1->v - s->etrial) * s->dt);
            ecan e;
            memset(&e, 0, sizeof e);
            addv(&e, 1, el, wt);
            flush_est(s, &e);
        }
        wput(s, out, k, w1);
    }
    out->n = n;
    in->n = 0;
    s->istin = 1 - s->istin;
    free(w1); free(xs); free(hr); free(dp); free(dg);
    sums[0] = ene; sums[1] = ene2; sums[2] = psi; sums[3] = psi2; sums[4] = psig; sums[5] = psig2;
    sums[6] = sgn; sums[7] = n; sums[8] = wtsum;
    if (dmc) {
        double vn[DMC_NEST_MAX], en[DMC_NEST_MAX];
        orc_block_update(s, vn, en);
        if (est) { est[0] = vn[0]; est[1] = en[0]; }
        /* operator pass: pop/push every walker once more (dmcbcs.f90:385-392) */
        wstack* a = &s->st[s->istin];
        wstack* b = &s->st[1 - s->istin];
        walker* w = (walker*)malloc(sizeof(walker));
        for (int k = 0; k < a->n; k++) { wget(s, a, a->n - 1 - k, w); wput(s, b, k, w); }
        free(w);
        b->n = a->n;
        a->n = 0;
        s->istin = 1 - s->istin;
    }
    orc_zero_estimators(s);
    return 0;
}

/* Copy the current stack out (index 0 = bottom). */
int orc_get_walkers(const orc_state* s, int cap, double* x, double* dpsi, double* dpsig, double* scal, int* is,
                    int64_t* irn, float* wt0)
{
    const wstack* st = &s->st[s->istin];
    int n = st->n, n3 = 3 * s->npart;
    if (n > cap) return -1;
    if (x) memcpy(x, st->x, sizeof(double) * (size_t)n * n3);
    if (dpsi) memcpy(dpsi, st->dpsi, sizeof(double) * (size_t)n * n3);
    if (dpsig) memcpy(dpsig, st->dpsig, sizeof(double) * (size_t)n * n3);
    if (scal)
        for (int k = 0; k < n; k++) {
            double* o = scal + (size_t)9 * k;
            o[0] = st->psil[k]; o[1] = st->psigl[k]; o[2] = st->d2psi[k]; o[3] = st->d2psig[k];
            o[4] = st->v[k]; o[5] = st->vext[k]; o[6] = st->weight[k]; o[7] = st->psil0[k]; o[8] = st->psigl0[k];
        }
    if (is) memcpy(is, st->is, sizeof(int) * n);
    if (irn) memcpy(irn, st->irn, sizeof(int64_t) * n);
    if (wt0) memcpy(wt0, st->wt0, sizeof(float) * n);
    return n;
}

void orc_get_wtisto(const orc_state* s, int64_t* h) { memcpy(h, s->wtisto, sizeof(s->wtisto)); }

/* updatepar, optimizer.f90:118-169 (one process): from the accumulated sums
 * ovec, ovecw, pmat (nparm^2, column-major), esum, esum2 over isteptot
 * samples, the parameter change newpars = delta0 * S^-1 f. */
int orc_sr_update(int nparm, const double* ovec_s, const double* ovecw_s, const double* pmat_s, double esum_s,
                  double esum2_s, int isteptot, double delta0, double eps, double* newpars, double* eave,
                  double* eerr)
{
    double* ovec = (double*)malloc(sizeof(double) * nparm);
    double* ovecw = (double*)malloc(sizeof(double) * nparm);
    double* pmat = (double*)malloc(sizeof(double) * (size_t)nparm * nparm);
    double* fvec = (double*)malloc(sizeof(double) * nparm);
    for (int i = 0; i < nparm; i++) { ovec[i] = ovec_s[i] / isteptot; ovecw[i] = ovecw_s[i] / isteptot; }
    for (int k = 0; k < nparm * nparm; k++) pmat[k] = pmat_s[k] / isteptot;
    double esum = esum_s / isteptot, esum2 = esum2_s / isteptot;
    *eerr = sqrt(fabs(esum * esum - esum2) / isteptot);
    for (int i = 0; i < nparm; i++) fvec[i] = -2.0 * ovecw[i] + 2.0 * ovec[i] * esum;
    for (int i = 0; i < nparm; i++) {
        for (int j = 0; j < nparm; j++) pmat[i + (size_t)j * nparm] = pmat[i + (size_t)j * nparm] - ovec[i] * ovec[j];
        pmat[i + (size_t)i * nparm] = pmat[i + (size_t)i * nparm] + eps;
    }
    double det;
    int is = 1;
    int rc = orc_matinv(nparm, pmat, &det, &is);
    for (int i = 0; i < nparm; i++) {
        double sm = 0.0;
        for (int j = 0; j < nparm; j++) sm += pmat[i + (size_t)j * nparm] * fvec[j];
        newpars[i] = delta0 * sm;
    }
    *eave = esum;
    free(ovec); free(ovecw); free(pmat); free(fvec);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* particle-by-particle sweeps (the library's own addition, restated in FP64) */
/* ------------------------------------------------------------------------ */

/* nsweep sweeps of every walker of the current stack, particles in order:
 * positions wrapped into the box first (as step.f90:59 wraps them), then per
 * move five ran1 draws of the walker's stream -- gaussian(3) from four
 * uniforms (ran.f90:74-104) and one acceptance uniform -- the proposal
 * x_i + sigma_i g wrapped into the box, and Metropolis acceptance with
 * exp(2 (log|Psi'| - log|Psi|)) from two full FP64 evaluations (hpsi): the
 * exact ratio the GPU's FP32 Sherman-Morrison path approximates.  The
 * walkers' stored values are then re-evaluated at the new positions.
 * Returns the accepted moves. */
int64_t orc_sm_sweeps(orc_state* s, int nsweep)
{
    wstack* st = &s->st[s->istin];
    int n = st->n, P = s->npart, n3 = 3 * P;
    int64_t total = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total) num_threads(s->nthreads)
    for (int w = 0; w < n; w++) {
        walker wk;
        wget(s, st, w, &wk);
        double x[3 * MAXP], xn[3 * MAXP], dp[3 * MAXP], dg[3 * MAXP];
        for (int e = 0; e < n3; e++) x[e] = wk.x[e] - s->el * fnint(wk.x[e] / s->el);
        hres h;
        hpsi(s, x, &h, dp, dg);
        double psil = h.psil;
        int64_t irn = wk.irn, acc = 0;
        for (int sw = 0; sw < nsweep; sw++) {
            for (int i = 0; i < P; i++) {
                double g[3];
                gaussian(&irn, 3, g);
                double rn = orc_ran1(&irn);
                double sig = s->sigma[i];
                memcpy(xn, x, sizeof(double) * n3);
                for (int c = 0; c < 3; c++) {
                    double v = x[3 * i + c] + sig * g[c];
                    xn[3 * i + c] = v - s->el * fnint(v / s->el);
                }
                hres hn;
                hpsi(s, xn, &hn, dp, dg);
                double prob = exp(2.0 * (hn.psil - psil));
                if (rn < prob) {
                    memcpy(x, xn, sizeof(double) * n3);
                    psil = hn.psil;
                    acc++;
                }
            }
        }
        memcpy(wk.x, x, sizeof(double) * n3);
        hpsi(s, x, &h, wk.dpsi, wk.dpsig);
        wk.psil = h.psil; wk.is = h.is; wk.d2psi = h.d2psi; wk.v = h.v; wk.vext = h.vext;
        wk.psigl = h.psigl; wk.d2psig = h.d2psig;
        wk.irn = irn;
        wput(s, st, w, &wk);
        total += acc;
    }
    return total;
}

/* ------------------------------------------------------------------------ */
/* operators: operators.f90:7-141 with gofr.f90 (g(r) and the density       */
/* profile), sofq.f90 (S(q)) and momentum3d.f90 (n(k))                      */
/* ------------------------------------------------------------------------ */

struct orc_ops {
    int ntabg, ntabq, ntabk, nsamp;
    /* gofr.f90:14-37: gnow(3,0:ntab), dnow(6,-ntab:ntab) */
    double drg, scaleg, wsg, totwg;
    double *gnow, *gerr, *g, *ge;       /* [itab][0..ntabg] */
    double *dnow, *derr, *d, *de;       /* [itab][-ntabg..ntabg] at i + ntabg */
    /* sofq.f90:17-33: snow(3,nqtot) */
    int nqtot, numshq[DMC_MAX_SHELLS];
    double *akq, *ak2q, wsq, totwq;
    double *snow, *serr, *sq, *se;      /* [itab][iq] */
    /* momentum3d.f90:14-71 */
    int nkv;
    int *ik, *indk, *nkk;               /* ik[3*nkv], indk/nkk[0..ntabk] */
    double dk, wsk, totwk;
    double *enknow, *enkerr, *enk, *enke;
};

static void free_ops(struct orc_ops* o)
{
    if (!o) return;
    free(o->gnow); free(o->gerr); free(o->g); free(o->ge);
    free(o->dnow); free(o->derr); free(o->d); free(o->de);
    free(o->akq); free(o->ak2q); free(o->snow); free(o->serr); free(o->sq); free(o->se);
    free(o->ik); free(o->indk); free(o->nkk);
    free(o->enknow); free(o->enkerr); free(o->enk); free(o->enke);
    free(o);
}

static double* zalloc(size_t n) { return (double*)calloc(n ? n : 1, sizeof(double)); }

/* zerooperators, operators.f90:75-88 */
void orc_zero_operators(orc_state* s)
{
    struct orc_ops* o = s->ops;
    if (!o) return;
    size_t ng = 3 * (size_t)(o->ntabg + 1), nd = 6 * (size_t)(2 * o->ntabg + 1), nq = 3 * (size_t)o->nqtot;
    size_t nk = (size_t)o->ntabk + 1;
    if (o->ntabg > 0) {
        memset(o->gnow, 0, ng * 8); memset(o->gerr, 0, ng * 8); memset(o->g, 0, ng * 8); memset(o->ge, 0, ng * 8);
        memset(o->dnow, 0, nd * 8); memset(o->derr, 0, nd * 8); memset(o->d, 0, nd * 8); memset(o->de, 0, nd * 8);
    }
    if (o->ntabq > 0) {
        memset(o->snow, 0, nq * 8); memset(o->serr, 0, nq * 8); memset(o->sq, 0, nq * 8); memset(o->se, 0, nq * 8);
    }
    if (o->nkv > 0) {
        memset(o->enknow, 0, nk * 8); memset(o->enkerr, 0, nk * 8); memset(o->enk, 0, nk * 8);
        memset(o->enke, 0, nk * 8);
    }
    o->wsg = o->wsq = o->wsk = 0.0;
}

/* setoperators for a periodic box (operators.f90:33-41,65-74): ntabg g(r)
 * bins (setupgofr, gofr.f90:14-37), ntabq S(q) shells (setupsofq,
 * sofq.f90:17-33), n(k) up to |ik|^2 <= ntabk (setupenk, momentum3d.f90:
 * 14-71).  Zero switches an operator off.  Returns the number of n(k)
 * shells + 1 (0 when off), or -1. */
int orc_set_operators(orc_state* s, int ntabg, int ntabq, int ntabk)
{
    free_ops(s->ops);
    struct orc_ops* o = (struct orc_ops*)calloc(1, sizeof(struct orc_ops));
    if (!o) return -1;
    s->ops = o;
    o->ntabg = ntabg > 0 ? ntabg : 0;
    o->ntabq = ntabq > 0 ? ntabq : 0;
    if (o->ntabg > 0) {
        size_t ng = 3 * (size_t)(o->ntabg + 1), nd = 6 * (size_t)(2 * o->ntabg + 1);
        o->gnow = zalloc(ng); o->gerr = zalloc(ng); o->g = zalloc(ng); o->ge = zalloc(ng);
        o->dnow = zalloc(nd); o->derr = zalloc(nd); o->d = zalloc(nd); o->de = zalloc(nd);
        o->drg = 0.5 * s->el / o->ntabg;
        o->scaleg = 1.0 / o->drg;
    }
    if (o->ntabq > 0) {
        int nq = 0;
        if (o->ntabq > DMC_MAX_SHELLS || kstates3d(s->el, o->ntabq, o->numshq, &o->akq, &o->ak2q, &nq) != 0) return -1;
        /* kstates3d lists k = 0 first (numsh(1) = 1); S(q) runs over all nqtot vectors */
        o->nqtot = 0;
        for (int i = 0; i < o->ntabq; i++) o->nqtot += o->numshq[i];
        if (o->nqtot > nq) return -1;
        size_t n3 = 3 * (size_t)o->nqtot;
        o->snow = zalloc(n3); o->serr = zalloc(n3); o->sq = zalloc(n3); o->se = zalloc(n3);
    }
    if (ntabk > 0) {
        o->nsamp = 10;
        o->dk = 2.0 * (4.0 * atan(1.0)) / s->el;   /* pi = 4 atan(1), momentum3d.f90:27-28 */
        int nnk = (int)(sqrt((double)ntabk) + 1.0);
        int ntot = 0;
        for (int ix = 0; ix <= nnk; ix++)
            for (int iy = 0; iy <= nnk; iy++)
                for (int iz = 0; iz <= nnk; iz++)
                    if (ix * ix + iy * iy + iz * iz <= ntabk) ntot++;
        o->nkv = ntot;
        o->ik = (int*)calloc(3 * (size_t)ntot, sizeof(int));
        int* ik2 = (int*)calloc(ntot, sizeof(int));
        ntot = 0;
        for (int ix = 0; ix <= nnk; ix++)
            for (int iy = 0; iy <= nnk; iy++)
                for (int iz = 0; iz <= nnk; iz++)
                    if (ix * ix + iy * iy + iz * iz <= ntabk) {
                        ik2[ntot] = ix * ix + iy * iy + iz * iz;
                        o->ik[3 * ntot] = ix; o->ik[3 * ntot + 1] = iy; o->ik[3 * ntot + 2] = iz;
                        ntot++;
                    }
        /* exchange sort of momentum3d.f90:46-57 */
        for (int i = 1; i < ntot; i++)
            for (int j = 0; j < i; j++)
                if (ik2[i] < ik2[j]) {
                    int t = ik2[i]; ik2[i] = ik2[j]; ik2[j] = t;
                    for (int c = 0; c < 3; c++) { t = o->ik[3 * i + c]; o->ik[3 * i + c] = o->ik[3 * j + c]; o->ik[3 * j + c] = t; }
                }
        o->indk = (int*)calloc((size_t)ntabk + 1, sizeof(int));
        o->nkk = (int*)calloc((size_t)ntabk + 1, sizeof(int));
        int itab = 0;
        o->indk[0] = 0;
        o->nkk[0] = 1;
        for (int i = 1; i < ntot; i++) {
            if (ik2[i] != ik2[i - 1]) {
                itab++;
                o->indk[itab] = i;
            }
            o->nkk[itab]++;
        }
        o->ntabk = itab;
        free(ik2);
        size_t nk = (size_t)o->ntabk + 1;
        o->enknow = zalloc(nk); o->enkerr = zalloc(nk); o->enk = zalloc(nk); o->enke = zalloc(nk);
    }
    orc_zero_operators(s);
    return o->nkv > 0 ? o->ntabk + 1 : 0;
}

/* addgofr, gofr.f90:53-92 */
static void addgofr(struct orc_ops* o, const orc_state* s, const double* x, double weight)
{
    int npart = s->npart, nup = s->nbin[0], ntab = o->ntabg;
    for (int i = 0; i < npart - 1; i++)
        for (int j = i + 1; j < npart; j++) {
            int itab = 0;
            if (i < nup && j < nup) itab = 1;
            if (i >= nup && j >= nup) itab = 2;
            double dx[3], r2 = 0.0;
            for (int c = 0; c < 3; c++) {
                dx[c] = x[3 * i + c] - x[3 * j + c];
                dx[c] = dx[c] - s->el * fnint(dx[c] / s->el);
                r2 += dx[c] * dx[c];
            }
            double r = sqrt(r2);
            int index = r < 0.5 * s->el ? (int)(o->scaleg * r) : ntab;
            o->gnow[itab * (ntab + 1) + index] += 2.0 * weight;
            o->gerr[itab * (ntab + 1) + index] += 4.0 * weight;
        }
    o->wsg += weight;
    for (int i = 0; i < npart; i++) {
        double dx[3];
        for (int c = 0; c < 3; c++) {
            dx[c] = x[3 * i + c];
            dx[c] = dx[c] - s->el * fnint(dx[c] / s->el);
        }
        for (int is = 0; is < 3; is++) {
            int itab = i < nup ? is : is + 3;
            int index = (int)(o->scaleg * dx[is]);
            size_t at = (size_t)itab * (2 * ntab + 1) + (index + ntab);
            if (index == 0) {
                o->dnow[at] += 0.5 * weight;
                o->derr[at] += 0.25 * weight;
            } else {
                o->dnow[at] += weight;
                o->derr[at] += weight;
            }
        }
    }
}

/* addsofq, sofq.f90:43-64 */
static void addsofq(struct orc_ops* o, const orc_state* s, const double* x, double weight)
{
    int nup = s->nbin[0], npart = s->npart, nq = o->nqtot;
    for (int iq = 0; iq < nq; iq++) {
        const double* a = &o->akq[3 * iq];   /* ak(:,1..nqtot): k = 0 first, as kstates3d lists it */
        double ur = 0, ui = 0, dr = 0, di = 0;
        for (int i = 0; i < nup; i++) {
            double arg = a[0] * x[3 * i] + a[1] * x[3 * i + 1] + a[2] * x[3 * i + 2];
            ur += cos(arg);
            ui -= sin(arg);
        }
        for (int i = nup; i < npart; i++) {
            double arg = a[0] * x[3 * i] + a[1] * x[3 * i + 1] + a[2] * x[3 * i + 2];
            dr += cos(arg);
            di -= sin(arg);
        }
        double uu = ur * ur + ui * ui, dd = dr * dr + di * di;
        double zr = ur * dr + ui * di, zi = ui * dr - ur * di;   /* rhokup * conjg(rhokdn) */
        o->snow[iq] += uu * weight;
        o->serr[iq] += uu * uu * weight;
        o->snow[nq + iq] += dd * weight;
        o->serr[nq + iq] += dd * dd * weight;
        o->snow[2 * nq + iq] += zr * weight;
        o->serr[2 * nq + iq] += (zr * zr - zi * zi) * weight;
    }
    o->wsq += weight;
}

/* addenk, momentum3d.f90:89-124: nsamp uniform displacements of every
 * particle from the walker's own random stream (not saved back), psi ratios
 * from move1 (getphione * bcsone with the walker's inverse), and the
 * symmetrised plane-wave products per |ik|^2 shell */
static void addenk(struct orc_ops* o, const orc_state* s, const walker* w, double wt)
{
    int npart = s->npart, nd = s->nd, ntab = o->ntabk;
    double* sinv = (double*)malloc(sizeof(double) * ((size_t)nd * nd + 1));
    double* dphi = (double*)malloc(sizeof(double) * 3 * npart);
    double* tmp = zalloc((size_t)ntab + 1);
    double phil, d2phi;
    int is;
    orc_bcs(s, w->x, &phil, &is, dphi, &d2phi, sinv);   /* hpsi(w) leaves the inverse in smatisave */
    int64_t irn = w->irn;                              /* setrn(w%irn) */
    for (int i = 0; i < npart; i++)
        for (int ii = 0; ii < o->nsamp; ii++) {
            double dx[3], drr[3];
            for (int c = 0; c < 3; c++) dx[c] = (orc_ran1(&irn) - 0.5) * s->el;
            for (int c = 0; c < 3; c++) drr[c] = -dx[c];   /* move1: drr = x - xnew */
            double rat1 = orc_getphione(s, w->x, drr, i + 1);
            double rat2 = orc_bcsone(s, w->x, drr, i + 1, sinv);
            double psirat = rat1 * rat2;
            for (int k = 0; k <= ntab; k++) {
                int in = o->indk[k];
                for (int j = 0; j < o->nkk[k]; j++) {
                    const int* v = &o->ik[3 * (in + j)];
                    tmp[k] += psirat * cos(o->dk * v[0] * dx[0]) * cos(o->dk * v[1] * dx[1]) * cos(o->dk * v[2] * dx[2]);
                }
            }
        }
    for (int k = 0; k <= ntab; k++) {
        double e = tmp[k] / o->nkk[k];
        o->enknow[k] += e * wt;
        o->enkerr[k] += e * e * wt;
    }
    o->wsk += wt * o->nsamp;
    free(sinv); free(dphi); free(tmp);
}

/* The operator pass of dmcbcs.f90:465-475 (addoperators, operators.f90:90-
 * 107): every walker popped, its estimators added with weight
 * w = weight exp(psil - psigl) is wt0, and pushed on the other stack. */
int orc_add_operators(orc_state* s)
{
    struct orc_ops* o = s->ops;
    if (!o) return -1;
    wstack* in = &s->st[s->istin];
    wstack* out = &s->st[1 - s->istin];
    walker w;
    out->n = 0;
    while (in->n > 0) {
        wget(s, in, in->n - 1, &w);
        in->n--;
        double wt = w.weight * exp(w.psil - w.psigl) * w.is * (double)w.wt0;
        if (o->ntabg > 0) addgofr(o, s, w.x, wt);
        if (o->ntabq > 0) addsofq(o, s, w.x, wt);
        if (o->nkv > 0) addenk(o, s, &w, wt);
        wput(s, out, out->n, &w);
        out->n++;
    }
    s->istin = 1 - s->istin;
    return 0;
}

static void block_norm(double* now, double* err, double* val, double* e, size_t n, double ws)
{
    double norm = 1.0 / ws;
    for (size_t k = 0; k < n; k++) {
        now[k] *= norm;
        val[k] = now[k];
        err[k] *= norm;
        e[k] = sqrt(fabs(err[k] - now[k] * now[k]) / ws);
        now[k] = 0.0;
        err[k] = 0.0;
    }
}

/* updateoperators (operators.f90:109-124): updategofr (gofr.f90:94-130),
 * updatesofq (sofq.f90:66-88), updateenk (momentum3d.f90:148-170) for one
 * process */
void orc_update_operators(orc_state* s)
{
    struct orc_ops* o = s->ops;
    if (!o) return;
    if (o->ntabg > 0 && o->wsg != 0.0) {
        block_norm(o->gnow, o->gerr, o->g, o->ge, 3 * (size_t)(o->ntabg + 1), o->wsg);
        block_norm(o->dnow, o->derr, o->d, o->de, 6 * (size_t)(2 * o->ntabg + 1), o->wsg);
        o->totwg = o->wsg;
        o->wsg = 0.0;
    }
    if (o->ntabq > 0 && o->wsq != 0.0) {
        block_norm(o->snow, o->serr, o->sq, o->se, 3 * (size_t)o->nqtot, o->wsq);
        o->totwq = o->wsq;
        o->wsq = 0.0;
    }
    if (o->nkv > 0 && o->wsk != 0.0) {
        block_norm(o->enknow, o->enkerr, o->enk, o->enke, (size_t)o->ntabk + 1, o->wsk);
        o->totwk = o->wsk;
        o->wsk = 0.0;
    }
}

/* Copy operator arrays: which 0 g(r) [3][ntabg+1] and its error, 1 the
 * density profile [6][2 ntabg+1] and error, 2 S(q) [3][nqtot] and error,
 * 3 n(k) [ntabk+1] and error; out gets values then errors; returns the
 * count of values (0 if off).  which +4: the running sums before the update
 * (now, err) instead. */
int orc_get_operators(const orc_state* s, int which, double* out, double* wsum)
{
    const struct orc_ops* o = s->ops;
    if (!o) return 0;
    int raw = which >= 4;
    which &= 3;
    size_t n = 0;
    const double *a = NULL, *b = NULL;
    double ws = 0.0;
    if (which == 0 && o->ntabg > 0) {
        n = 3 * (size_t)(o->ntabg + 1);
        a = raw ? o->gnow : o->g; b = raw ? o->gerr : o->ge; ws = raw ? o->wsg : o->totwg;
    } else if (which == 1 && o->ntabg > 0) {
        n = 6 * (size_t)(2 * o->ntabg + 1);
        a = raw ? o->dnow : o->d; b = raw ? o->derr : o->de; ws = raw ? o->wsg : o->totwg;
    } else if (which == 2 && o->ntabq > 0) {
        n = 3 * (size_t)o->nqtot;
        a = raw ? o->snow : o->sq; b = raw ? o->serr : o->se; ws = raw ? o->wsq : o->totwq;
    } else if (which == 3 && o->nkv > 0) {
        n = (size_t)o->ntabk + 1;
        a = raw ? o->enknow : o->enk; b = raw ? o->enkerr : o->enke; ws = raw ? o->wsk : o->totwk;
    }
    if (!n) return 0;
    if (out) {
        memcpy(out, a, n * 8);
        memcpy(out + n, b, n * 8);
    }
    if (wsum) *wsum = ws;
    return (int)n;
}
