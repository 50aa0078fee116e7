/*
 * dmcbcs_gpu.h -- C ABI of the GB300 (sm_103a) DMCBS walker hot path.
 *
 * The reference (CalebRHicks/DMCBS_Project, Fortran 90) has no plugin or FFI
 * layer: its hot path is a set of module procedures whose state is set once
 * by setup routines and then called once per walker.  Every entry point below
 * replaces one of those procedures (the replaced routine is cited file:line
 * beside it) and works on a whole batch of walkers at once.
 *
 * Conventions
 *  - Every function returns an int status (DMC_OK on success).  Nothing calls
 *    exit() or abort(); the message of the last failure on a context is
 *    returned by dmc_last_error().
 *  - Coordinates use the reference layout: one walker is x(3,npart) in
 *    Fortran column-major order, i.e. C double x[npart][3], up particles
 *    first (psislaterbcs.f90:44-45).  A batch is x[nw][npart][3].
 *  - Matrices returned to the caller (the BCS inverse) are column-major
 *    nd x nd like the Fortran array smati(nd,nd).
 *  - "_batch" functions take HOST pointers and are synchronous.
 *    "_device" variants take DEVICE pointers and a cudaStream_t (passed as
 *    void*), are stream-ordered and return once the work is enqueued.
 *  - One host thread per context.  Contexts are independent.
 *  - A singular BCS matrix is not an error: as in the reference
 *    (matrixlapack.f90:19-25, psislaterbcs.f90:210) log|det| is set to
 *    DMC_MINUSHUGE and the determinant drift and Laplacian are zero.
 */
#ifndef DMCBCS_GPU_H
#define DMCBCS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DMC_ABI_VERSION 1

#define DMC_MAX_SHELLS 32     /* s-wave pairing shells (norb) */
#define DMC_MAX_UNPAIRED 16   /* unpaired plane-wave states per spin */
#define DMC_MAX_PART 256      /* particles per system; above about N = 144 at seven shells
                                 the walker's orbitals live in global scratch, and
                                 dmc_create returns DMC_ERR_UNSUPPORTED only when the
                                 pair matrix and k records do not fit one CTA */
#define DMC_NEST_MAX 16       /* estimators (14 for DMC, 13 for idmc=2, 6 for VMC) */
#define DMC_WTISTO 500        /* multiplicity histogram bins (step.f90:9) */
#define DMC_MINUSHUGE (-1.0e30) /* log|det| of a singular matrix (matrixlapack.f90:19) */

/* status codes */
#define DMC_OK 0
#define DMC_ERR_INVALID 1      /* bad argument or deck value */
#define DMC_ERR_CUDA 2         /* a CUDA runtime call failed */
#define DMC_ERR_UNSUPPORTED 3  /* valid for the reference, not built here */
#define DMC_ERR_OVERFLOW 4     /* walker stack full (stack.f90:88-91) */
#define DMC_ERR_SETUP 5        /* table setup failed (rungekutta.f90:85-88, kshell.f90:137-140) */
#define DMC_ERR_EMPTY 6        /* population died out */
#define DMC_ERR_NOMEM 7        /* device or host allocation failed */
#define DMC_ERR_NOALLOC_LIMIT 8 /* size above the fixed scratch of dmc_branch_noalloc */

/* Failure flags (dmc_get_status, dmc_walker_status).  Neither is an error
 * of the call that met it: the reference carries on past a singular matrix
 * with its sentinel (matrixlapack.f90:19-25, psislaterbcs.f90:210) and
 * stops on a full stack (stack.f90:88-91), which here is the call's
 * DMC_ERR_OVERFLOW plus the flag. */
#define DMC_STATUS_SINGULAR 1   /* a pair matrix was singular: log|det| = DMC_MINUSHUGE, zero drift */
#define DMC_STATUS_NONFINITE 2  /* a walker's log|Psi|, Laplacian, potential or drift was NaN or infinite */
#define DMC_STATUS_OVERFLOW 4   /* branching made more copies than the stack holds; the excess was dropped */

/* Largest population dmc_branch_noalloc accepts (input walkers and output
 * capacity): its scratch is a fixed device array sized for this many. */
#define DMC_NOALLOC_MAX_WALKERS 65536

/*
 * System description: the deck values read by setpsi, setupbcs, setbeta and
 * setphi, as read (before the reference rescales any of them).
 */
typedef struct dmc_system_desc {
    /* main deck, dmcbcs.f90:61-66 */
    int ntab;             /* table points for Jastrow, potential and beta */
    double hbar;          /* hbar^2/2 without the mass */
    int ndim;             /* must be 3 */
    int nbin[2];          /* number of up and down particles */
    double mass[2];       /* mass of up and down particles */
    /* setpsi, wavefunction.f90:36-37 (node type must be 'bcs') */
    double a2;            /* constant in the importance function */
    /* setupbcs, psislaterbcs.f90:47-68 */
    double rho;           /* number density */
    int nexup;            /* unpaired up plane waves */
    int ikup[DMC_MAX_UNPAIRED][3];
    int nexdn;            /* unpaired down plane waves */
    int ikdn[DMC_MAX_UNPAIRED][3];
    int norb;             /* s-wave pairing shells */
    double vorb[DMC_MAX_SHELLS];
    int nqex[3];          /* q of the external cosine potential */
    double v0ex;          /* as read; the reference multiplies it by 1/2 */
    double v0exjas;       /* as read; the reference multiplies it by v0ex */
    int numq;             /* long-range Jastrow shells (0 = off) */
    double jbeta, jgamma; /* long-range Jastrow parameters */
    /* setbeta, betafun.f90:19-21 */
    double bbeta, dbeta;  /* b and d of the up-down beta function */
    double bfact;         /* beta strength; 0 = no beta (bfact<0 unsupported) */
    /* setphi, coshpot.f90:35-41 */
    double v0, amu;       /* cosh potential strength and width */
    double cjas[2];       /* opposite- and equal-spin Jastrow strength */
    double djas;          /* Jastrow healing distance */
    double v0op, v0eq;    /* effective strengths for the Jastrow (0 = v0) */
} dmc_system_desc;

/* Run parameters: dmcbcs.f90:44-60 plus the stack size factor (:224-230). */
typedef struct dmc_run_desc {
    int64_t seed;         /* random number seed for the initial walkers */
    int idmc;             /* -2,-1,0 (VMC), 1 (DMC local weight), 2 (DMC Metropolis),
                             10 (DMC without drift, two-point Green's function) */
    int isite;            /* 1 = random initial walkers, 0 = walkers loaded */
    int nwalk;            /* target population */
    int neq, nav, nstep;  /* equilibration blocks, averaging blocks, steps/block */
    double dt;            /* time step */
    double etrial;        /* trial energy per particle in energy units */
    int units;            /* 1 = energies in units of the free Fermi gas */
    double dcut;          /* drift cut off; <0 = no cut (step.f90:32-37) */
    int fn;               /* fixed node */
    double popup, popdn;  /* drastic population control factors */
    double dobal;         /* rebalance threshold (single process: unused) */
    double wtcut;         /* weight cut off */
    double stmax;         /* stack capacity factor: capacity = nwalk*stmax (10) */
} dmc_run_desc;

/* Derived sizes and units, filled by dmc_get_info. */
typedef struct dmc_info {
    int npart, nup, ndn, npair, nexup, nexdn, nd;
    int nk;               /* k vectors incl. k=0 (kshell.f90:136-143) */
    int ncol;             /* pair-orbital columns K = 2*nk-1 */
    int ntab;
    int capacity;         /* walker slots per stack */
    int nest;             /* estimators for this idmc */
    double el;            /* box side L */
    double eunit;         /* energy unit (dmcbcs.f90:146-159) */
    double nfac;          /* estimator normalisation (step.f90:24-25) */
    double etrial;        /* trial energy of the whole system */
    double sigma[2];      /* diffusion width per species (step.f90:29-30) */
    int64_t device_bytes; /* device memory held by the context */
} dmc_info;

typedef struct dmc_ctx dmc_ctx;

/* ---- lifecycle --------------------------------------------------------- */

/* Replaces setpsi (wavefunction.f90:13-96), setupbcs (psislaterbcs.f90:23-153),
 * setbeta/initbeta (betafun.f90:12-125), setphi (coshpot.f90:14-143),
 * setstep (step.f90:11-41) and create (stack.f90:51-80).  Builds the k
 * shells, the beta, Jastrow and potential tables on the host and uploads
 * them to the current CUDA device, and picks the walker layout (threads per
 * CTA, CTAs per SM, what stays in shared memory; dmc_tune_layout may change
 * it later).  DMC_ERR_INVALID for deck values out of range (checked on the
 * host first), DMC_ERR_UNSUPPORTED for ndim other than 3, a beta table read
 * from unit 80 (bfact < 0) or a system whose pair matrix and k records do
 * not fit one CTA's shared memory. */
int dmc_create(const dmc_system_desc* sys, const dmc_run_desc* run, dmc_ctx** out);
int dmc_destroy(dmc_ctx* ctx);
const char* dmc_last_error(const dmc_ctx* ctx);
const char* dmc_status_string(int status);
int dmc_abi_version(void);
int dmc_get_info(const dmc_ctx* ctx, dmc_info* out);

/* Copy a setup table to host memory.  which: 0 utab, 1 dutab, 2 d2utab,
 * 3 vtab (each 2*(ntab+1) values, layout [ic][0..ntab] i.e. Fortran
 * (2,0:ntab) transposed), 4 swbtab, 5 swdbtab, 6 swd2btab (ntab+1 each),
 * 7 ak (3*nk), 8 ak2 (nk), 9 numsh (norb, as doubles), 10 vorb (norb),
 * 11 (beta, gamma) of the long-range Jastrow, 12 (bfact, b, d) of the beta
 * function.  10 and 12 are the parameters getbcspar (psislaterbcs.f90:421-447,
 * through getdetparam, wavefunction.f90:260-287) returns. */
int dmc_get_table(const dmc_ctx* ctx, int which, double* out, int n);

/* Arithmetic of the walker kernel.  DMC_PREC_FP64 (the default) computes
 * everything in FP64.  DMC_PREC_MIXED computes the pair matrix, its inverse,
 * log-determinant and the drift/Laplacian contractions in double-float
 * arithmetic on the FP32 pipe (~48-bit significands) and the Jastrow and
 * potential in FP32, keeping the move, weights, branching and estimator
 * sums in FP64.  No counterpart in the reference (which is FP64 only). */
#define DMC_PREC_FP64 0
#define DMC_PREC_MIXED 1
int dmc_set_precision(dmc_ctx* ctx, int precision);
int dmc_get_precision(const dmc_ctx* ctx, int* precision);

/* Measured FMA throughput of the current device, TFLOP/s: kind 0 the FP64
 * pipe (DFMA), kind 1 the FP32 pipe (FFMA).  A measurement aid for roofline
 * fractions; no counterpart in the reference. */
int dmc_probe_peak(int kind, double* tflops);

/* The mixed path's double-float elementary functions evaluated on the device
 * for n host inputs (an accuracy check; no counterpart in the reference):
 * fn 0: in = double a[n], out[2i], out[2i+1] = sin(pi a), cos(pi a);
 * fn 1: in = uint64 m[n] (0 < m < 2^48), out = sin, cos of 2 pi m 2^-48, the
 *       Box-Muller angle of ran.f90:74-104;
 * fn 2: in = double x[n] > 0, out[i] = log x. */
int dmc_dfmath_eval(int fn, int n, const void* in, double* out);

/* Replaces setbcspar (psislaterbcs.f90:401-419, through setdetparam,
 * wavefunction.f90:231-258) with optbeta=.false.: new s-wave amplitudes
 * vorb(1:norb); dmc_set_beta covers its optbeta branch. */
int dmc_set_vorb(dmc_ctx* ctx, const double* vorb, int norb);

/* ---- wavefunction and local energy, batched ----------------------------- */

/* Replaces hpsi (wavefunction.f90:161-201): Jastrow+potential, one-body,
 * long-range Jastrow and BCS determinant for nw walkers.
 * x[nw][npart][3] -> psil[nw], is[nw], dpsi[nw][npart][3], d2psi[nw], v[nw],
 * vext[nw], psigl[nw], dpsig[nw][npart][3], d2psig[nw].  Any output pointer
 * may be NULL. */
int dmc_hpsi_batch(dmc_ctx* ctx, int nw, const double* x, double* psil, int* is,
                   double* dpsi, double* d2psi, double* v, double* vext,
                   double* psigl, double* dpsig, double* d2psig);
int dmc_hpsi_device(dmc_ctx* ctx, int nw, const double* x, double* psil, int* is,
                    double* dpsi, double* d2psi, double* v, double* vext,
                    double* psigl, double* dpsig, double* d2psig, void* stream);

/* Failure flags of the context (DMC_STATUS_* OR-ed over every walker of
 * every evaluation, step and generation since the last clear); clear != 0
 * resets them.  Reading them waits for the context's stream.  No
 * counterpart in the reference, which stops or carries a sentinel. */
int dmc_get_status(dmc_ctx* ctx, int* flags, int clear);

/* Per-walker DMC_STATUS_* flags of the last batched evaluation on this
 * context (dmc_hpsi_batch/_device, dmc_bcs_batch, dmc_getphi_batch) for its
 * first nw walkers (DMC_ERR_INVALID if nw exceeds that evaluation's batch).
 * No counterpart in the reference. */
int dmc_walker_status(dmc_ctx* ctx, int nw, int* status);

/* Replaces bcs (psislaterbcs.f90:155-225), which getpsi
 * (wavefunction.f90:98-131) calls for the BCS wavefunction: log|det|, sign,
 * drift dphi[nw][npart][3], Laplacian d2phi and (if smati != NULL) the
 * inverse smati[nw][nd*nd] column-major, which the reference keeps as
 * smatisave. */
int dmc_bcs_batch(dmc_ctx* ctx, int nw, const double* x, double* phil, int* is,
                  double* dphi, double* d2phi, double* smati);

/* Replaces getphi (coshpot.f90:154-205): Jastrow u, du[nw][npart][3], d2u and
 * the pair potential v. */
int dmc_getphi_batch(dmc_ctx* ctx, int nw, const double* x, double* u,
                     double* du, double* d2u, double* v);

/* Replaces rmatinv (matrixlapack.f90:13-41), i.e. MKL dgetrf+dgetri, on nb
 * column-major n x n matrices a[nb][n*n] in place: inverse, log|det| and
 * sign.  A singular matrix gives detl = DMC_MINUSHUGE and is left
 * unspecified, as the reference leaves it.  One matrix is held in one CTA's
 * shared memory: the blocked Gauss-Jordan form up to n of about 114, a
 * single-buffer form above it, DMC_ERR_UNSUPPORTED beyond about n = 160. */
int dmc_matinv_batch(dmc_ctx* ctx, int n, int nb, double* a, double* detl, int* is);

/* Replaces bcsone (psislaterbcs.f90:296-376): determinant ratio for moving
 * particle ipart[w] (1-based, as in the reference) of walker w by -dr[w][3]
 * (dr = xold - xnew), from that walker's inverse smati[w] (as returned by
 * dmc_bcs_batch). */
int dmc_bcsone_batch(dmc_ctx* ctx, int nw, const double* x, const double* smati,
                     const int* ipart, const double* dr, double* ratio);

/* Replaces getphione (coshpot.f90:207-264): Jastrow ratio exp(U'-U) for the
 * same single-particle moves (drr = xold - xnew). */
int dmc_getphione_batch(dmc_ctx* ctx, int nw, const double* x, const int* ipart,
                        const double* drr, double* ratio);

/* Replaces getderbcs (psislaterbcs.f90:449-524), which getderpsi
 * (wavefunction.f90:203-229) calls for the BCS wavefunction, with
 * optsw=.true., optbeta=.false.: d log|det| / d vorb(k), dpsi[nw][norb]. */
int dmc_getderbcs_batch(dmc_ctx* ctx, int nw, const double* x, double* dpsi);

/* Opt-in up-down Jastrow spline, no counterpart in the reference (whose
 * Jastrow is the zero-energy two-body solution, coshpot.f90:14-143): the
 * up-down pair Jastrow becomes the reference's plus
 *   u_s(r) = sum_{k=0}^{15} knots[k] phi_k(r),  h = L/34,
 *   phi_0(r) = B(r/h),  phi_k(r) = B(r/h - k) + B(r/h + k),
 * B the centred cubic B-spline on [-2, 2]: even in r and zero with its
 * first two derivatives at L/2.  nknots = DMC_JASTROW_KNOTS sets it,
 * nknots = 0 switches it off (the reference's wavefunction, the default).
 * The knots join the adjoint gradients' parameters. */
#define DMC_JASTROW_KNOTS 16
int dmc_set_jastrow_spline(dmc_ctx* ctx, const double* knots, int nknots);
int dmc_get_jastrow_spline(const dmc_ctx* ctx, double* knots, int cap, int* nknots);

/* No counterpart in the reference (its optimizer uses d log Psi only):
 * per-walker gradients with respect to theta = (vorb(1), ..., vorb(norb),
 * then bfact, b, d of the beta function when it is on (bfact != 0), then
 * the DMC_JASTROW_KNOTS knots when the Jastrow spline is on);
 * dmc_param_count gives their number np (7 + 3 + 16 = 26 at seven shells).
 * dlogpsi[nw][np] = d log|Psi| / d theta (the vorb part equals getderbcs,
 * psislaterbcs.f90:449-524) and deloc[nw][np] = d E_L / d theta with
 * E_L = -hbar d2psi + v in the units of v (step.f90:62,76), by the adjoint
 * of the determinant's kinetic terms: one extra pair of nd^3 products per
 * walker for all pair-function parameters.  The b and d derivatives are
 * those of the image-summed, shifted, bfact-scaled table that Psi uses
 * (betafun.f90:62-64,100-122), not of the single-image beta that the
 * reference's derbeta (betafun.f90:196-327) differentiates.  FP64 whatever
 * the context's precision. */
int dmc_param_count(const dmc_ctx* ctx, int* np);
/* New b, d and bfact of the up-down beta function (setbeta/initbeta,
 * betafun.f90:12-125): its tables are rebuilt.  The beta function must be
 * on (bfact != 0 at creation) and all three positive. */
int dmc_set_beta(dmc_ctx* ctx, double b, double d, double bfact);
int dmc_param_grad(dmc_ctx* ctx, int nw, const double* x, double* dlogpsi, double* deloc);

/* Replaces getjasder (jastrowlongrange.f90:63-78): dpsi[nw][2] = d U / d beta
 * (central differences with dp = 1e-4, as the reference takes them) and
 * d U / d gamma of the long-range Jastrow; DMC_ERR_INVALID when numq = 0. */
int dmc_getjasder_batch(dmc_ctx* ctx, int nw, const double* x, double* dpsi);

/* ---- stochastic reconfiguration (optimizer.f90:90-169) ----------------- */

/* Which parameters the SR step optimises, as iopt(1) and iopt(2) of the
 * optimizer input: the long-range Jastrow's (beta, gamma), then vorb(norb).
 * nparm = 2 opt_jastrow + norb opt_det; the default is (0, 1).  Clears the
 * sums. */
int dmc_sr_configure(dmc_ctx* ctx, int opt_jastrow, int opt_det);

/* No counterpart in the reference: the SR step over every parameter of
 * dmc_param_grad (vorb, then bfact, b, d, then the Jastrow knots when the
 * spline is on), with O_k = d log Psi / d theta_k from the adjoint kernel;
 * dmc_sr_update then moves all of them (dmc_set_vorb, dmc_set_beta,
 * dmc_set_jastrow_spline).  Set the spline first: nparm follows
 * dmc_param_count.  dmc_sr_configure switches back.  Clears the sums. */
int dmc_sr_configure_adjoint(dmc_ctx* ctx);

/* Replaces the calder loop of dmcbcs.f90:492-503 (optimizer.f90:90-116)
 * over the current population, in pop order: per walker the parameter
 * derivatives (getjasder, getderbcs) and ene = (-hbar*d2psi + v)/eunit/npart from its stored
 * evaluation are added to the context's sums ovec, ovecw, pmat, esum and
 * esum2; the walkers are left in reverse order, as that pop/push pass
 * leaves them.  *nsamples (may be NULL) receives the running count. */
int dmc_sr_accumulate(dmc_ctx* ctx, int64_t* nsamples);

/* The running sums: ovec[nparm], ovecw[nparm], pmat[nparm*nparm]
 * (column-major), e[2] = {esum, esum2} and the sample count; any pointer may
 * be NULL. */
int dmc_sr_get_sums(dmc_ctx* ctx, double* ovec, double* ovecw, double* pmat, double* e, int64_t* nsamples);

/* Clears the sums. */
int dmc_sr_zero(dmc_ctx* ctx);

/* Replaces updatepar (optimizer.f90:118-169) on one process: normalises the
 * sums by the sample count, f = -2 ovecw + 2 ovec esum,
 * P = pmat - ovec ovec^T + eps I, newpars = delta0 P^-1 f; adds newpars to
 * the parameters (setjasparam / setdetparam) and clears the sums.
 * newpars[nparm], eave and eerr may be NULL.  DMC_ERR_INVALID when no
 * sample was accumulated. */
int dmc_sr_update(dmc_ctx* ctx, double delta0, double eps, double* newpars, double* eave, double* eerr);

/* ---- walker population (device-resident stacks) ------------------------ */

/* Walker records as exchanged with the host; any array pointer may be NULL
 * on output.  Stack order: index 0 is the bottom of the reference's stack,
 * index n-1 its top (the next walker pop() returns). */
typedef struct dmc_walkers {
    int n;
    double* x;        /* [n][npart][3] */
    double* dpsi;     /* [n][npart][3] */
    double* dpsig;    /* [n][npart][3] */
    double* psil;     /* [n] */
    double* psigl;    /* [n] */
    double* d2psi;    /* [n] */
    double* d2psig;   /* [n] */
    double* v;        /* [n] */
    double* vext;     /* [n] */
    double* weight;   /* [n] */
    double* psil0;    /* [n] */
    double* psigl0;   /* [n] */
    double* wt0;      /* [n] (single precision in the reference, stack.f90:12) */
    int* is;          /* [n] */
    int64_t* irn;     /* [n] per-walker 48-bit random number state */
} dmc_walkers;

/* Replaces the random-configuration set-up of dmcbcs.f90:238-282 (isite):
 * nwalk walkers from the seed, pushed on the input stack. */
int dmc_init_walkers(dmc_ctx* ctx);

/* Replaces the walker read of dmcbcs.f90:254-258,283-294 (fort.9): push
 * w->n walkers with x, weight, psil0, psigl0 and irn (other fields ignored). */
int dmc_load_walkers(dmc_ctx* ctx, const dmc_walkers* w);

/* ---- operators (operators.f90, gofr.f90, sofq.f90, momentum3d.f90) ------ */

/* Replaces setoperators for a periodic box (operators.f90:7-74): ntabg g(r)
 * bins on [0, L/2] with the density profile (gofr.f90:14-37), ntabq S(q)
 * shells (sofq.f90:17-33), n(k) for |ik|^2 <= ntabk (momentum3d.f90:14-71;
 * at most 80 here); 0 switches one off.  Clears the sums. */
int dmc_set_operators(dmc_ctx* ctx, int ntabg, int ntabq, int ntabk);

/* zerooperators (operators.f90:75-88). */
int dmc_zero_operators(dmc_ctx* ctx);

/* The operator pass of dmcbcs.f90:465-473: every walker's addgofr, addsofq
 * and addenk with weight w exp(psil - psigl) is wt0 (operators.f90:90-107),
 * in pop order; the walkers are left in reverse order, as the pass leaves
 * them.  n(k) draws from each walker's stream without advancing it. */
int dmc_add_operators(dmc_ctx* ctx);

/* updateoperators (operators.f90:109-124): block averages and errors. */
int dmc_update_operators(dmc_ctx* ctx);

/* Results of the last update: which 0 g(r) [3][ntabg+1] (up-down, up-up,
 * down-down), 1 density profile [6][2 ntabg + 1] (x, y, z of up, then of
 * down; bin i at i + ntabg), 2 S(q) [3][nqtot] (up, down, up-down), 3 n(k)
 * [nshells]; which + 4: the running sums and their second-moment sums
 * instead.  *n gets the count (0 if off), *wsum the weight sum. */
int dmc_get_operators(dmc_ctx* ctx, int which, double* values, double* errors, int cap, int* n, double* wsum);

/* writeoperators (operators.f90:126-141): appends gofr.out, rho.out,
 * sofq.out and nofk.out in directory dir, in the reference's layouts. */
int dmc_write_operators(dmc_ctx* ctx, const char* dir, double tau);

/* ---- fort.9 walker files (dmcbcs.f90:254-294 read, :548-567 write) ----- */

/* Write n walkers in the reference's fort.9 layout: an (i10,f15.8) header
 * n, tau; per walker x (6e15.7, 3*npart values), weight, psil, psigl
 * (e15.7,2e25.15) and irn (i20).  Arrays are in file order (the reference
 * writes its stack top first).  No device or context is used. */
int dmc_fort9_write(const char* path, int npart, int n, const double* x, const double* weight, const double* psil,
                    const double* psigl, const int64_t* irn, double tau);

/* Read a fort.9 file (also the (i10)-header files of pairsconfig.f90):
 * *n walkers (DMC_ERR_OVERFLOW if more than cap; *n is still set), tau,
 * x[cap][3*npart], weight, psil0, psigl0 (may be NULL) and irn, in file
 * order.  Blank fields read as zero, as Fortran formatted input does. */
int dmc_fort9_read(const char* path, int npart, int cap, double* x, double* weight, double* psil0, double* psigl0,
                   int64_t* irn, int* n, double* tau);

/* Write the context's population to a fort.9 file, top of the stack first
 * (dmcbcs.f90:548-567). */
int dmc_save_walkers(dmc_ctx* ctx, const char* path, double tau);

/* Push the walkers of a fort.9 file in file order (dmcbcs.f90:283-294),
 * with x, weight, psil0, psigl0 and irn; *tau (may be NULL) gets the file's
 * tau.  Follow with dmc_initial_eval, as the reference does. */
int dmc_restore_walkers(dmc_ctx* ctx, const char* path, double* tau);

/* Copy the current walker stack to the host (fort.9 write,
 * dmcbcs.f90:548-567, and full walker state for checks).  w->n is the
 * capacity of the caller's arrays on entry and the count on return. */
int dmc_get_walkers(dmc_ctx* ctx, dmc_walkers* w);

/* Replaces the initial evaluation of dmcbcs.f90:314-395 for a run that
 * starts at tau = 0: hpsi on every walker, wt0=is, weight=1.  sums[11]:
 * ene, ene2, psi, psi2, psig, psig2, sgn, n, wtsum (the sums reduced to
 * rank 0 at dmcbcs.f90:354-362), then for DMC the block value and error of
 * estimator 1 printed at tau = 0 (dmcbcs.f90:337-340,379-384). */
int dmc_initial_eval(dmc_ctx* ctx, double* sums);

int dmc_num_walkers(dmc_ctx* ctx, int* n);

/* Replaces step1 (step.f90:43-285): one drift-diffusion move, Metropolis test
 * or DMC weight for every walker; opcomp selects the estimator step. */
int dmc_step(dmc_ctx* ctx, int opcomp);

/* Replaces branch (step.f90:287-315): stochastic-rounding copies with
 * weight*factor. */
int dmc_branch(dmc_ctx* ctx, double factor);

/* No counterpart in the reference: chooses the context's walker layout by
 * timing.  The candidates are the layout dmc_create picks (shared memory
 * for everything that fits, two CTAs per SM when they fit, else one CTA
 * with 16 warps for the mixed kernel), the same on chip with 256 threads
 * throughout, and the union region (orbitals, their powers, the second
 * inverse buffer, pair vectors) in an L2-resident global slice per CTA;
 * each is timed over `passes` wavefunction evaluations of the current
 * walkers (which do not change) and the fastest is kept.  kind_out: 0, 1 or
 * 2 in that order; ms_out: milliseconds per evaluation.  Captured
 * generations of the old layout are dropped (also those of a batch holding
 * the context, at its next call).  Results change only by the rounding of
 * the thread count's reduction order. */
int dmc_tune_layout(dmc_ctx* ctx, int passes, int* kind_out, double* ms_out);

/* Replaces one generation of dmcbcs.f90:436-448: step1, branch (DMC),
 * drastic population control; returns the population in *nt. */
int dmc_generation(dmc_ctx* ctx, int opcomp, int* nt);

/* Particle-by-particle VMC sweeps, no counterpart in the reference's walker
 * loop (its moves are all-particle, step.f90:43-285; it uses the
 * single-particle ratios of bcsone/getphione, psislaterbcs.f90:296-376 and
 * coshpot.f90:207-264, only for n(k)).  Every walker of the current stack
 * moves each particle in turn (nsweeps sweeps): proposal x_i + sigma_i g
 * (three deviates of gaussian, ran.f90:74-104, from the walker's stream,
 * then one uniform), Metropolis acceptance with |R|^2 exp(2 dU), R the
 * determinant ratio from the inverse pair matrix and the new row or column,
 * dU the Jastrow change.  Ratios, Jastrow and the Sherman-Morrison rank-one
 * updates of the inverse run in FP32; the inverse is recomputed from the
 * pair matrix in FP64 every recompute_every sweeps (0: only at the start of
 * the call).  Positions and random states are updated in place; the
 * walkers' stored wavefunction values are then re-evaluated at the new
 * positions in the context's precision.  accepted and moves (may be NULL)
 * receive the counts; nsweeps = 0 moves nothing and changes nothing.
 * DMC_ERR_UNSUPPORTED with the one-body or long-range Jastrow on or
 * a2 != 0. */
int dmc_sm_sweeps(dmc_ctx* ctx, int nsweeps, int recompute_every, int64_t* accepted, int64_t* moves);

/* The FP32 inverses the last dmc_sm_sweeps left, for the first nw walkers
 * of the stack: sinv[nw][nd*nd], column-major as smati.  No counterpart in
 * the reference. */
int dmc_sm_inverse(dmc_ctx* ctx, int nw, double* sinv);

/* Replaces zerest (estimator.f90:37-55). */
int dmc_zero_estimators(dmc_ctx* ctx);

/* Current block sums of the estimators (estimator.f90:72-82):
 * valblk, valblk2, wtblk, each [nest].  The library accumulates them across
 * a block's generations as compensated sums (Neumaier) and returns each
 * sum with its error term added. */
int dmc_get_estimators(dmc_ctx* ctx, double* valblk, double* valblk2, double* wtblk);

/* Replaces update (estimator.f90:84-113): block averages valnow[nest],
 * errors errnow[nest]; then zero the block sums. */
int dmc_block_update(dmc_ctx* ctx, double* valnow, double* errnow);

/* Walker multiplicity histogram (step.f90:310,317-334), hist[DMC_WTISTO]. */
int dmc_get_wtisto(dmc_ctx* ctx, int64_t* hist);

/* Device timing of the last dmc_step: milliseconds of the hpsi-dominated
 * step kernel, measured with CUDA events on the context's stream. */
int dmc_last_step_ms(dmc_ctx* ctx, double* ms);

/* Replaces the walker loop of dmcbcs.f90:435-449 for ngen generations (the
 * last one with opcomp): each generation is bracketed by CUDA events on the
 * context's stream and, when flush_l2 is set, preceded by a write of a
 * buffer twice the L2 size outside the timed interval.  Returns the summed
 * device milliseconds, the walker-steps (walkers entering step1, summed)
 * and the number of kernels launched inside the timed intervals. */
int dmc_timed_generations(dmc_ctx* ctx, int ngen, int opcomp_last, int flush_l2, int64_t* walker_steps,
                          double* device_ms, int64_t* launches);

/* One generation (dmcbcs.f90:436-448, as dmc_generation) for a host that
 * keeps its walker stacks in its own memory (stack.f90:82-110): the
 * population in->n walkers with every field set is read, the new population
 * is written to out (out->n: its capacity on entry, the new count on
 * return; out may be the same arrays as in).  With pinned (page-locked,
 * mapped) host arrays the walker kernel reads each walker's state directly
 * from them and one kernel writes the new population back, so the call
 * makes one round trip; other memory goes through dmc_put_walkers,
 * dmc_generation and dmc_get_walkers.  DMC_ERR_INVALID with out->n set to
 * the count needed when out is too small (the first out->n walkers are
 * written). */
int dmc_generation_host(dmc_ctx* ctx, const dmc_walkers* in, dmc_walkers* out, int opcomp);

/* Replace the current stack by w->n walkers with their full state (all
 * fields of dmc_walkers must be set): the inverse of dmc_get_walkers, for
 * hosts that keep the walker stacks in their own memory (stack.f90:82-110)
 * and hand them to the GPU for each generation. */
int dmc_put_walkers(dmc_ctx* ctx, const dmc_walkers* w);

/* A walker stack in device memory owned by the caller (all pointers are
 * device pointers; the layout is the library's own device layout). */
typedef struct dmc_dev_stack {
    double *x, *dpsi, *dpsig;   /* [cap][npart][3] */
    double *psil, *psigl, *d2psi, *d2psig, *v, *vext, *weight, *psil0, *psigl0;   /* [cap] */
    float* wt0;                 /* [cap] */
    int* is;                    /* [cap] */
    uint64_t* irn;              /* [cap] 48-bit random states */
} dmc_dev_stack;

/* No counterpart in the reference: this is the branching step of dmc_branch
 * for callers that may not allocate GPU memory.  Some hosts keep their walker
 * stacks in device memory that another allocator owns (a Fortran host with
 * its own device arrays, a memory pool) and must not call cudaMalloc or
 * cudaFree inside the walker loop, where an allocation would synchronise the
 * device and fragment the pool.  This call allocates nothing: the caller
 * passes the input stack `in` (n walkers, popped from the top as in
 * step.f90:287-315) and the output stack `out` (room for cap walkers), and the
 * copy counts, prefix offsets and advanced random states live in one
 * file-scope device array of about 1 MB that every GPU loading the library
 * keeps until the process exits.
 *  - n and cap must not exceed DMC_NOALLOC_MAX_WALKERS (else
 *    DMC_ERR_NOALLOC_LIMIT, nothing launched); more than cap copies gives
 *    DMC_ERR_OVERFLOW with *nout = cap.
 *  - wtisto: optional device array of DMC_WTISTO counters, incremented like
 *    the reference's multiplicity histogram; NULL to skip it.
 *  - The call waits on `stream` (a cudaStream_t, NULL for the default
 *    stream): it copies the new count to the host and synchronises the
 *    stream, so it must not be called while that stream, or any stream in a
 *    global-mode capture, is being captured.
 *  - The first call on a device looks up that device's scratch address and
 *    keeps it for the life of the process: cudaDeviceReset on that device
 *    (which unloads the library's device code) is not supported afterwards.
 *  - DMC_ERR_INVALID when a field of `in` overlaps a field of `out` (the
 *    scatter would read walkers it overwrites) or when factor is negative,
 *    above 1e6 or not finite.
 *  - All calls share the scratch and every value in it is written before it
 *    is read within a call, so nothing needs clearing; calls that overlap on
 *    the GPU (other streams, other host threads) race on it. */
int dmc_branch_noalloc(int n, int npart, int cap, double factor, const dmc_dev_stack* in,
                       const dmc_dev_stack* out, uint64_t* wtisto, int* nout, void* stream);

/* ---- Batches of systems of uneven size ----
 * No counterpart in the reference, where one MPI job runs one system: a
 * batch advances several contexts (one system each: its own N, polarisation,
 * wavefunction, walkers, trial energy and estimators) generation by
 * generation on one GPU.  Each batched generation is one CUDA graph: the
 * generation of every system (dmcbcs.f90:435-449 as in dmc_generation) on
 * its own stream, forked from and joined to the batch's stream, so that the
 * systems' walker kernels run concurrently.  grids[s] CTAs run system s's
 * walker kernel; the split and the launch order are what the batch tunes.  Each system's
 * walkers, random streams, estimators and populations come out exactly as
 * from dmc_generation on that context alone.  A context belongs to at most
 * one batch and must not be used on its own while a batched call runs. */
#define DMC_BATCH_MAX 16

typedef struct dmc_batch dmc_batch;

/* Group nsys contexts on the current device (DMC_ERR_INVALID if they are on
 * different devices, repeated or more than DMC_BATCH_MAX).  Initially every
 * system runs on its whole persistent grid: the CTA scheduler then starts a
 * system's CTAs as those of the systems launched before it retire.  Systems
 * are launched in decreasing order of cost per walker (algorithmic flops
 * until dmc_batch_tune measures them), so short walkers fill the tails. */
int dmc_batch_create(dmc_ctx* const* ctxs, int nsys, dmc_batch** out);
int dmc_batch_destroy(dmc_batch* b);
const char* dmc_batch_last_error(const dmc_batch* b);

/* The walker-kernel CTAs of each system in a batched generation:
 * 1 <= grids[s] <= the context's own persistent grid. */
int dmc_batch_set_grids(dmc_batch* b, const int* grids);
int dmc_batch_get_grids(const dmc_batch* b, int* grids);

/* Host-only planning step of the tuner (no GPU work): split the SMs over
 * nsys systems to minimise the predicted longest system.  System s has nw[s]
 * walkers, tau[s] seconds per walker on one of its CTAs, per_sm[s] of its
 * CTAs fit on one SM (1 or 2) and at most maxgrid[s] CTAs; a CTA takes
 * 2 / per_sm[s] of the 2 * nsm half-SM slots.  Predicted time of s:
 * ceil(nw[s] / grids[s]) * tau[s].  Starting from one CTA per system, one
 * CTA at a time goes to the system with the longest predicted time among
 * those that can still take one.  DMC_ERR_INVALID if the systems do not get
 * one CTA each. */
int dmc_batch_plan(int nsys, const double* tau, const int* nw, const int* per_sm, const int* maxgrid, int nsm,
                   int* grids);

/* Autotuner: time each system's walker kernel alone on its current walkers
 * (a wavefunction evaluation, which leaves every walker as it was) and order
 * the launches by the measured time per walker.  Then time concurrent
 * passes of all systems with the split in use, with every system on its
 * whole grid, and with `rounds` + 1 partitions from dmc_batch_plan (each
 * re-planned from the per-system times of the pass before); keep the split
 * with the shortest measured pass.  grids (optional, [nsys]) receives it,
 * ms (optional) its pass time in milliseconds. */
int dmc_batch_tune(dmc_batch* b, int rounds, int* grids, double* ms);

/* ngen batched generations, the last one with opcomp (estimators) when
 * opcomp_last is set; each generation is bracketed by CUDA events on the
 * batch's stream and, with flush_l2, preceded by an untimed write of a
 * buffer twice the L2 size.  Returns the summed device milliseconds, the
 * walker-steps of all systems and the kernels launched in the timed
 * intervals (each optional). */
int dmc_batch_generations(dmc_batch* b, int ngen, int opcomp_last, int flush_l2, int64_t* walker_steps,
                          double* device_ms, int64_t* launches);

#ifdef __cplusplus
}
#endif

#endif /* DMCBCS_GPU_H */
