"""Synthetic workloads of the unitary Fermi gas benchmark family.

There is no public dataset behind these runs: every workload is a seeded
synthetic system with the sizes and parameter ranges of the benchmark
configurations.  Common physical parameters (k_F = 1, hbar^2/2 = 0.5, m = 1,
cosh potential v0 = 1, mu = 24 k_F, opposite-spin Jastrow only, healing
distance 1.15, 10000-point tables, beta d = 5, bfact = 1) follow the
reference's production deck for N = 66; the s-wave amplitudes are drawn
from U(0.2, 1) * 0.5**shell and the beta parameter b from U(0.5, 1.5) with
a fixed seed per workload.
"""
import numpy as np

from .abi import make_run, make_system

RHO_KF1 = 0.0337737278          # k_F^3 / (3 pi^2) for k_F = 1
E_FG = 0.3                      # free-gas energy per particle, (3/5) E_F

# unpaired plane waves used for polarised systems (lowest shells first);
# the reference picks sin when the last non-zero component is negative
_UNPAIRED = [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0),
             (0, 0, 1), (0, 0, -1), (1, 1, 0)]


def system_params(nup, ndn, norb, seed=1234, ntab=10000, longrange=None):
    """Deck values of one synthetic system with nup >= ndn; longrange =
    (numq, beta, gamma) switches the long-range Jastrow on."""
    if ndn > nup:
        raise ValueError("put the larger spin species first")
    rng = np.random.default_rng(seed)
    vorb = (rng.uniform(0.2, 1.0, size=norb) * 0.5 ** np.arange(norb)).tolist()
    b = float(rng.uniform(0.5, 1.5))
    nexup = nup - ndn
    numq, jbeta, jgamma = longrange if longrange else (0, 0.0, 0.0)
    return dict(
        ntab=ntab, hbar=0.5, ndim=3, nbin=[nup, ndn], mass=[1.0, 1.0], a2=0.0,
        rho=RHO_KF1, nexup=nexup, ikup=[list(k) for k in _UNPAIRED[:nexup]],
        nexdn=0, ikdn=[], norb=norb, vorb=vorb, nqex=[0, 0, 0], v0ex=0.0, v0exjas=0.0,
        numq=numq, jbeta=jbeta, jgamma=jgamma, bbeta=b, dbeta=5.0, bfact=1.0,
        v0=1.0, amu=24.0, cjas=[1.0, 0.0], djas=1.15, v0op=0.0, v0eq=-10.0,
    )


def run_params(nwalk, dt_efg, idmc=1, nstep=1, seed=17, etrial=0.4):
    """Run values; dt is given in units of 1/E_FG as in the benchmark."""
    return dict(seed=seed, idmc=idmc, isite=1, nwalk=nwalk, neq=0, nav=1, nstep=nstep,
                dt=dt_efg / E_FG, etrial=etrial, units=1, dcut=-1.0, fn=1,
                popup=1.1, popdn=0.9, dobal=0.5, wtcut=10.0, stmax=10.0)


# name -> (nup, ndn, norb, walkers, dt [1/E_FG], steps)
WORKLOADS = {
    # plain FP64 VMC then DMC, 7 up / 7 down, shells 0..4, 200 walkers, 200 steps
    "n14": (7, 7, 5, 200, 0.002, 200),
    # plain FP64 DMC at 33 up / 33 down, shells 0..6, 4096 walkers, 2000 steps
    "n66": (33, 33, 7, 4096, 0.001, 2000),
    # 66 up / 66 down, shells 0..6
    "n132": (66, 66, 7, 8192, 0.001, 200),
    # polarised members of the uneven batch
    "p33_30": (33, 30, 7, 1024, 0.001, 200),
    "p38_33": (38, 33, 7, 1024, 0.001, 200),
    "n38": (19, 19, 7, 1024, 0.001, 200),
}


def workload(name, nwalk=None, idmc=1, seed=1234, ntab=10000, longrange=None):
    """Return ``(SystemDesc, RunDesc, meta)`` for a named workload."""
    nup, ndn, norb, nw, dt, steps = WORKLOADS[name]
    if nwalk is not None:
        nw = nwalk
    sp = system_params(nup, ndn, norb, seed=seed, ntab=ntab, longrange=longrange)
    rp = run_params(nw, dt, idmc=idmc)
    meta = dict(name=name, nup=nup, ndn=ndn, norb=norb, nwalk=nw, dt_efg=dt, steps=steps)
    return make_system(sp), make_run(rp), meta
