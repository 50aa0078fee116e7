"""The optional terms of hpsi (wavefunction.f90:161-201) that the benchmark
workloads leave off: the one-body external potential and its Jastrow
factor (v0ex, v0exjas, nqex: vext and the one-body cross terms of the
Laplacian), the guiding function psi_G = sqrt(psi^2 + a2) (psigl, dpsig,
d2psig, wavefunction.f90:525-535), alone and together, and the same-spin
pair Jastrow (cjas(2) != 0) with its own effective interaction, at N = 14,
66 and 132 (the last on the mixed path's 16-warp CTA).  Every hpsi output
against the oracle (FP64 to 1e-10 relative, the mixed path to the
benchmark's 1e-6, as in the other parity tests), and generations
with exact populations and random streams (idmc = 1 uses the guide's
Laplacian in the weights, idmc = 2 its ratio in the Metropolis test,
idmc = 10 its ratio in the two proposals' weights)."""
import numpy as np
import pytest

import oracle
from dmcbcs_project_gb300 import capi, configs
from dmcbcs_project_gb300.abi import make_run, make_system

pytestmark = pytest.mark.gpu

TERMS = {
    "onebody": dict(v0ex=0.5, v0exjas=0.3, nqex=[1, 0, 0]),
    "guide": dict(a2=0.05),
    "both": dict(a2=0.05, v0ex=0.5, v0exjas=0.3, nqex=[0, 1, 1]),
    # a same-spin Jastrow from a repulsive effective interaction next to a
    # weaker up-down one (coshpot.f90:40-43,90-133: v0op, v0eq = 0 would
    # mean v0; the workloads switch the same-spin factor off, cjas(2) = 0)
    "jastrow": dict(v0op=0.5, v0eq=-0.5, cjas=[1.0, 1.0]),
}


def system(term, nup=7, nwalk=16, idmc=1):
    sp = configs.system_params(nup, nup, 5 if nup < 20 else 7)
    sp.update(TERMS[term])
    return make_system(sp), make_run(configs.run_params(nwalk, 0.002, idmc=idmc))


def rel_each(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)))


@pytest.mark.parametrize("term", list(TERMS))
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-6)])
@pytest.mark.parametrize("nup", [7, 33, 66])
def test_hpsi_terms(term, precision, tol, nup):
    sysd, rund = system(term, nup=nup)
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    # the configurations of the other parity tests: permuted initial walkers
    # spread by a seeded displacement
    x = orc.walkers()["x"] + np.random.default_rng(1234).normal(scale=0.3, size=(16, orc.npart, 3))
    ho = orc.hpsi(x)
    with capi.Context(sysd, rund, precision=precision) as ctx:
        hg = ctx.hpsi(x)
    assert np.array_equal(hg["is_"], ho["is_"])
    for k in ("psil", "psigl", "d2psi", "d2psig", "v", "vext"):
        assert rel_each(hg[k], ho[k]) < tol, k
    for k in ("dpsi", "dpsig"):
        scale = max(float(np.max(np.abs(ho[k]))), 1.0)
        assert float(np.max(np.abs(hg[k] - ho[k]))) / scale < tol, k


@pytest.mark.parametrize("term,idmc", [("onebody", 1), ("guide", 1), ("guide", 2), ("both", 2), ("both", 10),
                                       ("jastrow", 1)])
def test_generations_with_terms(term, idmc):
    sysd, rund = system(term, nwalk=24, idmc=idmc)
    orc = oracle.Oracle(sysd, rund)
    with capi.Context(sysd, rund) as ctx:
        ctx.init_walkers()
        orc.init_walkers()
        ctx.initial_eval()
        orc.initial_eval()
        for g in range(4):
            assert ctx.generation(g == 3) == orc.generation(g == 3)
        wg, wo = ctx.walkers(), orc.walkers()
        eg, _, wbg = ctx.estimators()
        eo, _, wbo = orc.estimators()
    assert np.array_equal(wg["irn"], wo["irn"])
    assert np.array_equal(wg["is_"], wo["is_"])
    assert float(np.max(np.abs(wg["x"] - wo["x"]))) < 1e-9
    for k in ("psil", "psigl", "d2psig", "v", "vext", "weight"):
        assert rel_each(wg[k], wo[k]) < 1e-10, k
    assert rel_each(eg, eo) < 1e-9 and rel_each(wbg, wbo) < 1e-9
