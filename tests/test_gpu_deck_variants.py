"""Deck values the benchmark decks leave at one setting, against the oracle:
unequal masses of the two species (setstep's sigma_i = sqrt(2 hbar dt /
m_i), the drift's sqrt(m_i), the reduced mass of the up-down Jastrow and
beta Laplacians, step.f90:26-29,66-70, coshpot.f90:180-200), the drift cut
(dcut >= 0, step.f90:32-37,66-68), the fixed-node rule off (fn = .false.,
step.f90:131-136) and a weight cut that acts (wtcut, step.f90:130).
hpsi within 1e-10 (FP64) and 1e-6 (mixed); generations with identical
random streams, populations and signs, positions within 1e-10 and weights
within 1e-10 in FP64."""
import numpy as np
import pytest

import oracle
from dmcbcs_project_gb300 import abi, capi, configs

pytestmark = pytest.mark.gpu


def rel_each(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)))


def system(nup, norb, nwalk, idmc=1, sys_over=None, run_over=None):
    sp = configs.system_params(nup, nup, norb)
    sp.update(sys_over or {})
    rp = configs.run_params(nwalk, 0.002, idmc=idmc)
    rp.update(run_over or {})
    return abi.make_system(sp), abi.make_run(rp)


MASSES = dict(mass=[1.0, 2.5])


@pytest.mark.parametrize("nup,norb", [(7, 5), (33, 7)])
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("mixed", 1e-6)])
def test_unequal_masses_hpsi(nup, norb, prec, tol):
    sysd, rund = system(nup, norb, 8, sys_over=dict(MASSES, v0op=0.5, cjas=[1.0, 0.0]))
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    x = orc.walkers()["x"][:8] + np.random.default_rng(3).normal(scale=0.3, size=(8, 2 * nup, 3))
    ref = orc.hpsi(x)
    with capi.Context(sysd, rund, precision=prec) as ctx:
        got = ctx.hpsi(x)
    assert np.array_equal(got["is_"], ref["is_"])
    el_g = -sysd.hbar * got["d2psi"] + got["v"]
    el_r = -sysd.hbar * ref["d2psi"] + ref["v"]
    print(f"masses 1, 2.5 N = {2 * nup} {prec}: E_L rel err {rel_each(el_g, el_r):.2e}")
    for k in ("psil", "d2psi", "v"):
        assert rel_each(got[k], ref[k]) < tol, k
    for w in range(8):
        scale = max(1.0, float(np.max(np.abs(ref["dpsi"][w]))))
        assert float(np.max(np.abs(got["dpsi"][w] - ref["dpsi"][w]))) / scale < tol


CASES = {
    "masses": (dict(MASSES, v0op=0.5), {}),
    "dcut": ({}, dict(dcut=0.5)),
    "no_fixed_node": ({}, dict(fn=0)),
    "wtcut": ({}, dict(wtcut=1.001)),
}


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("idmc", [1, 2])
def test_generations_with_deck_variants(case, idmc):
    so, ro = CASES[case]
    ro = dict(ro)
    if case == "no_fixed_node":
        ro["dt"] = 5 * 0.002 / configs.E_FG            # moves that cross nodes
    sysd, rund = system(7, 5, 40, idmc=idmc, sys_over=so, run_over=ro)
    orc = oracle.Oracle(sysd, rund)
    with capi.Context(sysd, rund) as ctx:
        ctx.init_walkers()
        orc.init_walkers()
        ctx.initial_eval()
        orc.initial_eval()
        for g in range(4):
            assert ctx.generation(g == 3) == orc.generation(g == 3), g
        # one more move without branching: the weights it leaves are the
        # (cut) DMC weights themselves
        ctx.step(True)
        orc.step(True)
        wg, wo = ctx.walkers(), orc.walkers()
        eg, _, wbg = ctx.estimators()
        eo, _, wbo = orc.estimators()
    assert np.array_equal(wg["irn"], wo["irn"])
    assert np.array_equal(wg["is_"], wo["is_"])
    assert float(np.max(np.abs(wg["x"] - wo["x"]))) < 1e-10
    for k in ("psil", "d2psi", "v", "weight"):
        assert rel_each(wg[k], wo[k]) < 1e-10, k
    assert rel_each(eg, eo) < 1e-9 and rel_each(wbg, wbo) < 1e-9
    if case == "wtcut":
        assert np.max(wo["weight"]) == 1.001            # the cut acted
