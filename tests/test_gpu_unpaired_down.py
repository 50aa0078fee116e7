"""Systems with unpaired DOWN plane waves (nexdn > 0: extra rows of the pair
matrix that depend on one down particle each, psislaterbcs.f90:189-206, with
the gradient sign flipped in the drift, :211-223), alone (7 up / 8 down,
one unpaired down state) and together with an unpaired up state (9 up / 10
down: one unpaired up, two unpaired down).  The benchmark workloads put the
larger species up, so these rows are covered here: wavefunction and
local-energy parity (FP64 to 1e-10, mixed to 1e-7 relative), generation
parity (populations and random streams exactly), and the adjoint parameter
gradients against the oracle's extrapolated central differences."""
import numpy as np
import pytest

import oracle
from dmcbcs_project_gb300 import capi, configs
from dmcbcs_project_gb300.abi import make_run, make_system

pytestmark = pytest.mark.gpu

SYSTEMS = {
    "d7_8": (7, 8, [], [(0, 0, 0)]),
    "b9_10": (9, 10, [(0, 0, 0)], [(1, 0, 0), (-1, 0, 0)]),
}


def system(name, nwalk=16, idmc=1, seed=99):
    nup, ndn, ikup, ikdn = SYSTEMS[name]
    sp = configs.system_params(max(nup, ndn), max(nup, ndn), 5, seed=seed)
    sp.update(nbin=[nup, ndn], nexup=len(ikup), ikup=[list(k) for k in ikup], nexdn=len(ikdn),
              ikdn=[list(k) for k in ikdn])
    return make_system(sp), make_run(configs.run_params(nwalk, 0.002, idmc=idmc))


def rel_each(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)))


@pytest.mark.parametrize("name", list(SYSTEMS))
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-7)])
def test_hpsi_parity(name, precision, tol):
    sysd, rund = system(name)
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    x = orc.walkers()["x"] + np.random.default_rng(3).normal(scale=0.2, size=(16, orc.npart, 3))
    ho = orc.hpsi(x)
    with capi.Context(sysd, rund, precision=precision) as ctx:
        assert ctx.nd == orc.nd
        hg = ctx.hpsi(x)
    assert np.array_equal(hg["is_"], ho["is_"])
    for k in ("psil", "d2psi", "v"):
        assert rel_each(hg[k], ho[k]) < tol, k
    scale = max(float(np.max(np.abs(ho["dpsi"]))), 1.0)
    assert float(np.max(np.abs(hg["dpsi"] - ho["dpsi"]))) / scale < tol
    eg = -sysd.hbar * hg["d2psi"] + hg["v"]
    eo = -sysd.hbar * ho["d2psi"] + ho["v"]
    assert rel_each(eg, eo) < tol


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_generation_parity(name):
    sysd, rund = system(name, nwalk=24, idmc=1)
    orc = oracle.Oracle(sysd, rund)
    with capi.Context(sysd, rund) as ctx:
        ctx.init_walkers()
        orc.init_walkers()
        ctx.initial_eval()
        orc.initial_eval()
        for g in range(4):
            assert ctx.generation(g == 3) == orc.generation(g == 3)
        wg, wo = ctx.walkers(), orc.walkers()
    assert np.array_equal(wg["irn"], wo["irn"])
    assert np.array_equal(wg["is_"], wo["is_"])
    assert float(np.max(np.abs(wg["x"] - wo["x"]))) < 1e-9
    for k in ("psil", "d2psi", "v", "weight"):
        assert rel_each(wg[k], wo[k]) < 1e-10, k


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_param_grad(name):
    import test_gpu_pgrad as pg

    sysd, rund = system(name, nwalk=4)
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    x = orc.walkers()["x"][:4] + np.random.default_rng(5).normal(scale=0.2, size=(4, orc.npart, 3))
    with capi.Context(sysd, rund) as ctx:
        dl, de = ctx.param_grad(x)
    fl, fe = pg.fd_oracle(sysd, rund, x)
    el, ee = pg.rel_err(dl, fl), pg.rel_err(de, fe)
    print(f"{name}: d log Psi rel err {el:.2e}, d E_L rel err {ee:.2e}")
    assert el < pg.TOL and ee < pg.TOL
