"""The opt-in up-down Jastrow spline on the walker path, against the oracle.

The spline (16 knots, h = L/34, cubic B-spline basis even in r and zero at
L/2) is added to the reference's up-down Jastrow table; with it on, hpsi
must still match the oracle (which adds the same spline to its own table) to
1e-10 in FP64 and 1e-6 in mixed precision -- the mixed path then keeps the
whole up-down Jastrow in double-float out to L/2 -- and DMC generations must
keep identical random streams and populations.  Switching the spline off
restores the reference's wavefunction bit for bit.
"""
import numpy as np
import pytest

import oracle
from dmcbcs_project_gb300 import capi, configs

pytestmark = pytest.mark.gpu

KNOTS = np.random.default_rng(17).uniform(-0.3, 0.3, 16) * np.exp(-0.15 * np.arange(16))


def setup(name, nw, seed=23):
    sysd, rund, _ = configs.workload(name, nwalk=nw, seed=seed)
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    x = orc.walkers()["x"][:nw] + np.random.default_rng(seed).normal(scale=0.3, size=(nw, orc.npart, 3))
    orc.set_jastrow_spline(KNOTS)
    return sysd, rund, orc, x


def rel_each(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b)) / np.maximum(np.abs(b), 1.0)))


@pytest.mark.parametrize("name,nw,prec", [("n14", 32, "fp64"), ("n66", 32, "fp64"), ("n14", 32, "mixed"),
                                          ("n66", 32, "mixed"), ("p33_30", 16, "mixed")])
def test_spline_hpsi_against_oracle(name, nw, prec):
    sysd, rund, orc, x = setup(name, nw)
    ref = orc.hpsi(x)
    with capi.Context(sysd, rund, precision=prec) as ctx:
        base = ctx.hpsi(x)
        ctx.set_jastrow_spline(KNOTS)
        got = ctx.hpsi(x)
        ctx.set_jastrow_spline(None)
        back = ctx.hpsi(x)
    tol = 1e-10 if prec == "fp64" else 1e-6
    el_g = -sysd.hbar * got["d2psi"] + got["v"]
    el_r = -sysd.hbar * ref["d2psi"] + ref["v"]
    err = rel_each(el_g, el_r)
    print(f"{name} {prec}: E_L rel err with the spline {err:.2e}, "
          f"max |log Psi change| {np.max(np.abs(got['psil'] - base['psil'])):.3f}")
    assert err < tol
    assert rel_each(got["psil"], ref["psil"]) < tol
    for w in range(nw):
        assert np.max(np.abs(got["dpsi"][w] - ref["dpsi"][w])) < tol * max(1.0, np.max(np.abs(ref["dpsi"][w])))
    assert np.max(np.abs(got["psil"] - base["psil"])) > 1e-3       # the spline changes Psi
    for k in ("psil", "d2psi", "v"):
        assert np.array_equal(back[k], base[k]), k


def test_spline_generations_against_oracle():
    sysd, rund, _ = configs.workload("n14", nwalk=48)
    orc = oracle.Oracle(sysd, rund)
    orc.set_jastrow_spline(KNOTS)
    with capi.Context(sysd, rund) as ctx:
        ctx.set_jastrow_spline(KNOTS)
        ctx.init_walkers()
        orc.init_walkers()
        ctx.initial_eval()
        orc.initial_eval()
        for g in range(4):
            assert ctx.generation(g == 3) == orc.generation(g == 3)
        wg, wo = ctx.walkers(), orc.walkers()
    assert np.array_equal(wg["irn"], wo["irn"])
    assert np.max(np.abs(wg["x"] - wo["x"])) < 1e-10
    assert rel_each(wg["psil"], wo["psil"]) < 1e-10


def test_spline_rejects_wrong_sizes():
    sysd, rund, _ = configs.workload("n14", nwalk=4)
    with capi.Context(sysd, rund) as ctx:
        with pytest.raises(capi.DMCError):
            ctx.set_jastrow_spline(np.zeros(15))
        with pytest.raises(capi.DMCError):
            ctx.set_jastrow_spline(np.full(16, np.nan))
        assert ctx.jastrow_spline().size == 0
