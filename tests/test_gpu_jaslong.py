"""Long-range Jastrow (jastrowlongrange.f90:22-46, switched on by numq > 0)
on both GPU paths against the oracle: hpsi values (N = 132 runs the mixed
path on its 16-warp CTA) and whole generations."""
import numpy as np
import pytest

import oracle
from dmcbcs_project_gb300 import capi, configs

pytestmark = pytest.mark.gpu

LR = (3, 1.0, 0.3)   # numq, beta, gamma


def _x(name, nw, seed):
    sysd, rund, _ = configs.workload(name, nwalk=nw, seed=seed, longrange=LR)
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    x = orc.walkers()["x"] + np.random.default_rng(seed).normal(scale=0.3, size=(nw, orc.npart, 3))
    return sysd, rund, orc, x


@pytest.mark.parametrize("name", ["n14", "n66", "p33_30", "n132"])
def test_hpsi_with_long_range_jastrow(name):
    sysd, rund, orc, x = _x(name, 16, 31)
    ref = orc.hpsi(x)
    for prec, tol in (("fp64", 1e-10), ("mixed", 1e-6)):
        with capi.Context(sysd, rund, precision=prec) as ctx:
            got = ctx.hpsi(x)
        el_g = -sysd.hbar * got["d2psi"] + got["v"]
        el_r = -sysd.hbar * ref["d2psi"] + ref["v"]
        e_el = np.max(np.abs(el_g - el_r) / np.maximum(np.abs(el_r), 1.0))
        e_pl = np.max(np.abs(got["psil"] - ref["psil"]) / np.maximum(np.abs(ref["psil"]), 1.0))
        e_dr = np.max(np.abs(got["dpsi"] - ref["dpsi"])) / max(1.0, np.max(np.abs(ref["dpsi"])))
        print(f"{name} {prec}: E_L {e_el:.2e} log|Psi| {e_pl:.2e} drift {e_dr:.2e}")
        assert e_el < tol and e_pl < tol and e_dr < tol


def test_generations_with_long_range_jastrow():
    sysd, rund, _ = configs.workload("n14", nwalk=32, longrange=LR)
    orc = oracle.Oracle(sysd, rund)
    with capi.Context(sysd, rund) as ctx:
        for m in (ctx, orc):
            m.init_walkers()
            m.initial_eval()
            for g in range(3):
                m.generation(g == 2)
        wg, wo = ctx.walkers(), orc.walkers()
    assert wg["n"] == wo["n"]
    assert np.array_equal(wg["irn"], wo["irn"])
    assert np.max(np.abs(wg["x"] - wo["x"])) < 1e-10
    assert np.max(np.abs(wg["psil"] - wo["psil"])) < 1e-9


def test_getjasder_against_oracle():
    sysd, rund, orc, x = _x("n14", 12, 41)
    with capi.Context(sysd, rund) as ctx:
        got = ctx.getjasder(x)
    ref = np.array([orc.getjasder(x[w]) for w in range(x.shape[0])])
    err = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-6 * np.max(np.abs(ref), axis=0))
    print(f"getjasder rel err {err[:, 0].max():.2e} (d/d beta), {err[:, 1].max():.2e} (d/d gamma)")
    # d/d gamma = U/gamma agrees to rounding; d/d beta is the reference's
    # central difference with dp = 1e-4, which turns rounding-level
    # differences in U (pair sum there, |rho_q|^2 - N here) into ~1e-8
    assert err[:, 1].max() < 1e-11
    assert err[:, 0].max() < 1e-7


def test_sr_step_with_jastrow_and_determinant_parameters():
    """calder with iopt(1) and iopt(2): derpsi = (djas(2), dpsi(norb))."""
    sysd, rund, _ = configs.workload("n14", nwalk=40, idmc=-1, longrange=LR)
    orc = oracle.Oracle(sysd, rund)
    with capi.Context(sysd, rund) as ctx:
        ctx.init_walkers()
        ctx.initial_eval()
        for _ in range(2):
            ctx.generation(False)
        ctx.sr_configure(True, True)
        w = ctx.walkers()
        n = w["n"]
        assert ctx.sr_accumulate() == n
        s = ctx.sr_sums()
        bg0, vorb0 = ctx.table(11).copy(), ctx.table(10).copy()
        newp, eave, eerr = ctx.sr_update(0.02, 1e-3)
        bg1, vorb1 = ctx.table(11), ctx.table(10)
    d = np.array([np.concatenate([orc.getjasder(w["x"][k]), orc.getderbcs(w["x"][k])]) for k in range(n)])
    ene = (-sysd.hbar * w["d2psi"] + w["v"]) / orc.info.eunit / orc.npart
    ov = d[::-1].sum(axis=0)
    pm = sum(np.outer(d[k], d[k]) for k in range(n)[::-1])
    assert len(s["ovec"]) == 2 + sysd.norb
    assert np.allclose(s["ovec"], ov, rtol=1e-9, atol=1e-9 * np.abs(ov).max())
    assert np.allclose(s["ovecw"], (d * ene[:, None])[::-1].sum(axis=0), rtol=1e-9, atol=1e-8)
    assert np.allclose(s["pmat"], pm, rtol=1e-9, atol=1e-9 * np.abs(pm).max())
    refp, refe, _ = oracle.sr_update(s["ovec"], s["ovecw"], s["pmat"], s["e"][0], s["e"][1], n, 0.02, 1e-3)
    assert np.allclose(newp, refp, rtol=1e-8, atol=1e-12)
    assert np.allclose(bg1, bg0 + newp[:2], rtol=0, atol=1e-15)
    assert np.allclose(vorb1, vorb0 + newp[2:], rtol=0, atol=1e-15)
