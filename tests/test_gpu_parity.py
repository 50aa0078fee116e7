"""GPU parity of the CUDA walker path against the CPU oracle.

Tolerance: the FP64 path must match the oracle to 1e-10 relative (scalars
relative to max(|ref|, 1); vectors relative to max(max|ref|, 1)) for
log|Psi|, drift, Laplacian, potential and local energy.  Random-number
streams, walker counts and branching must match exactly.
"""
import numpy as np
import pytest

import oracle
from dmcbcs_project_gb300 import abi, capi, configs

TOL = 1e-10
pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1.0)) if a.size else 0.0


def rel_each(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)))


def configs_for(name, nw, seed=1234):
    sysd, rund, _ = configs.workload(name, nwalk=nw, seed=seed)
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    x = orc.walkers()["x"].copy()
    # spread the permuted copies with a seeded displacement so walkers differ
    rng = np.random.default_rng(seed)
    x = x + rng.normal(scale=0.3, size=x.shape)
    return sysd, rund, orc, x


@pytest.mark.parametrize("name,nw", [("n14", 64), ("n66", 96), ("p33_30", 32), ("p38_33", 32), ("n38", 32)])
def test_hpsi_parity(name, nw):
    sysd, rund, orc, x = configs_for(name, nw)
    ref = orc.hpsi(x)
    with capi.Context(sysd, rund) as ctx:
        got = ctx.hpsi(x)
    assert np.array_equal(got["is_"], ref["is_"])
    assert rel_each(got["psil"], ref["psil"]) < TOL
    assert rel_each(got["d2psi"], ref["d2psi"]) < TOL
    assert rel_each(got["v"], ref["v"]) < TOL
    hb = sysd.hbar
    el_g = -hb * got["d2psi"] + got["v"]
    el_r = -hb * ref["d2psi"] + ref["v"]
    assert rel_each(el_g, el_r) < TOL
    for w in range(nw):
        assert rel(got["dpsi"][w], ref["dpsi"][w]) < TOL, w


@pytest.mark.parametrize("name,nw", [("n14", 16), ("n66", 16), ("p38_33", 8)])
def test_bcs_and_inverse(name, nw):
    sysd, rund, orc, x = configs_for(name, nw, seed=7)
    ref = orc.bcs(x, want_inverse=True)
    with capi.Context(sysd, rund) as ctx:
        got = ctx.bcs(x, want_inverse=True)
    assert np.array_equal(got["is_"], ref["is_"])
    assert rel_each(got["phil"], ref["phil"]) < TOL
    assert rel_each(got["d2phi"], ref["d2phi"]) < TOL
    for w in range(nw):
        assert rel(got["dphi"][w], ref["dphi"][w]) < TOL
        assert rel(got["smati"][w], ref["smati"][w]) < 1e-9


@pytest.mark.parametrize("name,same_spin", [("n14", False), ("n66", False), ("n66", True)])
def test_getphi(name, same_spin):
    sysd, rund, orc, x = configs_for(name, 8, seed=3)
    if same_spin:
        # the same-spin Jastrow on (cjas(2) = 1, its own effective interaction)
        sysd.v0op, sysd.v0eq = 0.5, -0.5
        sysd.cjas[0], sysd.cjas[1] = 1.0, 1.0
        orc = oracle.Oracle(sysd, rund)
    with capi.Context(sysd, rund) as ctx:
        got = ctx.getphi(x)
    for w in range(x.shape[0]):
        r = orc.getphi(x[w])
        assert abs(got["u"][w] - r["u"]) <= TOL * max(1.0, abs(r["u"]))
        assert abs(got["d2u"][w] - r["d2u"]) <= TOL * max(1.0, abs(r["d2u"]))
        assert abs(got["v"][w] - r["v"]) <= TOL * max(1.0, abs(r["v"]))
        assert rel(got["du"][w], r["du"]) < TOL


@pytest.mark.parametrize("n", [1, 2, 7, 33, 66, 96, 110, 128, 150])
def test_matinv(n):
    """Blocked Gauss-Jordan with 2, 3 and 4 rows per lane (n <= 64, 96,
    ~114 where the second buffer fits) and the single-buffer form above."""
    rng = np.random.default_rng(n)
    a = rng.normal(size=(5, n, n))
    sysd, rund, _ = configs.workload("n14", nwalk=4)
    with capi.Context(sysd, rund) as ctx:
        inv, d, s = ctx.matinv(a)
    for b in range(a.shape[0]):
        ri, rd, rs, info = oracle.matinv(a[b])
        assert info == 0
        assert s[b] == rs
        assert abs(d[b] - rd) < 1e-11 * max(1.0, abs(rd))
        assert rel(inv[b], ri) < 1e-10


def test_matinv_too_large_is_unsupported():
    sysd, rund, _ = configs.workload("n14", nwalk=4)
    with capi.Context(sysd, rund) as ctx:
        with pytest.raises(capi.DMCError) as err:
            ctx.matinv(np.eye(200)[None])
    assert err.value.status == abi.DMC_ERR_UNSUPPORTED


def test_matinv_singular():
    a = np.zeros((1, 4, 4))
    a[0, :, 0] = 1.0
    a[0, :, 1] = 1.0   # two equal columns: exactly singular
    a[0, 2, 2] = a[0, 3, 3] = 1.0
    sysd, rund, _ = configs.workload("n14", nwalk=4)
    with capi.Context(sysd, rund) as ctx:
        _, d, s = ctx.matinv(a)
    assert d[0] == -1.0e30


@pytest.mark.parametrize("name,nw,idmc,gens", [("n14", 64, 1, 6), ("n14", 32, 0, 4), ("n66", 48, 1, 3),
                                               ("n14", 32, 2, 4)])
def test_generation_parity(name, nw, idmc, gens):
    sysd, rund, _ = configs.workload(name, nwalk=nw, idmc=idmc)
    orc = oracle.Oracle(sysd, rund)
    with capi.Context(sysd, rund) as ctx:
        ctx.init_walkers()
        orc.init_walkers()
        sg, eg = ctx.initial_eval()
        so, eo = orc.initial_eval()
        assert rel_each(sg, so) < 1e-9
        if idmc != 0:
            assert rel_each(eg, eo) < 1e-9
        for g in range(gens):
            op = g == gens - 1
            ng = ctx.generation(op)
            no = orc.generation(op)
            assert ng == no, (g, ng, no)
        wg, wo = ctx.walkers(), orc.walkers()
        assert np.array_equal(wg["irn"], wo["irn"])
        assert np.array_equal(wg["is_"], wo["is_"])
        assert rel(wg["x"], wo["x"]) < 1e-10
        for k in ("psil", "psigl", "d2psi", "d2psig", "v", "weight"):
            assert rel_each(wg[k], wo[k]) < TOL, k
        vb_g, vb2_g, wb_g = ctx.estimators()
        vb_o, vb2_o, wb_o = orc.estimators()
        assert rel_each(vb_g, vb_o) < 1e-9
        assert rel_each(wb_g, wb_o) < 1e-9
        assert np.array_equal(ctx.wtisto(), orc.wtisto())


@pytest.mark.parametrize("name,nw,idmc", [("n14", 48, 1), ("n14", 32, 0), ("p33_30", 16, 2)])
def test_step_and_branch_calls(name, nw, idmc):
    """The separate drop-ins for step1 (step.f90:43) and branch (step.f90:287),
    called the way the reference's loop calls them, against the oracle."""
    sysd, rund, _ = configs.workload(name, nwalk=nw, idmc=idmc)
    orc = oracle.Oracle(sysd, rund)
    with capi.Context(sysd, rund) as ctx:
        ctx.init_walkers()
        orc.init_walkers()
        ctx.initial_eval()
        orc.initial_eval()
        for g in range(3):
            op = g == 2
            ctx.step(op)
            orc.step(op)
            if idmc > 0:
                ctx.branch(1.0)
                orc.branch(1.0)
            assert ctx.num_walkers() == orc.num_walkers()
        wg, wo = ctx.walkers(), orc.walkers()
        assert np.array_equal(wg["irn"], wo["irn"])
        assert np.array_equal(wg["is_"], wo["is_"])
        assert rel(wg["x"], wo["x"]) < 1e-10
        for k in ("psil", "d2psi", "v", "weight"):
            assert rel_each(wg[k], wo[k]) < TOL, k
        vb_g, _, wb_g = ctx.estimators()
        vb_o, _, wb_o = orc.estimators()
        assert rel_each(vb_g, vb_o) < 1e-9 and rel_each(wb_g, wb_o) < 1e-9


def test_timed_generations_equal_generations():
    """dmc_timed_generations (graph replay with events) gives the same walkers
    as the same number of dmc_generation calls."""
    sysd, rund, _ = configs.workload("n66", nwalk=64, idmc=1)
    with capi.Context(sysd, rund) as a, capi.Context(sysd, rund) as b:
        for c in (a, b):
            c.init_walkers()
            c.initial_eval()
        steps, ms, nl = a.timed_generations(4, opcomp_last=True, flush_l2=True)
        n_in = []
        for g in range(4):
            n_in.append(b.num_walkers())
            b.generation(g == 3)
        assert steps == sum(n_in) and ms > 0 and nl > 0
        wa, wb = a.walkers(), b.walkers()
        for k in ("x", "irn", "weight", "psil", "d2psi"):
            assert np.array_equal(wa[k], wb[k]), k
        for ea, eb in zip(a.estimators(), b.estimators()):
            assert np.array_equal(ea, eb)
