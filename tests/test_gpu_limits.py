"""Size limits of the walker path.

The walker kernel keeps the pair matrix, its second inverse buffer and the
orbitals of one walker in shared memory up to about N = 144 at seven shells
(K = 81); above that the orbitals, their powers and the second buffer move
to an L2-resident global slice per CTA.  Both sides of the bound (70/70 on
chip, 80/80 at seven shells and 66/66 and 128/128 at ten with the slice)
must match the oracle (FP64 to 1e-10, mixed to 1e-6, generations with
identical streams); a system whose pair matrix and records do not fit even
then is refused with DMC_ERR_UNSUPPORTED at creation, before any launch;
the smallest systems and a single walker run like any other.
"""
import numpy as np
import pytest

import oracle
from dmcbcs_project_gb300 import abi, capi, configs

pytestmark = pytest.mark.gpu


def rel_each(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)))


def system(nup, ndn, norb=7, nwalk=4, idmc=1):
    return (abi.make_system(configs.system_params(nup, ndn, norb)),
            abi.make_run(configs.run_params(nwalk, 0.001, idmc=idmc)))


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("mixed", 1e-6)])
def test_largest_layout_against_oracle(prec, tol):
    sysd, rund = system(70, 70)
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    x = orc.walkers()["x"][:4] + np.random.default_rng(5).normal(scale=0.3, size=(4, 140, 3))
    ref = orc.hpsi(x)
    with capi.Context(sysd, rund, precision=prec) as ctx:
        got = ctx.hpsi(x)
    el_g = -sysd.hbar * got["d2psi"] + got["v"]
    el_r = -sysd.hbar * ref["d2psi"] + ref["v"]
    print(f"N = 140 {prec}: E_L rel err {rel_each(el_g, el_r):.2e}")
    assert np.array_equal(got["is_"], ref["is_"])
    assert rel_each(el_g, el_r) < tol
    assert rel_each(got["psil"], ref["psil"]) < tol
    for w in range(4):
        scale = max(1.0, float(np.max(np.abs(ref["dpsi"][w]))))
        assert float(np.max(np.abs(got["dpsi"][w] - ref["dpsi"][w]))) / scale < tol


def test_largest_layout_generations():
    sysd, rund = system(70, 70, nwalk=8)
    orc = oracle.Oracle(sysd, rund)
    with capi.Context(sysd, rund) as ctx:
        ctx.init_walkers()
        orc.init_walkers()
        ctx.initial_eval()
        orc.initial_eval()
        for g in range(2):
            assert ctx.generation(g == 1) == orc.generation(g == 1)
        wg, wo = ctx.walkers(), orc.walkers()
    assert np.array_equal(wg["irn"], wo["irn"])
    assert float(np.max(np.abs(wg["x"] - wo["x"]))) < 1e-9
    assert rel_each(wg["weight"], wo["weight"]) < 1e-10


@pytest.mark.parametrize("nup,norb,prec,tol", [(80, 7, "fp64", 1e-10), (80, 7, "mixed", 1e-6),
                                               (66, 10, "fp64", 1e-10), (66, 10, "mixed", 1e-6),
                                               (128, 10, "fp64", 1e-10), (128, 10, "mixed", 1e-6)])
def test_union_in_global_scratch_against_oracle(nup, norb, prec, tol):
    """Systems whose orbitals and second inverse buffer do not fit one CTA
    (N = 160 at seven shells, N = 132 and 256 at the production decks' ten
    shells) run with that region in an L2-resident global slice per CTA.
    (128 pairs need more than the 81 pair-function columns of seven shells:
    there the pair matrix is nearly singular and no two implementations
    agree to 1e-10.)"""
    sysd, rund = system(nup, nup, norb, nwalk=4)
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    x = orc.walkers()["x"][:4] + np.random.default_rng(nup + norb).normal(scale=0.3, size=(4, 2 * nup, 3))
    ref = orc.hpsi(x)
    with capi.Context(sysd, rund, precision=prec) as ctx:
        got = ctx.hpsi(x)
        held = ctx.info.device_bytes
    el_g = -sysd.hbar * got["d2psi"] + got["v"]
    el_r = -sysd.hbar * ref["d2psi"] + ref["v"]
    print(f"N = {2 * nup}, {norb} shells {prec}: E_L rel err {rel_each(el_g, el_r):.2e}, "
          f"device memory {held / 2**20:.0f} MiB")
    assert np.array_equal(got["is_"], ref["is_"])
    assert rel_each(el_g, el_r) < tol
    assert rel_each(got["psil"], ref["psil"]) < tol
    for w in range(4):
        scale = max(1.0, float(np.max(np.abs(ref["dpsi"][w]))))
        assert float(np.max(np.abs(got["dpsi"][w] - ref["dpsi"][w]))) / scale < tol


def test_union_in_global_scratch_generations():
    sysd, rund = system(80, 80, 7, nwalk=8)
    orc = oracle.Oracle(sysd, rund)
    with capi.Context(sysd, rund) as ctx:
        ctx.init_walkers()
        orc.init_walkers()
        ctx.initial_eval()
        orc.initial_eval()
        for g in range(2):
            assert ctx.generation(g == 1) == orc.generation(g == 1)
        wg, wo = ctx.walkers(), orc.walkers()
    assert np.array_equal(wg["irn"], wo["irn"])
    assert float(np.max(np.abs(wg["x"] - wo["x"]))) < 1e-9
    assert rel_each(wg["weight"], wo["weight"]) < 1e-10


def test_layout_beyond_one_cta_is_unsupported():
    """Even with the union region off chip, the pair matrix, positions and
    k-vector records must fit: 128/128 at 32 shells does not."""
    sysd, rund = system(128, 128, 32)
    with pytest.raises(capi.DMCError) as err:
        capi.Context(sysd, rund)
    assert err.value.status == abi.DMC_ERR_UNSUPPORTED


def test_single_walker_generations():
    sysd, rund, _ = configs.workload("n14", nwalk=1)
    orc = oracle.Oracle(sysd, rund)
    with capi.Context(sysd, rund) as ctx:
        ctx.init_walkers()
        orc.init_walkers()
        ctx.initial_eval()
        orc.initial_eval()
        for g in range(5):
            assert ctx.generation(g == 4) == orc.generation(g == 4)
        wg, wo = ctx.walkers(), orc.walkers()
    assert np.array_equal(wg["irn"], wo["irn"])
    assert rel_each(wg["psil"], wo["psil"]) < 1e-10


@pytest.mark.parametrize("nup,ndn,norb", [(1, 1, 2), (2, 1, 2), (3, 3, 3), (5, 2, 3)])
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("mixed", 1e-6)])
def test_smallest_systems_against_oracle(nup, ndn, norb, prec, tol):
    """The smallest systems: a 1 x 1 pair matrix, unpaired states with one
    or two pairs, fewer particles than a warp's tile rows in every stage."""
    sysd = abi.make_system(configs.system_params(nup, ndn, norb))
    rund = abi.make_run(configs.run_params(16, 0.002))
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    x = orc.walkers()["x"][:16] + np.random.default_rng(nup + 7 * ndn).normal(scale=0.3, size=(16, nup + ndn, 3))
    ref = orc.hpsi(x)
    with capi.Context(sysd, rund, precision=prec) as ctx:
        got = ctx.hpsi(x)
        if prec == "fp64":
            ctx.init_walkers()
            orc.init_walkers()
            ctx.initial_eval()
            orc.initial_eval()
            for g in range(3):
                assert ctx.generation(g == 2) == orc.generation(g == 2)
            wg, wo = ctx.walkers(), orc.walkers()
            assert np.array_equal(wg["irn"], wo["irn"])
            assert float(np.max(np.abs(wg["x"] - wo["x"]))) < 1e-10
    assert np.array_equal(got["is_"], ref["is_"])
    el_g = -sysd.hbar * got["d2psi"] + got["v"]
    el_r = -sysd.hbar * ref["d2psi"] + ref["v"]
    assert rel_each(el_g, el_r) < tol
    assert rel_each(got["psil"], ref["psil"]) < tol
    scale = max(1.0, float(np.max(np.abs(ref["dpsi"]))))
    assert float(np.max(np.abs(got["dpsi"] - ref["dpsi"]))) / scale < tol


def _fd_relative(sysd, rund, x, eps):
    """Central differences of log|Psi| and E_L with a step relative to each
    parameter (vorb(1..norb), bfact, b, d): the high-shell amplitudes are
    small, and an absolute step of 1e-5 moves them by ~1 % at N = 160."""
    norb = int(sysd.norb)
    theta = list(sysd.vorb[:norb]) + [sysd.bfact, sysd.bbeta, sysd.dbeta]
    dl = np.zeros((x.shape[0], len(theta)))
    de = np.zeros_like(dl)
    base = oracle.Oracle(sysd, rund)
    for k, t in enumerate(theta):
        h = eps * max(abs(t), 1e-3)
        vals = []
        for sgn in (1.0, -1.0):
            if k < norb:
                v = np.array(theta[:norb])
                v[k] += sgn * h
                base.set_vorb(v)
                vals.append(base.hpsi(x))
                base.set_vorb(np.array(theta[:norb]))
            else:
                s2 = type(sysd).from_buffer_copy(sysd)
                field = ("bfact", "bbeta", "dbeta")[k - norb]
                setattr(s2, field, getattr(sysd, field) + sgn * h)
                vals.append(oracle.Oracle(s2, rund).hpsi(x))
        dl[:, k] = (vals[0]["psil"] - vals[1]["psil"]) / (2 * h)
        e0 = -sysd.hbar * vals[0]["d2psi"] + vals[0]["v"]
        e1 = -sysd.hbar * vals[1]["d2psi"] + vals[1]["v"]
        de[:, k] = (e0 - e1) / (2 * h)
    return dl, de


def test_union_in_global_scratch_gradients_and_sweeps():
    """The entry points with layouts of their own at N = 160: the adjoint
    gradients (their scratch then spills from shared memory to global
    memory) against the oracle's analytic d log|det| / d vorb (getderbcs)
    and extrapolated central differences with relative steps, and the
    particle-by-particle sweeps against the oracle's exact ratios."""
    from test_gpu_pgrad import rel_err

    sysd, rund = system(80, 80, 10, nwalk=8, idmc=0)
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    x = orc.walkers()["x"][:2] + np.random.default_rng(12).normal(scale=0.3, size=(2, 160, 3))
    with capi.Context(sysd, rund) as ctx:
        dl, de = ctx.param_grad(x)
    norb = int(sysd.norb)
    od = np.array([orc.getderbcs(x[w]) for w in range(2)])
    assert np.max(np.abs(dl[:, :norb] - od)) < 1e-9 * np.max(np.abs(od))
    l1, e1 = _fd_relative(sysd, rund, x, 1e-4)
    l2, e2 = _fd_relative(sysd, rund, x, 5e-5)
    fl, fe = (4 * l2 - l1) / 3, (4 * e2 - e1) / 3
    print(f"N = 160 ({dl.shape[1]} parameters): d log Psi rel err {rel_err(dl, fl):.2e}, "
          f"d E_L rel err {rel_err(de, fe):.2e}")
    assert rel_err(dl, fl) < 1e-6 and rel_err(de, fe) < 1e-6
    ctx = capi.Context(sysd, rund)
    orc = oracle.Oracle(sysd, rund)
    try:
        for c in (ctx, orc):
            c.init_walkers()
            c.initial_eval()
        acc, moves = ctx.sm_sweeps(1, recompute_every=16)
        acc_o = orc.sm_sweeps(1)
        wg, wo = ctx.walkers(), orc.walkers()
    finally:
        ctx.close()
    assert np.array_equal(wg["irn"], wo["irn"])
    same = [float(np.max(np.abs(wg["x"][w] - wo["x"][w]))) < 1e-10 for w in range(8)]
    print(f"N = 160 sweeps: accepted {acc}/{moves} (oracle {acc_o}), on the oracle's path {sum(same)}/8")
    # the pair matrices here have |S^-1| ~ 3e3, so the FP32 ratios flip more
    # Metropolis decisions against the oracle's FP64 ratios than at N = 66;
    # every walker's state must still be that of its own positions
    assert sum(same) >= 4 and abs(acc - acc_o) < 0.02 * moves
    ref = orc.hpsi(wg["x"])
    assert rel_each(wg["psil"], ref["psil"]) < 1e-9


def test_gradients_with_the_adjoint_core_in_global_scratch():
    """At N = 256 (128/128, ten shells) the adjoint kernel's core (the
    inverse, M and the product buffer: 3 x 128^2 doubles) does not fit one
    CTA's shared memory and runs from a global slice per CTA: d log|det| /
    d vorb against the oracle's analytic getderbcs, and every parameter
    against relative-step central differences of the oracle."""
    from test_gpu_pgrad import rel_err

    sysd, rund = system(128, 128, 10, nwalk=4, idmc=0)
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    x = orc.walkers()["x"][:1] + np.random.default_rng(13).normal(scale=0.3, size=(1, 256, 3))
    with capi.Context(sysd, rund) as ctx:
        dl, de = ctx.param_grad(x)
    norb = int(sysd.norb)
    od = np.array([orc.getderbcs(x[0])])
    assert np.max(np.abs(dl[:, :norb] - od)) < 1e-9 * np.max(np.abs(od))
    l1, e1 = _fd_relative(sysd, rund, x, 1e-4)
    l2, e2 = _fd_relative(sysd, rund, x, 5e-5)
    fl, fe = (4 * l2 - l1) / 3, (4 * e2 - e1) / 3
    print(f"N = 256 ({dl.shape[1]} parameters): d log Psi rel err {rel_err(dl, fl):.2e}, "
          f"d E_L rel err {rel_err(de, fe):.2e}")
    assert rel_err(dl, fl) < 1e-5 and rel_err(de, fe) < 1e-5


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_union_in_global_scratch_two_point_moves(prec):
    """idmc = 10 (two wavefunction evaluations per move) with the union
    region in global scratch: the GF and BIG kernel instance together."""
    sysd, rund = system(80, 80, 10, nwalk=8, idmc=10)
    orc = oracle.Oracle(sysd, rund)
    with capi.Context(sysd, rund, precision=prec) as ctx:
        ctx.init_walkers()
        orc.init_walkers()
        ctx.initial_eval()
        orc.initial_eval()
        for g in range(2):
            assert ctx.generation(g == 1) == orc.generation(g == 1)
        wg, wo = ctx.walkers(), orc.walkers()
        eg, _, wbg = ctx.estimators()
        eo, _, wbo = orc.estimators()
    assert np.array_equal(wg["irn"], wo["irn"])
    assert float(np.max(np.abs(wg["x"] - wo["x"]))) < (1e-10 if prec == "fp64" else 1e-7)
    tol = 1e-10 if prec == "fp64" else 1e-6
    assert rel_each(wg["weight"], wo["weight"]) < tol
    assert rel_each(eg, eo) < (1e-9 if prec == "fp64" else 1e-6)


def test_batch_with_a_global_union_system():
    """A batch holding a system in the global-union layout next to an
    on-chip one: every system's walkers bit for bit those of its context
    run alone (FP64)."""
    specs = [(7, 7, 5, 48), (80, 80, 10, 24)]

    def make():
        out = []
        for i, (nup, ndn, norb, nw) in enumerate(specs):
            sysd = abi.make_system(configs.system_params(nup, ndn, norb, seed=500 + i))
            rund = abi.make_run(configs.run_params(nw, 0.001))
            c = capi.Context(sysd, rund)
            c.init_walkers()
            c.initial_eval()
            out.append(c)
        return out

    A, B = make(), make()
    try:
        with capi.Batch(A) as b:
            b.generations(3, opcomp_last=True)
        for g in range(3):
            for c in B:
                c.generation(g == 2)
        for a, c in zip(A, B):
            wa, wc = a.walkers(), c.walkers()
            for k in ("x", "irn", "weight", "psil", "d2psi"):
                assert np.array_equal(wa[k], wc[k]), k
    finally:
        for c in A + B:
            c.close()
