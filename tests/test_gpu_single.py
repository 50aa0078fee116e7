"""Single-particle ratios (bcsone, getphione, move1), parameter derivatives
(getderbcs) and the stochastic-reconfiguration sums and step, through the
C ABI, against the oracle (FP64, <= 1e-10 relative) and against properties
that need no oracle: a ratio equals the quotient of two full evaluations,
and the derivative equals a central finite difference of log|det| in vorb
(chkderp, optimizer.f90:171-225)."""
import numpy as np
import pytest

import oracle
from dmcbcs_project_gb300 import abi, capi, configs

pytestmark = pytest.mark.gpu

TOL = 1e-10
NAMES = ["n14", "n66", "p33_30", "p38_33"]
NAMES_RATIO = NAMES + ["n132"]   # nd = 66: three passes of the warp over a row


def setup(name, nw, seed, jastrow=False):
    sysd, rund, _ = configs.workload(name, nwalk=nw, seed=seed)
    if jastrow:
        # the same-spin Jastrow on (the workloads have cjas(2) = 0) with its
        # own effective interaction, and a weaker up-down one
        sysd.v0op, sysd.v0eq = 0.5, -0.5
        sysd.cjas[0], sysd.cjas[1] = 1.0, 1.0
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    x = orc.walkers()["x"][:nw] + np.random.default_rng(seed).normal(scale=0.3, size=(nw, orc.npart, 3))
    return sysd, rund, orc, x


def moves(npart, nw, seed, scale=0.4):
    rng = np.random.default_rng(seed)
    ip = rng.integers(1, npart + 1, size=nw).astype(np.int32)
    ip[:2] = [1, npart]   # first up and last down particle always covered
    dr = rng.normal(scale=scale, size=(nw, 3))
    return ip, dr


def rel(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-300)


@pytest.mark.parametrize("name", NAMES_RATIO)
def test_bcsone_against_oracle_and_full_evaluation(name):
    sysd, rund, orc, x = setup(name, 24, 3)
    ip, dr = moves(orc.npart, x.shape[0], 4)
    with capi.Context(sysd, rund) as ctx:
        old = ctx.bcs(x, want_inverse=True)
        got = ctx.bcsone(x, old["smati"], ip, dr)
        xn = x.copy()
        xn[np.arange(len(ip)), ip - 1] -= dr
        new = ctx.bcs(xn)
    ref = np.array([orc.bcsone(x[w], dr[w], ip[w], old["smati"][w]) for w in range(len(ip))])
    full = new["is_"] * old["is_"] * np.exp(new["phil"] - old["phil"])
    print(f"{name}: bcsone rel err vs oracle {rel(got, ref).max():.2e}, vs det quotient {rel(got, full).max():.2e}")
    assert rel(got, ref).max() < TOL
    assert rel(got, full).max() < 1e-8


@pytest.mark.parametrize("jastrow", [False, True])
@pytest.mark.parametrize("name", NAMES_RATIO)
def test_getphione_against_oracle_and_full_evaluation(name, jastrow):
    sysd, rund, orc, x = setup(name, 24, 5, jastrow)
    # small steps so that some pairs cross the healing distance
    ip, drr = moves(orc.npart, x.shape[0], 6, scale=0.2)
    with capi.Context(sysd, rund) as ctx:
        got = ctx.getphione(x, ip, drr)
        xn = x.copy()
        xn[np.arange(len(ip)), ip - 1] -= drr
        u0, u1 = ctx.getphi(x)["u"], ctx.getphi(xn)["u"]
    ref = np.array([orc.getphione(x[w], drr[w], ip[w]) for w in range(len(ip))])
    print(f"{name} (same-spin Jastrow {'on' if jastrow else 'off'}): getphione rel err vs oracle {rel(got, ref).max():.2e}, "
          f"ratios in [{got.min():.3g}, {got.max():.3g}]")
    assert rel(got, ref).max() < TOL
    assert rel(got, np.exp(u1 - u0)).max() < 1e-9
    if jastrow:
        assert np.max(np.abs(got - 1.0)) > 1e-3     # the moves change the Jastrow


def test_move1_is_the_product():
    sysd, rund, orc, x = setup("p33_30", 16, 7, jastrow=True)
    ip, dr = moves(orc.npart, x.shape[0], 8)
    xnew = x[np.arange(len(ip)), ip - 1] - dr
    with capi.Context(sysd, rund) as ctx:
        sm = ctx.bcs(x, want_inverse=True)["smati"]
        r = ctx.move1(x, sm, ip, xnew)
        r1 = ctx.getphione(x, ip, dr)
        r2 = ctx.bcsone(x, sm, ip, dr)
    assert np.array_equal(r, r1 * r2)


def test_ratio_arguments_are_checked():
    sysd, rund, orc, x = setup("n14", 2, 9)
    with capi.Context(sysd, rund) as ctx:
        with pytest.raises(capi.DMCError) as e:
            ctx.getphione(x, [0, 1], np.zeros((2, 3)))
        assert e.value.status == abi.DMC_ERR_INVALID
        with pytest.raises(capi.DMCError):
            ctx.getphione(x, [1, orc.npart + 1], np.zeros((2, 3)))


@pytest.mark.parametrize("name", NAMES)
def test_getderbcs_against_oracle(name):
    sysd, rund, orc, x = setup(name, 12, 11)
    with capi.Context(sysd, rund) as ctx:
        got = ctx.getderbcs(x)
    ref = np.array([orc.getderbcs(x[w]) for w in range(x.shape[0])])
    err = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max())
    print(f"{name}: getderbcs rel err {err.max():.2e}")
    assert err.max() < TOL


def test_getderbcs_is_the_vorb_derivative_of_log_det():
    """chkderp (optimizer.f90:171-225): central differences in vorb with a
    step relative to each amplitude (h = 1e-4 |vorb|), Richardson-
    extrapolated from h and h/2.  The outer shells have amplitudes ~1e-2 and
    derivatives ~1e3, so a fixed absolute step leaves ~1e-5 truncation
    error there."""
    sysd, rund, orc, x = setup("n66", 4, 13)
    with capi.Context(sysd, rund) as ctx:
        der = ctx.getderbcs(x)
        v0 = np.array(sysd.vorb[: sysd.norb])

        def central(p, step):
            vp, vm = v0.copy(), v0.copy()
            vp[p] += step
            vm[p] -= step
            ctx.set_vorb(vp)
            lp = ctx.bcs(x)["phil"]
            ctx.set_vorb(vm)
            lm = ctx.bcs(x)["phil"]
            return (lp - lm) / (2 * step)

        fd = np.zeros_like(der)
        for p in range(sysd.norb):
            h = 1e-4 * abs(v0[p])
            fd[:, p] = (4.0 * central(p, h / 2) - central(p, h)) / 3.0
        ctx.set_vorb(v0)
    err = np.abs(der - fd) / np.maximum(np.abs(fd), 1.0)
    print(f"getderbcs vs central FD: max err {err.max():.2e}")
    assert err.max() < 1e-6


def test_sr_sums_step_and_order():
    """calder over a VMC population (pop order, top first), then updatepar."""
    sysd, rund, _ = configs.workload("n14", nwalk=48, idmc=-1)
    orc = oracle.Oracle(sysd, rund)
    with capi.Context(sysd, rund) as ctx:
        ctx.init_walkers()
        ctx.initial_eval()
        for _ in range(3):
            ctx.generation(False)
        w = ctx.walkers()
        n = w["n"]
        assert ctx.sr_accumulate() == n
        after = ctx.walkers()
        assert np.array_equal(after["x"], w["x"][::-1])      # pushed back in reverse
        s = ctx.sr_sums()
        vorb0 = ctx.table(10).copy()
        newp, eave, eerr = ctx.sr_update(0.05, 1e-3)
        vorb1 = ctx.table(10)
        zero = ctx.sr_sums()
    d = np.array([orc.getderbcs(w["x"][k]) for k in range(n)])
    ene = (-sysd.hbar * w["d2psi"] + w["v"]) / orc.info.eunit / orc.npart
    order = np.arange(n)[::-1]
    ov = np.zeros(sysd.norb)
    ow = np.zeros(sysd.norb)
    pm = np.zeros((sysd.norb, sysd.norb))
    es = es2 = 0.0
    for k in order:
        ov += d[k]
        ow += d[k] * ene[k]
        pm += np.outer(d[k], d[k])
        es += ene[k]
        es2 += ene[k] ** 2
    scale = np.abs(ov).max()
    assert np.abs(s["ovec"] - ov).max() < TOL * max(scale, 1.0)
    assert np.abs(s["ovecw"] - ow).max() < TOL * max(np.abs(ow).max(), 1.0)
    assert np.abs(s["pmat"] - pm).max() < TOL * max(np.abs(pm).max(), 1.0)
    assert abs(s["e"][0] - es) < TOL * max(abs(es), 1.0)
    assert abs(s["e"][1] - es2) < TOL * max(abs(es2), 1.0)
    assert s["n"] == n
    refp, refe, referr = oracle.sr_update(s["ovec"], s["ovecw"], s["pmat"], s["e"][0], s["e"][1], n, 0.05, 1e-3)
    assert np.abs(newp - refp).max() < 1e-9 * max(np.abs(refp).max(), 1e-12)
    assert abs(eave - refe) < 1e-12 * max(abs(refe), 1.0)
    assert abs(eerr - referr) < 1e-9 * max(abs(referr), 1e-12)
    assert np.allclose(vorb1, vorb0 + newp, rtol=0, atol=1e-15)
    assert zero["n"] == 0 and not zero["ovec"].any()


def test_sr_update_without_samples_is_rejected():
    sysd, rund, _ = configs.workload("n14", nwalk=8, idmc=-1)
    with capi.Context(sysd, rund) as ctx:
        with pytest.raises(capi.DMCError) as e:
            ctx.sr_update(0.05, 1e-3)
        assert e.value.status == abi.DMC_ERR_INVALID
