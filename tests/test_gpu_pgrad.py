"""Adjoint parameter gradients (dmc_param_grad) for theta = (vorb(1..norb),
bfact, b, d, and the 16 knots of the opt-in up-down Jastrow spline):
d log|Psi| / d theta and d E_L / d theta per walker, E_L = -hbar d2psi + v.
At seven shells with the beta function and the spline on that is
7 + 3 + 16 = 26 parameters.

Checks:
  - the vorb part of d log|Psi| equals getderbcs (psislaterbcs.f90:449-524),
    which the single-walker parity tests hold to the oracle;
  - both gradients against central finite differences of the ORACLE's hpsi
    with the parameter moved up and down (vorb through set_vorb, bfact, b and
    d through beta tables rebuilt at the moved value -- the image-summed,
    shifted, bfact-scaled table of betafun.f90:62-64,100-122 -- and the
    knots through the oracle's spline), extrapolated from h = 1e-5 and h/2
    as chkderp does (optimizer.f90:171-225): plain central differences at
    h = 1e-5 carry an O(h^2) error of ~5e-6 relative for the small
    high-shell amplitudes of the polarised system; relative error <= 1e-6 of
    max(|FD|, 1e-3 * max over theta of |FD|);
  - a torch.autograd.Function whose forward is the GPU local energy at theta
    and whose backward is the adjoint passes torch.autograd.gradcheck
    (finite differences of the forward, float64), over vorb and over all
    26 parameters;
  - the SR step over every adjoint parameter: its sums equal the sums of the
    adjoint d log Psi over the population in pop order, and the update moves
    every parameter by the step it returns.
Systems: 7/7, polarised 33/30 (unpaired columns enter M but not S'), 33/33,
7/7 with the long-range Jastrow on (its gradient enters w), and 33/33 with
the same-spin Jastrow on (its pair terms enter w)."""
import numpy as np
import pytest

import oracle
from dmcbcs_project_gb300 import capi, configs

pytestmark = pytest.mark.gpu

H = 1e-5
TOL = 1e-6
LR = (3, 1.0, 0.3)


def knots_for(seed):
    """Seeded knot values of a smooth up-down Jastrow spline (|u_s| < ~0.3)."""
    rng = np.random.default_rng(seed)
    return rng.uniform(-0.3, 0.3, 16) * np.exp(-0.15 * np.arange(16))


def walkers(name, nw, seed=11, longrange=None, same_spin=False):
    sysd, rund, _ = configs.workload(name, nwalk=nw, seed=seed, longrange=longrange)
    if same_spin:
        # the same-spin Jastrow on: grad J, which the d E_L terms use, then
        # has same-spin pair terms
        sysd.v0op, sysd.v0eq = 0.5, -0.5
        sysd.cjas[0], sysd.cjas[1] = 1.0, 1.0
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    x = orc.walkers()["x"][:nw].copy()
    x += np.random.default_rng(seed).normal(scale=0.3, size=x.shape)
    return sysd, rund, x


def eloc(h, hbar):
    return -hbar * h["d2psi"] + h["v"]


def fd_oracle(sysd, rund, x, knots=None):
    """Extrapolated central differences (4 D(h/2) - D(h)) / 3 of log|Psi|
    and E_L over theta with the oracle."""
    l1, e1 = fd_central(sysd, rund, x, H, knots)
    l2, e2 = fd_central(sysd, rund, x, H / 2, knots)
    return (4 * l2 - l1) / 3, (4 * e2 - e1) / 3


def oracle_at(sysd, rund, knots):
    orc = oracle.Oracle(sysd, rund)
    if knots is not None:
        orc.set_jastrow_spline(knots)
    return orc


def fd_central(sysd, rund, x, H, knots=None):
    norb = int(sysd.norb)
    vorb = np.array(sysd.vorb[:norb], dtype=float)
    nbeta = 3 if sysd.bfact != 0.0 else 0
    nkn = 0 if knots is None else 16
    np_ = norb + nbeta + nkn
    dl = np.zeros((x.shape[0], np_))
    de = np.zeros((x.shape[0], np_))

    def put(t, vals):
        dl[:, t] = (vals[0]["psil"] - vals[1]["psil"]) / (2 * H)
        de[:, t] = (eloc(vals[0], sysd.hbar) - eloc(vals[1], sysd.hbar)) / (2 * H)

    orc = oracle_at(sysd, rund, knots)
    for t in range(norb):
        vals = []
        for sgn in (1.0, -1.0):
            v = vorb.copy()
            v[t] += sgn * H
            orc.set_vorb(v)
            vals.append(orc.hpsi(x))
        put(t, vals)
    orc.set_vorb(vorb)
    for q, field in enumerate(("bfact", "bbeta", "dbeta")[:nbeta]):
        vals = []
        for sgn in (1.0, -1.0):
            s2 = type(sysd).from_buffer_copy(sysd)
            setattr(s2, field, getattr(sysd, field) + sgn * H)
            vals.append(oracle_at(s2, rund, knots).hpsi(x))
        put(norb + q, vals)
    for k in range(nkn):
        vals = []
        for sgn in (1.0, -1.0):
            kn = np.array(knots, dtype=float)
            kn[k] += sgn * H
            orc.set_jastrow_spline(kn)
            vals.append(orc.hpsi(x))
        put(norb + nbeta + k, vals)
    return dl, de


def rel_err(a, ref):
    scale = np.maximum(np.abs(ref), 1e-3 * np.max(np.abs(ref), axis=1, keepdims=True))
    return float(np.max(np.abs(a - ref) / scale))


@pytest.mark.parametrize("name,nw,longrange,spline,same_spin", [("n14", 8, None, False, False),
                                                                ("p33_30", 4, None, False, False),
                                                                ("n66", 4, None, False, False),
                                                                ("n14", 6, LR, False, False),
                                                                ("n66", 4, None, True, False),
                                                                ("n14", 8, None, True, False),
                                                                ("p33_30", 4, None, True, False),
                                                                ("n66", 4, None, True, True),
                                                                ("n132", 2, None, True, False)])
def test_param_grad_against_oracle_fd(name, nw, longrange, spline, same_spin):
    sysd, rund, x = walkers(name, nw, longrange=longrange, same_spin=same_spin)
    knots = knots_for(5) if spline else None
    norb = int(sysd.norb)
    with capi.Context(sysd, rund) as ctx:
        if spline:
            ctx.set_jastrow_spline(knots)
            assert np.array_equal(ctx.jastrow_spline(), knots)
        dl, de = ctx.param_grad(x)
        assert dl.shape == (nw, norb + 3 + (16 if spline else 0)) == (nw, ctx.param_count())
        np.testing.assert_allclose(dl[:, :norb], ctx.getderbcs(x), rtol=1e-12, atol=1e-12)
    fl, fe = fd_oracle(sysd, rund, x, knots)
    el, ee = rel_err(dl, fl), rel_err(de, fe)
    print(f"{name} ({dl.shape[1]} parameters): d log Psi rel err {el:.2e}, d E_L rel err {ee:.2e} "
          f"(max |dE_L| {np.abs(fe).max():.3g})")
    assert el < TOL and ee < TOL


def test_param_grad_independent_of_precision():
    sysd, rund, x = walkers("n14", 6)
    with capi.Context(sysd, rund) as a, capi.Context(sysd, rund, precision="mixed") as b:
        ga, gb = a.param_grad(x), b.param_grad(x)
    assert np.array_equal(ga[0], gb[0]) and np.array_equal(ga[1], gb[1])


def test_param_grad_no_beta():
    sysd, rund, x = walkers("n14", 4)
    sysd.bfact = 0.0
    with capi.Context(sysd, rund) as ctx:
        assert ctx.param_count() == int(sysd.norb)
        dl, de = ctx.param_grad(x)
        with pytest.raises(capi.DMCError):
            ctx.set_beta(1.0, 5.0, 1.0)          # no beta function to change
    fl, fe = fd_oracle(sysd, rund, x)
    assert rel_err(dl, fl) < TOL and rel_err(de, fe) < TOL


def test_autograd_function_gradcheck():
    torch = pytest.importorskip("torch")
    sysd, rund, x = walkers("n14", 3)
    norb = int(sysd.norb)
    ctx = capi.Context(sysd, rund)

    class LocalEnergy(torch.autograd.Function):
        """E_L of the walkers at x as a function of vorb; backward = adjoint."""

        @staticmethod
        def forward(fctx, vorb):
            ctx.set_vorb(vorb.detach().cpu().numpy())
            h = ctx.hpsi(x)
            _, de = ctx.param_grad(x)
            fctx.save_for_backward(torch.from_numpy(de[:, :norb].copy()))
            return torch.from_numpy(eloc(h, sysd.hbar))

        @staticmethod
        def backward(fctx, gout):
            (de,) = fctx.saved_tensors
            return gout @ de

    v0 = torch.tensor(np.array(sysd.vorb[:norb]), dtype=torch.float64, requires_grad=True)
    ok = torch.autograd.gradcheck(LocalEnergy.apply, (v0,), eps=1e-6, atol=1e-7, rtol=1e-6)
    ctx.close()
    assert ok


def test_autograd_gradcheck_all_26_parameters():
    """The same autograd wrapper over theta = (vorb(1..7), bfact, b, d,
    16 knots) at N = 14 with 7 shells: forward moves every parameter on the
    context (set_vorb, set_beta, set_jastrow_spline)."""
    torch = pytest.importorskip("torch")
    sysd, rund, _ = configs.workload("n14", nwalk=3, seed=11)
    sysd.norb = 7
    sysd.vorb[:7] = (np.random.default_rng(3).uniform(0.2, 1.0, 7) * 0.5 ** np.arange(7)).tolist()
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    x = orc.walkers()["x"][:3] + np.random.default_rng(4).normal(scale=0.3, size=(3, 14, 3))
    ctx = capi.Context(sysd, rund)
    ctx.set_jastrow_spline(knots_for(9))
    assert ctx.param_count() == 26

    class LocalEnergy(torch.autograd.Function):
        @staticmethod
        def forward(fctx, theta):
            t = theta.detach().cpu().numpy()
            ctx.set_vorb(t[:7])
            ctx.set_beta(t[8], t[9], t[7])
            ctx.set_jastrow_spline(t[10:])
            h = ctx.hpsi(x)
            _, de = ctx.param_grad(x)
            fctx.save_for_backward(torch.from_numpy(de.copy()))
            return torch.from_numpy(eloc(h, sysd.hbar))

        @staticmethod
        def backward(fctx, gout):
            (de,) = fctx.saved_tensors
            return gout @ de

    theta = np.concatenate([np.array(sysd.vorb[:7]), [sysd.bfact, sysd.bbeta, sysd.dbeta], knots_for(9)])
    t0 = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
    ok = torch.autograd.gradcheck(LocalEnergy.apply, (t0,), eps=1e-6, atol=1e-6, rtol=1e-6)
    ctx.close()
    assert ok


def test_sr_step_over_adjoint_parameters():
    """dmc_sr_configure_adjoint: the SR sums are those of the adjoint
    d log Psi of the population in pop order, and dmc_sr_update moves vorb,
    beta and the knots by the returned step (optimizer.f90:118-169)."""
    sysd, rund, _ = configs.workload("n14", nwalk=64, idmc=0)
    with capi.Context(sysd, rund) as ctx:
        ctx.set_jastrow_spline(knots_for(2))
        ctx.init_walkers()
        ctx.initial_eval()
        ctx.generation(False)
        ctx.sr_configure_adjoint()
        w = ctx.walkers()
        x_pop = w["x"][::-1].copy()                 # pop order: top of the stack first
        e_pop = ((-sysd.hbar * w["d2psi"] + w["v"]) / ctx.info.eunit / ctx.npart)[::-1]
        dl, _ = ctx.param_grad(x_pop)
        n = ctx.sr_accumulate()
        assert n == 64
        sums = ctx.sr_sums()
        np_ = ctx.param_count()
        assert np_ == int(sysd.norb) + 3 + 16 and sums["ovec"].size == np_ and sums["n"] == 64
        np.testing.assert_allclose(sums["ovec"], dl.sum(0), rtol=1e-10, atol=1e-12)
        np.testing.assert_allclose(sums["ovecw"], (dl * e_pop[:, None]).sum(0), rtol=1e-10, atol=1e-12)
        np.testing.assert_allclose(sums["pmat"], dl.T @ dl, rtol=1e-10, atol=1e-12)
        before = np.concatenate([np.array(sysd.vorb[:int(sysd.norb)]), [sysd.bfact, sysd.bbeta, sysd.dbeta],
                                 ctx.jastrow_spline()])
        step, _, _ = ctx.sr_update(0.02, 1e-3)
        after = np.concatenate([ctx.table(10), ctx.beta_params(), ctx.jastrow_spline()])
        np.testing.assert_allclose(after, before + step, rtol=1e-14, atol=1e-15)
