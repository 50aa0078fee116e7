"""Adjoint parameter gradients (dmc_param_grad) for theta = (vorb(1..norb),
bfact): d log|Psi| / d theta and d E_L / d theta per walker, E_L =
-hbar d2psi + v.

Checks:
  - the vorb part of d log|Psi| equals getderbcs (psislaterbcs.f90:449-524),
    which the single-walker parity tests hold to the oracle;
  - both gradients against central finite differences of the ORACLE's hpsi
    with the parameter moved up and down (vorb through set_vorb, bfact
    through tables rebuilt at bfact +- h), extrapolated from h = 1e-5 and
    h/2 as chkderp does (optimizer.f90:171-225): plain central differences
    at h = 1e-5 carry an O(h^2) error of ~5e-6 relative for the small
    high-shell amplitudes of the polarised system; relative error
    <= 1e-6 of max(|FD|, 1e-3 * max over theta of |FD|);
  - a torch.autograd.Function whose forward is the GPU local energy at
    vorb and whose backward is the adjoint passes torch.autograd.gradcheck
    (finite differences of the forward, float64).
Systems: 7/7, polarised 33/30 (unpaired columns enter M but not S'), 33/33,
and 7/7 with the long-range Jastrow on (its gradient enters w)."""
import numpy as np
import pytest

import oracle
from dmcbcs_project_gb300 import capi, configs

pytestmark = pytest.mark.gpu

H = 1e-5
TOL = 1e-6
LR = (3, 1.0, 0.3)


def walkers(name, nw, seed=11, longrange=None):
    sysd, rund, _ = configs.workload(name, nwalk=nw, seed=seed, longrange=longrange)
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    x = orc.walkers()["x"][:nw].copy()
    x += np.random.default_rng(seed).normal(scale=0.3, size=x.shape)
    return sysd, rund, x


def eloc(h, hbar):
    return -hbar * h["d2psi"] + h["v"]


def fd_oracle(sysd, rund, x):
    """Extrapolated central differences (4 D(h/2) - D(h)) / 3 of log|Psi|
    and E_L over theta with the oracle."""
    l1, e1 = fd_central(sysd, rund, x, H)
    l2, e2 = fd_central(sysd, rund, x, H / 2)
    return (4 * l2 - l1) / 3, (4 * e2 - e1) / 3


def fd_central(sysd, rund, x, H):
    norb = int(sysd.norb)
    vorb = np.array(sysd.vorb[:norb], dtype=float)
    np_ = norb + (1 if sysd.bfact != 0.0 else 0)
    dl = np.zeros((x.shape[0], np_))
    de = np.zeros((x.shape[0], np_))
    orc = oracle.Oracle(sysd, rund)
    for t in range(norb):
        vals = []
        for sgn in (1.0, -1.0):
            v = vorb.copy()
            v[t] += sgn * H
            orc.set_vorb(v)
            vals.append(orc.hpsi(x))
        dl[:, t] = (vals[0]["psil"] - vals[1]["psil"]) / (2 * H)
        de[:, t] = (eloc(vals[0], sysd.hbar) - eloc(vals[1], sysd.hbar)) / (2 * H)
    if np_ > norb:
        vals = []
        for sgn in (1.0, -1.0):
            s2 = type(sysd).from_buffer_copy(sysd)
            s2.bfact = sysd.bfact + sgn * H
            vals.append(oracle.Oracle(s2, rund).hpsi(x))
        dl[:, norb] = (vals[0]["psil"] - vals[1]["psil"]) / (2 * H)
        de[:, norb] = (eloc(vals[0], sysd.hbar) - eloc(vals[1], sysd.hbar)) / (2 * H)
    return dl, de


def rel_err(a, ref):
    scale = np.maximum(np.abs(ref), 1e-3 * np.max(np.abs(ref), axis=1, keepdims=True))
    return float(np.max(np.abs(a - ref) / scale))


@pytest.mark.parametrize("name,nw,longrange", [("n14", 8, None), ("p33_30", 4, None), ("n66", 4, None),
                                               ("n14", 6, LR)])
def test_param_grad_against_oracle_fd(name, nw, longrange):
    sysd, rund, x = walkers(name, nw, longrange=longrange)
    with capi.Context(sysd, rund) as ctx:
        dl, de = ctx.param_grad(x)
        assert dl.shape == (nw, int(sysd.norb) + 1)
        np.testing.assert_allclose(dl[:, :int(sysd.norb)], ctx.getderbcs(x), rtol=1e-12, atol=1e-12)
    fl, fe = fd_oracle(sysd, rund, x)
    el, ee = rel_err(dl, fl), rel_err(de, fe)
    print(f"{name}: d log Psi rel err {el:.2e}, d E_L rel err {ee:.2e} (max |dE_L| {np.abs(fe).max():.3g})")
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
