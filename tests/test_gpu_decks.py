"""GPU parity on the reference's own production decks, and the free Fermi gas.

The two decks the reference ships (parsed into ``tests/golden/decks.json`` by
``tests/golden/make_decks.py``):

* ``dmcbcs.dat``: N = 66 (33/33) DMC, 10 s-wave shells with the fitted
  amplitudes of the deck (K = 147 pair-orbital columns), dt = 5e-5,
  beta b = 0.5, d = 5, bfact = 1;
* ``input.dat``: N = 17 (9 up / 8 down, one unpaired up plane wave at
  k = 0), 10 shells with large mixed-sign amplitudes, equal-spin Jastrow
  on, VMC optimisation run (idmc = -1) with the drift cut off at 0 (zero
  drift, step.f90:32-37).

Bars: FP64 path within 1e-10 of the oracle (relative, as in
test_gpu_parity.py), inverse within 1e-9; mixed path within 1e-6 (local
energy, Laplacian, drift) and 1e-6 absolute in log|Psi|.  Generations:
identical random streams, populations and signs, positions within 1e-10
(FP64) and 1e-7 (mixed, which follows the FP64 trajectories).

The free Fermi gas (v0 = 0, no Jastrow, no beta, phi = the seven lowest
plane waves of a 7/7 closed shell) has the constant local energy
E_free = 2 sum_k |k|^2 / 2 on every configuration; both precisions must
give it to 1e-10 (FP64) and 1e-9 (mixed).
"""
import json
import os

import numpy as np
import pytest

import oracle
from dmcbcs_project_gb300 import abi, capi, configs

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
DECKS = json.load(open(os.path.join(HERE, "golden", "decks.json")))
TOL = 1e-10
MIX = 1e-6


def deck(name, nwalk, idmc=None):
    d = DECKS[name]
    r = dict(d["run"])
    r["nwalk"] = nwalk
    if idmc is not None:
        r["idmc"] = idmc
    return abi.make_system(d["system"]), abi.make_run(r)


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1.0)) if a.size else 0.0


def rel_each(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)))


def configurations(sysd, rund, nw, seed):
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    x = orc.walkers()["x"][:nw] + np.random.default_rng(seed).normal(scale=0.3, size=(nw, orc.npart, 3))
    return orc, x


def local_energy(h, hbar):
    return -hbar * h["d2psi"] + h["v"]


@pytest.mark.parametrize("name,nw", [("dmcbcs.dat", 48), ("input.dat", 96)])
def test_deck_hpsi_and_bcs_fp64(name, nw):
    sysd, rund = deck(name, nw)
    orc, x = configurations(sysd, rund, nw, 31)
    ref = orc.hpsi(x)
    refb = orc.bcs(x, want_inverse=True)
    with capi.Context(sysd, rund) as ctx:
        assert ctx.info.ncol == 147          # 10 shells: 74 k vectors
        got = ctx.hpsi(x)
        gotb = ctx.bcs(x, want_inverse=True)
    assert np.array_equal(got["is_"], ref["is_"])
    for k in ("psil", "d2psi", "v", "psigl", "d2psig"):
        assert rel_each(got[k], ref[k]) < TOL, k
    assert rel_each(local_energy(got, sysd.hbar), local_energy(ref, sysd.hbar)) < TOL
    for w in range(nw):
        assert rel(got["dpsi"][w], ref["dpsi"][w]) < TOL, w
    assert np.array_equal(gotb["is_"], refb["is_"])
    assert rel_each(gotb["phil"], refb["phil"]) < TOL
    assert rel_each(gotb["d2phi"], refb["d2phi"]) < TOL
    for w in range(nw):
        assert rel(gotb["dphi"][w], refb["dphi"][w]) < TOL
        assert rel(gotb["smati"][w], refb["smati"][w]) < 1e-9


@pytest.mark.parametrize("name,nw", [("dmcbcs.dat", 64), ("input.dat", 96)])
def test_deck_hpsi_mixed(name, nw):
    sysd, rund = deck(name, nw)
    orc, x = configurations(sysd, rund, nw, 37)
    ref = orc.hpsi(x)
    with capi.Context(sysd, rund, precision="mixed") as ctx:
        got = ctx.hpsi(x)
    el_r = local_energy(ref, sysd.hbar)
    el_err = np.abs(local_energy(got, sysd.hbar) - el_r) / np.maximum(np.abs(el_r), 1.0)
    lap_err = np.abs(got["d2psi"] - ref["d2psi"]) / np.maximum(np.abs(ref["d2psi"]), 1.0)
    dr_err = max(rel(got["dpsi"][w], ref["dpsi"][w]) for w in range(nw))
    psil_err = np.max(np.abs(got["psil"] - ref["psil"]))
    print(f"{name} mixed: E_L {el_err.max():.2e}, d2psi {lap_err.max():.2e}, drift {dr_err:.2e}, "
          f"log|Psi| {psil_err:.2e}")
    assert np.array_equal(got["is_"], ref["is_"])
    assert el_err.max() < MIX and lap_err.max() < MIX and dr_err < MIX and psil_err < MIX


@pytest.mark.parametrize("name,nw,gens,prec", [("dmcbcs.dat", 48, 4, "fp64"), ("dmcbcs.dat", 48, 4, "mixed"),
                                               ("input.dat", 64, 4, "fp64"), ("input.dat", 64, 4, "mixed")])
def test_deck_generations(name, nw, gens, prec):
    """Generations of the deck's own run type (DMC for dmcbcs.dat, the VMC
    steps of the optimisation run for input.dat) against the oracle."""
    sysd, rund = deck(name, nw)
    orc = oracle.Oracle(sysd, rund)
    tol_x = 1e-10 if prec == "fp64" else 1e-7
    tol = TOL if prec == "fp64" else MIX
    with capi.Context(sysd, rund, precision=prec) as ctx:
        ctx.init_walkers()
        orc.init_walkers()
        sg, _ = ctx.initial_eval()
        so, _ = orc.initial_eval()
        assert rel_each(sg, so) < (1e-9 if prec == "fp64" else MIX)
        for g in range(gens):
            op = g == gens - 1
            assert ctx.generation(op) == orc.generation(op), g
        wg, wo = ctx.walkers(), orc.walkers()
        assert np.array_equal(wg["irn"], wo["irn"])
        assert np.array_equal(wg["is_"], wo["is_"])
        assert rel(wg["x"], wo["x"]) < tol_x
        for k in ("psil", "d2psi", "v", "weight"):
            assert rel_each(wg[k], wo[k]) < tol, k
        assert rel_each(ctx.estimators()[0], orc.estimators()[0]) < (1e-9 if prec == "fp64" else MIX)


def free_gas(nwalk=8):
    sp = configs.system_params(7, 7, 2)
    sp.update(vorb=[1.0, 1.0], bfact=0.0, cjas=[0.0, 0.0], v0=0.0)
    return abi.make_system(sp), abi.make_run(configs.run_params(nwalk, 0.002))


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("mixed", 1e-9)])
def test_free_fermi_gas_known_answer(prec, tol):
    """Closed-shell free Fermi gas: E_L = E_free exactly on any configuration
    (the BCS determinant factors into two Slater determinants of the seven
    lowest plane waves), and the local energy has no variance."""
    sysd, rund = free_gas()
    with capi.Context(sysd, rund, precision=prec) as ctx:
        el = ctx.info.el
        x = np.random.default_rng(3).uniform(-0.5, 0.5, size=(64, 14, 3)) * el
        h = ctx.hpsi(x)
    k2 = (2 * np.pi / el) ** 2
    e_free = 2 * 0.5 * 6 * k2
    e_l = local_energy(h, sysd.hbar)
    print(f"{prec}: max |E_L / E_free - 1| = {np.max(np.abs(e_l / e_free - 1)):.2e}")
    assert np.all(h["v"] == 0.0)
    assert np.allclose(e_l, e_free, rtol=tol, atol=0.0)
