"""Failure detection: per-walker status flags, faults made on the host.

Every failure here is made in the inputs on the host; no kernel is made to
fault, trap or wait forever.

* Two up particles at the same position make two rows of the pair matrix
  equal: the matrix is singular, log|det| takes the reference's sentinel
  (matrixlapack.f90:19-25) and the drift is zero (psislaterbcs.f90:210).
  The walker gets DMC_STATUS_SINGULAR; the other walkers of the batch are
  unaffected and still equal the oracle's values.
* A walker with NaN coordinates gets DMC_STATUS_NONFINITE; the others are
  unaffected and the context stays usable.
* A population pushed past the stack capacity (stack.f90:88-91) returns
  DMC_ERR_OVERFLOW with the count at the capacity, and DMC_STATUS_OVERFLOW.
* A NaN walker inside a DMC generation gets weight 0 and no estimator
  record, so branching drops it, and sets DMC_STATUS_NONFINITE; the rest of
  the population carries on with finite estimators.
"""
import numpy as np
import pytest

import oracle
from dmcbcs_project_gb300 import abi, capi, configs

pytestmark = pytest.mark.gpu


def setup(name, nw, seed=5):
    sysd, rund, _ = configs.workload(name, nwalk=nw, seed=seed)
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    x = orc.walkers()["x"][:nw] + np.random.default_rng(seed).normal(scale=0.3, size=(nw, orc.npart, 3))
    return sysd, rund, orc, x


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_coincident_up_particles_flag_singular(prec):
    sysd, rund, orc, x = setup("n14", 16)
    x[3, 1] = x[3, 0]          # walker 3: up particles 0 and 1 at one point
    ref = orc.hpsi(x)
    with capi.Context(sysd, rund, precision=prec) as ctx:
        ctx.status(clear=True)
        got = ctx.hpsi(x)
        ws = ctx.walker_status(16)
        flags = ctx.status()
        b = ctx.bcs(x)
    assert ws[3] & abi.DMC_STATUS_SINGULAR
    assert np.all(ws[np.arange(16) != 3] == 0)
    assert flags & abi.DMC_STATUS_SINGULAR and not flags & abi.DMC_STATUS_NONFINITE
    assert b["phil"][3] == abi.DMC_MINUSHUGE
    assert np.all(b["dphi"][3] == 0.0)
    assert ref["psil"][3] < -1e29 and got["psil"][3] < -1e29
    ok = np.arange(16) != 3
    tol = 1e-10 if prec == "fp64" else 1e-6
    assert np.max(np.abs(got["psil"][ok] - ref["psil"][ok])) < tol
    el_g = -sysd.hbar * got["d2psi"][ok] + got["v"][ok]
    el_r = -sysd.hbar * ref["d2psi"][ok] + ref["v"][ok]
    assert np.max(np.abs(el_g - el_r) / np.maximum(np.abs(el_r), 1.0)) < tol


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_nan_coordinates_flag_nonfinite(prec):
    sysd, rund, orc, x = setup("n66", 8)
    bad = x.copy()
    bad[5, 10, 1] = np.nan
    ref = orc.hpsi(x)
    with capi.Context(sysd, rund, precision=prec) as ctx:
        got = ctx.hpsi(bad)
        ws = ctx.walker_status(8)
        assert ctx.status(clear=True) & abi.DMC_STATUS_NONFINITE
        assert ctx.status() == 0
        # the context is still usable, and the walkers without NaN are exact
        again = ctx.hpsi(x)
        assert np.all(ctx.walker_status(8) == 0)
    assert ws[5] & abi.DMC_STATUS_NONFINITE
    assert np.all(ws[np.arange(8) != 5] == 0)
    tol = 1e-10 if prec == "fp64" else 1e-6
    ok = np.arange(8) != 5
    assert np.max(np.abs(got["psil"][ok] - ref["psil"][ok])) < tol
    assert np.max(np.abs(again["psil"] - ref["psil"])) < tol
    with pytest.raises(capi.DMCError):
        ctx_n = capi.Context(sysd, rund)
        try:
            ctx_n.walker_status(1)      # no batched evaluation yet
        finally:
            ctx_n.close()


def test_population_past_capacity_overflows():
    sysd, rund, _ = configs.workload("n14", nwalk=64)
    rund.stmax = 1.5                    # capacity 96 walkers
    with capi.Context(sysd, rund) as ctx:
        ctx.init_walkers()
        ctx.initial_eval()
        cap = ctx.info.capacity
        assert cap == 96
        with pytest.raises(capi.DMCError) as ei:
            ctx.branch(3.0)             # about 3 x 64 copies
        assert ei.value.status == abi.DMC_ERR_OVERFLOW
        assert ctx.num_walkers() == cap
        assert ctx.status(clear=True) & abi.DMC_STATUS_OVERFLOW
        w = ctx.walkers()
        assert np.all(np.isfinite(w["x"])) and np.all(w["irn"] > 0)
        ctx.step(False)                 # the context carries on from the kept copies
        assert ctx.num_walkers() == cap


def test_nan_walker_in_a_generation_is_dropped():
    sysd, rund, _ = configs.workload("n14", nwalk=32)
    with capi.Context(sysd, rund) as ctx:
        ctx.init_walkers()
        w = ctx.walkers()
    x = w["x"].copy()
    x[7, 2, 0] = np.nan
    with capi.Context(sysd, rund) as ctx:
        ctx.load_walkers(x, w["irn"])
        ctx.initial_eval()
        ctx.status(clear=True)
        n0 = ctx.num_walkers()
        n1 = ctx.generation(True)
        flags = ctx.status()
        wn = ctx.walkers()
        vb, _, wb = ctx.estimators()
    assert flags & abi.DMC_STATUS_NONFINITE
    assert n0 == 32 and n1 > 0
    assert np.all(np.isfinite(wn["x"])) and np.all(np.isfinite(wn["weight"]))
    assert np.all(np.isfinite(vb)) and np.all(np.isfinite(wb))
