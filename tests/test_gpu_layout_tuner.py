"""dmc_tune_layout: the walker layout chosen by timing (the layout dmc_create
picks, on chip with 256 threads throughout, or the union region in a global
slice per CTA).

Every layout runs the same FP64 arithmetic (the FP64 kernel always has 256
threads and the layouts differ only in where the data live), so an FP64
context keeps its results bit for bit whatever the tuner picks; the mixed
kernel's 16-warp CTA sums in another order, so a mixed context is held to
the oracle's bars instead.  A batch holding a tuned context follows the
change (its captured generations are dropped, its CTA split clamped).
"""
import numpy as np
import pytest

import oracle
from dmcbcs_project_gb300 import capi, configs

pytestmark = pytest.mark.gpu

FIELDS = ("x", "irn", "is_", "weight", "psil", "d2psi", "v")


def rel_each(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)))


@pytest.mark.parametrize("name,nw", [("n66", 512), ("p38_33", 256), ("n132", 304)])
def test_tuned_fp64_context_is_bit_identical(name, nw):
    sysd, rund, _ = configs.workload(name, nwalk=nw)
    with capi.Context(sysd, rund) as a, capi.Context(sysd, rund) as b:
        for c in (a, b):
            c.init_walkers()
            c.initial_eval()
        kind, ms = a.tune_layout(2)
        print(f"{name}: layout {kind}, {ms:.3f} ms per evaluation of {nw} walkers")
        assert kind in (0, 1, 2) and ms > 0
        for g in range(3):
            assert a.generation(g == 2) == b.generation(g == 2)
        wa, wb = a.walkers(), b.walkers()
        for k in FIELDS:
            assert np.array_equal(wa[k], wb[k]), k
        for ea, eb in zip(a.estimators(), b.estimators()):
            assert np.array_equal(ea, eb)


def test_tuned_mixed_context_against_oracle():
    sysd, rund, _ = configs.workload("n132", nwalk=16)
    orc = oracle.Oracle(sysd, rund)
    with capi.Context(sysd, rund, precision="mixed") as ctx:
        ctx.init_walkers()
        orc.init_walkers()
        ctx.initial_eval()
        orc.initial_eval()
        kind, _ = ctx.tune_layout(2)
        for g in range(2):
            assert ctx.generation(g == 1) == orc.generation(g == 1)
        wg, wo = ctx.walkers(), orc.walkers()
    print(f"n132 mixed: layout {kind}")
    assert np.array_equal(wg["irn"], wo["irn"])
    assert float(np.max(np.abs(wg["x"] - wo["x"]))) < 1e-7
    assert rel_each(-sysd.hbar * wg["d2psi"] + wg["v"], -sysd.hbar * wo["d2psi"] + wo["v"]) < 1e-6


def test_batch_follows_a_retuned_system():
    systems = [("n14", 64), ("n132", 32)]
    ctxs = []
    for i, (name, nw) in enumerate(systems):
        sysd, rund, _ = configs.workload(name, nwalk=nw, seed=77 + i)
        ctxs.append(capi.Context(sysd, rund))
        ctxs[-1].init_walkers()
        ctxs[-1].initial_eval()
    singles = []
    for i, (name, nw) in enumerate(systems):
        sysd, rund, _ = configs.workload(name, nwalk=nw, seed=77 + i)
        singles.append(capi.Context(sysd, rund))
        singles[-1].init_walkers()
        singles[-1].initial_eval()
    try:
        with capi.Batch(ctxs) as b:
            b.generations(1, opcomp_last=False)           # graphs captured with the first layouts
            for c in singles:
                c.generation(False)
            # force the other layouts by tuning each system, then go on
            for c in ctxs:
                c.tune_layout(1)
            b.generations(2, opcomp_last=True)
            for g in range(2):
                for c in singles:
                    c.generation(g == 1)
        for a, s in zip(ctxs, singles):
            wa, ws = a.walkers(), s.walkers()
            for k in FIELDS:
                assert np.array_equal(wa[k], ws[k]), k
    finally:
        for c in ctxs + singles:
            c.close()


def test_tune_arguments_and_empty_population():
    from dmcbcs_project_gb300 import abi

    sysd, rund, _ = configs.workload("n14", nwalk=8)
    with capi.Context(sysd, rund) as ctx:
        with pytest.raises(capi.DMCError) as e:
            ctx.tune_layout(0)
        assert e.value.status == abi.DMC_ERR_INVALID
        with pytest.raises(capi.DMCError) as e:
            ctx.tune_layout(1)                        # no walkers yet
        assert e.value.status == abi.DMC_ERR_EMPTY
