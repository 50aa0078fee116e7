"""Batches of systems of uneven size (dmc_batch_*): six systems of the
uneven-batch family (7/7, 19/19, 33/33, 33/30, 38/33, 66/66) advanced by
batched generations, one CUDA graph per generation.  Each system's walkers,
random streams, weights, populations, estimators and multiplicity histogram
must be identical, bit for bit, to the same context advanced alone by
dmc_generation (which the generation parity tests hold to the oracle), for
any CTA split: the planner's, a tuned one and one CTA per system.  The
smallest system is also checked against the oracle directly."""
import numpy as np
import pytest

import oracle
from dmcbcs_project_gb300 import capi, configs

pytestmark = pytest.mark.gpu

SYSTEMS = [("n14", 24), ("n38", 12), ("n66", 12), ("p33_30", 10), ("p38_33", 10), ("n132", 6)]
FIELDS = ("x", "irn", "is_", "weight", "psil", "psigl", "d2psi", "d2psig", "v", "wt0")


def make(idmc, precision, systems=SYSTEMS):
    out = []
    for i, (name, nw) in enumerate(systems):
        sysd, rund, _ = configs.workload(name, nwalk=nw, idmc=idmc, seed=1234 + i)
        ctx = capi.Context(sysd, rund, precision)
        ctx.init_walkers()
        ctx.initial_eval()
        out.append(ctx)
    return out


def assert_same(a, b, label):
    wa, wb = a.walkers(), b.walkers()
    assert wa["n"] == wb["n"], label
    for k in FIELDS:
        assert np.array_equal(wa[k], wb[k]), (label, k)
    for ea, eb in zip(a.estimators(), b.estimators()):
        assert np.array_equal(ea, eb), label
    assert np.array_equal(a.wtisto(), b.wtisto()), label


@pytest.mark.parametrize("idmc,precision,split", [(1, "fp64", "plan"), (0, "fp64", "ones"), (1, "mixed", "tuned"),
                                                  (2, "fp64", "plan"), (10, "fp64", "plan")])
def test_batch_matches_single(idmc, precision, split):
    gens = 5
    A, B = make(idmc, precision), make(idmc, precision)
    expect_steps = 0
    with capi.Batch(A) as b:
        if split == "ones":
            b.grids = [1] * len(A)
        elif split == "tuned":
            grids, ms = b.tune(2)
            assert ms > 0 and np.array_equal(grids, b.grids)
        # populations entering each generation, from the single-context runs
        pops = []
        for g in range(gens):
            pops.append(sum(ctx.num_walkers() for ctx in B))
            for ctx in B:
                ctx.generation(g == gens - 1)
        expect_steps = sum(pops)
        # two calls: graphs captured by the first are replayed by the second
        s1, ms1, nl1 = b.generations(gens - 2, opcomp_last=False)
        s2, ms2, nl2 = b.generations(2, opcomp_last=True)
        assert s1 + s2 == expect_steps
        assert nl1 > 0 and nl2 > 0 and ms1 > 0 and ms2 > 0
    for i, (a, bb) in enumerate(zip(A, B)):
        assert_same(a, bb, SYSTEMS[i][0])
    for ctx in A + B:
        ctx.close()


def test_batch_against_oracle():
    """The 7/7 system of a batch against the oracle's generations."""
    gens = 4
    A = make(1, "fp64")
    sysd, rund, _ = configs.workload("n14", nwalk=SYSTEMS[0][1], idmc=1, seed=1234)
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    orc.initial_eval()
    for g in range(gens):
        orc.generation(g == gens - 1)
    with capi.Batch(A) as b:
        b.generations(gens, opcomp_last=True)
    wg, wo = A[0].walkers(), orc.walkers()
    assert np.array_equal(wg["irn"], wo["irn"])
    assert np.array_equal(wg["is_"], wo["is_"])
    assert float(np.max(np.abs(wg["x"] - wo["x"]))) < 1e-9
    for k in ("psil", "d2psi", "v", "weight"):
        ref = np.asarray(wo[k], float)
        assert float(np.max(np.abs(wg[k] - ref) / np.maximum(np.abs(ref), 1.0))) < 1e-10, k
    vb_g, _, wb_g = A[0].estimators()
    vb_o, _, wb_o = orc.estimators()
    assert float(np.max(np.abs(vb_g - vb_o) / np.maximum(np.abs(vb_o), 1.0))) < 1e-9
    for ctx in A:
        ctx.close()


def test_batch_rejects_bad_grids():
    A = make(1, "fp64", SYSTEMS[:2])
    with capi.Batch(A) as b:
        g = b.grids
        assert g.min() >= 1
        with pytest.raises(capi.DMCError):
            b.grids = [0, 1]
        with pytest.raises(capi.DMCError):
            b.grids = [1, 100000]
        assert np.array_equal(b.grids, g)
    with pytest.raises(capi.DMCError):
        capi.Batch([A[0], A[0]])
    for ctx in A:
        ctx.close()
