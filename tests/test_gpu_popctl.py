"""Population control (dmcbcs.f90:441-448): when the walker count leaves
[popdn, popup] * nwalk after branching, a second branch with factor
nwalk / nt brings it back.  Here the population starts at twice and at half
the target, so the control acts in the first generation (conditional pass on
the device); counts, random streams, weights and estimators must equal the
oracle's exactly or to 1e-10."""
import numpy as np
import pytest

import oracle
from dmcbcs_project_gb300 import capi, configs

pytestmark = pytest.mark.gpu


def rel_each(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)))


@pytest.mark.parametrize("ratio", [2.0, 0.5])
@pytest.mark.parametrize("idmc", [1, -2])
def test_population_control_acts(ratio, idmc):
    target = 32
    sysd, rund, _ = configs.workload("n14", nwalk=target, idmc=idmc)
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    w0 = orc.walkers()
    n0 = int(target * ratio)
    reps = -(-n0 // w0["n"])
    x = np.concatenate([w0["x"]] * reps)[:n0] + np.random.default_rng(9).normal(scale=0.2, size=(n0, orc.npart, 3))
    irn = (np.arange(n0, dtype=np.int64) * 2654435761 + 12345) & ((1 << 48) - 1)
    with capi.Context(sysd, rund) as ctx:
        ctx.load_walkers(x, irn)
        orc.load_walkers(x, irn=irn)
        ctx.initial_eval()
        orc.initial_eval()
        counts = []
        for g in range(3):
            ng, no = ctx.generation(g == 2), orc.generation(g == 2)
            assert ng == no, (g, ng, no)
            counts.append(ng)
        wg, wo = ctx.walkers(), orc.walkers()
        eg = ctx.estimators()
        eo = orc.estimators()
    # the first generation was brought back into the band around the target
    assert 0.9 * target <= counts[0] <= 1.1 * target or abs(counts[0] - target) <= 3, counts
    assert np.array_equal(wg["irn"], wo["irn"])
    for k in ("psil", "d2psi", "v", "weight"):
        assert rel_each(wg[k], wo[k]) < 1e-10, k
    for a, b in zip(eg, eo):
        assert rel_each(a, b) < 1e-9


@pytest.mark.parametrize("weights", ["one_heavy", "spread"])
def test_branch_many_copies_of_one_walker(weights):
    """dmc_branch with walker weights far from one: one walker carrying
    almost the whole population (hundreds of copies, spread over many warps
    of the scatter) or weights spread over [0, 12); copies, their order and
    each copy's ran2-advanced stream against the oracle's branch."""
    sysd, rund, _ = configs.workload("n14", nwalk=40, idmc=1)
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    w0 = orc.walkers()
    n0 = w0["n"]
    rng = np.random.default_rng(21)
    wt = np.full(n0, 0.3) if weights == "one_heavy" else rng.uniform(0.0, 12.0, n0)
    if weights == "one_heavy":
        wt[7] = 311.6
    irn = (np.arange(n0, dtype=np.int64) * 2654435761 + 99991) & ((1 << 48) - 1)
    with capi.Context(sysd, rund) as ctx:
        ctx.load_walkers(w0["x"], irn, weight=wt)
        orc.load_walkers(w0["x"], weight=wt, irn=irn)
        ctx.branch(1.0)
        orc.branch(1.0)
        assert ctx.num_walkers() == orc.num_walkers()
        wg, wo = ctx.walkers(), orc.walkers()
        hg, ho = ctx.wtisto(), orc.wtisto()
    print(f"{weights}: {wg['n']} walkers after branching")
    assert wg["n"] > (300 if weights == "one_heavy" else n0)
    assert np.array_equal(wg["irn"], wo["irn"])
    assert np.array_equal(wg["x"], wo["x"])
    assert np.array_equal(wg["weight"], wo["weight"])
    assert np.array_equal(hg, ho)
