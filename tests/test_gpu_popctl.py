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
