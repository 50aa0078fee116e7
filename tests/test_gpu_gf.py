"""idmc = 10 on the GPU (step.f90:231-279: DMC without drift, direct sampling
of the Green's function with importance sampling) against the oracle.

Each move evaluates the wavefunction at x + sigma g and x - sigma g, keeps
one of the two with one more uniform from the walker's stream and weights
it by 0.5 (wt1 + wt2) exp(etrial dt).  Bars as for the other run types:
FP64 within 1e-10 of the oracle with identical random streams, populations,
signs and histogram of copies; the mixed path follows the FP64 trajectories
(positions within 1e-7, local energies within 1e-6).  The 512-thread mixed
kernel (one CTA per SM, N = 132) and graph replay run the same move (the
host-buffer and batched entry points are covered with the other run types).
"""
import numpy as np
import pytest

import oracle
from dmcbcs_project_gb300 import capi, configs

pytestmark = pytest.mark.gpu

TOL = 1e-10
MIX = 1e-6


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1.0)) if a.size else 0.0


def rel_each(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0))) if a.size else 0.0


def start(ctx, orc):
    ctx.init_walkers()
    orc.init_walkers()
    sg, eg = ctx.initial_eval()
    so, eo = orc.initial_eval()
    return sg, eg, so, eo


@pytest.mark.parametrize("name,nw,gens,prec", [("n14", 48, 5, "fp64"), ("n66", 32, 3, "fp64"),
                                               ("p33_30", 16, 3, "fp64"), ("n14", 48, 5, "mixed"),
                                               ("n66", 32, 3, "mixed"), ("n132", 6, 2, "mixed")])
def test_gf_generations_against_oracle(name, nw, gens, prec):
    sysd, rund, _ = configs.workload(name, nwalk=nw, idmc=10)
    orc = oracle.Oracle(sysd, rund)
    tol = TOL if prec == "fp64" else MIX
    with capi.Context(sysd, rund, precision=prec) as ctx:
        assert ctx.info.nest == 14
        sg, eg, so, eo = start(ctx, orc)
        assert rel_each(sg, so) < (1e-9 if prec == "fp64" else MIX)
        assert rel_each(eg, eo) < (1e-9 if prec == "fp64" else MIX)
        counts = []
        for g in range(gens):
            op = g == gens - 1
            ng, no = ctx.generation(op), orc.generation(op)
            assert ng == no, (g, ng, no)
            counts.append(ng)
        wg, wo = ctx.walkers(), orc.walkers()
        assert np.array_equal(wg["irn"], wo["irn"])
        assert np.array_equal(wg["is_"], wo["is_"])
        assert rel(wg["x"], wo["x"]) < (1e-10 if prec == "fp64" else 1e-7)
        for k in ("psil", "psigl", "d2psi", "d2psig", "v", "weight"):
            assert rel_each(wg[k], wo[k]) < tol, k
        for w in range(wg["n"]):
            assert rel(wg["dpsi"][w], wo["dpsi"][w]) < tol
        vb_g, vb2_g, wb_g = ctx.estimators()
        vb_o, vb2_o, wb_o = orc.estimators()
        print(f"{name} {prec}: populations {counts}, estimator rel err {rel_each(vb_g, vb_o):.2e}")
        assert rel_each(vb_g, vb_o) < (1e-9 if prec == "fp64" else MIX)
        assert rel_each(wb_g, wb_o) < (1e-9 if prec == "fp64" else MIX)
        assert np.array_equal(ctx.wtisto(), orc.wtisto())


def test_gf_moves_are_unwrapped_two_point_proposals():
    """The pushed walker sits at x_old +- sigma g with x_old wrapped into the
    box and the proposal itself not wrapped (step.f90:236-242), and both
    signs occur."""
    sysd, rund, _ = configs.workload("n14", nwalk=64, idmc=10)
    with capi.Context(sysd, rund) as ctx:
        ctx.init_walkers()
        ctx.initial_eval()
        before = ctx.walkers()
        ctx.step(False)
        after = ctx.walkers()
    el = ctx.info.el
    sig = np.array([ctx.info.sigma[0]] * ctx.info.nup + [ctx.info.sigma[1]] * ctx.info.ndn)
    n, npart = before["n"], sysd.nbin[0] + sysd.nbin[1]
    signs = set()
    outside = 0
    for k in range(n):
        src = n - 1 - k
        x1 = before["x"][src] - el * np.sign(before["x"][src]) * np.floor(np.abs(before["x"][src] / el) + 0.5)
        g, s = oracle.gaussian(int(before["irn"][src]) & ((1 << 48) - 1), 3 * npart)
        _, s = oracle.ran1(s)
        dx = sig[:, None] * g.reshape(npart, 3)
        d_plus = np.max(np.abs(after["x"][k] - (x1 + dx)))
        d_minus = np.max(np.abs(after["x"][k] - (x1 - dx)))
        assert min(d_plus, d_minus) < 1e-13
        signs.add(d_plus < d_minus)
        assert after["irn"][k] == s
        outside += int(np.any(np.abs(after["x"][k]) > 0.5 * el))
    assert signs == {True, False}
    assert outside > 0          # some proposals left the box unwrapped


def test_gf_step_and_branch_calls():
    sysd, rund, _ = configs.workload("n14", nwalk=40, idmc=10)
    orc = oracle.Oracle(sysd, rund)
    with capi.Context(sysd, rund) as ctx:
        start(ctx, orc)
        for g in range(3):
            op = g == 2
            ctx.step(op)
            orc.step(op)
            ctx.branch(1.0)
            orc.branch(1.0)
            assert ctx.num_walkers() == orc.num_walkers()
        wg, wo = ctx.walkers(), orc.walkers()
        assert np.array_equal(wg["irn"], wo["irn"])
        assert rel(wg["x"], wo["x"]) < 1e-10
        for k in ("psil", "d2psi", "v", "weight"):
            assert rel_each(wg[k], wo[k]) < TOL, k
        vb_g, _, wb_g = ctx.estimators()
        vb_o, _, wb_o = orc.estimators()
        assert rel_each(vb_g, vb_o) < 1e-9 and rel_each(wb_g, wb_o) < 1e-9


def test_gf_timed_generations_equal_generations():
    """Graph replay (dmc_timed_generations) runs the same idmc = 10 move as
    single dmc_generation calls, bit for bit."""
    sysd, rund, _ = configs.workload("n66", nwalk=48, idmc=10)
    with capi.Context(sysd, rund) as a, capi.Context(sysd, rund) as b:
        for c in (a, b):
            c.init_walkers()
            c.initial_eval()
        steps, ms, nl = a.timed_generations(3, opcomp_last=True, flush_l2=False)
        for g in range(3):
            b.generation(g == 2)
        wa, wb = a.walkers(), b.walkers()
        for k in ("x", "irn", "weight", "psil", "d2psi"):
            assert np.array_equal(wa[k], wb[k]), k
        for ea, eb in zip(a.estimators(), b.estimators()):
            assert np.array_equal(ea, eb)



@pytest.mark.parametrize("fn", [0, 1])
def test_gf_node_crossings_with_and_without_fixed_node(fn):
    """A larger time step makes proposals cross nodes: with fn on the
    crossing walker's weight is 0, with fn off it keeps 0.5 (wt1 + wt2)
    exp(etrial dt); populations, estimator 5 (the crossing rate) and the
    walkers follow the oracle either way."""
    sysd, rund, _ = configs.workload("n14", nwalk=64, idmc=10)
    rund.fn = fn
    rund.dt = rund.dt * 5           # about 12 % of the moves cross a node
    orc = oracle.Oracle(sysd, rund)
    with capi.Context(sysd, rund) as ctx:
        start(ctx, orc)
        for g in range(4):
            op = g == 3
            assert ctx.generation(op) == orc.generation(op)
        wg, wo = ctx.walkers(), orc.walkers()
        vb_g, _, wb_g = ctx.estimators()
        vb_o, _, wb_o = orc.estimators()
    assert np.array_equal(wg["irn"], wo["irn"])
    assert np.array_equal(wg["is_"], wo["is_"])
    assert rel(wg["x"], wo["x"]) < 1e-10
    assert rel_each(wg["weight"], wo["weight"]) < TOL
    assert rel_each(vb_g, vb_o) < 1e-9 and rel_each(wb_g, wb_o) < 1e-9
    crossings = vb_o[4] / wb_o[4]
    print(f"fn={fn}: node-crossing rate {crossings:.3f}")
    assert crossings > 0
