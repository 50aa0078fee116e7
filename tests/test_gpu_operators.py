"""Operators of the block loop (operators.f90 with gofr.f90, sofq.f90 and
momentum3d.f90) on the GPU against the oracle: the same population (the
generations follow identical random streams), one operator pass, the
running sums and the block averages."""
import numpy as np
import pytest

import oracle
from dmcbcs_project_gb300 import capi, configs

pytestmark = pytest.mark.gpu


def run_both(name, nwalk, gens, tabs, same_spin=False):
    sysd, rund, _ = configs.workload(name, nwalk=nwalk)
    if same_spin:
        # the same-spin Jastrow on: n(k)'s single-particle ratios then carry
        # both Jastrow tables
        sysd.v0op, sysd.v0eq = 0.5, -0.5
        sysd.cjas[0], sysd.cjas[1] = 1.0, 1.0
    orc = oracle.Oracle(sysd, rund)
    ctx = capi.Context(sysd, rund)
    for m in (ctx, orc):
        m.init_walkers()
        m.initial_eval()
        for g in range(gens):
            m.generation(False)
        m.set_operators(*tabs)
    return sysd, ctx, orc


def close(a, b, rtol):
    scale = max(np.max(np.abs(b)), 1e-300)
    return np.max(np.abs(a - b)) <= rtol * scale


@pytest.mark.parametrize("name,nwalk,tabs,same_spin", [("n14", 24, (25, 4, 12), False),
                                                       ("p33_30", 6, (20, 3, 6), False),
                                                       ("n66", 6, (20, 3, 6), True),
                                                       ("n132", 3, (20, 3, 4), False)])
def test_operator_pass_matches_oracle(name, nwalk, tabs, same_spin):
    sysd, ctx, orc = run_both(name, nwalk, 2, tabs, same_spin)
    try:
        wg0, wo0 = ctx.walkers(), orc.walkers()
        assert np.array_equal(wg0["irn"], wo0["irn"])
        ctx.add_operators()
        orc.add_operators()
        # the pass leaves the population reversed, on both sides
        assert np.array_equal(ctx.walkers()["irn"], wg0["irn"][::-1])
        assert np.array_equal(orc.walkers()["irn"], wo0["irn"][::-1])
        for which, label in enumerate(["g(r)", "density", "S(q)", "n(k)"]):
            gv, ge, gw = ctx.operators(which, raw=True)
            ov, oe, ow = orc.operators(which, raw=True)
            print(f"{name} {label}: {len(gv)} sums, max |diff| {np.max(np.abs(gv - ov)):.2e} of {np.max(np.abs(ov)):.2e}")
            assert len(gv) == len(ov) > 0
            assert abs(gw - ow) <= 1e-12 * abs(ow)
            assert close(gv, ov, 1e-10) and close(ge, oe, 1e-10)
        ctx.update_operators()
        orc.update_operators()
        for which in range(4):
            gv, ge, gw = ctx.operators(which)
            ov, oe, ow = orc.operators(which)
            assert abs(gw - ow) <= 1e-12 * abs(ow)
            assert close(gv, ov, 1e-10)
            # err^2 = |<x^2> - <x>^2| / wsum cancels where a bin has no spread:
            # compare squared errors against the scale of <x>^2 / wsum
            tol = 1e-11 * np.max(ov ** 2) / ow + 1e-10 * oe ** 2
            assert np.all(np.abs(ge ** 2 - oe ** 2) <= tol)
    finally:
        ctx.close()


def test_histogram_totals_and_files(tmp_path):
    sysd, ctx, orc = run_both("n14", 16, 1, (30, 2, 0))
    try:
        w = ctx.walkers()
        wt = w["weight"] * np.exp(w["psil"] - w["psigl"]) * w["is_"] * w["wt0"]
        ctx.add_operators()
        g, g2, ws = ctx.operators(0, raw=True)
        nup, ndn = sysd.nbin[0], sysd.nbin[1]
        pairs = np.array([nup * ndn, nup * (nup - 1) // 2, ndn * (ndn - 1) // 2])
        tot = g.reshape(3, -1).sum(axis=1)
        assert np.allclose(tot, 2.0 * wt.sum() * pairs, rtol=1e-12)
        assert abs(ws - wt.sum()) <= 1e-12 * abs(ws)
        d, _, _ = ctx.operators(1, raw=True)
        d = d.reshape(6, -1)
        ntab = (d.shape[1] - 1) // 2
        # every particle lands in one bin per axis; the centre bin counts a half
        full = d.copy()
        full[:, ntab] *= 2.0
        assert np.allclose(full.sum(axis=1), wt.sum() * np.array([nup] * 3 + [ndn] * 3), rtol=1e-12)
        ctx.update_operators()
        ctx.write_operators(tmp_path, tau=1.5)
        lines = (tmp_path / "gofr.out").read_text().split("\n")
        assert lines[0] == "# r*kF, g(r), err" and lines[2].startswith("# tau = ")
        assert len(lines[3]) == 7 * 15 and len([l for l in lines if l and not l.startswith("#") and l.strip()]) == 30
        assert (tmp_path / "rho.out").exists() and (tmp_path / "sofq.out").exists()
        assert not (tmp_path / "nofk.out").exists()
    finally:
        ctx.close()
