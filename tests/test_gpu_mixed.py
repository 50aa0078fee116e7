"""Mixed-precision walker path against the FP64 oracle.

The mixed path computes the pair matrix, inverse and drift/Laplacian
contractions in double-float arithmetic and the Jastrow and potential in
FP32.  Bars (per configuration, against the FP64 oracle): local energy and
Laplacian within 1e-6 relative (the benchmark's requirement), log|Psi|
within 1e-6 absolute, drift within 1e-6 relative to the largest component.
The measured errors are printed.
"""
import numpy as np
import pytest

import oracle
from dmcbcs_project_gb300 import capi, configs

pytestmark = pytest.mark.gpu

EL_TOL = 1e-6


def walkers(name, nw, seed):
    sysd, rund, _ = configs.workload(name, nwalk=nw, seed=seed)
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    x = orc.walkers()["x"] + np.random.default_rng(seed).normal(scale=0.3, size=(nw, orc.npart, 3))
    return sysd, rund, orc, x


@pytest.mark.parametrize("name,nw", [("n14", 64), ("n66", 128), ("p33_30", 32), ("p38_33", 32), ("n132", 16)])
def test_mixed_hpsi_against_fp64_oracle(name, nw):
    sysd, rund, orc, x = walkers(name, nw, 21)
    ref = orc.hpsi(x)
    with capi.Context(sysd, rund, precision="mixed") as ctx:
        got = ctx.hpsi(x)
    hb = sysd.hbar
    el_g = -hb * got["d2psi"] + got["v"]
    el_r = -hb * ref["d2psi"] + ref["v"]
    el_err = np.abs(el_g - el_r) / np.maximum(np.abs(el_r), 1.0)
    lap_err = np.abs(got["d2psi"] - ref["d2psi"]) / np.maximum(np.abs(ref["d2psi"]), 1.0)
    psil_err = np.abs(got["psil"] - ref["psil"])
    dr_err = np.array([np.max(np.abs(got["dpsi"][w] - ref["dpsi"][w])) / max(1.0, np.max(np.abs(ref["dpsi"][w])))
                       for w in range(nw)])
    print(f"{name}: max rel err E_L {el_err.max():.2e}, d2psi {lap_err.max():.2e}, "
          f"drift {dr_err.max():.2e}; max abs err log|Psi| {psil_err.max():.2e}")
    assert np.array_equal(got["is_"], ref["is_"])
    assert el_err.max() < EL_TOL
    assert lap_err.max() < EL_TOL
    assert dr_err.max() < EL_TOL
    assert psil_err.max() < 1e-6


@pytest.mark.parametrize("idmc", [1, 2, 0, -2])
def test_mixed_generations_track_fp64(idmc):
    """Short runs of every run type from the same walkers: the mixed path
    follows the FP64 trajectories (same random streams, same Metropolis
    decisions and branching; weights and positions differ only by the mixed
    path's rounding).  The pair matrix is accumulated against a bound of
    sum_q |v_q|, which leaves drift errors up to ~1e-8 relative for walkers
    near a node; after four generations the positions agree to 1e-7."""
    sysd, rund, _ = configs.workload("n66", nwalk=64, idmc=idmc)
    res = {}
    for prec in ("fp64", "mixed"):
        with capi.Context(sysd, rund, precision=prec) as ctx:
            ctx.init_walkers()
            ctx.initial_eval()
            for g in range(4):
                ctx.generation(g == 3)
            res[prec] = (ctx.walkers(), ctx.estimators())
    (w64, e64), (wmx, emx) = res["fp64"], res["mixed"]
    assert w64["n"] == wmx["n"]
    assert np.array_equal(w64["irn"], wmx["irn"])
    dx = np.max(np.abs(w64["x"] - wmx["x"]))
    print(f"max position difference after 4 generations {dx:.2e}")
    assert dx < 1e-7
    el64 = -sysd.hbar * w64["d2psi"] + w64["v"]
    elmx = -sysd.hbar * wmx["d2psi"] + wmx["v"]
    assert np.max(np.abs(el64 - elmx) / np.maximum(np.abs(el64), 1.0)) < EL_TOL
    assert np.allclose(e64[0], emx[0], rtol=1e-6)


@pytest.mark.parametrize("rel", [1.3e-8, -1.3e-8])
def test_mixed_pair_within_fp32_ulp_of_half_box(rel):
    """An up-down pair whose distance is within one FP32 ulp of L/2 (the end
    of the beta table) must land on the same side of the range as in FP64."""
    sysd, rund, orc, x = walkers("n66", 8, 5)
    el = orc.info.el
    u = np.array([0.3, 0.5, -0.81])
    u /= np.linalg.norm(u)
    nup = sysd.nbin[0]
    for w in range(x.shape[0]):
        x[w, nup + w] = x[w, w] + 0.5 * el * (1.0 + rel) * u
    ref = orc.hpsi(x)
    with capi.Context(sysd, rund, precision="mixed") as ctx:
        got = ctx.hpsi(x)
    hb = sysd.hbar
    el_g = -hb * got["d2psi"] + got["v"]
    el_r = -hb * ref["d2psi"] + ref["v"]
    err = np.abs(el_g - el_r) / np.maximum(np.abs(el_r), 1.0)
    print(f"rel {rel:+.1e}: max rel err E_L {err.max():.2e}")
    assert err.max() < EL_TOL


@pytest.mark.parametrize("name", ["n14", "n66", "p33_30"])
def test_mixed_bcs_and_getphi_against_oracle(name):
    """The determinant alone (dmc_bcs_batch, bcs) and the Jastrow with the
    potential alone (dmc_getphi_batch, getphi) from a mixed context: the
    same bars as hpsi (1e-6), the inverse within 1e-6 of its largest entry."""
    sysd, rund, orc, x = walkers(name, 16, 41)
    rb = orc.bcs(x, want_inverse=True)
    with capi.Context(sysd, rund, precision="mixed") as ctx:
        gb = ctx.bcs(x, want_inverse=True)
        gj = ctx.getphi(x)
    assert np.array_equal(gb["is_"], rb["is_"])
    assert np.max(np.abs(gb["phil"] - rb["phil"])) < 1e-6
    lap = np.abs(gb["d2phi"] - rb["d2phi"]) / np.maximum(np.abs(rb["d2phi"]), 1.0)
    assert lap.max() < EL_TOL
    for w in range(16):
        assert np.max(np.abs(gb["dphi"][w] - rb["dphi"][w])) < EL_TOL * max(1.0, np.max(np.abs(rb["dphi"][w])))
        assert np.max(np.abs(gb["smati"][w] - rb["smati"][w])) < 1e-6 * np.max(np.abs(rb["smati"][w]))
        r = orc.getphi(x[w])
        assert abs(gj["u"][w] - r["u"]) < EL_TOL * max(1.0, abs(r["u"]))
        assert abs(gj["d2u"][w] - r["d2u"]) < EL_TOL * max(1.0, abs(r["d2u"]))
        assert abs(gj["v"][w] - r["v"]) < EL_TOL * max(1.0, abs(r["v"]))
        assert np.max(np.abs(gj["du"][w] - r["du"])) < EL_TOL * max(1.0, np.max(np.abs(r["du"])))
