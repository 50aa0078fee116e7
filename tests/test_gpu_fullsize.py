"""The benchmark configuration at full size (N = 66, 4096 walkers, DMC)
through size-independent properties: after 20 mixed-precision generations,
every running configuration's local energy, log|Psi| and drift agree with
the FP64 path to the benchmark's 1e-6 (relative to max(|E_L|, 1); drift
relative to its largest component), the population stays in the
population-control band, weights are finite in [0, wtcut] and every random
state is a 48-bit value."""
import numpy as np
import pytest

from dmcbcs_project_gb300 import capi, configs

pytestmark = pytest.mark.gpu


def test_mixed_against_fp64_on_running_configurations():
    sysd, rund, meta = configs.workload("n66")
    assert meta["nwalk"] == 4096
    with capi.Context(sysd, rund, precision="mixed") as m, capi.Context(sysd, rund) as f:
        m.init_walkers()
        m.initial_eval()
        for g in range(20):
            n = m.generation(g == 19)
            assert rund.popdn * rund.nwalk <= n <= rund.popup * rund.nwalk, (g, n)
        w = m.walkers()
        x = w["x"]
        hm, hf = m.hpsi(x), f.hpsi(x)
    el_m = -sysd.hbar * hm["d2psi"] + hm["v"]
    el_f = -sysd.hbar * hf["d2psi"] + hf["v"]
    err = float(np.max(np.abs(el_m - el_f) / np.maximum(np.abs(el_f), 1.0)))
    derr = float(np.max(np.abs(hm["dpsi"] - hf["dpsi"])) / np.max(np.abs(hf["dpsi"])))
    lerr = float(np.max(np.abs(hm["psil"] - hf["psil"])))
    print(f"{x.shape[0]} running configurations: E_L rel err {err:.1e}, drift {derr:.1e}, log|Psi| {lerr:.1e}")
    assert err < 1e-6 and derr < 1e-6 and lerr < 1e-6
    assert np.array_equal(hm["is_"], hf["is_"])
    wt = w["weight"]
    assert np.all(np.isfinite(wt)) and np.all(wt >= 0) and np.all(wt <= rund.wtcut)
    assert np.all((w["irn"] >= 0) & (w["irn"] < (1 << 48)))
    assert np.all(np.isfinite(x))
