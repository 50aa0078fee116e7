"""Restart through fort.9 files (dmcbcs.f90:254-294, :548-567): a GPU
population written with dmc_save_walkers and pushed back with
dmc_restore_walkers continues like the oracle started from the same file."""
import numpy as np
import pytest

import oracle
from dmcbcs_project_gb300 import capi, configs

pytestmark = pytest.mark.gpu


def test_save_restore_continue(tmp_path):
    path = tmp_path / "fort.9"
    sysd, rund, _ = configs.workload("n14", nwalk=48)
    with capi.Context(sysd, rund) as ctx:
        ctx.init_walkers()
        ctx.initial_eval()
        for g in range(3):
            ctx.generation(g == 2)
        w = ctx.walkers()
        ctx.save_walkers(path, tau=0.75)
    f = capi.fort9_read(path, w["x"].shape[1])
    n = w["n"]
    assert f["tau"] == 0.75 and len(f["irn"]) == n
    # the file holds the stack top first
    assert np.array_equal(f["irn"], w["irn"][::-1])
    assert np.allclose(f["x"], w["x"][::-1], rtol=6e-7, atol=1e-12)
    assert np.allclose(f["psil0"], w["psil"][::-1], rtol=1e-14)
    assert np.allclose(f["weight"], w["weight"][::-1], rtol=6e-7)

    # restart: the GPU context and the oracle both start from the file
    with capi.Context(sysd, rund) as ctx:
        assert ctx.restore_walkers(path) == 0.75
        r = ctx.walkers()
        assert np.array_equal(r["irn"], f["irn"])                  # pushed in file order
        assert np.array_equal(r["x"], f["x"])
        s_gpu, _ = ctx.initial_eval()
        for g in range(2):
            ctx.generation(g == 1)
        wg = ctx.walkers()
    orc = oracle.Oracle(sysd, rund)
    orc.load_walkers(f["x"], weight=f["weight"], psil0=f["psil0"], psigl0=f["psigl0"], irn=f["irn"])
    s_orc, _ = orc.initial_eval()
    for g in range(2):
        orc.generation(g == 1)
    wo = orc.walkers()
    assert np.allclose(s_gpu, s_orc, rtol=1e-10, atol=1e-12)
    assert wg["n"] == wo["n"]
    assert np.array_equal(wg["irn"], wo["irn"])
    assert np.max(np.abs(wg["x"] - wo["x"])) < 1e-10
