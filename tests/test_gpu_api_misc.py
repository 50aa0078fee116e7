"""Entry points the other tests reach only indirectly: the device-pointer
hpsi (stream-ordered, CUDA tensors in and out) against the host-staged batch
call, precision get/set, and the zeroing calls of the estimators, the SR
sums and the operators, and the step timer."""
import ctypes as C

import numpy as np
import pytest

from dmcbcs_project_gb300 import abi, capi, configs

pytestmark = pytest.mark.gpu


def test_hpsi_device_equals_batch():
    torch = pytest.importorskip("torch")
    sysd, rund, _ = configs.workload("n66", nwalk=32)
    with capi.Context(sysd, rund, precision="mixed") as ctx:
        ctx.init_walkers()
        x = ctx.walkers()["x"][:32].copy()
        ref = ctx.hpsi(x)
        nw, P = x.shape[0], ctx.npart
        dev = torch.device("cuda")
        xd = torch.from_numpy(x).to(dev)
        out = {k: torch.zeros(nw, dtype=torch.float64, device=dev) for k in
               ("psil", "d2psi", "v", "vext", "psigl", "d2psig")}
        out["is_"] = torch.zeros(nw, dtype=torch.int32, device=dev)
        out["dpsi"] = torch.zeros(nw, P, 3, dtype=torch.float64, device=dev)
        out["dpsig"] = torch.zeros(nw, P, 3, dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream()
        order = ("psil", "is_", "dpsi", "d2psi", "v", "vext", "psigl", "dpsig", "d2psig")
        st = capi.load().dmc_hpsi_device(ctx._h, nw, C.c_void_p(xd.data_ptr()),
                                         *[C.c_void_p(out[k].data_ptr()) for k in order],
                                         C.c_void_p(stream.cuda_stream))
        assert st == abi.DMC_OK
        stream.synchronize()
        for k in order:
            assert np.array_equal(out[k].cpu().numpy(), ref[k]), k


def test_precision_and_zeroing_calls():
    sysd, rund, _ = configs.workload("n14", nwalk=24, idmc=-1)
    with capi.Context(sysd, rund, precision="mixed") as ctx:
        p = C.c_int()
        assert capi.load().dmc_get_precision(ctx._h, C.byref(p)) == abi.DMC_OK and p.value == capi.PREC_MIXED
        ctx.set_precision("fp64")
        assert capi.load().dmc_get_precision(ctx._h, C.byref(p)) == abi.DMC_OK and p.value == capi.PREC_FP64
        assert capi.load().dmc_set_precision(ctx._h, 7) == abi.DMC_ERR_INVALID
        ctx.init_walkers()
        ctx.initial_eval()
        ctx.generation(True)
        vb, vb2, wb = ctx.estimators()
        assert np.any(wb != 0)
        ctx.zero_estimators()
        for a in ctx.estimators():
            assert not np.any(a)
        ctx.step(True)
        assert ctx.last_step_ms() > 0
        ctx.sr_configure(False, True)
        assert ctx.sr_accumulate() == ctx.num_walkers()
        ctx.sr_zero()
        s = ctx.sr_sums()
        assert s["n"] == 0 and not np.any(s["ovec"]) and not np.any(s["pmat"])
        ctx.set_operators(10, 2, 4)
        ctx.add_operators()
        v0, _, w0 = ctx.operators(0, raw=True)
        assert w0 > 0 and np.any(v0)
        ctx.zero_operators()
        v, _, w = ctx.operators(0, raw=True)
        assert w == 0 and not np.any(v)
