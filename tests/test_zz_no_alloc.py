"""dmc_branch_noalloc: branching for callers that may not allocate GPU memory.

Hosts whose walker stacks live in device memory owned by another allocator
(their own device arrays or a memory pool) cannot call cudaMalloc inside the
walker loop.  dmc_branch_noalloc takes their input and output stacks and
keeps its scratch in a fixed device array.  These checks give it the same
walkers as the context-based dmc_branch and compare the two results, for two
branching calls in a row (tolerance 1e-10 relative on floating-point fields,
exact on random states and signs).  The file is named so that pytest
collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from dmcbcs_project_gb300 import abi, capi, configs

pytestmark = pytest.mark.gpu

TOL = 1e-10
FLOAT_FIELDS = ("x", "dpsi", "dpsig", "psil", "psigl", "d2psi", "d2psig", "v", "vext", "weight", "psil0", "psigl0")


def device_stack(torch, cap, npart):
    f64 = dict(dtype=torch.float64, device="cuda")
    s = {k: torch.zeros((cap, npart, 3), **f64) for k in ("x", "dpsi", "dpsig")}
    for k in ("psil", "psigl", "d2psi", "d2psig", "v", "vext", "weight", "psil0", "psigl0"):
        s[k] = torch.zeros(cap, **f64)
    s["wt0"] = torch.zeros(cap, dtype=torch.float32, device="cuda")
    s["is_"] = torch.zeros(cap, dtype=torch.int32, device="cuda")
    s["irn"] = torch.zeros(cap, dtype=torch.int64, device="cuda")
    return s


def as_struct(s):
    d = abi.DevStack()
    for k, t in s.items():
        setattr(d, k, t.data_ptr())
    return d


def upload(torch, s, w):
    n = w["n"]
    for k in FLOAT_FIELDS:
        s[k][:n] = torch.from_numpy(np.ascontiguousarray(w[k])).cuda()
    s["wt0"][:n] = torch.from_numpy(w["wt0"].astype(np.float32)).cuda()
    s["is_"][:n] = torch.from_numpy(w["is_"].astype(np.int32)).cuda()
    s["irn"][:n] = torch.from_numpy(w["irn"].astype(np.int64)).cuda()


def download(s, n):
    out = {k: s[k][:n].cpu().numpy() for k in FLOAT_FIELDS}
    out["wt0"] = s["wt0"][:n].cpu().numpy().astype(np.float64)
    out["is_"] = s["is_"][:n].cpu().numpy()
    out["irn"] = s["irn"][:n].cpu().numpy()
    out["n"] = n
    return out


def assert_same(got, ref):
    assert got["n"] == ref["n"]
    assert np.array_equal(got["irn"], ref["irn"])
    assert np.array_equal(got["is_"], ref["is_"])
    assert np.array_equal(got["wt0"], ref["wt0"])
    for k in FLOAT_FIELDS:
        a, b = np.asarray(got[k]), np.asarray(ref[k])
        assert np.max(np.abs(a - b), initial=0.0) <= TOL * max(1.0, float(np.max(np.abs(b), initial=0.0))), k


def test_branch_noalloc_matches_branch():
    torch = pytest.importorskip("torch")
    L = capi.load()
    sysd, rund, _ = configs.workload("n14", nwalk=256)
    with capi.Context(sysd, rund) as ctx:
        ctx.init_walkers()
        ctx.initial_eval()
        ctx.step(False)                      # weights of one DMC move, before branching
        w0 = ctx.walkers()
        ctx.branch(1.0)
        ref1 = ctx.walkers()
        ctx.branch(0.8)
        ref2 = ctx.walkers()
        hist_ref = ctx.wtisto()
        cap, npart = ctx.info.capacity, ctx.npart

    a = device_stack(torch, cap, npart)
    b = device_stack(torch, cap, npart)
    hist = torch.zeros(abi.DMC_WTISTO, dtype=torch.int64, device="cuda")
    upload(torch, a, w0)
    torch.cuda.synchronize()
    nout = C.c_int(-1)
    # first call: the same input stack and factor as the first dmc_branch
    st = L.dmc_branch_noalloc(w0["n"], npart, cap, 1.0, C.byref(as_struct(a)), C.byref(as_struct(b)),
                              C.c_void_p(hist.data_ptr()), C.byref(nout), None)
    assert st == abi.DMC_OK
    got1 = download(b, nout.value)
    assert_same(got1, ref1)
    # second call in a row, on the first call's output
    st = L.dmc_branch_noalloc(nout.value, npart, cap, 0.8, C.byref(as_struct(b)), C.byref(as_struct(a)),
                              C.c_void_p(hist.data_ptr()), C.byref(nout), None)
    assert st == abi.DMC_OK
    got2 = download(a, nout.value)
    assert_same(got2, ref2)
    assert np.array_equal(hist.cpu().numpy(), hist_ref)


def test_branch_noalloc_rejects_sizes_above_its_scratch():
    torch = pytest.importorskip("torch")
    L = capi.load()
    a = device_stack(torch, 2, 2)
    nout = C.c_int(-1)
    big = abi.DMC_NOALLOC_MAX_WALKERS + 1
    st = L.dmc_branch_noalloc(big, 2, 2, 1.0, C.byref(as_struct(a)), C.byref(as_struct(a)), None,
                              C.byref(nout), None)
    assert st == abi.DMC_ERR_NOALLOC_LIMIT
    st = L.dmc_branch_noalloc(2, 2, big, 1.0, C.byref(as_struct(a)), C.byref(as_struct(a)), None,
                              C.byref(nout), None)
    assert st == abi.DMC_ERR_NOALLOC_LIMIT


def test_branch_noalloc_rejects_aliased_stacks_and_bad_factors():
    """The scatter must not read walkers it overwrites, and int(w * factor + u)
    is undefined for a non-finite factor: both are argument errors."""
    torch = pytest.importorskip("torch")
    L = capi.load()
    a = device_stack(torch, 8, 2)
    b = device_stack(torch, 8, 2)
    nout = C.c_int(-1)
    st = L.dmc_branch_noalloc(4, 2, 8, 1.0, C.byref(as_struct(a)), C.byref(as_struct(a)), None, C.byref(nout), None)
    assert st == abi.DMC_ERR_INVALID
    for f in (float("nan"), float("inf"), -1.0):
        st = L.dmc_branch_noalloc(4, 2, 8, f, C.byref(as_struct(a)), C.byref(as_struct(b)), None, C.byref(nout),
                                  None)
        assert st == abi.DMC_ERR_INVALID, f
