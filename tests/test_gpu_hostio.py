"""Walker state through host memory (dmc_put_walkers / dmc_get_walkers,
stack.f90:82-110 hand-over of the whole population): with pinned host arrays
one kernel reads or writes every field over the host link; with pageable
arrays the library copies field by field.  Both must give the same bits, and
generations after a pinned put must match generations after a pageable put
exactly.  dmc_generation_host (the walker kernel reading the population from
pinned host arrays, the new population written back in the same call) must
match put + generation + get bit for bit."""
import numpy as np
import pytest

from dmcbcs_project_gb300 import capi, configs

pytestmark = pytest.mark.gpu

FIELDS = ("x", "dpsi", "dpsig", "psil", "psigl", "d2psi", "d2psig", "v", "vext", "weight", "psil0", "psigl0", "wt0",
          "is_", "irn")


def pinned_arrays(torch, ctx):
    cap, npart = ctx.info.capacity, ctx.npart
    pin = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=True).numpy()
    host = {k: pin((cap, npart, 3), torch.float64) for k in ("x", "dpsi", "dpsig")}
    for k in ("psil", "psigl", "d2psi", "d2psig", "v", "vext", "weight", "psil0", "psigl0", "wt0"):
        host[k] = pin((cap,), torch.float64)
    host["is_"] = pin((cap,), torch.int32)
    host["irn"] = pin((cap,), torch.int64)
    host["cap"] = cap
    return host


@pytest.mark.parametrize("name,nw,idmc", [("n14", 64, 1), ("p33_30", 24, 0)])
def test_pinned_and_pageable_walker_io(name, nw, idmc):
    torch = pytest.importorskip("torch")
    sysd, rund, _ = configs.workload(name, nwalk=nw, idmc=idmc)
    with capi.Context(sysd, rund) as a, capi.Context(sysd, rund) as b:
        for c in (a, b):
            c.init_walkers()
            c.initial_eval()
            c.generation(False)
        host = pinned_arrays(torch, a)
        n = a.get_walkers_into(host)
        ref = b.walkers()
        assert n == ref["n"]
        for k in FIELDS:
            assert np.array_equal(host[k][:n], ref[k]), k
        # change the population on the host, hand it back both ways
        rng = np.random.default_rng(5)
        dx = rng.normal(scale=0.05, size=ref["x"].shape)
        host["x"][:n] += dx
        ref["x"] = ref["x"] + dx
        host["weight"][:n] *= 0.5
        ref["weight"] = ref["weight"] * 0.5
        a.put_walkers(dict(host, n=n))
        b.put_walkers({k: np.ascontiguousarray(v) if isinstance(v, np.ndarray) else v for k, v in ref.items()})
        for g in range(3):
            na = a.generation(g == 2)
            nb = b.generation(g == 2)
            assert na == nb
        wa, wb = a.walkers(), b.walkers()
        for k in FIELDS:
            assert np.array_equal(wa[k], wb[k]), k
        for ea, eb in zip(a.estimators(), b.estimators()):
            assert np.array_equal(ea, eb)
        # a second read into the same pinned arrays (cached device views)
        m = a.get_walkers_into(host)
        assert m == wa["n"] and np.array_equal(host["x"][:m], wa["x"])


@pytest.mark.parametrize("name,nw,idmc", [("n14", 64, 1), ("n14", 40, 0), ("p33_30", 24, 2), ("n66", 32, -2),
                                         ("n14", 32, 10)])
def test_generation_host_matches_device_stacks(name, nw, idmc):
    torch = pytest.importorskip("torch")
    sysd, rund, _ = configs.workload(name, nwalk=nw, idmc=idmc)
    with capi.Context(sysd, rund) as a, capi.Context(sysd, rund) as b:
        for c in (a, b):
            c.init_walkers()
            c.initial_eval()
        host = pinned_arrays(torch, a)
        n = a.get_walkers_into(host)
        gens = 4
        for g in range(gens):
            op = g == gens - 1
            n = a.generation_host(dict(host, n=n), host, op)
            nb = b.generation(op)
            assert n == nb, (g, n, nb)
        wb = b.walkers()
        for k in FIELDS:
            assert np.array_equal(host[k][:n], wb[k]), k
        for ea, eb in zip(a.estimators(), b.estimators()):
            assert np.array_equal(ea, eb)
        assert np.array_equal(a.wtisto(), b.wtisto())
        # pageable arrays take the copy path with the same result
        pg = {k: np.array(v) if isinstance(v, np.ndarray) else v for k, v in host.items()}
        n2 = a.generation_host(dict(pg, n=n), pg, False)
        nb2 = b.generation(False)
        wb = b.walkers()
        assert n2 == nb2
        for k in FIELDS:
            assert np.array_equal(pg[k][:n2], wb[k]), k
        # an output too small is reported with the count it needs
        small = dict(host, cap=1)
        with pytest.raises(capi.DMCError):
            a.generation_host(dict(pg, n=n2), small, False)
