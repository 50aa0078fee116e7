"""Every public entry point of the library once, on small synthetic inputs:
wavefunction batches (hpsi, bcs, getphi, matinv), single-particle ratios
(bcsone, getphione), parameter derivatives (getderbcs, getjasder, the adjoint
gradients), the stochastic-reconfiguration sums and step, the operators
(g(r), density, S(q), n(k)), the layout tuner, generations on device
stacks and on pinned host arrays, and a batch of two systems.  The calls raise on any status other
than DMC_OK; the values are checked by the other tests.  Also the one
process in which the secondary kernels are profiled:

    python -m pytest tests/test_gpu_exercise.py -q
"""
import numpy as np
import pytest

from dmcbcs_project_gb300 import capi, configs

pytestmark = pytest.mark.gpu


def _pinned(torch, ctx):
    cap, npart = ctx.info.capacity, ctx.npart
    pin = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=True).numpy()
    host = {k: pin((cap, npart, 3), torch.float64) for k in ("x", "dpsi", "dpsig")}
    for k in ("psil", "psigl", "d2psi", "d2psig", "v", "vext", "weight", "psil0", "psigl0", "wt0"):
        host[k] = pin((cap,), torch.float64)
    host["is_"] = pin((cap,), torch.int32)
    host["irn"] = pin((cap,), torch.int64)
    host["cap"] = cap
    return host


def test_every_entry_point_once(nwalk=256):
    torch = pytest.importorskip("torch")

    rng = np.random.default_rng(7)
    sysd, rund, _ = configs.workload("n66", nwalk=nwalk, idmc=-1, longrange=(3, 1.0, 0.3))
    with capi.Context(sysd, rund) as ctx:
        ctx.init_walkers()
        ctx.initial_eval()
        x = ctx.walkers()["x"][:64].copy()
        ctx.hpsi(x)
        ctx.getphi(x)
        old = ctx.bcs(x, want_inverse=True)
        ctx.matinv(rng.normal(size=(16, ctx.nd, ctx.nd)))
        ip = rng.integers(1, ctx.npart + 1, size=x.shape[0]).astype(np.int32)
        dr = rng.normal(scale=0.3, size=(x.shape[0], 3))
        ctx.bcsone(x, old["smati"], ip, dr)
        ctx.getphione(x, ip, dr)
        ctx.getderbcs(x)
        ctx.getjasder(x)
        ctx.param_grad(x)
        ctx.sr_configure(True, True)
        ctx.sr_accumulate()
        ctx.sr_update(0.02, 1e-3)
        ctx.set_operators(20, 3, 6)
        ctx.generation(False)
        ctx.add_operators()
        ctx.update_operators()
        ctx.tune_layout(1)
        host = _pinned(torch, ctx)
        n = ctx.get_walkers_into(host)
        ctx.put_walkers(dict(host, n=n))
        n = ctx.generation_host(dict(host, n=n), host, True)
        ctx.estimators()
    capi.dfmath_eval(0, rng.uniform(-1, 1, 4096))
    # a batch of two systems, DMC
    ctxs = []
    for name in ("n14", "p33_30"):
        s, r, _ = configs.workload(name, nwalk=nwalk)
        c = capi.Context(s, r, precision="mixed")
        c.init_walkers()
        c.initial_eval()
        ctxs.append(c)
    with capi.Batch(ctxs) as b:
        b.tune(1)
        b.generations(2, opcomp_last=True)
    for c in ctxs:
        c.close()
