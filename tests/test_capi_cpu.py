"""C ABI checks that need no GPU: the library loads and exports every entry
point declared in include/dmcbcs_gpu.h; the deck reader."""
import ctypes
import os
import re

import pytest

from dmcbcs_project_gb300 import abi, capi, deck

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "dmcbcs_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(dmc_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from dmcbcs_project_gb300 import build

    build.build()
    return ctypes.CDLL(capi.LIB_PATH)


def test_exports_every_declared_symbol(lib):
    declared = header_functions()
    assert len(declared) >= 30
    missing = [f for f in declared if not hasattr(lib, f)]
    assert not missing, missing
    assert sorted(capi.EXPORTS) == declared


def test_abi_version_and_status_strings(lib):
    lib.dmc_abi_version.restype = ctypes.c_int
    assert lib.dmc_abi_version() == abi.DMC_ABI_VERSION
    lib.dmc_status_string.restype = ctypes.c_char_p
    assert lib.dmc_status_string(abi.DMC_ERR_OVERFLOW) == b"walker stack overflow"


def test_struct_sizes_match_header():
    # offsets/sizes of the descriptor structs as compiled by gcc from the header
    import subprocess
    import tempfile

    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "dmcbcs_gpu.h"
int main(void){ printf("%zu %zu %zu %zu %zu %zu\n", sizeof(dmc_system_desc), sizeof(dmc_run_desc),
  sizeof(dmc_info), sizeof(dmc_walkers), offsetof(dmc_system_desc, v0eq), offsetof(dmc_run_desc, stmax)); return 0; }
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    got = [int(v) for v in out]
    exp = [ctypes.sizeof(abi.SystemDesc), ctypes.sizeof(abi.RunDesc), ctypes.sizeof(abi.Info),
           ctypes.sizeof(abi.Walkers), abi.SystemDesc.v0eq.offset, abi.RunDesc.stmax.offset]
    assert got == exp


DECK = """17             # seed
1              # idmc
.true.         # isite
64             # walkers
0              # neq
2              # nav
5              # nstep
0.00005        # dt
0.40           # etrial
.true.         # units
-1.0           # dcut
.true.         # fn
1.1
0.9
0.5
10.0
10000
0.5
3
17
9    1.0
8    1.0
bcs
0.0
0.0337737278
1
0 0 0
0
3
2.5
0.5
0.1
0 0 0
0.0
0.0
0
0.0
0.0
0.5
5.0
1.0
1.0
24.0
1.0
1.0
1.15
0
0
0
0
0
0
"""


def test_deck_reader():
    s, r, e = deck.load_deck(DECK)
    assert (s.nbin[0], s.nbin[1]) == (9, 8)
    assert s.nexup == 1 and list(s.ikup[0]) == [0, 0, 0]
    assert s.norb == 3 and abs(s.vorb[1] - 0.5) < 1e-15
    assert r.idmc == 1 and r.nwalk == 64 and r.dcut == -1.0 and r.fn == 1
    assert s.cjas[1] == 1.0 and s.djas == 1.15
    assert e["operators"] == [0, 0, 0, 0]


DECKS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "decks.json")


@pytest.mark.parametrize("name", ["dmcbcs.dat", "input.dat"])
def test_reference_decks_fixture(name):
    """The committed parse of the reference's two decks builds valid
    descriptors: 10 shells each, 33/33 DMC and polarised 9/8 VMC."""
    import json

    d = json.load(open(DECKS))[name]
    s, r = abi.make_system(d["system"]), abi.make_run(d["run"])
    assert s.norb == 10 and r.dt == 5e-5
    if name == "dmcbcs.dat":
        assert (s.nbin[0], s.nbin[1], r.idmc, r.dcut) == (33, 33, 1, -1.0)
    else:
        assert (s.nbin[0], s.nbin[1], s.nexup, r.idmc, r.dcut) == (9, 8, 1, -1, 0.0)


@pytest.mark.parametrize("name", ["dmcbcs.dat", "input.dat"])
def test_reference_decks_parse(name):
    """Where the reference tree is available (DMCBCS_REFERENCE names its
    directory), the deck reader still gives the committed values."""
    import json

    ref = os.environ.get("DMCBCS_REFERENCE")
    if not ref or not os.path.exists(os.path.join(ref, name)):
        pytest.skip("reference decks not present (set DMCBCS_REFERENCE)")
    s, r, e = deck.parse_deck(open(os.path.join(ref, name)).read())
    want = json.load(open(DECKS))[name]
    assert json.loads(json.dumps({"system": s, "run": r, "extra": e}, sort_keys=True)) == want


def _plan_units(grids, per_sm):
    return sum(g * (2 // p) for g, p in zip(grids, per_sm))


def test_batch_plan_balances_and_fits(lib):
    """dmc_batch_plan (host only): the split fits the SMs, every system gets a
    CTA, no system gets more CTAs than walkers or its own grid, and the
    predicted longest system cannot be shortened by moving one CTA."""
    import numpy as np

    nsm = 152
    nw = [2731, 2712, 2745, 2698, 2760, 2738]
    tau = [1.0, 4.0, 21.0, 19.0, 26.0, 150.0]
    per_sm = [2, 2, 2, 2, 2, 1]
    maxg = [304, 304, 304, 304, 304, 152]
    g = capi.batch_plan(tau, nw, per_sm, maxg, nsm)
    assert g.min() >= 1 and all(g[s] <= min(maxg[s], nw[s]) for s in range(6))
    assert _plan_units(g, per_sm) <= 2 * nsm
    pred = [-(-nw[s] // g[s]) * tau[s] for s in range(6)]
    worst = int(np.argmax(pred))
    # taking one CTA from any other system and giving it to the worst one does
    # not shorten the makespan
    for s in range(6):
        if s == worst or g[s] == 1:
            continue
        g2 = g.copy()
        g2[s] -= 1
        free = 2 * nsm - _plan_units(g2, per_sm)
        add = free // (2 // per_sm[worst])
        g2[worst] = min(maxg[worst], g2[worst] + add)
        pred2 = [-(-nw[k] // g2[k]) * tau[k] for k in range(6)]
        assert max(pred2) >= max(pred) * (1 - 1e-12)


def test_batch_plan_small_and_invalid(lib):
    import numpy as np

    # fewer walkers than SMs: never more CTAs than walkers
    g = capi.batch_plan([1.0, 1.0], [3, 5], [2, 2], [304, 304], 152)
    assert list(g) == [3, 5]
    # equal systems: the makespan of the even split (14 waves of 76 CTAs)
    g = capi.batch_plan([1.0] * 4, [1000] * 4, [2] * 4, [304] * 4, 152)
    assert max(-(-1000 // int(x)) for x in g) == 14 and sum(g) <= 304
    # one-per-SM systems take two slots per CTA
    g = capi.batch_plan([1.0, 1.0], [1000, 1000], [1, 2], [152, 304], 152)
    assert _plan_units(g, [1, 2]) <= 304 and g[0] * 2 + g[1] >= 300
    for bad in (dict(tau=[0.0]), dict(nw=[0]), dict(per_sm=[3]), dict(maxgrid=[0])):
        args = dict(tau=[1.0], nw=[10], per_sm=[2], maxgrid=[10])
        args.update(bad)
        with pytest.raises(capi.DMCError):
            capi.batch_plan(args["tau"], args["nw"], args["per_sm"], args["maxgrid"], 152)
    with pytest.raises(capi.DMCError):   # more systems than slots
        capi.batch_plan([1.0] * 3, [10] * 3, [1] * 3, [10] * 3, 1)
    assert np.all(capi.batch_plan([2.0], [100], [1], [152], 152) == 100)


def test_new_entry_points_reject_bad_arguments(lib):
    """Argument checks of the batch, gradient and host-generation entry
    points (no context, no GPU work)."""
    c_int, vp = ctypes.c_int, ctypes.c_void_p
    lib.dmc_batch_create.argtypes = [vp, c_int, vp]
    lib.dmc_batch_destroy.argtypes = [vp]
    lib.dmc_batch_tune.argtypes = [vp, c_int, vp, vp]
    lib.dmc_batch_generations.argtypes = [vp, c_int, c_int, c_int, vp, vp, vp]
    lib.dmc_batch_set_grids.argtypes = [vp, vp]
    lib.dmc_param_count.argtypes = [vp, vp]
    lib.dmc_param_grad.argtypes = [vp, c_int, vp, vp, vp]
    lib.dmc_generation_host.argtypes = [vp, vp, vp, c_int]
    out = vp()
    assert lib.dmc_batch_create(None, 1, ctypes.byref(out)) == abi.DMC_ERR_INVALID
    assert lib.dmc_batch_create(None, 0, ctypes.byref(out)) == abi.DMC_ERR_INVALID
    arr = (vp * 17)()
    assert lib.dmc_batch_create(arr, 17, ctypes.byref(out)) == abi.DMC_ERR_INVALID   # more than DMC_BATCH_MAX
    assert lib.dmc_batch_destroy(None) == abi.DMC_ERR_INVALID
    assert lib.dmc_batch_tune(None, 1, None, None) == abi.DMC_ERR_INVALID
    assert lib.dmc_batch_generations(None, 1, 1, 0, None, None, None) == abi.DMC_ERR_INVALID
    assert lib.dmc_batch_set_grids(None, None) == abi.DMC_ERR_INVALID
    n = c_int()
    assert lib.dmc_param_count(None, ctypes.byref(n)) == abi.DMC_ERR_INVALID
    assert lib.dmc_param_grad(None, 1, None, None, None) == abi.DMC_ERR_INVALID
    assert lib.dmc_generation_host(None, None, None, 0) == abi.DMC_ERR_INVALID


def test_create_rejects_bad_decks_before_any_device_call(lib):
    """dmc_create checks the deck values on the host first: more particles
    than DMC_MAX_PART, more shells than DMC_MAX_SHELLS, an idmc the
    reference does not have, a non-positive time step or no walkers give
    DMC_ERR_INVALID (no device is needed to see it)."""
    from dmcbcs_project_gb300 import configs

    lib.dmc_create.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    cases = []
    sp = configs.system_params(150, 150, 7)
    cases.append((sp, configs.run_params(4, 0.001)))
    sp = configs.system_params(7, 7, 5)
    sp["norb"] = abi.DMC_MAX_SHELLS + 1
    cases.append((sp, configs.run_params(4, 0.001)))
    for idmc in (3, 11, -3):
        cases.append((configs.system_params(7, 7, 5), configs.run_params(4, 0.001, idmc=idmc)))
    r = configs.run_params(4, 0.001)
    r["dt"] = 0.0
    cases.append((configs.system_params(7, 7, 5), r))
    r = configs.run_params(4, 0.001)
    r["nwalk"] = 0
    cases.append((configs.system_params(7, 7, 5), r))
    for sp, rp in cases:
        s = abi.make_system(sp) if sp["norb"] <= abi.DMC_MAX_SHELLS else None
        if s is None:
            sp2 = dict(sp)
            sp2["norb"] = 5
            s = abi.make_system(sp2)
            s.norb = abi.DMC_MAX_SHELLS + 1
        out = ctypes.c_void_p()
        st = lib.dmc_create(ctypes.byref(s), ctypes.byref(abi.make_run(rp)), ctypes.byref(out))
        assert st == abi.DMC_ERR_INVALID, (sp["nbin"], sp["norb"], rp)
        assert not out.value


def test_walker_views_are_cached_per_slot_and_array_set():
    """The dmc_walkers view of a population is built once per slot and set
    of arrays (the host generation hands the same arrays over every time):
    its pointers are the arrays' data, n follows every call, the in and out
    slots never share a view, and the cache stays bounded."""
    import numpy as np

    def population(cap, npart):
        h = {k: np.zeros((cap, npart, 3)) for k in ("x", "dpsi", "dpsig")}
        for k in ("psil", "psigl", "d2psi", "d2psig", "v", "vext", "weight", "psil0", "psigl0", "wt0"):
            h[k] = np.zeros(cap)
        h["is_"] = np.zeros(cap, np.int32)
        h["irn"] = np.zeros(cap, np.int64)
        return h

    class Holder:
        pass

    ctx = Holder()
    view = capi.Context.walker_struct
    host = population(16, 2)
    a = view(ctx, dict(host, n=5), "in")
    b = view(ctx, dict(host, n=16), "out")
    assert a is not b and a.n == 5 and b.n == 16
    for k in capi._WALKER_FIELDS:
        ptr = ctypes.cast(getattr(a, k), ctypes.c_void_p).value
        assert ptr == host[k].ctypes.data == ctypes.cast(getattr(b, k), ctypes.c_void_p).value
    assert view(ctx, dict(host, n=7), "in") is a and a.n == 7
    other = population(16, 2)
    c = view(ctx, dict(other, n=3), "in")
    assert c is not a and ctypes.cast(c.x, ctypes.c_void_p).value == other["x"].ctypes.data
    keep = [population(4, 1) for _ in range(12)]
    for h in keep:
        view(ctx, dict(h, n=1), "in")
    assert len(ctx._wcache) <= 8
    # without a slot a fresh view every call
    assert view(ctx, dict(host, n=2)) is not view(ctx, dict(host, n=2))
