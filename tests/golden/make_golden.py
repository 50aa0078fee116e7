"""Generate the committed golden fixtures of the test suite.

Run from the repository root:  python tests/golden/make_golden.py

* rng.json: first outputs of the two 48-bit generators of ran.f90:8-48,
  computed here with Python integers straight from the recurrence
  s' = (mult * s + add) mod 2^48, u = (s' | 1) * 2^-48 (independent of the
  oracle's limb arithmetic).
* lapack.npz: seeded matrices with log|det|, sign and inverse from LAPACK
  dgetrf/dgetri (scipy's bundled LAPACK), the library the reference calls
  through matrixlapack.f90:20,34.
* kshell.json: half-set integer k vectors of each |n|^2 shell counted by a
  direct enumeration (every n with n > -n in lexicographic order).
* oracle_*.npz: oracle outputs (hpsi) on seeded configurations, so the GPU
  tests have fixed expected values even if the oracle changes.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

M48 = 1 << 48
GENS = {"ran1": (44485709377909, 96309754297), "ran2": (34522712143931, 55789347517)}


def lcg(name, seed, n):
    mult, add = GENS[name]
    s = seed % M48
    out = []
    for _ in range(n):
        s = (mult * s + add) % M48
        out.append({"state": s, "u": float((s | 1) / M48)})
    return out


def rng_fixture():
    seeds = [17, 1, 123456789, M48 - 1, 2 ** 47 + 12345]
    return {name: {str(sd): lcg(name, sd, 24) for sd in seeds} for name in GENS}


def lapack_fixture():
    import scipy.linalg.lapack as la

    rng = np.random.default_rng(20240601)
    out = {}
    for k, n in enumerate([1, 2, 3, 7, 16, 33]):
        a = rng.normal(size=(n, n))
        if n >= 3:
            a[0, :] *= 1e-3      # forces row interchanges
        lu, piv, info = la.dgetrf(a)
        assert info == 0
        logdet = float(np.sum(np.log(np.abs(np.diag(lu)))))
        sign = int(np.prod(np.sign(np.diag(lu))) * (-1) ** int(np.sum(piv != np.arange(n))))
        inv, info = la.dgetri(lu, piv)
        assert info == 0
        out[f"a{k}"] = a
        out[f"inv{k}"] = inv
        out[f"logdet{k}"] = np.array(logdet)
        out[f"sign{k}"] = np.array(sign)
        out[f"piv{k}"] = piv
    return out


def kshell_fixture(nshell=10):
    shells = {}
    r = 4
    for nx in range(-r, r + 1):
        for ny in range(-r, r + 1):
            for nz in range(-r, r + 1):
                n = (nx, ny, nz)
                if n > (-nx, -ny, -nz):       # one of each +-n pair
                    shells.setdefault(nx * nx + ny * ny + nz * nz, []).append(n)
    keys = sorted(shells)[:nshell]
    return {"n2": [0] + keys, "count": [1] + [len(shells[k]) for k in keys]}


def oracle_fixtures():
    import oracle
    from dmcbcs_project_gb300 import configs

    out = {}
    for name, nw in (("n14", 24), ("p38_33", 6), ("n66", 8)):
        sysd, rund, _ = configs.workload(name, nwalk=nw, seed=99)
        o = oracle.Oracle(sysd, rund, threads=1)
        o.init_walkers()
        x = o.walkers()["x"] + np.random.default_rng(5).normal(scale=0.3, size=(nw, o.npart, 3))
        h = o.hpsi(x)
        out[name] = dict(x=x, **{k: v for k, v in h.items()})
    return out


def main():
    with open(os.path.join(HERE, "rng.json"), "w") as f:
        json.dump(rng_fixture(), f, indent=0)
    np.savez_compressed(os.path.join(HERE, "lapack.npz"), **lapack_fixture())
    with open(os.path.join(HERE, "kshell.json"), "w") as f:
        json.dump(kshell_fixture(), f)
    for name, d in oracle_fixtures().items():
        np.savez_compressed(os.path.join(HERE, f"oracle_{name}.npz"), **d)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
