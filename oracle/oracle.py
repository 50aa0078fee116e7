"""ctypes front end of the CPU oracle (``oracle/dmc_oracle.c``).

TEST INFRASTRUCTURE ONLY: the tests, the smoke check and the CPU-baseline
leg of the benchmark use this module, as the reference to compare with.  The product library
never imports it.  See the header of ``dmc_oracle.c`` for what the oracle
restates and how far its parity with the reference is pinned.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from dmcbcs_project_gb300.abi import DMC_NEST_MAX, DMC_WTISTO, Info

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle_dmc.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lp = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")


def build(force=False):
    """Compile the oracle with its Makefile (gcc, portable flags)."""
    src = os.path.join(HERE, "dmc_oracle.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_set_threads.argtypes = [C.c_void_p, C.c_int]
        L.orc_info.argtypes = [C.c_void_p, C.POINTER(Info)]
        L.orc_get_table.argtypes = [C.c_void_p, C.c_int, _dp, C.c_int]
        L.orc_set_vorb.argtypes = [C.c_void_p, _dp, C.c_int]
        L.orc_set_jastrow_spline.argtypes = [C.c_void_p, _dp, C.c_int]
        L.orc_knot_basis.argtypes = [C.c_int, C.c_double, C.c_double, _dp]
        L.orc_sm_sweeps.restype = C.c_int64
        L.orc_sm_sweeps.argtypes = [C.c_void_p, C.c_int]
        L.orc_ran1.restype = C.c_double
        L.orc_ran1.argtypes = [C.POINTER(C.c_int64)]
        L.orc_ran2.restype = C.c_double
        L.orc_ran2.argtypes = [C.POINTER(C.c_int64)]
        L.orc_gaussian.argtypes = [C.POINTER(C.c_int64), C.c_int, _dp]
        L.orc_radialfun.argtypes = [C.c_void_p, C.c_double, _dp]
        L.orc_getphi.argtypes = [C.c_void_p, _dp, C.POINTER(C.c_double), C.POINTER(C.c_int), _dp,
                                 C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_getphione.restype = C.c_double
        L.orc_getphione.argtypes = [C.c_void_p, _dp, _dp, C.c_int]
        L.orc_bcsone.restype = C.c_double
        L.orc_bcsone.argtypes = [C.c_void_p, _dp, _dp, C.c_int, _dp]
        L.orc_getderbcs.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_getjasder.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_matinv.argtypes = [C.c_int, _dp, C.POINTER(C.c_double), C.POINTER(C.c_int)]
        L.orc_hpsi_batch.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.orc_bcs_batch.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _ip, _dp, _dp, C.c_void_p]
        L.orc_init_walkers.argtypes = [C.c_void_p]
        L.orc_load_walkers.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp, _lp]
        L.orc_initial_eval.argtypes = [C.c_void_p, C.c_double, _dp, _dp]
        L.orc_step.argtypes = [C.c_void_p, C.c_int]
        L.orc_branch.argtypes = [C.c_void_p, C.c_double]
        L.orc_generation.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int)]
        L.orc_num_walkers.argtypes = [C.c_void_p]
        L.orc_zero_estimators.argtypes = [C.c_void_p]
        L.orc_get_estimators.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.orc_block_update.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_get_walkers.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp, _ip, _lp, _fp]
        L.orc_get_wtisto.argtypes = [C.c_void_p, _lp]
        L.orc_sr_update.argtypes = [C.c_int, _dp, _dp, _dp, C.c_double, C.c_double, C.c_int, C.c_double,
                                    C.c_double, _dp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_set_operators.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int]
        L.orc_zero_operators.argtypes = [C.c_void_p]
        L.orc_add_operators.argtypes = [C.c_void_p]
        L.orc_update_operators.argtypes = [C.c_void_p]
        L.orc_get_operators.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.POINTER(C.c_double)]
        _lib = L
    return _lib


def ran1(irn):
    s = C.c_int64(irn)
    r = lib().orc_ran1(C.byref(s))
    return r, s.value


def ran2(irn):
    s = C.c_int64(irn)
    r = lib().orc_ran2(C.byref(s))
    return r, s.value


def gaussian(irn, n):
    s = C.c_int64(irn)
    g = np.zeros(n)
    lib().orc_gaussian(C.byref(s), n, g)
    return g, s.value


def matinv(a):
    """rmatinv on one matrix given as a numpy (n,n) array (row, col)."""
    n = a.shape[0]
    f = np.asfortranarray(a, dtype=np.float64).ravel(order="F").copy()
    d = C.c_double(0.0)
    s = C.c_int(1)
    info = lib().orc_matinv(n, f, C.byref(d), C.byref(s))
    return f.reshape((n, n), order="F"), d.value, s.value, info


class Oracle:
    """One system + run, as the reference's module state after set-up."""

    def __init__(self, sysdesc, rundesc, threads=None):
        L = lib()
        st = C.c_int(0)
        self._h = L.orc_create(C.byref(sysdesc), C.byref(rundesc), C.byref(st))
        if not self._h:
            raise RuntimeError(f"oracle set-up failed (status {st.value})")
        self.info = Info()
        L.orc_info(self._h, C.byref(self.info))
        self.npart = self.info.npart
        self.nd = self.info.nd
        self.nest = self.info.nest
        self.norb = int(sysdesc.norb)
        self.set_threads(threads or os.cpu_count() or 1)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().orc_destroy(h)
            self._h = None

    def set_threads(self, n):
        self.threads = int(n)
        lib().orc_set_threads(self._h, self.threads)

    def table(self, which):
        ntab = self.info.ntab
        n = {0: 2 * (ntab + 1), 1: 2 * (ntab + 1), 2: 2 * (ntab + 1), 3: 2 * (ntab + 1),
             4: ntab + 1, 5: ntab + 1, 6: ntab + 1, 7: 3 * self.info.nk, 8: self.info.nk,
             9: 32}[which]
        out = np.zeros(n)
        if lib().orc_get_table(self._h, which, out, n) != 0:
            raise RuntimeError("table")
        return out

    def set_vorb(self, vorb):
        v = np.ascontiguousarray(vorb, dtype=np.float64)
        if lib().orc_set_vorb(self._h, v, len(v)) != 0:
            raise ValueError("norb mismatch")

    def set_jastrow_spline(self, knots):
        """The opt-in up-down Jastrow spline (16 knots; None or [] = off)."""
        k = np.ascontiguousarray(knots if knots is not None else np.zeros(0), dtype=np.float64)
        if lib().orc_set_jastrow_spline(self._h, k if k.size else np.zeros(1), int(k.size)) != 0:
            raise ValueError("the spline has 16 knots")

    def sm_sweeps(self, nsweeps):
        """Particle-by-particle Metropolis sweeps with exact FP64 ratios;
        returns the accepted moves."""
        return int(lib().orc_sm_sweeps(self._h, int(nsweeps)))

    def radialfun(self, r):
        o = np.zeros(3)
        lib().orc_radialfun(self._h, float(r), o)
        return o

    def hpsi(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, self.npart, 3)
        nw = x.shape[0]
        o = dict(psil=np.zeros(nw), is_=np.zeros(nw, np.int32), dpsi=np.zeros((nw, self.npart, 3)),
                 d2psi=np.zeros(nw), v=np.zeros(nw), vext=np.zeros(nw), psigl=np.zeros(nw),
                 dpsig=np.zeros((nw, self.npart, 3)), d2psig=np.zeros(nw))
        lib().orc_hpsi_batch(self._h, nw, x, o["psil"], o["is_"], o["dpsi"], o["d2psi"], o["v"], o["vext"],
                             o["psigl"], o["dpsig"], o["d2psig"])
        return o

    def bcs(self, x, want_inverse=False):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, self.npart, 3)
        nw = x.shape[0]
        phil, is_ = np.zeros(nw), np.zeros(nw, np.int32)
        dphi, d2phi = np.zeros((nw, self.npart, 3)), np.zeros(nw)
        sinv = np.zeros((nw, self.nd * self.nd)) if want_inverse else None
        lib().orc_bcs_batch(self._h, nw, x, phil, is_, dphi, d2phi,
                            sinv.ctypes.data_as(C.c_void_p) if want_inverse else None)
        return dict(phil=phil, is_=is_, dphi=dphi, d2phi=d2phi, smati=sinv)

    def getphi(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(self.npart, 3)
        u, d2u, v = C.c_double(), C.c_double(), C.c_double()
        isj = C.c_int()
        du = np.zeros((self.npart, 3))
        lib().orc_getphi(self._h, x, C.byref(u), C.byref(isj), du, C.byref(d2u), C.byref(v))
        return dict(u=u.value, du=du, d2u=d2u.value, v=v.value)

    def getphione(self, x, drr, i1):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(self.npart, 3)
        return lib().orc_getphione(self._h, x, np.ascontiguousarray(drr, dtype=np.float64), int(i1))

    def bcsone(self, x, dr, i1, smati):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(self.npart, 3)
        return lib().orc_bcsone(self._h, x, np.ascontiguousarray(dr, dtype=np.float64), int(i1),
                                np.ascontiguousarray(smati, dtype=np.float64))

    def getjasder(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(self.npart, 3)
        d = np.zeros(2)
        lib().orc_getjasder(self._h, x, d)
        return d

    def getderbcs(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(self.npart, 3)
        d = np.zeros(max(1, self.norb))
        lib().orc_getderbcs(self._h, x, d)
        return d[: self.norb]

    # ---- population --------------------------------------------------------
    def init_walkers(self):
        rc = lib().orc_init_walkers(self._h)
        if rc:
            raise RuntimeError(f"init_walkers {rc}")

    def load_walkers(self, x, weight=None, psil0=None, psigl0=None, irn=None):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, self.npart, 3)
        n = x.shape[0]
        weight = np.ones(n) if weight is None else np.ascontiguousarray(weight, dtype=np.float64)
        psil0 = np.zeros(n) if psil0 is None else np.ascontiguousarray(psil0, dtype=np.float64)
        psigl0 = np.zeros(n) if psigl0 is None else np.ascontiguousarray(psigl0, dtype=np.float64)
        irn = np.ascontiguousarray(irn, dtype=np.int64)
        rc = lib().orc_load_walkers(self._h, n, x, weight, psil0, psigl0, irn)
        if rc:
            raise RuntimeError(f"load_walkers {rc}")

    def initial_eval(self, tau=0.0):
        sums = np.zeros(9)
        est = np.zeros(2)
        lib().orc_initial_eval(self._h, float(tau), sums, est)
        return sums, est

    def step(self, opcomp):
        rc = lib().orc_step(self._h, int(bool(opcomp)))
        if rc:
            raise RuntimeError(f"step {rc}")

    def branch(self, factor):
        return lib().orc_branch(self._h, float(factor))

    def generation(self, opcomp):
        nt = C.c_int(0)
        rc = lib().orc_generation(self._h, int(bool(opcomp)), C.byref(nt))
        if rc:
            raise RuntimeError(f"generation {rc}")
        return nt.value

    def num_walkers(self):
        return lib().orc_num_walkers(self._h)

    def zero_estimators(self):
        lib().orc_zero_estimators(self._h)

    def estimators(self):
        a, b, c = np.zeros(self.nest), np.zeros(self.nest), np.zeros(self.nest)
        lib().orc_get_estimators(self._h, a, b, c)
        return a, b, c

    def block_update(self):
        a, b = np.zeros(self.nest), np.zeros(self.nest)
        lib().orc_block_update(self._h, a, b)
        return a, b

    def walkers(self):
        n = self.num_walkers()
        cap = max(n, 1)
        x = np.zeros((cap, self.npart, 3))
        dpsi = np.zeros((cap, self.npart, 3))
        dpsig = np.zeros((cap, self.npart, 3))
        scal = np.zeros((cap, 9))
        is_ = np.zeros(cap, np.int32)
        irn = np.zeros(cap, np.int64)
        wt0 = np.zeros(cap, np.float32)
        lib().orc_get_walkers(self._h, cap, x, dpsi, dpsig, scal, is_, irn, wt0)
        names = ["psil", "psigl", "d2psi", "d2psig", "v", "vext", "weight", "psil0", "psigl0"]
        out = {k: scal[:n, i].copy() for i, k in enumerate(names)}
        out.update(n=n, x=x[:n], dpsi=dpsi[:n], dpsig=dpsig[:n], is_=is_[:n], irn=irn[:n],
                   wt0=wt0[:n].astype(np.float64))
        return out

    # ---- operators: g(r) + density profile, S(q), n(k) ----------------------
    def set_operators(self, ntabg, ntabq, ntabk):
        """Returns the number of n(k) shells (0 when n(k) is off)."""
        r = lib().orc_set_operators(self._h, int(ntabg), int(ntabq), int(ntabk))
        if r < 0:
            raise RuntimeError("set_operators failed")
        return r

    def zero_operators(self):
        lib().orc_zero_operators(self._h)

    def add_operators(self):
        lib().orc_add_operators(self._h)

    def update_operators(self):
        lib().orc_update_operators(self._h)

    def operators(self, which, raw=False):
        """which: 0 g(r) [3][ntabg+1], 1 density [6][2 ntabg+1], 2 S(q)
        [3][nqtot], 3 n(k) [ntabk+1]; returns (values, errors, weight sum);
        raw=True gives the running sums before the block update."""
        code = int(which) + (4 if raw else 0)
        n = lib().orc_get_operators(self._h, code, None, None)
        out = np.zeros(2 * max(n, 1))
        ws = C.c_double()
        lib().orc_get_operators(self._h, code, out.ctypes.data_as(C.c_void_p), C.byref(ws))
        return out[:n].copy(), out[n:2 * n].copy(), ws.value

    def wtisto(self):
        h = np.zeros(DMC_WTISTO, np.int64)
        lib().orc_get_wtisto(self._h, h)
        return h


def sr_update(ovec, ovecw, pmat, esum, esum2, nstep, delta0, eps):
    n = len(ovec)
    newp = np.zeros(n)
    eave, eerr = C.c_double(), C.c_double()
    lib().orc_sr_update(n, np.ascontiguousarray(ovec, float), np.ascontiguousarray(ovecw, float),
                        np.asfortranarray(pmat, float).ravel(order="F").copy(), float(esum), float(esum2),
                        int(nstep), float(delta0), float(eps), newp, C.byref(eave), C.byref(eerr))
    return newp, eave.value, eerr.value


__all__ = ["Oracle", "build", "lib", "ran1", "ran2", "gaussian", "matinv", "sr_update", "DMC_NEST_MAX"]
