"""ctypes binding of the C ABI in ``include/dmcbcs_gpu.h`` and a thin
Python front end over it.

This is plumbing for tests and the benchmark: every computation runs in the
CUDA library ``libdmcbcs_gb300.so``.  There is no CPU fallback; loading
fails loudly when the library has not been built.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from .abi import DMC_NEST_MAX, DMC_WTISTO, Info, RunDesc, SystemDesc, Walkers

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdmcbcs_gb300.so")

# the array fields of dmc_walkers: thirteen double arrays, then is and irn
_WALKER_FIELDS = ("x", "dpsi", "dpsig", "psil", "psigl", "d2psi", "d2psig", "v", "vext", "weight", "psil0",
                  "psigl0", "wt0", "is_", "irn")

# every entry point declared in include/dmcbcs_gpu.h
EXPORTS = [
    "dmc_abi_version", "dmc_status_string", "dmc_last_error", "dmc_create", "dmc_destroy", "dmc_get_info",
    "dmc_get_table", "dmc_set_vorb", "dmc_hpsi_batch", "dmc_hpsi_device", "dmc_bcs_batch", "dmc_getphi_batch",
    "dmc_matinv_batch", "dmc_bcsone_batch", "dmc_getphione_batch", "dmc_getderbcs_batch", "dmc_init_walkers",
    "dmc_tune_layout",
    "dmc_load_walkers", "dmc_get_walkers", "dmc_initial_eval", "dmc_num_walkers", "dmc_step", "dmc_branch",
    "dmc_generation", "dmc_zero_estimators", "dmc_get_estimators", "dmc_block_update", "dmc_get_wtisto",
    "dmc_last_step_ms", "dmc_timed_generations", "dmc_put_walkers", "dmc_branch_noalloc",
    "dmc_set_precision", "dmc_get_precision", "dmc_probe_peak", "dmc_sr_accumulate", "dmc_sr_get_sums",
    "dmc_sr_zero", "dmc_sr_update", "dmc_fort9_write", "dmc_fort9_read", "dmc_save_walkers", "dmc_restore_walkers",
    "dmc_set_operators", "dmc_zero_operators", "dmc_add_operators", "dmc_update_operators", "dmc_get_operators",
    "dmc_write_operators", "dmc_getjasder_batch", "dmc_sr_configure", "dmc_dfmath_eval",
    "dmc_batch_create", "dmc_batch_destroy", "dmc_batch_last_error", "dmc_batch_set_grids", "dmc_batch_get_grids",
    "dmc_batch_plan", "dmc_batch_tune", "dmc_batch_generations", "dmc_param_count", "dmc_param_grad",
    "dmc_generation_host", "dmc_get_status", "dmc_walker_status", "dmc_set_jastrow_spline",
    "dmc_get_jastrow_spline", "dmc_set_beta", "dmc_sr_configure_adjoint", "dmc_sm_sweeps", "dmc_sm_inverse",
]

PREC_FP64 = 0
PREC_MIXED = 1

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lp = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


class DMCError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


_lib = None


def _opt(arr):
    return None if arr is None else arr.ctypes.data_as(C.c_void_p)


def load(path=LIB_PATH):
    """Load the CUDA library (built by ``dmcbcs_project_gb300.build``)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: run __graft_entry__.build() (nvcc, sm_103a) first; "
                          "there is no CPU fallback")
    L = C.CDLL(path)
    vp = C.c_void_p
    L.dmc_abi_version.restype = C.c_int
    L.dmc_status_string.restype = C.c_char_p
    L.dmc_status_string.argtypes = [C.c_int]
    L.dmc_last_error.restype = C.c_char_p
    L.dmc_last_error.argtypes = [vp]
    L.dmc_create.argtypes = [C.POINTER(SystemDesc), C.POINTER(RunDesc), C.POINTER(vp)]
    L.dmc_destroy.argtypes = [vp]
    L.dmc_get_info.argtypes = [vp, C.POINTER(Info)]
    L.dmc_get_table.argtypes = [vp, C.c_int, _dp, C.c_int]
    L.dmc_set_vorb.argtypes = [vp, _dp, C.c_int]
    L.dmc_hpsi_batch.argtypes = [vp, C.c_int, _dp] + [vp] * 9
    L.dmc_hpsi_device.argtypes = [vp, C.c_int, vp] + [vp] * 9 + [vp]
    L.dmc_bcs_batch.argtypes = [vp, C.c_int, _dp] + [vp] * 5
    L.dmc_getphi_batch.argtypes = [vp, C.c_int, _dp] + [vp] * 4
    L.dmc_matinv_batch.argtypes = [vp, C.c_int, C.c_int, _dp, _dp, _ip]
    L.dmc_bcsone_batch.argtypes = [vp, C.c_int, _dp, _dp, _ip, _dp, _dp]
    L.dmc_getphione_batch.argtypes = [vp, C.c_int, _dp, _ip, _dp, _dp]
    L.dmc_getderbcs_batch.argtypes = [vp, C.c_int, _dp, _dp]
    L.dmc_init_walkers.argtypes = [vp]
    L.dmc_load_walkers.argtypes = [vp, C.POINTER(Walkers)]
    L.dmc_get_walkers.argtypes = [vp, C.POINTER(Walkers)]
    L.dmc_initial_eval.argtypes = [vp, _dp]
    L.dmc_num_walkers.argtypes = [vp, C.POINTER(C.c_int)]
    L.dmc_step.argtypes = [vp, C.c_int]
    L.dmc_branch.argtypes = [vp, C.c_double]
    L.dmc_generation.argtypes = [vp, C.c_int, C.POINTER(C.c_int)]
    L.dmc_tune_layout.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    L.dmc_zero_estimators.argtypes = [vp]
    L.dmc_get_estimators.argtypes = [vp, _dp, _dp, _dp]
    L.dmc_block_update.argtypes = [vp, _dp, _dp]
    L.dmc_get_wtisto.argtypes = [vp, _lp]
    L.dmc_last_step_ms.argtypes = [vp, C.POINTER(C.c_double)]
    L.dmc_timed_generations.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int64),
                                        C.POINTER(C.c_double), C.POINTER(C.c_int64)]
    L.dmc_put_walkers.argtypes = [vp, C.POINTER(Walkers)]
    L.dmc_set_precision.argtypes = [vp, C.c_int]
    L.dmc_probe_peak.argtypes = [C.c_int, C.POINTER(C.c_double)]
    L.dmc_dfmath_eval.argtypes = [C.c_int, C.c_int, vp, vp]
    L.dmc_get_precision.argtypes = [vp, C.POINTER(C.c_int)]
    L.dmc_fort9_write.argtypes = [C.c_char_p, C.c_int, C.c_int, vp, vp, vp, vp, vp, C.c_double]
    L.dmc_fort9_read.argtypes = [C.c_char_p, C.c_int, C.c_int, vp, vp, vp, vp, vp, C.POINTER(C.c_int),
                                 C.POINTER(C.c_double)]
    L.dmc_save_walkers.argtypes = [vp, C.c_char_p, C.c_double]
    L.dmc_restore_walkers.argtypes = [vp, C.c_char_p, C.POINTER(C.c_double)]
    L.dmc_set_operators.argtypes = [vp, C.c_int, C.c_int, C.c_int]
    L.dmc_zero_operators.argtypes = [vp]
    L.dmc_add_operators.argtypes = [vp]
    L.dmc_update_operators.argtypes = [vp]
    L.dmc_get_operators.argtypes = [vp, C.c_int, vp, vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    L.dmc_write_operators.argtypes = [vp, C.c_char_p, C.c_double]
    L.dmc_getjasder_batch.argtypes = [vp, C.c_int, _dp, _dp]
    L.dmc_sr_configure.argtypes = [vp, C.c_int, C.c_int]
    L.dmc_sr_accumulate.argtypes = [vp, C.POINTER(C.c_int64)]
    L.dmc_sr_get_sums.argtypes = [vp, vp, vp, vp, vp, C.POINTER(C.c_int64)]
    L.dmc_sr_zero.argtypes = [vp]
    L.dmc_sr_update.argtypes = [vp, C.c_double, C.c_double, vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.dmc_branch_noalloc.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.POINTER(abi.DevStack),
                                     C.POINTER(abi.DevStack), vp, C.POINTER(C.c_int), vp]
    L.dmc_generation_host.argtypes = [vp, C.POINTER(Walkers), C.POINTER(Walkers), C.c_int]
    L.dmc_get_status.argtypes = [vp, C.POINTER(C.c_int), C.c_int]
    L.dmc_set_jastrow_spline.argtypes = [vp, vp, C.c_int]
    L.dmc_set_beta.argtypes = [vp, C.c_double, C.c_double, C.c_double]
    L.dmc_sm_sweeps.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.dmc_sm_inverse.argtypes = [vp, C.c_int, _dp]
    L.dmc_sr_configure_adjoint.argtypes = [vp]
    L.dmc_get_jastrow_spline.argtypes = [vp, vp, C.c_int, C.POINTER(C.c_int)]
    L.dmc_walker_status.argtypes = [vp, C.c_int, _ip]
    L.dmc_param_count.argtypes = [vp, C.POINTER(C.c_int)]
    L.dmc_param_grad.argtypes = [vp, C.c_int, _dp, _dp, _dp]
    L.dmc_batch_create.argtypes = [C.POINTER(vp), C.c_int, C.POINTER(vp)]
    L.dmc_batch_destroy.argtypes = [vp]
    L.dmc_batch_last_error.restype = C.c_char_p
    L.dmc_batch_last_error.argtypes = [vp]
    L.dmc_batch_set_grids.argtypes = [vp, _ip]
    L.dmc_batch_get_grids.argtypes = [vp, _ip]
    L.dmc_batch_plan.argtypes = [C.c_int, _dp, _ip, _ip, _ip, C.c_int, _ip]
    L.dmc_batch_tune.argtypes = [vp, C.c_int, _ip, C.POINTER(C.c_double)]
    L.dmc_batch_generations.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int64),
                                        C.POINTER(C.c_double), C.POINTER(C.c_int64)]
    _lib = L
    return L


def dfmath_eval(fn, values):
    """The mixed path's double-float sin/cos (fn 0: of pi a; fn 1: of 2 pi m 2^-48
    for integers m) and log (fn 2), evaluated on the GPU; returns (n, 2) or (n,)."""
    if fn == 1:
        arr = np.ascontiguousarray(values, dtype=np.uint64)
    else:
        arr = np.ascontiguousarray(values, dtype=np.float64)
    n = arr.shape[0]
    out = np.zeros(n if fn == 2 else 2 * n)
    st = load().dmc_dfmath_eval(int(fn), n, _opt(arr), _opt(out))
    if st != abi.DMC_OK:
        raise DMCError(st, "dfmath_eval")
    return out if fn == 2 else out.reshape(n, 2)


def fort9_write(path, x, weight, psil, psigl, irn, tau=0.0):
    """Write walkers (file order) in the reference's fort.9 layout; no GPU used."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    n, npart = x.shape[0], x.shape[1]
    arr = [np.ascontiguousarray(a, dtype=t) for a, t in ((weight, np.float64), (psil, np.float64),
                                                           (psigl, np.float64), (irn, np.int64))]
    st = load().dmc_fort9_write(os.fsencode(path), npart, n, _opt(x), *[_opt(a) for a in arr], float(tau))
    if st != abi.DMC_OK:
        raise DMCError(st, f"fort9_write {path}")


def fort9_read(path, npart, cap=None):
    """Read a fort.9 file; returns dict(x, weight, psil0, psigl0, irn, tau) in file order."""
    n = C.c_int()
    tau = C.c_double()
    st = load().dmc_fort9_read(os.fsencode(path), npart, 0, None, None, None, None, None, C.byref(n), C.byref(tau))
    if st not in (abi.DMC_OK, abi.DMC_ERR_OVERFLOW):
        raise DMCError(st, f"fort9_read {path}")
    m = n.value if cap is None else cap
    o = dict(x=np.zeros((max(m, 1), npart, 3)), weight=np.zeros(max(m, 1)), psil0=np.zeros(max(m, 1)),
             psigl0=np.zeros(max(m, 1)), irn=np.zeros(max(m, 1), np.int64))
    st = load().dmc_fort9_read(os.fsencode(path), npart, m, *[_opt(o[k]) for k in ("x", "weight", "psil0", "psigl0",
                                                                                    "irn")],
                               C.byref(n), C.byref(tau))
    if st != abi.DMC_OK:
        raise DMCError(st, f"fort9_read {path}")
    out = {k: v[: n.value] for k, v in o.items()}
    out["tau"] = tau.value
    return out


def probe_peak(kind):
    """Measured FMA throughput (TFLOP/s) of the FP64 ('fp64') or FP32 ('fp32') pipe."""
    v = C.c_double()
    st = load().dmc_probe_peak({"fp64": 0, "fp32": 1}[kind], C.byref(v))
    if st != abi.DMC_OK:
        raise DMCError(st, "dmc_probe_peak")
    return v.value


def _walker_view(arrs):
    w = Walkers()
    w.n = int(arrs["n"])
    for k in _WALKER_FIELDS[:13]:
        setattr(w, k, arrs[k].ctypes.data_as(C.POINTER(C.c_double)))
    w.is_ = arrs["is_"].ctypes.data_as(C.POINTER(C.c_int))
    w.irn = arrs["irn"].ctypes.data_as(C.POINTER(C.c_int64))
    return w


class Context:
    """One system and run on the current CUDA device (``dmc_create``)."""

    def __init__(self, sysdesc, rundesc, precision="fp64"):
        L = load()
        h = C.c_void_p()
        st = L.dmc_create(C.byref(sysdesc), C.byref(rundesc), C.byref(h))
        if st != abi.DMC_OK:
            raise DMCError(st, "dmc_create failed")
        self._h = h
        self.info = Info()
        self._check(L.dmc_get_info(h, C.byref(self.info)))
        self.npart = self.info.npart
        self.nd = self.info.nd
        self.nest = self.info.nest
        self.norb = int(sysdesc.norb)
        self.set_precision(precision)

    def set_precision(self, precision):
        """'fp64' (plain FP64) or 'mixed' (double-float determinant, FP32 Jastrow)."""
        code = {"fp64": PREC_FP64, "mixed": PREC_MIXED}[precision]
        self._check(load().dmc_set_precision(self._h, code))
        self.precision = precision

    def close(self):
        if getattr(self, "_h", None):
            load().dmc_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, st):
        if st != abi.DMC_OK:
            msg = load().dmc_last_error(self._h)
            raise DMCError(st, msg.decode() if msg else "")

    # ---- set-up -----------------------------------------------------------
    def table(self, which):
        ntab = self.info.ntab
        n = {0: 2, 1: 2, 2: 2, 3: 2}.get(which, 1) * (ntab + 1)
        if which == 7:
            n = 3 * self.info.nk
        elif which == 8:
            n = self.info.nk
        elif which in (9, 10):
            n = self.norb
        elif which == 11:
            n = 2
        elif which == 12:
            n = 3
        out = np.zeros(n)
        self._check(load().dmc_get_table(self._h, which, out, n))
        return out

    def set_vorb(self, vorb):
        v = np.ascontiguousarray(vorb, dtype=np.float64)
        self._check(load().dmc_set_vorb(self._h, v, len(v)))

    # ---- batched evaluation -------------------------------------------------
    def _x(self, x):
        return np.ascontiguousarray(x, dtype=np.float64).reshape(-1, self.npart, 3)

    def hpsi(self, x):
        x = self._x(x)
        nw = x.shape[0]
        o = dict(psil=np.zeros(nw), is_=np.zeros(nw, np.int32), dpsi=np.zeros((nw, self.npart, 3)),
                 d2psi=np.zeros(nw), v=np.zeros(nw), vext=np.zeros(nw), psigl=np.zeros(nw),
                 dpsig=np.zeros((nw, self.npart, 3)), d2psig=np.zeros(nw))
        self._check(load().dmc_hpsi_batch(self._h, nw, x, *[_opt(o[k]) for k in
                                          ("psil", "is_", "dpsi", "d2psi", "v", "vext", "psigl", "dpsig",
                                           "d2psig")]))
        return o

    def bcs(self, x, want_inverse=False):
        x = self._x(x)
        nw = x.shape[0]
        o = dict(phil=np.zeros(nw), is_=np.zeros(nw, np.int32), dphi=np.zeros((nw, self.npart, 3)),
                 d2phi=np.zeros(nw), smati=np.zeros((nw, self.nd * self.nd)) if want_inverse else None)
        self._check(load().dmc_bcs_batch(self._h, nw, x, _opt(o["phil"]), _opt(o["is_"]), _opt(o["dphi"]),
                                         _opt(o["d2phi"]), _opt(o["smati"])))
        return o

    def getphi(self, x):
        x = self._x(x)
        nw = x.shape[0]
        o = dict(u=np.zeros(nw), du=np.zeros((nw, self.npart, 3)), d2u=np.zeros(nw), v=np.zeros(nw))
        self._check(load().dmc_getphi_batch(self._h, nw, x, _opt(o["u"]), _opt(o["du"]), _opt(o["d2u"]),
                                            _opt(o["v"])))
        return o

    def matinv(self, a):
        """Batched rmatinv on a[nb, n, n] (row, col); returns inverse, logdet, sign."""
        a = np.asarray(a, dtype=np.float64)
        nb, n = a.shape[0], a.shape[1]
        f = np.array(np.transpose(a, (0, 2, 1)), dtype=np.float64, order="C").reshape(nb, n * n)   # column-major copy
        d = np.zeros(nb)
        s = np.zeros(nb, np.int32)
        self._check(load().dmc_matinv_batch(self._h, n, nb, f, d, s))
        return np.transpose(f.reshape(nb, n, n), (0, 2, 1)), d, s

    # ---- single-particle moves and parameter derivatives --------------------
    def _moves(self, x, ipart, d):
        x = self._x(x)
        nw = x.shape[0]
        ip = np.ascontiguousarray(np.broadcast_to(np.asarray(ipart, dtype=np.int32), (nw,)))
        d = np.ascontiguousarray(np.broadcast_to(np.asarray(d, dtype=np.float64), (nw, 3)))
        return x, nw, ip, d

    def bcsone(self, x, smati, ipart, dr):
        """Determinant ratio for moving particle ipart (1-based) of each walker
        by -dr (dr = xold - xnew), from the inverse smati returned by bcs()."""
        x, nw, ip, d = self._moves(x, ipart, dr)
        sm = np.ascontiguousarray(smati, dtype=np.float64).reshape(nw, self.nd * self.nd)
        out = np.zeros(nw)
        self._check(load().dmc_bcsone_batch(self._h, nw, x, sm, ip, d, out))
        return out

    def getphione(self, x, ipart, drr):
        """Jastrow ratio exp(U' - U) for the same single-particle moves."""
        x, nw, ip, d = self._moves(x, ipart, drr)
        out = np.zeros(nw)
        self._check(load().dmc_getphione_batch(self._h, nw, x, ip, d, out))
        return out

    def move1(self, x, smati, ipart, xnew):
        """Psi ratio of move1 (wavefunction.f90:393-404): xnew[nw, 3]."""
        x = self._x(x)
        ip = np.broadcast_to(np.asarray(ipart, dtype=np.int64), (x.shape[0],))
        drr = x[np.arange(x.shape[0]), ip - 1] - np.asarray(xnew, dtype=np.float64)
        return self.getphione(x, ipart, drr) * self.bcsone(x, smati, ipart, drr)

    def getderbcs(self, x):
        """d log|det| / d vorb(shell), shape [nw, norb]."""
        x = self._x(x)
        nw = x.shape[0]
        out = np.zeros((nw, self.norb))
        self._check(load().dmc_getderbcs_batch(self._h, nw, x, out))
        return out

    def save_walkers(self, path, tau=0.0):
        """Write the population to a fort.9 file (top of the stack first)."""
        self._check(load().dmc_save_walkers(self._h, os.fsencode(path), float(tau)))

    def restore_walkers(self, path):
        """Push the walkers of a fort.9 file; returns its tau."""
        t = C.c_double()
        self._check(load().dmc_restore_walkers(self._h, os.fsencode(path), C.byref(t)))
        return t.value

    # ---- operators: g(r) + density profile, S(q), n(k) ----------------------
    def set_operators(self, ntabg, ntabq, ntabk):
        self._check(load().dmc_set_operators(self._h, int(ntabg), int(ntabq), int(ntabk)))

    def zero_operators(self):
        self._check(load().dmc_zero_operators(self._h))

    def add_operators(self):
        self._check(load().dmc_add_operators(self._h))

    def update_operators(self):
        self._check(load().dmc_update_operators(self._h))

    def operators(self, which, raw=False):
        """which: 0 g(r) [3][ntabg+1], 1 density [6][2 ntabg+1], 2 S(q)
        [3][nqtot], 3 n(k); returns (values, errors, weight sum); raw=True:
        the running sums before the block update."""
        code = int(which) + (4 if raw else 0)
        n = C.c_int()
        ws = C.c_double()
        self._check(load().dmc_get_operators(self._h, code, None, None, 0, C.byref(n), None))
        v, e = np.zeros(max(n.value, 1)), np.zeros(max(n.value, 1))
        self._check(load().dmc_get_operators(self._h, code, _opt(v), _opt(e), n.value, C.byref(n), C.byref(ws)))
        return v[: n.value], e[: n.value], ws.value

    def write_operators(self, directory, tau=0.0):
        self._check(load().dmc_write_operators(self._h, os.fsencode(str(directory)), float(tau)))

    def param_count(self):
        n = C.c_int()
        self._check(load().dmc_param_count(self._h, C.byref(n)))
        return n.value

    def param_grad(self, x):
        """Adjoint gradients for theta = (vorb(1..norb)[, bfact, b, d][, the
        16 Jastrow knots]): returns (d log|Psi|/d theta, d E_L/d theta), each
        (nw, np)."""
        x = self._x(x)
        nw, np_ = x.shape[0], self.param_count()
        dl = np.zeros((nw, np_))
        de = np.zeros((nw, np_))
        self._check(load().dmc_param_grad(self._h, nw, x.reshape(-1), dl.reshape(-1), de.reshape(-1)))
        return dl, de

    def getjasder(self, x):
        """d U_long / d beta, d U_long / d gamma per walker, shape [nw, 2]."""
        x = self._x(x)
        out = np.zeros((x.shape[0], 2))
        self._check(load().dmc_getjasder_batch(self._h, x.shape[0], x, out))
        return out

    def sr_configure(self, opt_jastrow, opt_det):
        self._check(load().dmc_sr_configure(self._h, int(bool(opt_jastrow)), int(bool(opt_det))))
        self._nparm = 2 * bool(opt_jastrow) + self.norb * bool(opt_det)

    @property
    def nparm(self):
        return getattr(self, "_nparm", self.norb)

    def sr_accumulate(self):
        n = C.c_int64()
        self._check(load().dmc_sr_accumulate(self._h, C.byref(n)))
        return n.value

    def sr_sums(self):
        npr = self.nparm
        o = dict(ovec=np.zeros(npr), ovecw=np.zeros(npr), pmat=np.zeros(npr * npr), e=np.zeros(2))
        n = C.c_int64()
        self._check(load().dmc_sr_get_sums(self._h, *[_opt(o[k]) for k in ("ovec", "ovecw", "pmat", "e")],
                                           C.byref(n)))
        o["pmat"] = o["pmat"].reshape(npr, npr, order="F")
        o["n"] = n.value
        return o

    def sr_zero(self):
        self._check(load().dmc_sr_zero(self._h))

    def sr_update(self, delta0, eps):
        """One SR step; returns (newpars, eave, eerr) and applies newpars to vorb."""
        newp = np.zeros(self.nparm)
        ea, ee = C.c_double(), C.c_double()
        self._check(load().dmc_sr_update(self._h, float(delta0), float(eps), _opt(newp), C.byref(ea),
                                         C.byref(ee)))
        return newp, ea.value, ee.value

    # ---- population ----------------------------------------------------------
    def init_walkers(self):
        self._check(load().dmc_init_walkers(self._h))

    def load_walkers(self, x, irn, weight=None, psil0=None, psigl0=None):
        x = self._x(x)
        n = x.shape[0]
        irn = np.ascontiguousarray(irn, dtype=np.int64)
        keep = [x, irn]
        w = Walkers()
        w.n = n
        w.x = x.ctypes.data_as(C.POINTER(C.c_double))
        w.irn = irn.ctypes.data_as(C.POINTER(C.c_int64))
        for name, arr in (("weight", weight), ("psil0", psil0), ("psigl0", psigl0)):
            if arr is not None:
                a = np.ascontiguousarray(arr, dtype=np.float64)
                keep.append(a)
                setattr(w, name, a.ctypes.data_as(C.POINTER(C.c_double)))
        self._check(load().dmc_load_walkers(self._h, C.byref(w)))

    def num_walkers(self):
        n = C.c_int()
        self._check(load().dmc_num_walkers(self._h, C.byref(n)))
        return n.value

    def walkers(self):
        n = self.num_walkers()
        cap = max(n, 1)
        arrs = {k: np.zeros((cap, self.npart, 3)) for k in ("x", "dpsi", "dpsig")}
        for k in ("psil", "psigl", "d2psi", "d2psig", "v", "vext", "weight", "psil0", "psigl0", "wt0"):
            arrs[k] = np.zeros(cap)
        arrs["is_"] = np.zeros(cap, np.int32)
        arrs["irn"] = np.zeros(cap, np.int64)
        w = Walkers()
        w.n = cap
        for k, a in arrs.items():
            ct = {np.dtype(np.float64): C.c_double, np.dtype(np.int32): C.c_int, np.dtype(np.int64): C.c_int64}[a.dtype]
            setattr(w, k, a.ctypes.data_as(C.POINTER(ct)))
        self._check(load().dmc_get_walkers(self._h, C.byref(w)))
        out = {k: a[:n] for k, a in arrs.items()}
        out["n"] = n
        return out

    def initial_eval(self):
        s = np.zeros(11)
        self._check(load().dmc_initial_eval(self._h, s))
        return s[:9], s[9:11]

    def step(self, opcomp):
        self._check(load().dmc_step(self._h, int(bool(opcomp))))

    def branch(self, factor):
        self._check(load().dmc_branch(self._h, float(factor)))

    def generation(self, opcomp):
        nt = C.c_int()
        self._check(load().dmc_generation(self._h, int(bool(opcomp)), C.byref(nt)))
        return nt.value

    def zero_estimators(self):
        self._check(load().dmc_zero_estimators(self._h))

    def estimators(self):
        a, b, c = np.zeros(self.nest), np.zeros(self.nest), np.zeros(self.nest)
        self._check(load().dmc_get_estimators(self._h, a, b, c))
        return a, b, c

    def block_update(self):
        a, b = np.zeros(self.nest), np.zeros(self.nest)
        self._check(load().dmc_block_update(self._h, a, b))
        return a, b

    def wtisto(self):
        h = np.zeros(DMC_WTISTO, np.int64)
        self._check(load().dmc_get_wtisto(self._h, h))
        return h

    def tune_layout(self, passes=3):
        """dmc_tune_layout: time the candidate walker layouts on the current
        walkers and keep the fastest; returns (kind, ms per evaluation)."""
        k, ms = C.c_int(), C.c_double()
        self._check(load().dmc_tune_layout(self._h, int(passes), C.byref(k), C.byref(ms)))
        return k.value, ms.value

    def timed_generations(self, ngen, opcomp_last=True, flush_l2=True):
        """Run ngen generations; returns (walker_steps, device_ms, kernel_launches)."""
        st, ms, nl = C.c_int64(), C.c_double(), C.c_int64()
        self._check(load().dmc_timed_generations(self._h, int(ngen), int(bool(opcomp_last)), int(bool(flush_l2)),
                                                 C.byref(st), C.byref(ms), C.byref(nl)))
        return st.value, ms.value, nl.value

    def walker_struct(self, arrs, slot=None):
        """dmc_walkers view of a dict of arrays (as returned by walkers()).

        With a slot name the view is kept for the next call with the same
        array objects in that slot (only n is set again): a host that hands
        the same population arrays over every generation pays the fifteen
        pointer conversions once.  The cache holds references to the arrays,
        so their ids (and data pointers) stay theirs while cached."""
        if slot is not None:
            key = (slot,) + tuple(id(arrs[k]) for k in _WALKER_FIELDS)
            cache = self.__dict__.setdefault("_wcache", {})
            hit = cache.get(key)
            if hit is None:
                if len(cache) >= 8:
                    cache.pop(next(iter(cache)))
                hit = (_walker_view(arrs), [arrs[k] for k in _WALKER_FIELDS])
                cache[key] = hit
            hit[0].n = int(arrs["n"])
            return hit[0]
        return _walker_view(arrs)

    def put_walkers(self, arrs):
        self._check(load().dmc_put_walkers(self._h, C.byref(self.walker_struct(arrs))))

    def generation_host(self, arrs_in, arrs_out, opcomp):
        """One generation on a population held in host arrays (dicts as for
        put_walkers; arrs_out['cap'] is its capacity); returns the new count."""
        wi = self.walker_struct(arrs_in, "in")
        wo = self.walker_struct(dict(arrs_out, n=arrs_out["cap"]), "out")
        self._check(load().dmc_generation_host(self._h, C.byref(wi), C.byref(wo), int(bool(opcomp))))
        return wo.n

    def get_walkers_into(self, arrs):
        """dmc_get_walkers into caller-owned arrays (capacity arrs['cap']); returns n."""
        w = self.walker_struct(dict(arrs, n=arrs["cap"]))
        self._check(load().dmc_get_walkers(self._h, C.byref(w)))
        return w.n

    def set_jastrow_spline(self, knots):
        """The opt-in up-down Jastrow spline (16 knots; None or [] = off)."""
        k = np.ascontiguousarray(knots if knots is not None else [], dtype=np.float64)
        self._check(load().dmc_set_jastrow_spline(self._h, _opt(k) if k.size else None, int(k.size)))

    def set_beta(self, b, d, bfact):
        """New b, d and bfact of the beta function (tables rebuilt)."""
        self._check(load().dmc_set_beta(self._h, float(b), float(d), float(bfact)))

    def sr_configure_adjoint(self):
        """SR over every adjoint-gradient parameter."""
        self._check(load().dmc_sr_configure_adjoint(self._h))
        self._nparm = self.param_count()

    def beta_params(self):
        """(bfact, b, d) of the beta function."""
        return self.table(12)

    def jastrow_spline(self):
        n = C.c_int()
        buf = np.zeros(abi.DMC_JASTROW_KNOTS)
        self._check(load().dmc_get_jastrow_spline(self._h, _opt(buf), buf.size, C.byref(n)))
        return buf[:n.value].copy()

    def sm_sweeps(self, nsweeps, recompute_every=16):
        """Particle-by-particle sweeps with FP32 Sherman-Morrison updates;
        returns (accepted, moves)."""
        a, m = C.c_int64(), C.c_int64()
        self._check(load().dmc_sm_sweeps(self._h, int(nsweeps), int(recompute_every), C.byref(a), C.byref(m)))
        return a.value, m.value

    def sm_inverse(self, nw):
        """The FP32 inverses carried by the last sweeps, (nw, nd, nd) with
        [w, r, c] = (S^-1)_{rc}."""
        out = np.zeros(nw * self.nd * self.nd)
        self._check(load().dmc_sm_inverse(self._h, int(nw), out))
        return out.reshape(nw, self.nd, self.nd).transpose(0, 2, 1)

    def status(self, clear=False):
        """DMC_STATUS_* flags met since the last clear (dmc_get_status)."""
        f = C.c_int()
        self._check(load().dmc_get_status(self._h, C.byref(f), int(bool(clear))))
        return f.value

    def walker_status(self, nw):
        """Per-walker DMC_STATUS_* flags of the last batched evaluation."""
        out = np.zeros(nw, np.int32)
        self._check(load().dmc_walker_status(self._h, int(nw), out))
        return out

    def last_step_ms(self):
        ms = C.c_double()
        self._check(load().dmc_last_step_ms(self._h, C.byref(ms)))
        return ms.value


def batch_plan(tau, nw, per_sm, maxgrid, nsm):
    """The batch tuner's host-only split (dmc_batch_plan): CTAs per system."""
    ns = len(tau)
    grids = np.zeros(ns, dtype=np.int32)
    st = load().dmc_batch_plan(ns, np.ascontiguousarray(tau, dtype=np.float64),
                               np.ascontiguousarray(nw, dtype=np.int32), np.ascontiguousarray(per_sm, dtype=np.int32),
                               np.ascontiguousarray(maxgrid, dtype=np.int32), int(nsm), grids)
    if st != abi.DMC_OK:
        raise DMCError(st, "dmc_batch_plan")
    return grids


class Batch:
    """Several contexts (systems of uneven size) advanced together, one CUDA
    graph per generation (``dmc_batch_create``)."""

    def __init__(self, contexts):
        L = load()
        self.contexts = list(contexts)
        arr = (C.c_void_p * len(self.contexts))(*[c._h.value for c in self.contexts])
        h = C.c_void_p()
        st = L.dmc_batch_create(arr, len(self.contexts), C.byref(h))
        if st != abi.DMC_OK:
            raise DMCError(st, "dmc_batch_create failed")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            load().dmc_batch_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, st):
        if st != abi.DMC_OK:
            msg = load().dmc_batch_last_error(self._h)
            raise DMCError(st, msg.decode() if msg else "")

    @property
    def grids(self):
        g = np.zeros(len(self.contexts), dtype=np.int32)
        self._check(load().dmc_batch_get_grids(self._h, g))
        return g

    @grids.setter
    def grids(self, values):
        self._check(load().dmc_batch_set_grids(self._h, np.ascontiguousarray(values, dtype=np.int32)))

    def tune(self, rounds=3):
        """Autotune the CTA split; returns (grids, pass_ms)."""
        g = np.zeros(len(self.contexts), dtype=np.int32)
        ms = C.c_double()
        self._check(load().dmc_batch_tune(self._h, int(rounds), g, C.byref(ms)))
        return g, ms.value

    def generations(self, ngen, opcomp_last=True, flush_l2=False):
        """ngen batched generations; returns (walker_steps, device_ms, kernel_launches)."""
        st, ms, nl = C.c_int64(), C.c_double(), C.c_int64()
        self._check(load().dmc_batch_generations(self._h, int(ngen), int(bool(opcomp_last)), int(bool(flush_l2)),
                                                 C.byref(st), C.byref(ms), C.byref(nl)))
        return st.value, ms.value, nl.value


__all__ = ["Context", "Batch", "DMCError", "load", "EXPORTS", "LIB_PATH", "DMC_NEST_MAX", "fort9_write",
           "fort9_read", "dfmath_eval", "batch_plan"]
