"""ctypes mirror of ``include/dmcbcs_gpu.h`` (descriptor structs and constants).

The structs here are the plain-data descriptors of the C ABI; they carry the
deck values read by the reference's set-up routines (dmcbcs.f90:44-66,
wavefunction.f90:36-37, psislaterbcs.f90:47-68, betafun.f90:19-21,
coshpot.f90:35-41) exactly as read.
"""
import ctypes as C

DMC_ABI_VERSION = 1
DMC_MAX_SHELLS = 32
DMC_MAX_UNPAIRED = 16
DMC_MAX_PART = 256
DMC_NEST_MAX = 16
DMC_WTISTO = 500
DMC_MINUSHUGE = -1.0e30

DMC_OK = 0
DMC_ERR_INVALID = 1
DMC_ERR_CUDA = 2
DMC_ERR_UNSUPPORTED = 3
DMC_ERR_OVERFLOW = 4
DMC_ERR_SETUP = 5
DMC_ERR_EMPTY = 6
DMC_ERR_NOMEM = 7
DMC_ERR_NOALLOC_LIMIT = 8
DMC_NOALLOC_MAX_WALKERS = 65536

DMC_JASTROW_KNOTS = 16

# failure flags of dmc_get_status / dmc_walker_status
DMC_STATUS_SINGULAR = 1
DMC_STATUS_NONFINITE = 2
DMC_STATUS_OVERFLOW = 4

STATUS_NAMES = {
    DMC_OK: "ok",
    DMC_ERR_INVALID: "invalid argument",
    DMC_ERR_CUDA: "CUDA error",
    DMC_ERR_UNSUPPORTED: "unsupported",
    DMC_ERR_OVERFLOW: "walker stack overflow",
    DMC_ERR_SETUP: "table set-up failed",
    DMC_ERR_EMPTY: "population died out",
    DMC_ERR_NOMEM: "out of memory",
    DMC_ERR_NOALLOC_LIMIT: "size above the no-allocation scratch maximum",
}


class SystemDesc(C.Structure):
    _fields_ = [
        ("ntab", C.c_int),
        ("hbar", C.c_double),
        ("ndim", C.c_int),
        ("nbin", C.c_int * 2),
        ("mass", C.c_double * 2),
        ("a2", C.c_double),
        ("rho", C.c_double),
        ("nexup", C.c_int),
        ("ikup", (C.c_int * 3) * DMC_MAX_UNPAIRED),
        ("nexdn", C.c_int),
        ("ikdn", (C.c_int * 3) * DMC_MAX_UNPAIRED),
        ("norb", C.c_int),
        ("vorb", C.c_double * DMC_MAX_SHELLS),
        ("nqex", C.c_int * 3),
        ("v0ex", C.c_double),
        ("v0exjas", C.c_double),
        ("numq", C.c_int),
        ("jbeta", C.c_double),
        ("jgamma", C.c_double),
        ("bbeta", C.c_double),
        ("dbeta", C.c_double),
        ("bfact", C.c_double),
        ("v0", C.c_double),
        ("amu", C.c_double),
        ("cjas", C.c_double * 2),
        ("djas", C.c_double),
        ("v0op", C.c_double),
        ("v0eq", C.c_double),
    ]


class RunDesc(C.Structure):
    _fields_ = [
        ("seed", C.c_int64),
        ("idmc", C.c_int),
        ("isite", C.c_int),
        ("nwalk", C.c_int),
        ("neq", C.c_int),
        ("nav", C.c_int),
        ("nstep", C.c_int),
        ("dt", C.c_double),
        ("etrial", C.c_double),
        ("units", C.c_int),
        ("dcut", C.c_double),
        ("fn", C.c_int),
        ("popup", C.c_double),
        ("popdn", C.c_double),
        ("dobal", C.c_double),
        ("wtcut", C.c_double),
        ("stmax", C.c_double),
    ]


class Info(C.Structure):
    _fields_ = [
        ("npart", C.c_int),
        ("nup", C.c_int),
        ("ndn", C.c_int),
        ("npair", C.c_int),
        ("nexup", C.c_int),
        ("nexdn", C.c_int),
        ("nd", C.c_int),
        ("nk", C.c_int),
        ("ncol", C.c_int),
        ("ntab", C.c_int),
        ("capacity", C.c_int),
        ("nest", C.c_int),
        ("el", C.c_double),
        ("eunit", C.c_double),
        ("nfac", C.c_double),
        ("etrial", C.c_double),
        ("sigma", C.c_double * 2),
        ("device_bytes", C.c_int64),
    ]

    def as_dict(self):
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            d[name] = list(v) if name == "sigma" else v
        return d


class Walkers(C.Structure):
    _fields_ = [
        ("n", C.c_int),
        ("x", C.POINTER(C.c_double)),
        ("dpsi", C.POINTER(C.c_double)),
        ("dpsig", C.POINTER(C.c_double)),
        ("psil", C.POINTER(C.c_double)),
        ("psigl", C.POINTER(C.c_double)),
        ("d2psi", C.POINTER(C.c_double)),
        ("d2psig", C.POINTER(C.c_double)),
        ("v", C.POINTER(C.c_double)),
        ("vext", C.POINTER(C.c_double)),
        ("weight", C.POINTER(C.c_double)),
        ("psil0", C.POINTER(C.c_double)),
        ("psigl0", C.POINTER(C.c_double)),
        ("wt0", C.POINTER(C.c_double)),
        ("is_", C.POINTER(C.c_int)),
        ("irn", C.POINTER(C.c_int64)),
    ]


class DevStack(C.Structure):
    """dmc_dev_stack: a walker stack in caller-owned device memory."""
    _fields_ = [(k, C.c_void_p) for k in ("x", "dpsi", "dpsig", "psil", "psigl", "d2psi", "d2psig", "v", "vext",
                                          "weight", "psil0", "psigl0", "wt0", "is_", "irn")]


def _set(struct, name, value):
    field = getattr(struct, name)
    if isinstance(field, C.Array):
        if len(value) > len(field):
            raise ValueError(f"{name}: {len(value)} values, room for {len(field)}")
        for i, v in enumerate(value):
            if isinstance(field[i], C.Array):
                for j, vv in enumerate(v):
                    field[i][j] = vv
            else:
                field[i] = v
    else:
        setattr(struct, name, value)


def make_system(params):
    """Build a :class:`SystemDesc` from a dict of deck values."""
    s = SystemDesc()
    s.ndim = 3
    for k, v in params.items():
        _set(s, k, v)
    return s


def make_run(params):
    """Build a :class:`RunDesc` from a dict of run values."""
    r = RunDesc()
    r.stmax = 10.0
    r.popup, r.popdn, r.wtcut, r.dcut, r.fn, r.units = 1.1, 0.9, 10.0, -1.0, 1, 1
    for k, v in params.items():
        _set(r, k, v)
    return r
