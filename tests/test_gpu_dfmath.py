"""The mixed path's double-float elementary functions against extended
precision: sin/cos of pi a (orbital base angles 2 pi x / L), sin/cos of
2 pi u for the Box-Muller deviates u = m 2^-48 of ran.f90:74-104, and log
(Box-Muller radius and log|det|).  The references use numpy's long double
(binary128 on aarch64, 80-bit on x86) on the value the device actually sees,
i.e. after the double -> double-float split.  Bars: 2e-14 absolute for
sin/cos, 2e-14 relative to max(1, |log x|) and 1e-13 relative near x = 1."""
import numpy as np
import pytest

from dmcbcs_project_gb300 import capi

pytestmark = pytest.mark.gpu

LD = np.longdouble
PI = LD("3.14159265358979323846264338327950288419716939937510")


def as_df(a):
    """The double a as the device holds it: hi = fl32(a), lo = fl32(a - hi)."""
    a = np.asarray(a, dtype=np.float64)
    hi = a.astype(np.float32).astype(np.float64)
    lo = (a - hi).astype(np.float32).astype(np.float64)
    return hi.astype(LD) + lo.astype(LD)


def test_sincospi_double_float():
    rng = np.random.default_rng(3)
    edges = [0.0, 0.25, -0.25, 0.5, -0.5, 0.75, -0.75, 1.0, -1.0, 1e-9, -3e-12, 0.2500001, 0.7499999,
             1.2, -1.2]
    a = np.concatenate([rng.uniform(-1.25, 1.25, 20000), edges])
    got = capi.dfmath_eval(0, a)
    x = as_df(a)
    es = np.abs(got[:, 0].astype(LD) - np.sin(PI * x)).max()
    ec = np.abs(got[:, 1].astype(LD) - np.cos(PI * x)).max()
    print(f"sin(pi a) max abs err {float(es):.2e}, cos {float(ec):.2e}")
    assert es < 2e-14 and ec < 2e-14


def test_box_muller_angle():
    rng = np.random.default_rng(4)
    m = rng.integers(1, 2 ** 48, size=20000, dtype=np.uint64) | np.uint64(1)
    edges = np.array([1, 2 ** 46 - 1, 2 ** 46 + 1, 2 ** 47 - 1, 2 ** 47 + 1, 3 * 2 ** 46 - 1, 3 * 2 ** 46 + 1,
                      2 ** 45 + 1, 2 ** 48 - 1], dtype=np.uint64)
    m = np.concatenate([m, edges])
    got = capi.dfmath_eval(1, m)
    ang = 2 * PI * (m.astype(LD) / LD(2 ** 48))
    es = np.abs(got[:, 0].astype(LD) - np.sin(ang)).max()
    ec = np.abs(got[:, 1].astype(LD) - np.cos(ang)).max()
    print(f"sin(2 pi u) max abs err {float(es):.2e}, cos {float(ec):.2e}")
    assert es < 2e-14 and ec < 2e-14


def test_log_double_float():
    rng = np.random.default_rng(5)
    u = (rng.integers(1, 2 ** 48, size=10000, dtype=np.uint64) | np.uint64(1)).astype(np.float64) * 2.0 ** -48
    wide = 10.0 ** rng.uniform(-12, 12, size=10000)
    near1 = 1.0 + rng.uniform(-1e-6, 1e-6, size=2000)
    edges = np.array([2.0 ** -48, 1.0 - 2.0 ** -48, 0.5, 2.0, 0.70710678, 0.7071068, 1.4142135, 1.0 + 2.0 ** -40])
    x = np.concatenate([u, wide, near1, edges])
    got = capi.dfmath_eval(2, x).astype(LD)
    ref = np.log(as_df(x))
    err = np.abs(got - ref)
    e_abs = float((err / np.maximum(1.0, np.abs(ref))).max())
    small = (np.abs(ref) < 1e-3) & (ref != 0)
    e_rel = float((err[small] / np.abs(ref[small])).max())
    print(f"log: max err / max(1,|log x|) {e_abs:.2e}; relative near 1 {e_rel:.2e}")
    assert e_abs < 2e-14
    assert e_rel < 1e-13
