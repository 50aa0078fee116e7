"""fort.9 walker files (dmcbcs.f90:254-294 read, :548-567 write) through the
library's context-free C entry points; no GPU is needed.

The expected strings below are what the Fortran edit descriptors produce:
Ew.d writes [-]0.<d digits>E+ee right-justified in w columns and drops the
letter E for a three-digit exponent; formatted input ignores blanks, reads a
blank field as zero, accepts D exponents and signed exponents without a
letter, and places an implied decimal point d digits from the right when the
field has none."""
import os

import numpy as np
import pytest

from dmcbcs_project_gb300 import abi, capi


def _lines(path):
    with open(path) as f:
        return f.read().split("\n")


def test_edit_descriptors_match_fortran(tmp_path):
    p = tmp_path / "fort.9"
    x = np.array([[[1.0, -0.000123456789, 0.0], [12.5022538359, -6.25, 1e120]]])
    capi.fort9_write(p, x, [1.0], [-14.888230832246244], [2.5e-7], [123456789012], tau=0.125)
    lines = _lines(p)
    assert lines[0] == "         1     0.12500000"
    assert lines[1] == ("  0.1000000E+01" " -0.1234568E-03" "  0.0000000E+00"
                        "  0.1250225E+02" " -0.6250000E+01" "  0.1000000+121")
    assert lines[2] == "  0.1000000E+01" + "   -0.148882308322462E+02" + "    0.250000000000000E-06"
    assert lines[3] == "        123456789012"
    assert lines[4] == ""


def test_record_layout_six_values_per_line(tmp_path):
    p = tmp_path / "fort.9"
    npart = 7                                   # 21 values: 6 + 6 + 6 + 3 per walker
    rng = np.random.default_rng(1)
    x = rng.uniform(-4, 4, size=(2, npart, 3))
    capi.fort9_write(p, x, np.ones(2), np.zeros(2), np.zeros(2), [5, 6])
    lines = _lines(p)
    assert [len(l) for l in lines[1:5]] == [90, 90, 90, 45]
    assert len(lines[5]) == 65 and lines[6].strip() == "5"
    assert len(lines) == 1 + 2 * 6 + 1


def test_round_trip(tmp_path):
    p = tmp_path / "fort.9"
    rng = np.random.default_rng(2)
    n, npart = 5, 14
    x = rng.uniform(-3.7, 3.7, size=(n, npart, 3))
    w = rng.uniform(0.1, 3.0, size=n)
    pl = rng.normal(scale=20, size=n)
    pg = rng.normal(scale=20, size=n)
    irn = rng.integers(0, 2 ** 48, size=n)
    capi.fort9_write(p, x, w, pl, pg, irn, tau=3.25)
    r = capi.fort9_read(p, npart)
    assert r["tau"] == 3.25
    assert np.array_equal(r["irn"], irn)
    def half_ulp(v, d):
        # 0.<d digits> x 10^e with e = floor(log10|v|) + 1: half a unit in the last digit
        return 0.5001 * 10.0 ** (np.floor(np.log10(np.abs(v))) + 1 - d)

    assert np.all(np.abs(r["x"] - x) <= half_ulp(x, 7))
    assert np.all(np.abs(r["weight"] - w) <= half_ulp(w, 7))
    assert np.all(np.abs(r["psil0"] - pl) <= half_ulp(pl, 15) + 1e-15 * np.abs(pl))
    assert np.all(np.abs(r["psigl0"] - pg) <= half_ulp(pg, 15) + 1e-15 * np.abs(pg))
    # a second write of what was read is byte-identical
    q = tmp_path / "fort.9b"
    capi.fort9_write(q, r["x"], r["weight"], r["psil0"], r["psigl0"], r["irn"], tau=3.25)
    assert _lines(p) == _lines(q)


def test_pairsconfig_layout_and_fortran_input_forms(tmp_path):
    """pairsconfig.f90:25-37 writes an (i10) header and a weight-only record;
    missing fields read as zero."""
    p = tmp_path / "pairs.9"
    vals = ["  0.5000000D+01", "0.1234567+100  ", "               ", "        1234567", "   -0.25       ", " 1.5E-3        "]
    with open(p, "w") as f:
        f.write("%10d\n" % 1)
        f.write("".join(vals) + "\n")
        f.write("  0.1000000E+01\n")
        f.write("%20d\n" % 987654321)
    r = capi.fort9_read(p, 2)
    assert r["tau"] == 0.0
    assert np.allclose(r["x"][0].ravel(), [5.0, 0.1234567e100, 0.0, 0.1234567, -0.25, 1.5e-3], rtol=1e-15)
    assert r["weight"][0] == 1.0 and r["psil0"][0] == 0.0 and r["psigl0"][0] == 0.0
    assert r["irn"][0] == 987654321


def test_capacity_and_malformed_files(tmp_path):
    p = tmp_path / "fort.9"
    capi.fort9_write(p, np.zeros((3, 1, 3)), np.ones(3), np.zeros(3), np.zeros(3), [1, 2, 3])
    with pytest.raises(capi.DMCError) as e:
        capi.fort9_read(p, 1, cap=2)
    assert e.value.status == abi.DMC_ERR_OVERFLOW
    q = tmp_path / "bad.9"
    with open(q, "w") as f:
        f.write("%10d\n" % 2)
        f.write("  0.1000000E+01  0.2000000E+01  0.3000000E+01\n")
    with pytest.raises(capi.DMCError):
        capi.fort9_read(q, 1)
    with pytest.raises(capi.DMCError):
        capi.fort9_read(os.path.join(tmp_path, "missing.9"), 1)
