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


@pytest.mark.parametrize("name", ["dmcbcs.dat", "input.dat"])
def test_reference_decks_parse(name):
    path = os.path.join("/root/reference", name)
    if not os.path.exists(path):
        pytest.skip("reference decks not present")
    s, r, e = deck.load_deck(open(path).read())
    assert s.norb == 10
