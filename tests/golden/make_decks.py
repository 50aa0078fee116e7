"""Parse the reference's two production decks into a committed fixture.

Run from the repository root where the reference tree is present:

    python tests/golden/make_decks.py /path/to/reference

The reference ships two input decks for its walker path:

* ``dmcbcs.dat``: DMC (idmc = 1) at N = 66 (33 up / 33 down), 10 s-wave
  shells with fitted amplitudes, dt = 5e-5, beta b = 0.5, d = 5;
* ``input.dat``: a VMC optimisation (idmc = -1) of a polarised N = 17
  system (9 up / 8 down, one unpaired up plane wave at k = 0), 10 shells,
  both Jastrow strengths on.

The values are read with this library's deck reader (the reference's
positional list-directed order) and written to ``decks.json``, so the GPU
parity tests can run the decks on a machine without the reference tree.
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from dmcbcs_project_gb300 import deck  # noqa: E402

DECKS = ("dmcbcs.dat", "input.dat")


def main(ref_dir):
    out = {}
    for name in DECKS:
        with open(os.path.join(ref_dir, name)) as f:
            s, r, e = deck.parse_deck(f.read())
        out[name] = {"system": s, "run": r, "extra": e}
    path = os.path.join(HERE, "decks.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print(path)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DMCBCS_REFERENCE", "."))
