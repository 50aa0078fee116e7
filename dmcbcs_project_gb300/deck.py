"""Reader for the reference's positional stdin deck.

The reference reads its input with list-directed Fortran reads, one record
per value, in the order in which its modules are set up:

* main program, dmcbcs.f90:44-66
* setpsi, wavefunction.f90:36-37 (node type, a2)
* setupbcs, psislaterbcs.f90:47-68
* setbeta, betafun.f90:19-21
* setphi, coshpot.f90:35-41
* setoperators, operators.f90:32-42 (periodic box: four table sizes)
* setupopt when idmc is -1 or -2, optimizer.f90:23-27

A list-directed read takes the values it needs from the start of a record and
ignores the rest, so trailing comments need no special syntax.
"""
from .abi import make_run, make_system


class DeckError(ValueError):
    pass


def _tokens(line):
    return line.replace(",", " ").split()


def _logical(tok):
    t = tok.strip().lower().lstrip(".")
    if t.startswith("t"):
        return True
    if t.startswith("f"):
        return False
    raise DeckError(f"not a logical value: {tok!r}")


class _Reader:
    def __init__(self, text):
        self.lines = text.splitlines()
        self.pos = 0

    def record(self):
        if self.pos >= len(self.lines):
            raise DeckError("deck ended early")
        line = self.lines[self.pos]
        self.pos += 1
        return line

    def values(self, n, conv):
        toks = _tokens(self.record())
        if len(toks) < n:
            raise DeckError(f"line {self.pos}: expected {n} values, got {toks}")
        return [conv(t) for t in toks[:n]]

    def one(self, conv):
        return self.values(1, conv)[0]


def _float(t):
    return float(t.lower().replace("d", "e"))


def parse_deck(text):
    """Parse a deck; returns ``(system_dict, run_dict, extra_dict)``.

    ``system_dict`` and ``run_dict`` feed :func:`abi.make_system` and
    :func:`abi.make_run`; ``extra_dict`` keeps the values this library reads
    but does not consume (operator table sizes, optimizer settings, node
    type)."""
    r = _Reader(text)
    run, sys_, extra = {}, {}, {}
    run["seed"] = r.one(int)
    run["idmc"] = r.one(int)
    run["isite"] = int(r.one(_logical))
    run["nwalk"] = r.one(int)
    run["neq"] = r.one(int)
    run["nav"] = r.one(int)
    run["nstep"] = r.one(int)
    run["dt"] = r.one(_float)
    run["etrial"] = r.one(_float)
    run["units"] = int(r.one(_logical))
    run["dcut"] = r.one(_float)
    run["fn"] = int(r.one(_logical))
    run["popup"] = r.one(_float)
    run["popdn"] = r.one(_float)
    run["dobal"] = r.one(_float)
    run["wtcut"] = r.one(_float)
    sys_["ntab"] = r.one(int)
    sys_["hbar"] = r.one(_float)
    sys_["ndim"] = r.one(int)
    npart = r.one(int)
    n1, m1 = r.values(2, str)
    n2, m2 = r.values(2, str)
    sys_["nbin"] = [int(n1), int(n2)]
    sys_["mass"] = [_float(m1), _float(m2)]
    if sum(sys_["nbin"]) != npart:
        raise DeckError("wrong number of particles")
    nodes = r.record()[:8].strip()
    extra["nodes"] = nodes
    if nodes != "bcs":
        raise DeckError(f"node type {nodes!r}: only 'bcs' is on this path")
    sys_["a2"] = r.one(_float)
    sys_["rho"] = r.one(_float)
    nexup = r.one(int)
    sys_["nexup"] = nexup
    sys_["ikup"] = [r.values(3, int) for _ in range(nexup)]
    nexdn = r.one(int)
    sys_["nexdn"] = nexdn
    sys_["ikdn"] = [r.values(3, int) for _ in range(nexdn)]
    norb = r.one(int)
    sys_["norb"] = norb
    sys_["vorb"] = [r.one(_float) for _ in range(norb)]
    sys_["nqex"] = r.values(3, int)
    sys_["v0ex"] = r.one(_float)
    sys_["v0exjas"] = r.one(_float)
    sys_["numq"] = r.one(int)
    sys_["jbeta"] = r.one(_float)
    sys_["jgamma"] = r.one(_float)
    sys_["bbeta"] = r.one(_float)
    sys_["dbeta"] = r.one(_float)
    sys_["bfact"] = r.one(_float)
    sys_["v0"] = r.one(_float)
    sys_["amu"] = r.one(_float)
    sys_["cjas"] = [r.one(_float), r.one(_float)]
    sys_["djas"] = r.one(_float)
    sys_["v0op"] = r.one(_float)
    sys_["v0eq"] = r.one(_float)
    extra["operators"] = [r.one(int) for _ in range(4)]
    if run["idmc"] in (-1, -2):
        extra["optiter"] = r.one(int)
        extra["iopt"] = [r.one(_logical), r.one(_logical)]
        extra["delta0"] = r.one(_float)
        extra["eps"] = r.one(_float)
    return sys_, run, extra


def load_deck(text):
    """Parse a deck and return ``(SystemDesc, RunDesc, extra)``."""
    s, r, e = parse_deck(text)
    return make_system(s), make_run(r), e
