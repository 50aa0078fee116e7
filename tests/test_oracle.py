"""Pins of the CPU oracle (no GPU).

The reference ships no golden outputs and cannot be built here, so the
oracle is pinned piece by piece: random numbers against the integer
recurrence, the dense inverse against LAPACK, the wavefunction against
analytic answers and against the finite-difference self-checks the
reference itself carries (chkder, chkone: wavefunction.f90:289-391;
chkderp: optimizer.f90:171-225).
"""
import json
import os

import numpy as np
import pytest

import oracle
from dmcbcs_project_gb300 import abi, configs

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


# ---- random numbers (ran.f90) ---------------------------------------------

def test_rng_golden():
    g = json.load(open(os.path.join(GOLD, "rng.json")))
    fn = {"ran1": oracle.ran1, "ran2": oracle.ran2}
    for name, per_seed in g.items():
        for seed, seq in per_seed.items():
            s = int(seed)
            for e in seq:
                u, s = fn[name](s)
                assert s == e["state"]
                assert u == e["u"]


def test_gaussian_box_muller():
    g = json.load(open(os.path.join(GOLD, "rng.json")))
    seq = g["ran1"]["17"]
    for n in (6, 7):
        out, st = oracle.gaussian(17, n)
        u = [e["u"] for e in seq]
        exp = []
        for i in range(n // 2):
            r = np.sqrt(-2.0 * np.log(u[2 * i + 1]))
            a = 2.0 * np.pi * u[2 * i]
            exp += [np.sin(a) * r, np.cos(a) * r]
        if n % 2:
            exp.append(np.cos(2.0 * np.pi * u[n - 1]) * np.sqrt(-2.0 * np.log(u[n])))
        assert np.allclose(out, exp, rtol=1e-14, atol=1e-15)
        assert st == seq[2 * ((n + 1) // 2) - 1]["state"]


# ---- dense inverse (matrixlapack.f90 + LAPACK) ------------------------------

def test_matinv_lapack_golden():
    d = np.load(os.path.join(GOLD, "lapack.npz"))
    k = 0
    while f"a{k}" in d:
        inv, ld, s, info = oracle.matinv(d[f"a{k}"])
        assert info == 0
        assert s == int(d[f"sign{k}"])
        assert abs(ld - float(d[f"logdet{k}"])) < 1e-12 * max(1, abs(float(d[f"logdet{k}"])))
        ref = d[f"inv{k}"]
        assert np.max(np.abs(inv - ref)) < 1e-12 * max(1.0, np.max(np.abs(ref)))
        k += 1
    assert k >= 6


def test_matinv_singular_and_sign():
    a = np.array([[1.0, 2.0], [2.0, 4.0]])
    _, ld, _, info = oracle.matinv(a)
    assert info > 0 and ld == abi.DMC_MINUSHUGE
    p = np.array([[0.0, 1.0], [1.0, 0.0]])          # a permutation: det = -1
    inv, ld, s, info = oracle.matinv(p)
    assert info == 0 and s == -1 and abs(ld) < 1e-15
    assert np.allclose(inv, p)


# ---- set-up tables ----------------------------------------------------------

def test_kshell_counts():
    g = json.load(open(os.path.join(GOLD, "kshell.json")))
    sysd, rund, _ = configs.workload("n66", nwalk=4)
    sysd.norb = 10
    for i in range(10):
        sysd.vorb[i] = 0.5 ** i
    o = oracle.Oracle(sysd, rund, threads=1)
    numsh = o.table(9)[:10]
    assert list(numsh.astype(int)) == g["count"][:10]
    ak = o.table(7).reshape(-1, 3) * o.info.el / (2 * np.pi)
    n2 = np.rint(np.sum(ak ** 2, axis=1)).astype(int)
    assert list(n2) == sorted(n2)                     # shells in increasing |n|^2
    vecs = {tuple(np.rint(v).astype(int)) for v in ak}
    assert len(vecs) == len(ak)                       # no vector twice
    assert all(tuple(-np.array(v)) not in vecs for v in vecs if any(v))   # half set only


def test_jastrow_and_potential_tables():
    sysd, rund, _ = configs.workload("n66", nwalk=4)
    o = oracle.Oracle(sysd, rund, threads=1)
    nt = o.info.ntab + 1
    u, du, d2u, vt = (o.table(i).reshape(2, nt) for i in range(4))
    el = o.info.el
    dr = 0.5 * el / o.info.ntab
    n0 = int(o.info.ntab * sysd.djas / (0.5 * el))
    assert u[0, n0] == 0.0 and np.all(u[0, n0:] == 0.0)   # log f = 0 from the healing distance on
    assert abs(du[0, n0]) < 1e-7                          # f'/f converged to 0 there
    assert np.all(du[0, n0 + 1:] == 0.0) and np.all(d2u[0, n0 + 1:] == 0.0)
    assert np.all(u[1] == 0.0)                            # no same-spin Jastrow (cjas(2)=0)
    mu = sysd.amu
    assert abs(vt[0, 0] - (-2.0 * sysd.v0 * mu * mu * 1.0)) < 1e-9
    r = np.arange(nt) * dr
    assert np.allclose(vt[0], -2.0 * mu * mu / np.cosh(mu * r) ** 2, rtol=1e-12, atol=1e-300)
    assert np.all(vt[1] == 0.0)
    # u'' table is f''/f - (f'/f)^2: check against finite differences of u' inside the Jastrow range
    i = np.arange(50, n0 - 50, 97)
    fd = (du[0, i + 1] - du[0, i - 1]) / (2 * dr)
    assert np.allclose(d2u[0, i], fd, rtol=1e-4, atol=1e-6)


@pytest.mark.parametrize("ic", [0, 1])
def test_jastrow_table_solves_the_pair_equation(ic):
    """The RK4 + bisection Jastrow (rungekutta.f90:8-100, coshpot.f90:90-133)
    for non-zero effective interactions, against an independent solve of the
    same radial equation f'' + 2 f'/r = (v(r) - E) f / hbar: E from the
    tables' own residual, f integrated from the origin with scipy's adaptive
    Runge-Kutta, u = cjas ln(f / f(d)) compared on the grid up to the healing
    distance d, where f' vanishes."""
    integrate = pytest.importorskip("scipy.integrate")
    sp = configs.system_params(33, 33, 7)
    sp.update(v0op=0.5, v0eq=-0.5, cjas=[1.0, 0.7])
    sysd = abi.make_system(sp)
    o = oracle.Oracle(sysd, abi.make_run(configs.run_params(4, 0.001)), threads=1)
    nt = o.info.ntab + 1
    u, du, d2u = (o.table(i).reshape(2, nt)[ic] for i in range(3))
    cj = sysd.cjas[ic]
    dr = 0.5 * o.info.el / o.info.ntab
    n0 = int(o.info.ntab * sysd.djas / (0.5 * o.info.el))
    v0 = (sysd.v0op, sysd.v0eq)[ic]
    hb, mu = sysd.hbar, sysd.amu
    vpot = lambda r: -2.0 * v0 * mu * mu * hb / np.cosh(mu * r) ** 2
    i = np.arange(5, n0, 11)
    r = i * dr
    # the tables are cjas ln f, cjas f'/f, cjas (f''/f - (f'/f)^2)
    a, b, c = u[i] / cj, du[i] / cj, d2u[i] / cj
    e_res = -hb * (c + b * b + 2.0 * b / r - vpot(r) / hb)
    assert np.ptp(e_res) < 1e-9 * max(1.0, abs(e_res.mean()))
    ene = float(e_res.mean())
    assert ene < 0.0 if v0 > 0 else ene > 0.0      # bound (attractive) or scattering (repulsive)

    def rhs(rr, y):
        return [y[1], (vpot(rr) - ene) * y[0] / hb - 2.0 * y[1] / rr]

    r0 = 1e-6
    f0 = 1.0 + (vpot(0.0) - ene) * r0 * r0 / (6.0 * hb)
    sol = integrate.solve_ivp(rhs, (r0, n0 * dr), [f0, (vpot(0.0) - ene) * r0 / (3.0 * hb)],
                              t_eval=np.append(r, n0 * dr), rtol=1e-12, atol=1e-14, method="DOP853")
    f = sol.y[0]
    lnf = np.log(f[:-1] / f[-1])
    print(f"ic={ic}: E = {ene:.6g}, max |ln f - u| = {np.max(np.abs(lnf - a)):.2e}, "
          f"max |f'/f - du| = {np.max(np.abs(sol.y[1][:-1] / f[:-1] - b)):.2e}")
    assert np.max(np.abs(lnf - a)) < 1e-6 * max(1.0, np.max(np.abs(a)))
    assert np.max(np.abs(sol.y[1][:-1] / f[:-1] - b)) < 1e-5 * max(1.0, np.max(np.abs(b)))
    assert abs(du[n0]) < 1e-6 and np.max(np.abs(a)) > 0.1        # f'(d) = 0; a non-trivial Jastrow


def test_beta_table():
    sysd, rund, _ = configs.workload("n14", nwalk=4)
    o = oracle.Oracle(sysd, rund, threads=1)
    b, db, d2b = o.table(4), o.table(5), o.table(6)
    assert b[-1] == 0.0                          # shifted to zero at L/2
    assert db[0] == 0.0
    dr = 0.5 * o.info.el / o.info.ntab
    i = np.arange(100, o.info.ntab - 100, 211)
    fd = (b[i + 1] - b[i - 1]) / (2 * dr)
    assert np.allclose(db[i], fd, rtol=1e-5, atol=1e-8)
    # beyond L/2 the radial function is zero
    assert np.all(o.radialfun(0.5 * o.info.el * 1.0001) == 0.0)


# ---- known answers ------------------------------------------------------------

def free_gas(nwalk=8):
    """7 up + 7 down with phi = sum of the 7 lowest plane waves: closed-shell
    free Fermi gas, E_L = 2 * sum_k k^2/2 exactly."""
    sp = configs.system_params(7, 7, 2)
    sp.update(vorb=[1.0, 1.0], bfact=0.0, cjas=[0.0, 0.0], v0=0.0)
    return abi.make_system(sp), abi.make_run(configs.run_params(nwalk, 0.002))


def test_free_fermi_gas_energy():
    sysd, rund = free_gas()
    o = oracle.Oracle(sysd, rund, threads=1)
    rng = np.random.default_rng(1)
    x = rng.uniform(-0.5, 0.5, size=(16, 14, 3)) * o.info.el
    h = o.hpsi(x)
    k2 = (2 * np.pi / o.info.el) ** 2
    e_free = 2 * 0.5 * 6 * k2                      # two spins, six |k|=2pi/L waves, hbar^2/2m = 0.5
    el = -0.5 * h["d2psi"] + h["v"]
    assert np.allclose(el, e_free, rtol=1e-10)
    assert np.all(h["v"] == 0.0)


def test_single_pair_is_pair_function():
    sp = configs.system_params(1, 1, 3)
    sp.update(cjas=[0.0, 0.0], v0=0.0)
    sysd, rund = abi.make_system(sp), abi.make_run(configs.run_params(4, 0.002))
    o = oracle.Oracle(sysd, rund, threads=1)
    el = o.info.el
    rng = np.random.default_rng(2)
    ak = o.table(7).reshape(-1, 3)
    numsh = o.table(9).astype(int)
    for _ in range(5):
        x = rng.uniform(-0.5, 0.5, size=(2, 3)) * el
        d = x[0] - x[1]
        d -= el * np.round(d / el)
        phi = sysd.vorb[0]
        k = 1
        for sh in range(1, sysd.norb):
            for _ in range(numsh[sh]):
                phi += 2 * sysd.vorb[sh] * np.cos(ak[k] @ (x[0] - x[1]))
                k += 1
        phi += o.radialfun(np.linalg.norm(d))[0]
        h = o.hpsi(x[None])
        assert abs(h["psil"][0] - np.log(abs(phi))) < 1e-12
        assert h["is_"][0] == (1 if phi > 0 else -1)


# ---- finite-difference self-checks (the reference's chkder/chkone/chkderp) ----

def _near_half_box(x, nup, el, ntab, cells=6):
    """True if an up-down pair is within `cells` table spacings of L/2.

    The reference's beta table has a doubled second derivative at its last
    point r = L/2 (betafun.f90:106-112: the image term beta(el-r) equals
    beta(L/2) there), so the tabulated Laplacian and the tabulated values
    disagree within two spacings of L/2; finite differences must stay away."""
    d = x[:nup, None, :] - x[None, nup:, :]
    d -= el * np.round(d / el)
    r = np.linalg.norm(d, axis=-1)
    return bool(np.any(np.abs(r - 0.5 * el) < cells * 0.5 * el / ntab))


def _walkers(name, nw, seed=11, longrange=None):
    sysd, rund, _ = configs.workload(name, nwalk=nw, seed=seed, longrange=longrange)
    o = oracle.Oracle(sysd, rund, threads=1)
    o.init_walkers()
    base = o.walkers()["x"]
    rng = np.random.default_rng(seed)
    out = []
    for w in range(nw):
        while True:
            x = base[w] + rng.normal(scale=0.2, size=(o.npart, 3))
            if not _near_half_box(x, o.info.nup, o.info.el, o.info.ntab):
                break
        out.append(x)
    return sysd, o, np.array(out)


@pytest.mark.parametrize("name,longrange", [("n14", None), ("p38_33", None), ("n14", (3, 1.0, 0.3))])
def test_chkder_gradient_and_laplacian(name, longrange):
    """wavefunction.f90:289-321: central differences of log|Psi| give dpsi;
    differences of dpsi*Psi give the Laplacian d2psi (also with the
    long-range Jastrow of jastrowlongrange.f90 on)."""
    sysd, o, x = _walkers(name, 1, longrange=longrange)
    x = x[0]
    h0 = o.hpsi(x[None])
    h = 1e-5
    d2num = 0.0
    for i in range(o.npart):
        for c in range(3):
            xp = x.copy(); xp[i, c] += h
            xm = x.copy(); xm[i, c] -= h
            hp, hm = o.hpsi(xp[None]), o.hpsi(xm[None])
            dnum = (hp["psil"][0] - hm["psil"][0]) / (2 * h)
            assert abs(h0["dpsi"][0, i, c] - dnum) < 1e-5 * max(1.0, abs(dnum)), (i, c)
            gp = hp["dpsi"][0, i, c] * np.exp(hp["psil"][0] - h0["psil"][0])
            gm = hm["dpsi"][0, i, c] * np.exp(hm["psil"][0] - h0["psil"][0])
            d2num += (gp - gm) / (2 * h)
    assert abs(d2num - h0["d2psi"][0]) < 1e-4 * max(1.0, abs(h0["d2psi"][0]))


@pytest.mark.parametrize("name", ["n14", "p38_33"])
def test_chkone_single_particle_ratios(name):
    """wavefunction.f90:351-391: bcsone and getphione against full recomputes."""
    sysd, o, x = _walkers(name, 1, seed=4)
    x = x[0]
    b0 = o.bcs(x[None], want_inverse=True)
    sinv = b0["smati"][0]
    rng = np.random.default_rng(8)
    for i1 in (1, o.npart // 2, o.npart):
        dr = rng.normal(scale=0.3, size=3)
        xn = x.copy()
        xn[i1 - 1] -= dr
        b1 = o.bcs(xn[None])
        rat_full = np.exp(b1["phil"][0] - b0["phil"][0]) * b1["is_"][0] * b0["is_"][0]
        rat = o.bcsone(x, dr, i1, sinv)
        assert abs(rat - rat_full) < 1e-9 * max(1.0, abs(rat_full))
        j0, j1 = o.getphi(x), o.getphi(xn)
        assert abs(o.getphione(x, dr, i1) - np.exp(j1["u"] - j0["u"])) < 1e-10 * np.exp(j1["u"] - j0["u"])


def test_chkderp_vorb_derivatives():
    """optimizer.f90:171-225: d log|det| / d vorb(k) against central differences."""
    sysd, o, x = _walkers("n14", 1, seed=6)
    x = x[0]
    d = o.getderbcs(x)
    vorb = np.array(sysd.vorb[: sysd.norb])
    hstep = 1e-6
    for k in range(sysd.norb):
        vp, vm = vorb.copy(), vorb.copy()
        vp[k] += hstep
        vm[k] -= hstep
        o.set_vorb(vp)
        lp = o.bcs(x[None])["phil"][0]
        o.set_vorb(vm)
        lm = o.bcs(x[None])["phil"][0]
        o.set_vorb(vorb)
        fd = (lp - lm) / (2 * hstep)
        assert abs(d[k] - fd) < 1e-6 * max(1.0, abs(fd)), (k, d[k], fd)


# ---- population dynamics -------------------------------------------------------

def test_generation_independent_of_threads():
    res = []
    for threads in (1, 4):
        sysd, rund, _ = configs.workload("n14", nwalk=40)
        o = oracle.Oracle(sysd, rund, threads=threads)
        o.init_walkers()
        o.initial_eval()
        for g in range(4):
            o.generation(g == 3)
        res.append((o.walkers(), o.estimators()))
    (w1, e1), (w2, e2) = res
    assert np.array_equal(w1["x"], w2["x"]) and np.array_equal(w1["irn"], w2["irn"])
    assert all(np.array_equal(a, b) for a, b in zip(e1, e2))


def _fnint(a):
    return np.sign(a) * np.floor(np.abs(a) + 0.5)


def test_gf_step_restates_step_f90():
    """idmc = 10 (step.f90:231-279) restated in numpy around the oracle's own
    hpsi: the two proposals x +- sigma g (no drift, not wrapped) from the
    walker's stream, the pick with one more uniform (the first with its
    share of exp(-v dt) Psi_G'/Psi_G, or always when the second crossed a
    node), weight 0.5 (wt1 + wt2) exp(etrial dt), 0 on a node crossing."""
    sysd, rund, _ = configs.workload("n14", nwalk=24, idmc=10)
    o = oracle.Oracle(sysd, rund, threads=1)
    o.init_walkers()
    o.initial_eval()
    o.generation(False)      # a populated stack with non-unit weights
    before = o.walkers()
    o.step(True)
    after = o.walkers()
    n, npart = before["n"], o.npart
    assert after["n"] == n
    sig = np.array([o.info.sigma[0]] * o.info.nup + [o.info.sigma[1]] * o.info.ndn)
    el, dt, et = o.info.el, rund.dt, o.info.etrial
    picks = [0, 0]
    for k in range(n):
        src = n - 1 - k
        x1 = before["x"][src] - el * _fnint(before["x"][src] / el)
        g, s = oracle.gaussian(int(before["irn"][src]) & ((1 << 48) - 1), 3 * npart)
        rn, s = oracle.ran1(s)
        dx = sig[:, None] * g.reshape(npart, 3)
        xa, xb = x1 + dx, x1 - dx
        ha, hb = o.hpsi(xa[None]), o.hpsi(xb[None])
        wt1 = np.exp(-ha["v"][0] * dt) * np.exp(ha["psigl"][0] - before["psigl"][src])
        wt2 = np.exp(-hb["v"][0] * dt) * np.exp(hb["psigl"][0] - before["psigl"][src])
        first = rn < wt1 / (wt1 + wt2) or hb["is_"][0] != before["is_"][src]
        h, xc = (ha, xa) if first else (hb, xb)
        picks[0 if first else 1] += 1
        wt = 0.0 if h["is_"][0] != before["is_"][src] else wt1 + wt2
        assert np.max(np.abs(after["x"][k] - xc)) < 1e-13
        assert after["irn"][k] == s
        assert after["is_"][k] == h["is_"][0]
        assert abs(after["weight"][k] - 0.5 * wt * np.exp(et * dt)) <= 1e-13 * max(1.0, abs(after["weight"][k]))
        assert abs(after["psil"][k] - h["psil"][0]) < 1e-12
        assert after["wt0"][k] == before["wt0"][src]
    assert picks[0] > 0 and picks[1] > 0
    # estimators: node crossings (5), the walker count of 10 (sign), 11 (weight)
    vb, _, wb = o.estimators()
    assert wb[10] >= n and vb[10] > 0


def test_branch_copies_are_contiguous_and_advance_ran2():
    sysd, rund, _ = configs.workload("n14", nwalk=20)
    o = oracle.Oracle(sysd, rund, threads=1)
    o.init_walkers()
    o.initial_eval()
    o.step(False)
    before = o.walkers()
    o.branch(1.0)
    after = o.walkers()
    # expected copies, walking the stack from the top (step.f90:295-311)
    exp_irn = []
    for j in range(before["n"] - 1, -1, -1):
        u, s = oracle.ran1(int(before["irn"][j]))
        iwt = int(before["weight"][j] + u)
        for _ in range(iwt):
            _, s = oracle.ran2(s)
            exp_irn.append(s)
    assert list(after["irn"]) == exp_irn
    assert set(np.unique(after["weight"])) <= {1.0, -1.0}


def test_vmc_acceptance_reasonable():
    sysd, rund, _ = configs.workload("n14", nwalk=32, idmc=0)
    o = oracle.Oracle(sysd, rund, threads=2)
    o.init_walkers()
    o.initial_eval()
    for g in range(5):
        o.generation(True)
    vn, en = o.block_update()
    assert 0.3 < vn[5] <= 1.0            # acceptance (estimator 6)
    assert o.num_walkers() == 32         # VMC never branches


def _operator_setup(nwalk=6):
    sysd, rund, _ = configs.workload("n14", nwalk=nwalk)
    orc = oracle.Oracle(sysd, rund)
    orc.init_walkers()
    orc.initial_eval()
    orc.generation(False)
    return sysd, orc


def test_oracle_gofr_and_sofq_against_numpy():
    """addgofr / addsofq (gofr.f90:53-92, sofq.f90:43-64) recomputed with numpy
    on the same population, walkers in pop order (top of the stack first)."""
    sysd, orc = _operator_setup()
    ntabg, ntabq = 16, 3
    orc.set_operators(ntabg, ntabq, 0)
    w = orc.walkers()
    el = orc.info.el
    nup = sysd.nbin[0]
    orc.add_operators()
    g, g2, ws = orc.operators(0, raw=True)
    d, d2, _ = orc.operators(1, raw=True)
    s, s2, _ = orc.operators(2, raw=True)
    scale = ntabg / (0.5 * el)
    G = np.zeros((3, ntabg + 1))
    Dn = np.zeros((6, 2 * ntabg + 1))
    wt = w["weight"] * np.exp(w["psil"] - w["psigl"]) * w["is_"] * w["wt0"]
    npart = w["x"].shape[1]
    for k in range(w["n"])[::-1]:
        x = w["x"][k]
        for i in range(npart - 1):
            for j in range(i + 1, npart):
                itab = 1 if (i < nup and j < nup) else (2 if (i >= nup and j >= nup) else 0)
                dx = x[i] - x[j]
                dx = dx - el * np.sign(dx / el) * np.floor(np.abs(dx / el) + 0.5)
                r = np.sqrt(np.sum(dx * dx))
                G[itab, int(scale * r) if r < 0.5 * el else ntabg] += 2 * wt[k]
        for i in range(npart):
            dx = x[i] - el * np.sign(x[i] / el) * np.floor(np.abs(x[i] / el) + 0.5)
            for c in range(3):
                idx = int(scale * dx[c])
                Dn[c + (0 if i < nup else 3), idx + ntabg] += (0.5 if idx == 0 else 1.0) * wt[k]
    assert np.allclose(g, G.ravel(), rtol=1e-12, atol=0)
    assert np.allclose(d, Dn.ravel(), rtol=1e-12, atol=1e-300)
    assert abs(ws - wt.sum()) < 1e-12 * abs(ws)
    # S(q): half-shell k vectors k = 0 first; rho_k = sum exp(-i k.x)
    ak = orc.table(7).reshape(-1, 3)
    nq = s.size // 3
    S = np.zeros((3, nq))
    for k in range(w["n"])[::-1]:
        x = w["x"][k]
        ru = np.exp(-1j * (x[:nup] @ ak[:nq].T)).sum(axis=0)
        rd = np.exp(-1j * (x[nup:] @ ak[:nq].T)).sum(axis=0)
        S[0] += np.real(ru * np.conj(ru)) * wt[k]
        S[1] += np.real(rd * np.conj(rd)) * wt[k]
        S[2] += np.real(ru * np.conj(rd)) * wt[k]
    assert np.allclose(s, S.ravel(), rtol=1e-11, atol=1e-9)
    assert np.allclose(s[:1], wt.sum() * nup ** 2)            # k = 0: |rho_0|^2 = N_up^2


def test_oracle_nofk_against_python_loop():
    """addenk (momentum3d.f90:89-124) for one walker from the oracle's own
    primitives: ran1 draws from the walker's stream, move1 = getphione *
    bcsone with the walker's inverse, the plane-wave products per shell."""
    sysd, orc = _operator_setup(nwalk=1)
    ntabk = 6
    nsh = orc.set_operators(0, 0, ntabk)
    w = orc.walkers()
    el = orc.info.el
    x = w["x"][0]
    wt = (w["weight"] * np.exp(w["psil"] - w["psigl"]) * w["is_"] * w["wt0"])[0]
    sm = orc.bcs(x[None], want_inverse=True)["smati"][0]
    nnk = int(np.sqrt(ntabk) + 1)
    ik = [(a, b, c) for a in range(nnk + 1) for b in range(nnk + 1) for c in range(nnk + 1)
          if a * a + b * b + c * c <= ntabk]
    shells = sorted(set(a * a + b * b + c * c for a, b, c in ik))
    dk = 2 * np.pi / el
    tmp = np.zeros(len(shells))
    irn = int(w["irn"][0])
    for i in range(x.shape[0]):
        for _ in range(10):
            dx = np.zeros(3)
            for c in range(3):
                u, irn = oracle.ran1(irn)
                dx[c] = (u - 0.5) * el
            rat = orc.getphione(x, -dx, i + 1) * orc.bcsone(x, -dx, i + 1, sm)
            for si, s2 in enumerate(shells):
                for v in ik:
                    if v[0] ** 2 + v[1] ** 2 + v[2] ** 2 == s2:
                        tmp[si] += rat * np.cos(dk * v[0] * dx[0]) * np.cos(dk * v[1] * dx[1]) * np.cos(dk * v[2] * dx[2])
    nk = np.array([sum(1 for v in ik if v[0] ** 2 + v[1] ** 2 + v[2] ** 2 == s2) for s2 in shells])
    orc.add_operators()
    e, e2, ws = orc.operators(3, raw=True)
    assert nsh == len(shells)
    assert np.allclose(e, tmp / nk * wt, rtol=1e-10, atol=1e-12)
    assert np.allclose(e2, (tmp / nk) ** 2 * wt, rtol=1e-10, atol=1e-12)
    assert abs(ws - 10 * wt) < 1e-12


def _custom_walker(extra, nbin=(7, 7), ikup=(), ikdn=(), seed=13):
    from dmcbcs_project_gb300.abi import make_run, make_system

    nup, ndn = nbin
    sp = configs.system_params(max(nup, ndn), max(nup, ndn), 5, seed=seed)
    sp.update(nbin=[nup, ndn], nexup=len(ikup), ikup=[list(k) for k in ikup], nexdn=len(ikdn),
              ikdn=[list(k) for k in ikdn])
    sp.update(extra)
    sysd = make_system(sp)
    o = oracle.Oracle(sysd, make_run(configs.run_params(4, 0.002)), threads=1)
    o.init_walkers()
    rng = np.random.default_rng(seed)
    while True:
        x = o.walkers()["x"][0] + rng.normal(scale=0.2, size=(o.npart, 3))
        if not _near_half_box(x, o.info.nup, o.info.el, o.info.ntab):
            return o, x


@pytest.mark.parametrize("label,extra,nbin,ikup,ikdn", [
    ("one-body", dict(v0ex=0.5, v0exjas=0.3, nqex=[1, 0, 0]), (7, 7), (), ()),
    ("guide", dict(a2=0.05), (7, 7), (), ()),
    ("unpaired down", {}, (7, 8), (), ((0, 0, 0),)),
    ("unpaired both", {}, (9, 10), ((0, 0, 0),), ((1, 0, 0), (-1, 0, 0))),
])
def test_chkder_optional_terms(label, extra, nbin, ikup, ikdn):
    """chkder (wavefunction.f90:289-321) for the hpsi terms and determinant
    rows the benchmark systems leave off: the one-body potential and Jastrow,
    the guiding function (its gradient and Laplacian checked the same way
    against psi_G) and unpaired down states."""
    o, x = _custom_walker(extra, nbin, ikup, ikdn)
    h0 = o.hpsi(x[None])
    h = 1e-5
    d2num = d2gnum = 0.0
    for i in range(o.npart):
        for c in range(3):
            xp = x.copy(); xp[i, c] += h
            xm = x.copy(); xm[i, c] -= h
            hp, hm = o.hpsi(xp[None]), o.hpsi(xm[None])
            for lg, dg in (("psil", "dpsi"), ("psigl", "dpsig")):
                dnum = (hp[lg][0] - hm[lg][0]) / (2 * h)
                assert abs(h0[dg][0, i, c] - dnum) < 1e-5 * max(1.0, abs(dnum)), (label, dg, i, c)
            gp = hp["dpsi"][0, i, c] * np.exp(hp["psil"][0] - h0["psil"][0])
            gm = hm["dpsi"][0, i, c] * np.exp(hm["psil"][0] - h0["psil"][0])
            d2num += (gp - gm) / (2 * h)
            gp = hp["dpsig"][0, i, c] * np.exp(hp["psigl"][0] - h0["psigl"][0])
            gm = hm["dpsig"][0, i, c] * np.exp(hm["psigl"][0] - h0["psigl"][0])
            d2gnum += (gp - gm) / (2 * h)
    assert abs(d2num - h0["d2psi"][0]) < 1e-4 * max(1.0, abs(h0["d2psi"][0])), label
    assert abs(d2gnum - h0["d2psig"][0]) < 1e-4 * max(1.0, abs(h0["d2psig"][0])), label


def test_jastrow_spline_table_against_scipy_bsplines():
    """The oracle's opt-in up-down Jastrow spline (the 16-knot basis the
    library shares through its spline header) against an independent
    construction: scipy's cardinal cubic B-spline on the knots -2..2,
    phi_0(r) = B(r/h), phi_k(r) = B(r/h - k) + B(r/h + k), h = L/34, summed
    with the knot values and differentiated in r, on every point of the
    up-down table grid (r_i = i L / (2 ntab)); also zero with its first two
    derivatives at L/2."""
    interpolate = pytest.importorskip("scipy.interpolate")
    sysd, rund, _ = configs.workload("n14", nwalk=4, ntab=2000)
    knots = np.random.default_rng(21).uniform(-0.3, 0.3, 16)
    base = oracle.Oracle(sysd, rund, threads=1)
    spl = oracle.Oracle(sysd, rund, threads=1)
    spl.set_jastrow_spline(knots)
    nt = base.info.ntab + 1
    diff = [spl.table(m).reshape(2, nt)[0] - base.table(m).reshape(2, nt)[0] for m in range(3)]
    for m in range(3):   # the same-spin rows are untouched
        assert np.array_equal(spl.table(m).reshape(2, nt)[1], base.table(m).reshape(2, nt)[1])
    el = base.info.el
    h = el / 34.0
    r = np.arange(nt) * (0.5 * el / base.info.ntab)
    B = interpolate.BSpline.basis_element(np.arange(-2.0, 3.0), extrapolate=False)
    dB, d2B = B.derivative(1), B.derivative(2)

    def ev(f, t):
        return np.nan_to_num(f(t), nan=0.0)

    want = [np.zeros(nt) for _ in range(3)]
    for k, tk in enumerate(knots):
        for m, f in enumerate((B, dB, d2B)):
            v = ev(f, r / h - k) + (ev(f, r / h + k) if k > 0 else 0.0)
            want[m] += tk * v / h ** m
    scale = [np.max(np.abs(w)) for w in want]
    for m in range(3):
        assert np.max(np.abs(diff[m] - want[m])) < 1e-12 * scale[m], m
    assert max(abs(want[m][-1]) for m in range(3)) < 1e-12 * max(scale)
