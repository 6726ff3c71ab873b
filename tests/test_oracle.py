"""CPU tests of the oracle: pinned against the reference's own known answer
(the 9x9 Hamiltonian of mathematica/MO-DMFT-ED.nb), against an independent
Jordan-Wigner construction, and against brute-force / textbook checks."""
import itertools
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _nb():
    with open(os.path.join(GOLDEN, "notebook_hmat.json")) as f:
        return json.load(f)


def _model(O, d):
    m = d["model"]
    return O.Model(m["norb"], m["nbath"], m["U"], m["J"], np.array(m["ek"]), np.array(m["vk"]))


def test_notebook_spectrum(oracle):
    """mathematica/MO-DMFT-ED.nb:1498-1590: same spectrum in sectors (2,1) and (1,2)."""
    d = _nb()
    m = _model(oracle, d)
    ref = np.linalg.eigvalsh(np.array(d["hmat"]))
    for nu, nd in [(2, 1), (1, 2)]:
        H = oracle.dense_H(m, oracle.Basis(3, nu, nd))
        assert np.allclose(H, H.T)
        np.testing.assert_allclose(np.linalg.eigvalsh(H), ref, rtol=0, atol=1e-9)


def test_notebook_matrix_up_to_gauge(oracle):
    """The oracle's H equals the notebook matrix entry by entry, in the
    notebook's basis order, up to a diagonal +-1 gauge of the basis states."""
    d = _nb()
    m = _model(oracle, d)
    b = oracle.Basis(3, 2, 1)
    H = oracle.dense_H(m, b)
    Hn = np.array(d["hmat"])
    modes = {"orb1_up": (1, 1), "orb1_dn": (1, 2), "orb2_up": (2, 1), "orb2_dn": (2, 2),
             "bath_up": (3, 1), "bath_dn": (3, 2)}
    order = [modes[k] for k in d["vc_order"]]
    rows = []
    for vc in d["basis_vc"]:
        w = sum(1 << ((sp - 1) * 3 + s - 1) for (s, sp), n in zip(order, vc) if n)
        rows.append(b.idx(w) - 1)
    P = H[np.ix_(rows, rows)]
    assert np.array_equal(np.abs(P), np.abs(Hn))
    s = np.zeros(9)
    s[0] = 1
    for _ in range(9):
        for i, j in itertools.product(range(9), range(9)):
            if s[i] and not s[j] and Hn[i, j]:
                s[j] = np.sign(Hn[i, j] / P[i, j]) * s[i]
    assert np.all(s != 0)
    assert np.array_equal(np.outer(s, s) * P, Hn)


@pytest.mark.parametrize("norb,nbath,dense", [(1, 3, True), (2, 2, True), (2, 2, False), (3, 1, True), (3, 2, False)])
def test_restatement_vs_jordan_wigner(oracle, norb, nbath, dense):
    rng = np.random.default_rng(norb * 10 + nbath)
    ns = norb + nbath
    vk = rng.uniform(-0.6, 0.6, (norb, nbath))
    if not dense:
        vk[rng.random((norb, nbath)) < 0.5] = 0.0
    m = oracle.Model(norb, nbath, 2.7, 0.45, rng.uniform(-1, 1, ns), vk)
    for nu in range(ns + 1):
        for nd in range(ns + 1):
            H = oracle.dense_H(m, oracle.Basis(ns, nu, nd))
            Hj = oracle.jw_sector_H(m, nu, nd)
            assert np.abs(H - Hj).max() < 1e-12, (nu, nd)


@pytest.mark.parametrize("nsite", [1, 4, 7, 10])
def test_basis_ranks_brute_force(oracle, nsite):
    """generate_basis: ascending popcount-N words, 1-based inverse tables, and
    ed_basis_get / ed_basis_idx as inverse maps (ed_basis.F90:35-139)."""
    for ne in range(nsite + 1):
        words = [w for w in range(1 << nsite) if bin(w).count("1") == ne]
        b = oracle.Basis(nsite, ne, nsite - ne)
        assert b.nup == len(words) == oracle.icom(nsite, ne)
        assert list(b.up) == words
        for r, w in enumerate(words):
            assert b.idx_up[w] == r + 1
    b = oracle.Basis(nsite, nsite // 2, (nsite + 1) // 2)
    for i in range(1, b.ntot + 1, max(1, b.ntot // 97)):
        assert b.idx(b.get(i)) == i


def test_icom_matches_binomial(oracle):
    from math import comb
    for n in range(0, 16):
        for m in range(0, n + 1):
            assert oracle.icom(n, m) == comb(n, m)


def test_operator_signs(oracle):
    """destruction/creation signs = parity of occupied bits below the target."""
    L = oracle.lib()
    import ctypes as C
    out = C.c_uint32()
    for w in range(64):
        for site in (1, 2, 3):
            for spin in (1, 2):
                bit = (spin - 1) * 3 + site - 1
                par = -1 if bin(w & ((1 << bit) - 1)).count("1") % 2 else 1
                s = L.or_destruction_op(w, site, spin, 3, C.byref(out))
                assert s == (par if (w >> bit) & 1 else 0)
                s = L.or_creation_op(w, site, spin, 3, C.byref(out))
                assert s == (0 if (w >> bit) & 1 else par)


def test_heapsort_and_boltzmann(oracle):
    rng = np.random.default_rng(5)
    a = rng.standard_normal(37)
    ind = oracle.sort(a)
    assert np.all(np.diff(a[ind - 1]) >= 0)
    assert sorted(ind.tolist()) == list(range(1, 38))
    assert list(oracle.sort(np.array([3.0]))) == [1]
    e = np.array([0.0, 0.01, 0.5, 1.5, np.finfo(np.float64).max])
    p = oracle.boltzmann_factor(e, 10.0)
    Z = np.exp(-10 * (e[:4] - e[0])).sum()
    assert abs(p[0] - 1 / Z) < 1e-15
    assert abs(p[2] - 1 / np.exp(-10 * (e[:4] - e[2])).sum()) < 1e-15
    # -beta*(E_k - E_i) > 10 for some k -> p_i = 0 (ed_solver.F90:207-212)
    assert p[3] == 0.0 and p[4] == 0.0


def test_ev_x_roundtrip(oracle):
    rng = np.random.default_rng(1)
    norb, nbath = 3, 12
    ns = norb + nbath
    ek = rng.standard_normal(ns)
    vk = rng.standard_normal((norb, nbath))
    ef = ek[:norb].copy()
    x = oracle.ev_to_x(ek, vk, ef, ns, nbath)
    assert np.array_equal(x[:nbath], ek[norb:])
    assert np.array_equal(x[nbath:nbath + norb * nbath], vk.ravel())
    assert np.array_equal(x[-norb:], ef)
    ef2, ek2, vk2 = oracle.x_to_ev(x, ns, nbath, norb)
    assert np.array_equal(ef2, ef) and np.array_equal(ek2, ek) and np.array_equal(vk2, vk)


def _fit_problem(seed=0, norb=2, nbath=4, nw=64, beta=50.0):
    rng = np.random.default_rng(seed)
    ns = norb + nbath
    om = (2 * np.arange(nw) + 1) * np.pi / beta
    eps = rng.uniform(-2, 2, nbath)
    vk = rng.uniform(0.1, 0.6, (norb, nbath))
    ef = rng.uniform(-0.5, 0.5, norb)
    z = 1j * om[None, :, None] - eps[None, None, :]
    dev = (vk[:, None, :] ** 2 / z).sum(-1) + ef[:, None]
    return ns, om, dev, eps, vk, ef


def test_func_matches_formula(oracle):
    """FUNC (func.f90:1-45) against the closed form with CMPLX-rounded i*w."""
    ns, om, dev, eps, vk, ef = _fit_problem()
    norb, nbath = 2, 4
    rng = np.random.default_rng(3)
    x = oracle.ev_to_x(np.concatenate([ef, eps]), vk, ef, ns, nbath) + 0.1 * rng.standard_normal(nbath + nbath * norb + norb)
    ef2, ek2, vk2 = oracle.x_to_ev(x, ns, nbath, norb)
    omf = om.astype(np.float32).astype(np.float64)
    z = 1j * omf[None, :, None] - ek2[norb:][None, None, :]
    delta = (vk2[:, None, :] ** 2 / z).sum(-1) + ef2[:, None]
    f = (np.abs(delta - dev) ** 2 / om[None, :]).sum() / (norb * norb * len(om))
    assert abs(oracle.func(x, ns, om, dev, nbath, norb) - f) < 1e-13 * abs(f)


def test_dfunc_finite_difference(oracle):
    ns, om, dev, eps, vk, ef = _fit_problem(seed=2)
    norb, nbath = 2, 4
    rng = np.random.default_rng(4)
    x = oracle.ev_to_x(np.concatenate([ef, eps]), vk, ef, ns, nbath) + 0.2 * rng.standard_normal(nbath + nbath * norb + norb)
    g = oracle.dfunc(x, ns, om, dev, nbath, norb)
    h = 1e-6
    for i in range(len(x)):
        xp, xm = x.copy(), x.copy()
        xp[i] += h
        xm[i] -= h
        fd = (oracle.func(xp, ns, om, dev, nbath, norb) - oracle.func(xm, ns, om, dev, nbath, norb)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1e-3, abs(g[i])), (i, fd, g[i])


def test_frprmn_recovers_bath(oracle):
    ns, om, dev, eps, vk, ef = _fit_problem(seed=7)
    norb, nbath = 2, 4
    rng = np.random.default_rng(8)
    x_true = oracle.ev_to_x(np.concatenate([ef, eps]), vk, ef, ns, nbath)
    x0 = x_true + 0.05 * rng.standard_normal(len(x_true))
    f0 = oracle.func(x0, ns, om, dev, nbath, norb)
    x, fret, it, rc = oracle.frprmn(x0, ns, om, dev, nbath, norb)
    assert rc == 0 and it >= 1
    assert fret < 1e-3 * f0


def test_calc_dev_formula(oracle):
    norb, nbath = 3, 6
    rng = np.random.default_rng(9)
    om = (2 * np.arange(32) + 1) * np.pi / 40.0
    ek = rng.standard_normal(norb + nbath)
    vk = rng.standard_normal((norb, nbath))
    ef = rng.standard_normal(norb)
    d = oracle.calc_dev(norb, norb + nbath, om, ek, vk, ef)
    omf = om.astype(np.float32).astype(np.float64)
    z = 1j * omf[None, :, None] - ek[norb:][None, None, :]
    ref = (vk[:, None, :] ** 2 / z).sum(-1) + ef[:, None]
    assert np.abs(d - ref).max() < 1e-13


def test_green_cf_equals_exact_resolvent(oracle):
    """Lanczos continued fraction with nstep >= dimension reproduces the exact
    sum over poles of the reference's particle / hole G (ed_green.F90:136-185)."""
    rng = np.random.default_rng(11)
    norb, nbath = 1, 3
    ns = norb + nbath
    m = oracle.Model(norb, nbath, 2.0, 0.0, np.concatenate([[-1.0], rng.uniform(-1, 1, nbath)]),
                     rng.uniform(0.2, 0.5, (norb, nbath)))
    nu = nd = 2
    b = oracle.Basis(ns, nu, nd)
    w, V = np.linalg.eigh(oracle.dense_H(m, b))
    E0, psi = w[0], V[:, 0]
    om = (2 * np.arange(16) + 1) * np.pi / 10.0
    gr = np.zeros(16, complex)
    oracle.green_diag(m, b, psi, E0, 1.0, 1.0, 1, 1, 40, om, gr)
    # exact
    bo, v = oracle.apply_c(m, b, psi, 1, 1, 1)
    wp, Vp = np.linalg.eigh(oracle.dense_H(m, bo))
    wts = (Vp.T @ v) ** 2
    bo2, v2 = oracle.apply_c(m, b, psi, 2, 1, 1)
    wm, Vm = np.linalg.eigh(oracle.dense_H(m, bo2))
    wts2 = (Vm.T @ v2) ** 2
    z = 1j * om.astype(np.float32).astype(np.float64)
    e0f = float(np.float32(E0))
    exact = (wts[None, :] / (z[:, None] + e0f - wp[None, :])).sum(1) + \
            (wts2[None, :] / (z[:, None] - e0f + wm[None, :])).sum(1)
    # the hole weight uses the sum rule 1 - ||c+psi||^2
    assert abs(wts.sum() + wts2.sum() - 1.0) < 1e-12
    assert np.abs(gr - exact).max() < 1e-9 * np.abs(exact).max()


def test_lanczos_iteration_tridiagonal(oracle):
    """a/b from lanczos_iteration reproduce the Krylov projection of H."""
    rng = np.random.default_rng(12)
    norb, nbath = 2, 2
    m = oracle.Model(norb, nbath, 3.0, 0.6, rng.uniform(-1, 1, 4), rng.uniform(0.1, 0.5, (2, 2)))
    b = oracle.Basis(4, 2, 2)
    H = oracle.dense_H(m, b)
    v0 = rng.standard_normal(b.ntot)
    n, a, bb = oracle.lanczos_iteration(m, b, v0, 8)
    assert n == 8
    # explicit Lanczos in numpy (modified, with reorthogonalisation)
    Q = [v0 / np.linalg.norm(v0)]
    al, be2 = [], []
    for j in range(6):
        w = H @ Q[-1]
        al.append(Q[-1] @ w)
        for q in Q:
            w -= (q @ w) * q
        be2.append(w @ w)
        Q.append(w / np.sqrt(be2[-1]))
    np.testing.assert_allclose(a[:6], al, rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(bb[1:6], be2[:5], rtol=1e-10)


# ---------------------------------------------------------------- DMFT loop pieces
def test_band_structure(oracle):
    """ed_hamiltonian.F90:29-85: -0.5 (cos kx + cos ky) on the k grid, kx outer;
    the k-average vanishes on a full even grid; a non-square Nq is refused."""
    hk, ef = oracle.set_band_structure(3, 16)
    k = 2 * np.pi / 4 * np.arange(4)
    ref = (-0.5 * (np.cos(k)[:, None] + np.cos(k)[None, :])).ravel()
    assert np.abs(hk - ref).max() < 1e-15
    assert np.abs(ef).max() < 1e-15 and ef.shape == (3,)
    with pytest.raises(ValueError):
        oracle.set_band_structure(1, 10)


def test_delta_new_and_occupation(oracle):
    """ed_green.F90:187-253 against a vectorised restatement."""
    rng = np.random.default_rng(21)
    norb, nw = 3, 16
    hk, _ = oracle.set_band_structure(norb, 64)
    gr = rng.standard_normal((norb, nw)) + 1j * (rng.standard_normal((norb, nw)) - 3.0)
    dev = 0.1 * (rng.standard_normal((norb, nw)) + 1j * rng.standard_normal((norb, nw)))
    dn, gk = oracle.delta_new(hk, 0.7, gr, dev)
    gi = 1.0 / gr
    gk2 = np.mean(1.0 / ((gi + dev + 0.7)[:, :, None] - hk[None, None, :]), axis=2)
    assert np.abs(gk - gk2).max() < 1e-14 * np.abs(gk2).max()
    assert np.abs(dn - (gi - 1.0 / gk2 + dev)).max() < 1e-13 * np.abs(dn).max()
    beta = 50.0
    assert np.abs(oracle.n_from_gksum(gk, beta) - (2.0 * gk.real.sum(axis=1) / beta + 0.5)).max() < 1e-14


def _cf(z, a, b, n, sgn):
    g = b[n] / (z + sgn * a[n])
    for j in range(n - 1, -1, -1):
        g = b[j] / (z + sgn * a[j] - g)
    return g


def test_dos_records(oracle):
    """dos.f90:1-106: last record of an orbital assigns A (the reference's
    dos_diag), or the probability-weighted sum; runs with nstep_calc = -1 add
    nothing; CMPLX rounds E + w and small to default REAL."""
    rng = np.random.default_rng(5)
    norb, ld = 2, 6
    recs = []
    for r in range(5):
        recs.append(dict(iorb=r % norb + 1, ev=-1.3 + 0.1 * r, prob=0.2 + 0.1 * r, even=r % 2,
                         np=int(rng.integers(0, ld)) if r != 2 else -1, nn=int(rng.integers(0, ld)),
                         ap=rng.standard_normal(ld), bp=rng.uniform(0.1, 1, ld), an=rng.standard_normal(ld),
                         bn=rng.uniform(0.1, 1, ld)))
    w = np.linspace(-3, 3, 41)
    small = 0.05
    f32 = lambda v: np.float64(np.float32(v))
    A0 = oracle.dos(norb, recs, w, small, weighted=False)
    A1 = oracle.dos(norb, recs, w, small, weighted=True)
    R0 = np.zeros((norb, len(w)))
    R1 = np.zeros((norb, len(w)))
    for r in recs:
        for i, x in enumerate(w):
            g = 0j
            if r["np"] >= 0:
                g += _cf(complex(f32(r["ev"] + x), f32(small)), r["ap"], r["bp"], r["np"], -1)
            if r["nn"] >= 0:
                g += _cf(complex(f32(x - r["ev"]), f32(small)), r["an"], r["bn"], r["nn"], +1)
            a = -g.imag / np.pi
            R0[r["iorb"] - 1, i] = a
            R1[r["iorb"] - 1, i] += r["prob"] * (1.0 if r["even"] else 0.5) * a
    assert np.abs(A0 - R0).max() < 1e-12 * np.abs(R0).max()
    assert np.abs(A1 - R1).max() < 1e-12 * np.abs(R1).max()


def test_fdf_round_trip_and_parsing(tmp_path):
    """FDF input (ed_config.f90:52-126): a written configuration reads back
    exactly; labels ignore case and '.', '_', '-'; '#' comments; absent
    labels take the reference's defaults; D exponents."""
    import importlib.util
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("moed_configs", os.path.join(root, "mo-dmft_gb300", "configs.py"))
    cf = importlib.util.module_from_spec(spec)
    sys.modules["moed_configs"] = cf   # dataclasses resolve their module by name
    spec.loader.exec_module(cf)
    cfg = cf.config("C2")
    p = tmp_path / "input.fdf"
    cf.write_fdf(cfg, p, nev=6)
    d = cf.read_fdf(str(p))
    ek, vk = cfg.model()
    assert d["DMFT.Norbs"] == 2 and d["DMFT.Nbaths"] == 6 and d["DMFT.Nev"] == 6
    assert d["sectors"] == cfg.sectors and d["DMFT.U"] == cfg.U and d["DMFT.beta"] == cfg.beta
    assert np.array_equal(d["eps_bath"], ek[cfg.norb:]) and np.array_equal(d["vk"], vk)
    text = "\n".join(["dmft_norbs 1   # one orbital", "DMFT-NBATHS 2", "DMFT.Nsectors 1",
                      "%block dmft.sectors", " 3 2", " 9 9", "%endblock dmft.sectors",
                      "%block DMFT.Baths", " -0.5d0", " 0.5D0", "%endblock DMFT.Baths",
                      "%block DMFT.BathCouplings", " 0.25", " 0.3", "%endblock DMFT.BathCouplings",
                      "DMFT.U 2.0d0"])
    d = cf.read_fdf(text)
    assert d["DMFT.Norbs"] == 1 and d["DMFT.Nbaths"] == 2 and d["sectors"] == [(3, 2)]
    assert np.array_equal(d["eps_bath"], [-0.5, 0.5]) and np.array_equal(d["vk"], [[0.25, 0.3]])
    assert d["DMFT.U"] == 2.0 and d["DMFT.J"] == 0.3 and d["DMFT.Nq"] == 10000


@pytest.mark.parametrize("nsite,nu,nd", [(4, 2, 1), (5, 2, 3), (6, 3, 3)])
def test_apply_c_dense_operator(oracle, nsite, nu, nd):
    """apply_c (ed_operators.F90:10-61) against the creation / annihilation
    operator built as a dense matrix in Python from the basis words: row
    index up-rank fastest, sign (-1)^(occupied bits below the target bit of
    the 2*Nsite-bit word, spin-down bits above the spin-up ones)."""
    m = oracle.Model(min(2, nsite - 1), nsite - min(2, nsite - 1), 1.0, 0.2, np.zeros(nsite),
                     np.zeros((min(2, nsite - 1), nsite - min(2, nsite - 1))))
    b = oracle.Basis(nsite, nu, nd)
    rng = np.random.default_rng(nsite * 10 + nu)
    v = rng.standard_normal(b.ntot)
    for ispin in (1, 2):
        for iorb in range(1, m.norb + 1):
            for pm in (1, 2):
                tu = nu + ((1 if pm == 1 else -1) if ispin == 1 else 0)
                td = nd + ((1 if pm == 1 else -1) if ispin == 2 else 0)
                if not (0 <= tu <= nsite and 0 <= td <= nsite):
                    continue
                bo, out = oracle.apply_c(m, b, v, pm, iorb, ispin)
                ref = np.zeros(bo.ntot)
                bit = (ispin - 1) * nsite + iorb - 1
                for idn in range(b.ndown):
                    for iup in range(b.nup):
                        w = int(b.up[iup]) | (int(b.down[idn]) << nsite)
                        occ = (w >> bit) & 1
                        if (pm == 1) == bool(occ):
                            continue          # c+ on an occupied / c on an empty orbital
                        sgn = -1.0 if bin(w & ((1 << bit) - 1)).count("1") % 2 else 1.0
                        w2 = w ^ (1 << bit)
                        u2, d2 = w2 & ((1 << nsite) - 1), w2 >> nsite
                        j = (int(bo.idx_down[d2]) - 1) * bo.nup + int(bo.idx_up[u2]) - 1
                        ref[j] += sgn * v[idn * b.nup + iup]
                assert np.array_equal(out, ref), (ispin, iorb, pm)


def test_sector_eigs_arpack_path_matches_dense(oracle):
    """The oracle's diag() stand-in for large sectors (scipy ARPACK eigsh, 'SA',
    tol = 0 as ed_solver.F90:149 asks of PARPACK) agrees with dense eigh on a
    sector small enough for both (D = 1,225): eigenvalues to 1e-10 and
    residuals of the returned vectors."""
    rng = np.random.default_rng(17)
    norb, nbath = 2, 5
    vk = np.zeros((norb, nbath))
    vk[0, :3] = rng.uniform(0.1, 0.5, 3)
    vk[1, 3:] = rng.uniform(0.1, 0.5, 2)
    m = oracle.Model(norb, nbath, 3.0, 0.5, np.concatenate([[-2.0, -2.0], rng.uniform(-1, 1, nbath)]), vk)
    b, ev_a, vec_a = oracle.sector_eigs(m, 3, 3, 6, dense_max=0)
    _, ev_d, _ = oracle.sector_eigs(m, 3, 3, 6, dense_max=10**6)
    assert b.ntot == 1225
    assert np.abs(ev_a - ev_d).max() < 1e-10
    for i in range(6):
        r = oracle.multiply_H(m, b, vec_a[:, i]) - ev_a[i] * vec_a[:, i]
        assert np.linalg.norm(r) < 1e-8
