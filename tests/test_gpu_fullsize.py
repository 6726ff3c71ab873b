"""Parity at the full benchmark sizes, against the oracle.

* C3 (3 orbitals x 3 bath levels, sector (6,6), D = 853,776): the device's
  ed_solve, Green's function and 150-step Lanczos against the oracle's FP64
  results stored in tests/golden/c3_oracle.npz (made by
  tests/golden/make_c3_golden.py; ed_solver.F90:28-105, ed_green.F90:60-185,
  ed_lanczos.F90:14-68).
* C4 (3 orbitals x 4 bath levels, ground sector (7,8), D = 41,409,225): the
  device H*v against the oracle's multiply_H (ed_hamiltonian.F90:88-191) on
  100,000 sampled rows.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(1e-300, np.abs(np.asarray(b)).max())


@pytest.fixture(scope="module")
def c3gold():
    return np.load(os.path.join(HERE, "golden", "c3_oracle.npz"))


def c3_solver(solver, pkg, gold, precision):
    cfg = pkg.configs.config("C3")
    ek, vk = cfg.model()
    solver.set_options(precision=precision.split("+")[0], green_fp64=precision.endswith("+g64"),
                       nstep=cfg.nstep, nev=int(gold["nev"]), beta=cfg.beta)
    solver.set_model(cfg.norb, cfg.nbath, cfg.U, cfg.J, ek, vk)
    solver.set_sectors([n for n, _ in cfg.sectors], [u for _, u in cfg.sectors])
    solver.set_omega(gold["omega"])
    return cfg


# G tolerances: FP64 device path; FP32-mixed (FP32 eigenvectors and
# recurrence); FP32 eigensolve with the FP64 Green's-function recurrence
@pytest.mark.parametrize("precision,etol,gtol", [("fp64", 1e-9, 1e-8), ("fp32", 1e-8, 2e-5),
                                                 ("fp32+g64", 1e-8, 1e-7)])
def test_c3_solve_and_green_vs_oracle(solver, pkg, c3gold, precision, etol, gtol):
    c3_solver(solver, pkg, c3gold, precision)
    st = solver.ed_solve()
    assert len(st) == len(c3gold["state_val"])
    for a, v, p in zip(st, c3gold["state_val"], c3gold["state_prob"]):
        assert abs(a["val"] - v) < etol
        assert abs(a["prob"] - p) < 1e3 * etol
    G = solver.ed_calc_green_ftn()
    err = rel(G, c3gold["Gr"])
    print(precision, "dE0", abs(st[0]["val"] - c3gold["state_val"][0]), "dG", err)
    assert err < gtol


def test_c3_eigenvalues_vs_oracle(solver, pkg, c3gold):
    c3_solver(solver, pkg, c3gold, "fp64")
    vals, _ = solver.diag(6, 6, int(c3gold["nev"]), vectors=False)
    assert np.abs(np.asarray(vals) - c3gold["eigvals"]).max() < 1e-9


def cfrac(a, b, z):
    """b(0) / (z - a(0) - b(1) / (z - a(1) - ...)) with b(0) = 1 (ed_green.F90:151-157)."""
    g = np.zeros_like(z)
    for j in range(len(a) - 1, 0, -1):
        g = b[j] / (z - a[j] - g)
    return 1.0 / (z - a[0] - g)


def test_c3_lanczos_coefficients_vs_oracle(solver, pkg, c3gold):
    """The reference recurrence (no reorthogonalisation) over all 150 steps from
    the fixture's seeded start vector.  Both FP64 codes round differently and
    the recurrence amplifies the difference once orthogonality is lost: the
    individual a, b agree to 1e-10 over the first 60 steps (69 measured on
    GB300) and then drift apart in both codes alike.  The continued fraction of
    all 150 steps at broadening 2 (where the leading ~60 steps fix it to
    1e-11) agrees to 1e-9."""
    cfg = c3_solver(solver, pkg, c3gold, "fp64")
    D = 924 * 924
    v0 = np.random.default_rng(int(c3gold["start_seed"])).standard_normal(D)
    n, a, b = solver.lanczos_iteration(6, 6, v0)
    assert n == int(c3gold["lz_nstep_calc"]) == cfg.nstep
    ao, bo = c3gold["lz_a"], c3gold["lz_b"]
    da = np.abs(a - ao) / np.abs(ao).max()
    db = np.abs(b[1:] - bo[1:]) / np.abs(bo[1:]).max()
    lead = next((j for j in range(len(da)) if max(da[j], db[j - 1] if j else 0.0) > 1e-10), len(da))
    z = np.linspace(ao.min(), ao.max(), 64) + 2j
    dcf = rel(cfrac(a, b, z), cfrac(ao, bo, z))
    print("steps agreeing to 1e-10:", lead, "continued fraction over 150 steps:", dcf)
    assert lead >= 60
    assert dcf < 1e-9


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 2e-6)])
def test_c4_hv_rows_vs_oracle(solver, oracle, pkg, precision, tol):
    """C4 ground sector at full size: the device H*v (every element computed)
    against the oracle's row loop on 10 blocks of 10,000 rows at random
    offsets (100,000 rows)."""
    cfg = pkg.configs.config("C4")
    ek, vk = cfg.model()
    solver.set_options(precision=precision)
    solver.set_model(cfg.norb, cfg.nbath, cfg.U, cfg.J, ek, vk)
    nu, nd = 7, 8
    b = oracle.Basis(cfg.nsite, nu, nd)
    rng = np.random.default_rng(31)
    x = rng.standard_normal(b.ntot)
    if precision == "fp32":
        x = x.astype(np.float32)
    y = solver.multiply_H(nu, nd, x)
    m = oracle.Model(cfg.norb, cfg.nbath, cfg.U, cfg.J, ek, vk)
    x64 = np.ascontiguousarray(x, dtype=np.float64)
    yo = np.zeros(b.ntot)
    worst = 0.0
    for r0 in rng.integers(0, b.ntot - 10000, 10):
        r0 = int(r0)
        oracle.multiply_H_rows(m, b, x64, yo, r0, r0 + 10000)
        worst = max(worst, rel(y[r0:r0 + 10000], yo[r0:r0 + 10000]))
    print(precision, "max rel error over the sampled rows", worst)
    assert worst < tol


@pytest.fixture(scope="module")
def c5gold():
    return np.load(os.path.join(HERE, "golden", "c5_oracle.npz"))


def test_c5_fits_vs_oracle(solver, pkg, c5gold):
    """The 256 C5 bath fits (3 orbitals x 4 bath levels, 512 w_n) on the
    device against the oracle's frprmn from the same starts
    (tests/golden/c5_oracle.npz, made by tests/golden/make_c5_golden.py;
    frprmn.f90 driven as func.f90:144-163 drives it).

    frprmn stops on a relative change of chi^2 below FTOL = 1e-7 between CG
    iterations, so two FP64 codes that sum in different orders follow the
    same trajectory only as long as their roundings do not steer a line
    search apart; after that they stop at different points of the same flat
    valley or in different minima.  Measured on GB300 the parity shows as:
      * where both end at the same point (final parameters within 1e-4 of
        each other; 5 to 7 starts with the kernels measured), chi^2 agrees
        to 1e-6 (measured: 2e-8);
      * the reference's own limits (itmax 20000, brent ITMAX 100) stop
        nearly the same starts (measured: 242 of 256 agree);
      * where both converge, neither is systematically lower (device lower
        on 48 %), the median relative chi^2 difference is 7e-4 and the
        median CG iteration counts agree to 20 %."""
    P = pkg.configs.fit_config(seed=4, nbatch=256)
    norb, nbath = P["norb"], P["nbath"]
    solver.set_options(precision="fp64")
    X, fret, it, st = solver.fit_batch(P["X0"], P["omega"], P["dev"], nbath, norb)
    fo, io, so, Xo = c5gold["fret"], c5gold["iter"], c5gold["status"], c5gold["X"]
    both = (st == 0) & (so == 0)
    d = np.abs(fret - fo) / np.abs(fo)
    dx = np.abs(X - Xo).max(axis=1)
    same = both & (dx < 1e-4)
    print(f"status agree {int((((st == 0) == (so == 0))).sum())}/256, both converged {int(both.sum())}, "
          f"same end point {int(same.sum())} (max rel dchi2 {d[same].max() if same.any() else 0:.2e}), "
          f"median rel dchi2 {np.median(d[both]):.2e}, device lower on {int((fret[both] < fo[both]).sum())}, "
          f"median CG iterations {np.median(it[both]):.0f} vs {np.median(io[both]):.0f}")
    assert ((st == 0) == (so == 0)).mean() >= 0.9
    assert same.sum() >= 3
    assert d[same].max() < 1e-6
    assert np.median(d[both]) < 1e-2
    assert 0.3 <= (fret[both] < fo[both]).mean() <= 0.7
    assert 0.8 <= np.median(it[both]) / np.median(io[both]) <= 1.25
    # the clusters took turns: fits were parked and resumed, and a parked
    # fit ends where it ends when run alone, bit for bit
    stats = solver.fit_stats()
    print("fit scheduler", stats)
    assert 1 <= stats["clusters"] < 256 and stats["suspensions"] > 0
    for b in np.flatnonzero(it > 600)[np.argsort(it[it > 600])][:3]:
        Xs, fs, its, sts = solver.fit_batch(P["X0"][b:b + 1], P["omega"], P["dev"], nbath, norb)
        assert sts[0] == st[b] and its[0] == it[b] and fs[0] == fret[b] and np.array_equal(Xs[0], X[b]), b
