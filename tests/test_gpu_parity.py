"""GPU parity tests: CUDA path through the C-ABI vs the CPU oracle.

Tolerances (stated per test):
  * basis words, ranks, rows, apply_c signs / values: bit-exact;
  * FP64 H*v: 1e-13 relative (max-norm) -- summation order only;
  * FP32 H*v: 2e-6 relative (max-norm) on FP32-rounded input;
  * FP32-in / FP64-accumulated H*v: 1e-13 relative on the same FP32 input;
  * FP64 Lanczos coefficients: 1e-9 relative over the first 12 steps (later
    steps amplify rounding after loss of orthogonality in both codes);
  * FP64 eigenvalues: 1e-9 absolute; FP32-mixed eigenvalues: 1e-8 absolute;
  * G(i w_n): FP64 1e-8, FP32-mixed 1e-5 (2e-5 on config 2), FP32-mixed
    eigensolve with green_fp64 (FP64 refinement of the kept eigenvectors and
    an FP64 Green's-function recurrence) 1e-7, relative to max |G|;
  * chi^2 / gradient: 1e-12 relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(1e-300, np.abs(np.asarray(b)).max())


MODELS = {
    # name: (norb, nbath, U, J, dense V)
    "1x4": (1, 4, 2.0, 0.0, True),
    "2x6_block": (2, 6, 4.0, 1.0, False),
    "2x3_dense": (2, 3, 3.1, 0.7, True),
    "3x3_dense": (3, 3, 3.0, 0.5, True),
    "3x6_block": (3, 6, 3.0, 0.5, False),
    "4x4_mixed": (4, 4, 2.5, 0.4, None),
    "5x2_dense": (5, 2, 2.0, 0.3, True),
}


def make_model(name, seed=0):
    norb, nbath, U, J, dense = MODELS[name]
    rng = np.random.default_rng(seed + 17 * norb + nbath)
    ek = np.concatenate([rng.uniform(-2, 0, norb), rng.uniform(-1, 1, nbath)])
    vk = rng.uniform(0.1, 0.6, (norb, nbath))
    if dense is False:
        per = nbath // norb
        mask = np.zeros_like(vk)
        for a in range(norb):
            mask[a, a * per:(a + 1) * per] = 1
        vk *= mask
    elif dense is None:
        vk[rng.random(vk.shape) < 0.4] = 0.0
    return norb, nbath, U, J, ek, vk


@pytest.fixture
def setup(solver, oracle):
    def f(name, seed=0, precision="fp64", **opt):
        norb, nbath, U, J, ek, vk = make_model(name, seed)
        solver.set_options(precision=precision, **opt)
        solver.set_model(norb, nbath, U, J, ek, vk)
        return solver, oracle.Model(norb, nbath, U, J, ek, vk)
    return f


# ---------------------------------------------------------------- basis
@pytest.mark.parametrize("norb,nbath", [(1, 4), (2, 6), (3, 9), (3, 12)])
def test_generate_basis_bitexact(solver, oracle, norb, nbath):
    ns = norb + nbath
    solver.set_model(norb, nbath, 1.0, 0.1, np.zeros(ns), np.full((norb, nbath), 0.2))
    for ne in sorted({0, 1, ns // 2, (ns + 1) // 2, ns - 1, ns}):
        ne2 = ns - ne
        g = solver.generate_basis(ne, ne2)
        b = oracle.Basis(ns, ne, ne2)
        assert g["nup"] == b.nup and g["ndown"] == b.ndown
        assert np.array_equal(g["up"], b.up) and np.array_equal(g["down"], b.down)
        assert np.array_equal(g["idx_up"], b.idx_up) and np.array_equal(g["idx_down"], b.idx_down)


def test_basis_get_idx_bitexact(solver, oracle):
    ns = 12
    solver.set_model(3, 9, 1.0, 0.1, np.zeros(ns), np.full((3, 9), 0.2))
    b = oracle.Basis(ns, 6, 5)
    rng = np.random.default_rng(0)
    rows = rng.integers(1, b.ntot + 1, 5000)
    st = solver.ed_basis_get(6, 5, rows)
    assert np.array_equal(st, [b.get(int(i)) for i in rows])
    assert np.array_equal(solver.ed_basis_idx(6, 5, st), rows)
    # a word outside the sector maps to 0
    assert solver.ed_basis_idx(6, 5, np.array([0], np.uint32))[0] == 0


# ---------------------------------------------------------------- H*v
def sectors_of(ns):
    out = {(ns // 2, (ns + 1) // 2), (1, 0), (0, ns), (ns, ns - 1), (ns // 2, ns // 2), (2, ns - 3)}
    return sorted(s for s in out if 0 <= s[0] <= ns and 0 <= s[1] <= ns)


@pytest.mark.parametrize("name", list(MODELS))
def test_multiply_h_fp64(setup, oracle, name):
    s, m = setup(name)
    ns = m.nsite
    rng = np.random.default_rng(1)
    for nu, nd in sectors_of(ns):
        b = oracle.Basis(ns, nu, nd)
        x = rng.standard_normal(b.ntot)
        y = s.multiply_H(nu, nd, x)
        assert rel(y, oracle.multiply_H(m, b, x)) < 1e-13, (name, nu, nd)


@pytest.mark.parametrize("name", ["1x4", "2x6_block", "3x6_block", "4x4_mixed", "5x2_dense"])
def test_multiply_h_fp32(setup, oracle, name):
    s, m = setup(name, precision="fp32")
    ns = m.nsite
    rng = np.random.default_rng(2)
    for nu, nd in sectors_of(ns):
        b = oracle.Basis(ns, nu, nd)
        x = rng.standard_normal(b.ntot).astype(np.float32)
        y = s.multiply_H(nu, nd, x)
        assert y.dtype == np.float32
        assert rel(y, oracle.multiply_H(m, b, x.astype(np.float64))) < 2e-6, (name, nu, nd)


@pytest.mark.parametrize("name", ["3x6_block", "4x4_mixed", "5x2_dense"])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-13), ("fp32", 2e-6)])
def test_multiply_h_every_variant(setup, oracle, pkg, name, precision, tol):
    """Each tile-shape variant (k_hv, the double-buffered staged k_hv_async, the
    split k_hv_down + k_hv_async and the split k_hv_down_rows + k_hv_async),
    pinned in turn, against the oracle on several sectors.  The k_hv_down split
    variants need every down-spin block of the model in one CTA's shared
    memory: the dense-V model has one block per sector and rejects them with
    MO_ED_ERR_ARG."""
    s, m = setup(name, precision=precision)
    dt = pkg.FP32 if precision == "fp32" else pkg.FP64
    ns = m.nsite
    rng = np.random.default_rng(11)
    for nu, nd in sectors_of(ns):
        b = oracle.Basis(ns, nu, nd)
        x = rng.standard_normal(b.ntot)
        if precision == "fp32":
            x = x.astype(np.float32)
        ref = oracle.multiply_H(m, b, x.astype(np.float64))
        variants, _ = s.hv_tuning(nu, nd, dt)
        ran, staged, split = 0, 0, 0
        for v, (shape, ms) in enumerate(variants):
            try:
                s.hv_set_variant(nu, nd, v, dt)
                y = s.multiply_H(nu, nd, x)
            except pkg.EDError as e:
                assert e.code == 1, e       # MO_ED_ERR_ARG: the shape does not fit this sector
                continue
            ran += 1
            staged += shape[3] == 1
            split += shape[3] >= 2
            assert rel(y, ref) < tol, (name, nu, nd, v, shape)
        assert ran >= 2 and staged >= 1
        if name == "3x6_block":
            assert split >= 2


def test_multiply_h_mixed(setup, oracle):
    import torch
    s, m = setup("3x6_block")
    nu, nd = 4, 5
    b = oracle.Basis(m.nsite, nu, nd)
    x = np.random.default_rng(3).standard_normal(b.ntot).astype(np.float32)
    ld, nelem = s.vector_layout(nu, nd)
    assert ld % 32 == 0 and nelem == ld * b.ndown
    xp = np.zeros((b.ndown, ld), np.float32)
    xp[:, :b.nup] = x.reshape(b.ndown, b.nup)
    dx = torch.from_numpy(xp.ravel()).cuda()
    dy = torch.empty(nelem, dtype=torch.float64, device="cuda")
    s.multiply_H_mixed_dev(nu, nd, dx.data_ptr(), dy.data_ptr())
    torch.cuda.synchronize()
    yp = dy.cpu().numpy().reshape(b.ndown, ld)
    assert np.all(yp[:, b.nup:] == 0)
    assert rel(yp[:, :b.nup].ravel(), oracle.multiply_H(m, b, x.astype(np.float64))) < 1e-13


def test_multiply_h_symmetric_c3(setup, oracle):
    """Full C3 sector (D = 853,776): <x|H y> = <y|H x> and FP32 vs FP64 agreement."""
    from __graft_entry__ import load_package
    cfg = load_package().configs.config("C3")
    ek, vk = cfg.model()
    s = setup("1x4")[0]
    s.set_model(cfg.norb, cfg.nbath, cfg.U, cfg.J, ek, vk)
    rng = np.random.default_rng(4)
    D = 924 * 924
    x, y = rng.standard_normal(D), rng.standard_normal(D)
    hx, hy = s.multiply_H(6, 6, x), s.multiply_H(6, 6, y)
    assert abs(x @ hy - y @ hx) < 1e-11 * abs(x @ hy)
    hx32 = s.multiply_H(6, 6, x.astype(np.float32))
    assert rel(hx32, s.multiply_H(6, 6, x.astype(np.float32).astype(np.float64))) < 2e-6
    # linearity
    assert rel(s.multiply_H(6, 6, 2.0 * x - y), 2.0 * hx - hy) < 1e-13


def test_multiply_h_c4_full_size(solver, pkg):
    """C4 ground sector at full size (D = 41,409,225): FP64 symmetry <x|Hy> =
    <y|Hx>, linearity, and every FP32 tile-shape variant (previous, staged and
    both split kernels) against the FP64 product of the same FP32 input; the
    FP64 split variants against the FP64 product."""
    cfg = pkg.configs.config("C4")
    ek, vk = cfg.model()
    solver.set_options(precision="fp64")
    solver.set_model(cfg.norb, cfg.nbath, cfg.U, cfg.J, ek, vk)
    nu, nd = 7, 8
    D = solver.sector_dims(nu, nd)[2]
    assert D == 41409225
    rng = np.random.default_rng(14)
    x, y = rng.standard_normal(D), rng.standard_normal(D)
    hx, hy = solver.multiply_H(nu, nd, x), solver.multiply_H(nu, nd, y)
    assert abs(x @ hy - y @ hx) < 1e-11 * abs(x @ hy)
    assert rel(solver.multiply_H(nu, nd, 2.0 * x - y), 2.0 * hx - hy) < 1e-13
    del y, hy
    x32 = x.astype(np.float32)
    h64 = solver.multiply_H(nu, nd, x32.astype(np.float64))
    variants, chosen = solver.hv_tuning(nu, nd, pkg.FP32)
    kinds = set()
    for v, (shape, ms) in enumerate(variants):
        if ms < 0:
            continue
        solver.hv_set_variant(nu, nd, v, pkg.FP32)
        assert rel(solver.multiply_H(nu, nd, x32), h64) < 2e-6, (v, shape)
        kinds.add(shape[3])
    assert kinds == {0, 1, 2, 3, 4}
    variants, chosen = solver.hv_tuning(nu, nd, pkg.FP64)
    for v, (shape, ms) in enumerate(variants):
        if shape[3] >= 2:
            try:   # FP64 move lists and slices may not fit one CTA for C4's blocks
                solver.hv_set_variant(nu, nd, v, pkg.FP64)
            except pkg.EDError as e:
                assert e.code == 1, e
                continue
            assert rel(solver.multiply_H(nu, nd, x), hx) < 1e-13, (v, shape)


# ---------------------------------------------------------------- apply_c
@pytest.mark.parametrize("name", ["1x4", "3x3_dense", "4x4_mixed"])
def test_apply_c_bitexact(setup, oracle, name):
    s, m = setup(name)
    ns = m.nsite
    rng = np.random.default_rng(5)
    for nu, nd in [(ns // 2, (ns + 1) // 2), (1, ns - 1)]:
        b = oracle.Basis(ns, nu, nd)
        v = rng.standard_normal(b.ntot)
        for ispin in (1, 2):
            for iorb in range(1, m.norb + 1):
                for pm in (1, 2):
                    tu = nu + ((1 if pm == 1 else -1) if ispin == 1 else 0)
                    td = nd + ((1 if pm == 1 else -1) if ispin == 2 else 0)
                    if not (0 <= tu <= ns and 0 <= td <= ns):
                        continue
                    _, out = s.apply_c(nu, nd, v, pm, iorb, ispin)
                    _, ref = oracle.apply_c(m, b, v, pm, iorb, ispin)
                    assert np.array_equal(out, ref), (nu, nd, pm, iorb, ispin)


# ---------------------------------------------------------------- Lanczos
@pytest.mark.parametrize("name,sector", [("2x6_block", (4, 4)), ("3x3_dense", (3, 3)), ("1x4", (2, 3))])
def test_lanczos_iteration_fp64(setup, oracle, name, sector):
    s, m = setup(name, nstep=40)
    b = oracle.Basis(m.nsite, *sector)
    v = np.random.default_rng(6).standard_normal(b.ntot)
    n, a, bb = s.lanczos_iteration(*sector, v)
    n0, a0, b0 = oracle.lanczos_iteration(m, b, v, 40)
    k = min(12, n0)
    assert n == n0
    assert rel(a[:k], a0[:k]) < 1e-9 and rel(bb[:k], b0[:k]) < 1e-9


def test_lanczos_breakdown_small_sector(setup, oracle):
    """A sector of dimension 5: b(j) falls below 1e-12 and nstep_calc stops there."""
    s, m = setup("1x4", nstep=30)
    b = oracle.Basis(m.nsite, 1, 0)
    v = np.random.default_rng(7).standard_normal(b.ntot)
    n, a, bb = s.lanczos_iteration(1, 0, v)
    n0, a0, b0 = oracle.lanczos_iteration(m, b, v, 30)
    assert n == n0 <= 6
    assert rel(a[:n], a0[:n]) < 1e-9


def test_lanczos_iteration_fp32(setup, oracle):
    s, m = setup("3x6_block", precision="fp32", nstep=20)
    b = oracle.Basis(m.nsite, 4, 5)
    v = np.random.default_rng(8).standard_normal(b.ntot)
    n, a, bb = s.lanczos_iteration(4, 5, v)
    n0, a0, b0 = oracle.lanczos_iteration(m, b, v.astype(np.float32).astype(np.float64), 20)
    assert rel(a[:6], a0[:6]) < 1e-5 and rel(bb[1:6], b0[1:6]) < 1e-5
    # all 20 steps through the continued fraction they define
    # (ed_green.F90:151-157), at broadening 0.5 over the spectral range
    assert n == n0
    z = np.linspace(a0[:n0].min(), a0[:n0].max(), 64) + 0.5j

    def cf(aa, bbb):
        g = np.zeros_like(z)
        for j in range(n0 - 1, 0, -1):
            g = bbb[j] / (z - aa[j] - g)
        return 1.0 / (z - aa[0] - g)
    assert rel(cf(a, bb), cf(a0, b0)) < 1e-5


# ---------------------------------------------------------------- diag
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32", 1e-8)])
def test_diag_vs_dense(setup, oracle, precision, tol):
    s, m = setup("2x6_block", precision=precision)
    for nu, nd in [(4, 4), (3, 5), (1, 1), (8, 7)]:
        b = oracle.Basis(m.nsite, nu, nd)
        w = np.linalg.eigvalsh(oracle.dense_H(m, b))
        nev = min(4, b.ntot)
        ev, vec = s.diag(nu, nd, nev)
        print(precision, (nu, nd), s.diag_stats(), np.abs(ev[:nev] - w[:nev]).max())
        assert np.abs(ev[:nev] - w[:nev]).max() < tol, (nu, nd, ev[:nev], w[:nev], s.diag_stats())
        H = oracle.dense_H(m, b)
        for i in range(nev):
            r = H @ vec[:, i] - ev[i] * vec[:, i]
            assert np.linalg.norm(r) < (1e-7 if precision == "fp64" else 1e-4)


# ---------------------------------------------------------------- ed_solve + G
@pytest.mark.parametrize("precision,etol,gtol", [("fp64", 1e-9, 1e-8), ("fp32", 1e-8, 1e-5),
                                                  ("fp32+g64", 1e-8, 1e-7)])
def test_ed_solve_green_c1(solver, oracle, pkg, precision, etol, gtol):
    """Config 1 (single band, 4 bath levels, all 36 sectors, beta = 50, 1024 w,
    100 steps): states, probabilities and G(i w_n) vs the oracle."""
    cfg = pkg.configs.config("C1")
    ek, vk = cfg.model()
    nev = 8
    solver.set_options(precision=precision.split("+")[0], green_fp64=precision.endswith("+g64"),
                       nstep=cfg.nstep, nev=nev, beta=cfg.beta)
    solver.set_model(cfg.norb, cfg.nbath, cfg.U, cfg.J, ek, vk)
    solver.set_sectors([n for n, _ in cfg.sectors], [u for _, u in cfg.sectors])
    om = cfg.omega()
    solver.set_omega(om)
    st = solver.ed_solve()
    m = oracle.Model(cfg.norb, cfg.nbath, cfg.U, cfg.J, ek, vk)
    st_o, vecs = oracle.ed_solve(m, cfg.sectors, nev, cfg.beta)
    assert len(st) == len(st_o)
    for a, c in zip(st, st_o):
        assert abs(a["val"] - c["val"]) < etol
        assert abs(a["prob"] - c["prob"]) < 1e3 * etol
    # spin-partner sectors (a,b), (b,a) are exactly degenerate: their order in
    # the heapsort depends on the last bit, so compare per energy tie group
    def groups(sts):
        out, cur = [], []
        for e in sts:
            if cur and abs(e["val"] - cur[-1]["val"]) > 1e-7:
                out.append(sorted((x["sector"], x["level"]) for x in cur))
                cur = []
            cur.append(e)
        out.append(sorted((x["sector"], x["level"]) for x in cur))
        return out
    assert groups(st) == groups(st_o)
    G = solver.ed_calc_green_ftn()
    Go = oracle.ed_calc_green_ftn(m, cfg.sectors, st_o, vecs, cfg.nstep, om)
    assert rel(G, Go) < gtol


@pytest.mark.parametrize("precision,etol,gtol", [("fp64", 1e-9, 1e-8), ("fp32", 1e-8, 2e-5),
                                                  ("fp32+g64", 1e-8, 1e-7)])
def test_ed_solve_green_c2(solver, oracle, pkg, precision, etol, gtol):
    """Config 2 (2-orbital Kanamori, 3 bath levels per orbital, all 81 sectors,
    largest 4,900; beta = 100, 2048 w): kept states, probabilities and G(i w_n)
    vs the oracle (dense / Lanczos eigensolves on the host)."""
    cfg = pkg.configs.config("C2")
    ek, vk = cfg.model()
    nev = 6
    solver.set_options(precision=precision.split("+")[0], green_fp64=precision.endswith("+g64"),
                       nstep=cfg.nstep, nev=nev, beta=cfg.beta)
    solver.set_model(cfg.norb, cfg.nbath, cfg.U, cfg.J, ek, vk)
    solver.set_sectors([n for n, _ in cfg.sectors], [u for _, u in cfg.sectors])
    om = cfg.omega()
    solver.set_omega(om)
    st = solver.ed_solve()
    m = oracle.Model(cfg.norb, cfg.nbath, cfg.U, cfg.J, ek, vk)
    st_o, vecs = oracle.ed_solve(m, cfg.sectors, nev, cfg.beta)
    assert len(st) == len(st_o) >= 1
    for a, c in zip(st, st_o):
        assert abs(a["val"] - c["val"]) < etol
        assert abs(a["prob"] - c["prob"]) < 1e3 * etol
    G = solver.ed_calc_green_ftn()
    Go = oracle.ed_calc_green_ftn(m, cfg.sectors, st_o, vecs, cfg.nstep, om)
    print(precision, rel(G, Go), solver.green_stats())
    assert rel(G, Go) < gtol
    if precision == "fp32+g64":
        assert 0 < solver.green_stats() < 1e-7   # Ritz residual of the FP64 refinement
    else:
        assert solver.green_stats() == 0


# ---------------------------------------------------------------- DMFT loop pieces, spectra
def test_ed_solve_threads_bitexact(solver, pkg):
    """mo_ed_solve over C2's 81 sectors from 8 host threads (worker contexts
    with their own streams and workspace) gives bit for bit the kept states
    and G(i w_n) of one thread, in FP32 and FP64."""
    cfg = pkg.configs.config("C2")
    ek, vk = cfg.model()
    for prec in ("fp32", "fp64"):
        out = {}
        for nt in (1, 8):
            solver.set_options(precision=prec, nstep=cfg.nstep, nev=6, beta=cfg.beta, solve_threads=nt)
            solver.set_model(cfg.norb, cfg.nbath, cfg.U, cfg.J, ek, vk)
            solver.set_sectors([n for n, _ in cfg.sectors], [u for _, u in cfg.sectors])
            solver.set_omega(cfg.omega())
            st = solver.ed_solve()
            out[nt] = (st, solver.ed_calc_green_ftn())
        (s1, g1), (s8, g8) = out[1], out[8]
        assert [(a["val"], a["prob"], a["sector"], a["level"]) for a in s1] == \
               [(a["val"], a["prob"], a["sector"], a["level"]) for a in s8]
        assert np.array_equal(g1, g8)
    solver.set_options(solve_threads=0)


def test_band_delta_new_occupation(solver, oracle, pkg):
    """ed_hamiltonian.F90:29-85 and ed_green.F90:187-253 at the reference's
    default Nq = 10,000 (100 x 100 grid), 3 orbitals, 512 w_n: band average,
    Gksum and the new D_ev to 1e-12 relative (the device sums the k grid in
    another order), occupations to 1e-12."""
    cfg = pkg.configs.config("C4")
    ek, vk = cfg.model()
    solver.set_model(cfg.norb, cfg.nbath, cfg.U, cfg.J, ek, vk)
    nq, nw, beta = 10000, 512, cfg.beta
    ef = solver.set_band_structure(nq)
    hk, ef_o = oracle.set_band_structure(cfg.norb, nq)
    assert np.abs(ef - ef_o).max() < 1e-15
    rng = np.random.default_rng(8)
    om = pkg.matsubara(nw, beta)
    gr = 1.0 / (1j * om[None, :] + 0.3 * rng.standard_normal((cfg.norb, 1)))
    dev = 0.2 * (rng.standard_normal((cfg.norb, nw)) + 1j * rng.standard_normal((cfg.norb, nw)))
    dn, gk = solver.delta_new(gr, dev, 1.0)
    dn_o, gk_o = oracle.delta_new(hk, 1.0, gr, dev)
    assert rel(gk, gk_o) < 1e-12 and rel(dn, dn_o) < 1e-12
    assert np.abs(solver.n_from_gksum(gk, beta) - oracle.n_from_gksum(gk_o, beta)).max() < 1e-12
    with pytest.raises(pkg.EDError):
        solver.set_band_structure(10001)   # not a square grid


@pytest.mark.parametrize("weighted", [False, True])
def test_dos_vs_oracle(solver, oracle, pkg, weighted):
    """dos.f90:1-106 on the records of a C1 solve + Green's function: the
    device spectral function against the oracle on the same records, 1e-12
    relative (runs that leave the Fock space are covered on the CPU)."""
    cfg = pkg.configs.config("C1")
    ek, vk = cfg.model()
    solver.set_options(precision="fp64", nstep=cfg.nstep, nev=8, beta=cfg.beta)
    solver.set_model(cfg.norb, cfg.nbath, cfg.U, cfg.J, ek, vk)
    solver.set_sectors([n for n, _ in cfg.sectors], [u for _, u in cfg.sectors])
    solver.set_omega(cfg.omega())
    st = solver.ed_solve()
    solver.ed_calc_green_ftn()
    recs = solver.green_coeffs()
    meta = []
    for e in st:
        nelec, nup = cfg.sectors[e["sector"] - 1]
        even = nelec - nup == nup
        for _ in range(1 if even else 2):
            for iorb in range(1, cfg.norb + 1):
                meta.append(dict(iorb=iorb, ev=e["val"], prob=e["prob"], even=int(even)))
    assert len(meta) == len(recs)
    for m, r in zip(meta, recs):
        r.update(m)
    w = np.linspace(-4.0, 4.0, 801)
    A = solver.dos(w, 0.05, weighted=weighted)
    A_o = oracle.dos(cfg.norb, recs, w, 0.05, weighted=weighted)
    assert rel(A, A_o) < 1e-12
    assert np.all(np.isfinite(A))


def _fortran_records(path):
    """Records of a gfortran unformatted sequential file (4-byte markers)."""
    data, out, o = open(path, "rb").read(), [], 0
    while o < len(data):
        n = int(np.frombuffer(data, np.int32, 1, o)[0])
        out.append(data[o + 4:o + 4 + n])
        assert int(np.frombuffer(data, np.int32, 1, o + 4 + n)[0]) == n
        o += 8 + n
    return out


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_eigvec_and_apbpanbn_files(pkg, oracle, tmp_path, precision):
    """ed_io.F90 / apbpanbn.dat round trips on C2: the exported eigenpairs
    have the reference's file layout and are eigenvectors of the oracle's H;
    a fresh context that imports them (no ed_solve) gives the same G(i w_n)
    bit for bit; apbpanbn.dat holds the same records as mo_ed_green_coeffs,
    and a context that reads it gives the same spectral function."""
    cfg = pkg.configs.config("C2")
    ek, vk = cfg.model()

    def fresh():
        s = pkg.EDSolver(0)
        s.set_options(precision=precision, nstep=cfg.nstep, nev=4, beta=cfg.beta)
        s.set_model(cfg.norb, cfg.nbath, cfg.U, cfg.J, ek, vk)
        s.set_sectors([n for n, _ in cfg.sectors], [u for _, u in cfg.sectors])
        s.set_omega(cfg.omega())
        return s

    s1 = fresh()
    st = s1.ed_solve()
    G1 = s1.ed_calc_green_ftn()
    s1.export_eigvec(str(tmp_path))
    s1.write_apbpanbn(str(tmp_path / "apbpanbn.dat"))
    w = np.linspace(-3.0, 3.0, 301)
    A1 = s1.dos(w, 0.05)
    recs = s1.green_coeffs()
    # eigenvalues.dat: nev_calc, then {ind, E, pev} per kept state
    r = _fortran_records(tmp_path / "eigenvalues.dat")
    assert len(r) == 2 and int(np.frombuffer(r[0], np.int32)[0]) == len(st)
    ent = np.frombuffer(r[1], np.dtype([("ind", "<i4"), ("val", "<f8"), ("pev", "<f8")]))
    assert [int(e["ind"]) for e in ent] == [(e["sector"] - 1) * 4 + e["level"] for e in st]
    assert np.array_equal(ent["val"], [e["val"] for e in st])
    m = oracle.Model(cfg.norb, cfg.nbath, cfg.U, cfg.J, ek, vk)
    for e in st[:3]:
        nelec, nup = cfg.sectors[e["sector"] - 1]
        r = _fortran_records(tmp_path / f"eigvec-{e['sector']:02d}-{e['level']:03d}-0000")
        v = np.frombuffer(r[1], "<f8")
        assert int(np.frombuffer(r[0], np.int32)[0]) == len(v)
        b = oracle.Basis(m.nsite, nup, nelec - nup)
        res = np.linalg.norm(oracle.multiply_H(m, b, v) - e["val"] * v) / np.linalg.norm(v)
        assert res < (1e-8 if precision == "fp64" else 1e-4)
    s1.close()
    # import: same states, same G without ed_solve
    s2 = fresh()
    assert s2.import_eigvec(str(tmp_path)) == len(st)
    assert np.array_equal(s2.ed_calc_green_ftn(), G1)
    s2.close()
    # apbpanbn.dat: the records of mo_ed_green_coeffs, read back for dos
    r = _fortran_records(tmp_path / "apbpanbn.dat")
    assert len(r) == 2 * len(recs)
    for k, rec in enumerate(recs):
        npp, nn = np.frombuffer(r[2 * k], np.int32)
        assert (npp, nn) == (rec["np"], rec["nn"])
        body = r[2 * k + 1]
        iev, iorb = np.frombuffer(body[:8], np.int32)
        ev, prob = np.frombuffer(body[8:24], "<f8")
        assert 1 <= iorb <= cfg.norb and ev == st[iev - 1]["val"] and prob == st[iev - 1]["prob"]
        coef = np.frombuffer(body[28:], "<f8")
        want = np.concatenate([rec["ap"][:npp + 1], rec["bp"][:npp + 1], rec["an"][:nn + 1], rec["bn"][:nn + 1]])
        assert np.array_equal(coef, want)
    s3 = fresh()
    assert s3.read_apbpanbn(str(tmp_path / "apbpanbn.dat")) == len(recs)
    assert np.array_equal(s3.dos(w, 0.05), A1)
    s3.close()


def test_dmft_loop_two_iterations(pkg, oracle, tmp_path):
    """main.f90's DMFT loop through the C-ABI (dmft_loop) on C1 written as an
    FDF input, two iterations, each against the oracle's chain from the same
    starting bath: G(i w_n), Gksum, the new D_ev and the occupations
    (ed_solve, ed_calc_green_ftn, ed_delta_new, n_from_gksum) to 1e-8, the
    fitted chi^2 no worse than the oracle's frprmn from the same start, and
    scf_diff.  The second iteration starts from the first's fitted bath
    (x_to_ev of its x, impurity levels included) bit for bit."""
    cfg = pkg.configs.config("C1")
    p = tmp_path / "input.fdf"
    pkg.configs.write_fdf(cfg, p, nev=8, nq=400)
    inp = pkg.configs.read_fdf(str(p))
    s = pkg.EDSolver(0)
    trace = []
    out = pkg.dmft_loop(s, inp, nloop=2, precision="fp64", trace=trace)
    s.close()
    assert out["iterations"] == 2 and len(trace) == 2 and np.all(np.isfinite(out["Sigma"]))
    norb, nbath, ns = cfg.norb, cfg.nbath, cfg.nsite
    hk, ef_band = oracle.set_band_structure(norb, 400)
    om = oracle.matsubara(cfg.nw, cfg.beta)
    assert np.abs(trace[0]["ef"] - ef_band).max() < 1e-14
    Gr_prev = np.zeros_like(trace[0]["Gr"])
    for i, t in enumerate(trace):
        if i:
            ef1, ek1, vk1 = oracle.x_to_ev(trace[i - 1]["x"], ns, nbath, norb)
            assert np.array_equal(t["ek"], ek1) and np.array_equal(t["vk"], vk1) and np.array_equal(t["ef"], ef1)
        assert rel(t["D_ev_in"], oracle.calc_dev(norb, ns, om, t["ek"], t["vk"], t["ef"])) < 1e-13
        m = oracle.Model(norb, nbath, cfg.U, cfg.J, t["ek"], t["vk"])
        st_o, vecs = oracle.ed_solve(m, inp["sectors"], 8, cfg.beta)
        Gr_o = oracle.ed_calc_green_ftn(m, inp["sectors"], st_o, vecs, cfg.nstep, om)
        assert rel(t["Gr"], Gr_o) < 1e-8
        dn_o, gk_o = oracle.delta_new(hk, inp["DMFT.Mu"], Gr_o, t["D_ev_in"])
        assert rel(t["Gksum"], gk_o) < 1e-8
        assert rel(t["D_ev"], dn_o) < 1e-8
        rec = out["history"][i]
        assert np.abs(np.array(rec["nocc"]) - oracle.n_from_gksum(gk_o, cfg.beta)).max() < 1e-8
        x0 = oracle.ev_to_x(t["ek"], t["vk"], t["ef"], ns, nbath)
        _, f_o, _, _ = oracle.frprmn(x0, ns, om, t["D_ev"], nbath, norb)
        assert rec["chi2"] <= 1.1 * f_o + 1e-10
        scf = np.sum(np.abs(Gr_prev - Gr_o).sum(axis=1) / float(np.float32(cfg.nw))) / norb
        assert abs(rec["scf_diff"] - scf) < 1e-8 * max(1.0, scf)
        Gr_prev = t["Gr"]


# ---------------------------------------------------------------- bath fit
def fit_problem(pkg, nbatch=8):
    return pkg.configs.fit_config(seed=4, nbatch=nbatch)


def test_func_dfunc_vs_oracle(solver, oracle, pkg):
    P = fit_problem(pkg)
    solver.set_options(precision="fp64")
    norb, nbath = P["norb"], P["nbath"]
    ns, nx = norb + nbath, P["X0"].shape[1]
    for x in P["X0"][:4]:
        f = solver.FUNC(x, ns, P["nw"], nx, P["omega"], P["dev"], nbath, norb)
        fo = oracle.func(x, ns, P["omega"], P["dev"], nbath, norb)
        assert abs(f - fo) < 1e-12 * abs(fo)
        g = solver.dfunc(x, P["nw"], ns, nx, P["omega"], P["dev"], nbath, norb)
        go = oracle.dfunc(x, ns, P["omega"], P["dev"], nbath, norb)
        assert rel(g, go) < 1e-12


def test_dfunc_finite_difference_device(solver, pkg):
    """Device adjoint gradient vs central differences of the device chi^2."""
    P = fit_problem(pkg)
    norb, nbath = P["norb"], P["nbath"]
    ns, nx = norb + nbath, P["X0"].shape[1]
    x = P["X0"][1]
    g = solver.dfunc(x, P["nw"], ns, nx, P["omega"], P["dev"], nbath, norb)
    for i in range(nx):
        h = 1e-5 * max(1.0, abs(x[i]))
        xp, xm = x.copy(), x.copy()
        xp[i] += h
        xm[i] -= h
        fd = (solver.FUNC(xp, ns, P["nw"], nx, P["omega"], P["dev"], nbath, norb) -
              solver.FUNC(xm, ns, P["nw"], nx, P["omega"], P["dev"], nbath, norb)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(abs(g[i]), 1e-6 * np.abs(g).max()), (i, fd, g[i])


def test_minimization_vs_oracle_and_batch(solver, oracle, pkg):
    """frprmn on the device chi^2 vs the oracle's frprmn, from starts near the
    hidden bath (one basin); a fit run alone equals the same fit in a batch bit
    for bit.  Near the noise floor of the target the reference's own limits
    (brent ITMAX, frprmn.f90:205) may stop a run whatever the arithmetic, so
    statuses are compared between the device paths and the final chi^2
    against the oracle wherever both runs converged."""
    P = fit_problem(pkg, nbatch=4)
    norb, nbath = P["norb"], P["nbath"]
    ns, nx = norb + nbath, P["X0"].shape[1]
    h = P["hidden"]
    x_true = oracle.ev_to_x(np.concatenate([h["ef"], h["eps"]]), h["vk"], h["ef"], ns, nbath)
    rng = np.random.default_rng(12)
    X0 = x_true[None, :] + 0.03 * rng.standard_normal((4, nx)) * (x_true[None, :] != 0)
    X, fret, it, st = solver.fit_batch(X0, P["omega"], P["dev"], nbath, norb)
    both = 0
    for b in range(4):
        # batching does not change a fit: bit-identical to the fit run alone
        Xs, fs, its, sts = solver.fit_batch(X0[b:b + 1], P["omega"], P["dev"], nbath, norb)
        assert sts[0] == st[b] and its[0] == it[b] and fs[0] == fret[b] and np.array_equal(Xs[0], X[b])
        xo, fo, io, rc = oracle.frprmn(X0[b], ns, P["omega"], P["dev"], nbath, norb)
        f0 = oracle.func(X0[b], ns, P["omega"], P["dev"], nbath, norb)
        assert fret[b] < 1e-2 * f0 and fo < 1e-2 * f0          # both reach the basin floor
        if st[b] == 0 and rc == 0:
            both += 1
            # the relative-change stop test of frprmn lets trajectories that
            # differ in rounding stop a few per cent apart on the floor
            assert abs(fret[b] - fo) <= 1e-1 * max(fret[b], fo) + 1e-14
    assert both >= 1
    # the reference-facing single-fit entry point (minimization, FTOL 1e-7)
    # from the hidden bath itself: a short run to the noisy target's optimum
    x1, f1, i1 = solver.minimization(x_true, P["nw"], ns, nx, P["omega"], P["dev"], nbath, norb)
    assert f1 <= oracle.func(x_true, ns, P["omega"], P["dev"], nbath, norb)


def test_fit_small_grid_one_cta(solver, oracle, pkg):
    """Below 256 w_n a fit runs on one CTA of 256 threads (no cluster): FUNC /
    dfunc on 128 w_n against the oracle, and fits from starts near the hidden
    bath that reach the oracle's floor, alone and in a batch bit for bit."""
    P = pkg.configs.fit_config(seed=4, nbatch=3)
    norb, nbath = P["norb"], P["nbath"]
    ns, nx = norb + nbath, P["X0"].shape[1]
    om, dev = P["omega"][:128], P["dev"][:, :128]
    solver.set_options(precision="fp64")
    for x in P["X0"][:2]:
        f = solver.FUNC(x, ns, 128, nx, om, dev, nbath, norb)
        assert abs(f - oracle.func(x, ns, om, dev, nbath, norb)) < 1e-12 * f
        g = solver.dfunc(x, 128, ns, nx, om, dev, nbath, norb)
        assert rel(g, oracle.dfunc(x, ns, om, dev, nbath, norb)) < 1e-12
    h = P["hidden"]
    x_true = oracle.ev_to_x(np.concatenate([h["ef"], h["eps"]]), h["vk"], h["ef"], ns, nbath)
    X0 = x_true[None, :] + 0.02 * np.random.default_rng(3).standard_normal((3, nx)) * (x_true[None, :] != 0)
    X, fret, it, st = solver.fit_batch(X0, om, dev, nbath, norb)
    for b in range(3):
        Xs, fs, its, sts = solver.fit_batch(X0[b:b + 1], om, dev, nbath, norb)
        assert its[0] == it[b] and fs[0] == fret[b] and np.array_equal(Xs[0], X[b])
        _, fo, _, rc = oracle.frprmn(X0[b], ns, om, dev, nbath, norb)
        f0 = oracle.func(X0[b], ns, om, dev, nbath, norb)
        assert fret[b] < 1e-2 * f0 and fo < 1e-2 * f0


def test_fit_parking_does_not_change_results(solver, oracle, pkg):
    """A fit that gives up its cluster to a waiting fit, and is resumed later,
    ends where it ends without a break, bit for bit.  The batches hold more
    fits than the GPU runs at once, and fits look for waiting fits every 3 CG
    iterations (fit_quantum).  They are compared with the same batches at the
    default 256 and with fits run alone, on the one-CTA shape (128 w_n) and
    on 4-CTA clusters (512 w_n).  ftol = 1e-5 keeps the fits short."""
    P = pkg.configs.fit_config(seed=4, nbatch=3)
    norb, nbath = P["norb"], P["nbath"]
    ns, nx = norb + nbath, P["X0"].shape[1]
    h = P["hidden"]
    x_true = oracle.ev_to_x(np.concatenate([h["ef"], h["eps"]]), h["vk"], h["ef"], ns, nbath)
    rng = np.random.default_rng(21)
    solver.set_options(precision="fp64")
    try:
        for nw, nb in ((128, 160), (512, 80)):
            om, dev = P["omega"][:nw], P["dev"][:, :nw]
            X0 = x_true[None, :] + 0.05 * rng.standard_normal((nb, nx)) * (x_true[None, :] != 0)
            solver.set_options(fit_quantum=3)
            Xa, fa, ia, sa = solver.fit_batch(X0, om, dev, nbath, norb, ftol=1e-5)
            stats = solver.fit_stats()
            print(nw, stats, "CG iterations", int(ia.min()), int(np.median(ia)), int(ia.max()))
            assert stats["suspensions"] > 0 and stats["clusters"] < nb
            solver.set_options(fit_quantum=0)
            Xb, fb, ib, sb = solver.fit_batch(X0, om, dev, nbath, norb, ftol=1e-5)
            assert np.array_equal(Xa, Xb) and np.array_equal(fa, fb)
            assert np.array_equal(ia, ib) and np.array_equal(sa, sb)
            order = np.argsort(ia, kind="stable")
            for b in order[[nb // 2, (3 * nb) // 4]]:
                Xs, fs, its, sts = solver.fit_batch(X0[b:b + 1], om, dev, nbath, norb, ftol=1e-5)
                assert sts[0] == sa[b] and its[0] == ia[b] and fs[0] == fa[b] and np.array_equal(Xs[0], Xa[b])
    finally:
        solver.set_options(fit_quantum=0)


def test_calc_dev_vs_oracle(solver, oracle):
    rng = np.random.default_rng(10)
    norb, nbath = 3, 12
    om = (2 * np.arange(200) + 1) * np.pi / 200.0
    ek, vk, ef = rng.standard_normal(norb + nbath), rng.standard_normal((norb, nbath)), rng.standard_normal(norb)
    d = solver.calc_dev(norb, norb + nbath, om, ek, vk, ef)
    assert rel(d, oracle.calc_dev(norb, norb + nbath, om, ek, vk, ef)) < 1e-14
