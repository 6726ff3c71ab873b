"""CPU test of the DMFT loop driver (dmft.py, main.f90:40-160): dmft_loop runs
against a stand-in solver whose methods are the oracle's restatements, so the
order of the steps, the scf_diff formula and the self-energy are checked
without a GPU.  The device solver behind the same methods is checked against
the oracle by the GPU parity tests."""
import numpy as np


class OracleSolver:
    """The EDSolver methods dmft_loop calls, on the CPU oracle."""

    def __init__(self, O):
        self.O = O
        self.calls = []

    def set_options(self, **kw):
        self.opt = kw
        self.calls.append("set_options")

    def set_model(self, norb, nbath, U, J, ek, vk):
        self.norb, self.nbath = norb, nbath
        self.m = self.O.Model(norb, nbath, U, J, np.array(ek), np.array(vk))
        self.calls.append("set_model")

    def set_band_structure(self, nq):
        self.hk, ef = self.O.set_band_structure(self.norb, nq)
        self.calls.append("set_band_structure")
        return ef

    def set_omega(self, om):
        self.om = np.array(om)

    def set_sectors(self, nelec, nup):
        self.sectors = list(zip(nelec, nup))

    def calc_dev(self, norb, nsite, om, ek, vk, ef):
        self.calls.append("calc_dev")
        return self.O.calc_dev(norb, nsite, om, ek, vk, ef)

    def ed_solve(self):
        self.states, self.vecs = self.O.ed_solve(self.m, self.sectors, self.opt["nev"], self.opt["beta"])
        self.calls.append("ed_solve")
        return self.states

    def ed_calc_green_ftn(self):
        self.calls.append("green")
        return self.O.ed_calc_green_ftn(self.m, self.sectors, self.states, self.vecs, self.opt["nstep"], self.om)

    def delta_new(self, gr, dev, mu):
        self.calls.append("delta_new")
        return self.O.delta_new(self.hk, mu, gr, dev)

    def n_from_gksum(self, gk, beta):
        self.calls.append("n_from_gksum")
        return self.O.n_from_gksum(gk, beta)

    def minimization(self, x, nw, ns, nx, om, dev, nbath, norb):
        self.calls.append("minimization")
        p, f, it, rc = self.O.frprmn(x, ns, om, dev, nbath, norb)
        assert rc == 0
        return p, f, it


def test_dmft_loop_order_and_outputs(pkg, oracle):
    text = "\n".join([
        "DMFT.Norbs 1", "DMFT.Nbaths 3", "DMFT.Nsectors 3",
        "%block DMFT.Sectors", "  4 2", "  3 2", "  5 3", "%endblock DMFT.Sectors",
        "DMFT.U 2.0", "DMFT.J 0.0", "DMFT.Mu 1.0", "DMFT.beta 20.0",
        "%block DMFT.Baths", "  -0.6", "  0.1", "  0.7", "%endblock DMFT.Baths",
        "%block DMFT.BathCouplings", "  0.3", "  0.25", "  0.4", "%endblock DMFT.BathCouplings",
        "DMFT.ContinuedFractionSteps 40", "DMFT.Nev 4", "DMFT.Nq 64", "DMFT.Nw 64",
        "DMFT.ScfTolerance 1d-12"])
    inp = pkg.configs.read_fdf(text)
    s = OracleSolver(oracle)
    hist = []
    out = pkg.dmft_loop(s, inp, nloop=2, callback=lambda i, r: hist.append(r))
    # main.f90's order: set-up, then per iteration solve, G, delta_new, occupations,
    # minimization, calc_dev
    it = ["set_model", "ed_solve", "green", "delta_new", "n_from_gksum", "minimization", "calc_dev"]
    assert s.calls == ["set_options", "set_model", "set_band_structure", "calc_dev"] + it + it
    assert out["iterations"] == 2 and not out["converged"] and len(hist) == 2
    # scf_diff of the first iteration: Gr_prev = 0, so mean_orb sum_w |Gr| / Nw
    # of that iteration's Gr; recompute it from the same chain
    ek = np.concatenate([np.zeros(1), inp["eps_bath"]])
    hk, ef = oracle.set_band_structure(1, 64)
    ek[:1] = ef
    m = oracle.Model(1, 3, 2.0, 0.0, ek, inp["vk"])
    om = oracle.matsubara(64, 20.0)
    st, vecs = oracle.ed_solve(m, inp["sectors"], 4, 20.0)
    g1 = oracle.ed_calc_green_ftn(m, inp["sectors"], st, vecs, 40, om)
    assert abs(hist[0]["scf_diff"] - np.abs(g1).sum() / 64) < 1e-12
    # Sigma = CMPLX(0, w) - D_ev - 1/Gr with the final D_ev (calc_dev of the fitted bath)
    dev = oracle.calc_dev(1, 4, om, out["ek"], out["vk"], out["ef"])
    w32 = om.astype(np.float32).astype(np.float64)
    assert np.allclose(out["Sigma"], 1j * w32[None, :] - dev - 1.0 / out["Gr"], rtol=0, atol=1e-12)
    assert np.all(np.isfinite(out["Sigma"])) and 0.0 < out["nocc"][0] < 2.0


class MultiStartSolver(OracleSolver):
    """The stand-in with fit_batch: the oracle's frprmn per start, and the
    second start reported as stopped by frprmn's iteration limit."""

    def fit_batch(self, X, om, dev, nbath, norb):
        self.calls.append("fit_batch")
        self.starts = np.array(X)
        out = [self.O.frprmn(x, nbath + norb, om, dev, nbath, norb) for x in X]
        P = np.array([o[0] for o in out])
        F = np.array([o[1] for o in out])
        IT = np.array([o[2] for o in out], np.int32)
        ST = np.array([o[3] for o in out], np.int32)
        ST[1] = 6
        F[1] = -1.0            # the lowest chi^2, but stopped: must not be taken
        self.F, self.ST = F, ST
        return P, F, IT, ST


def test_dmft_loop_multistart_fit(pkg, oracle):
    """fit_starts > 1: the current bath plus seeded perturbations in one batch
    (zero couplings stay zero); the lowest chi^2 among the fits that ended
    within frprmn's limits is taken."""
    text = "\n".join([
        "DMFT.Norbs 1", "DMFT.Nbaths 3", "DMFT.Nsectors 2",
        "%block DMFT.Sectors", "  4 2", "  3 2", "%endblock DMFT.Sectors",
        "DMFT.U 2.0", "DMFT.J 0.0", "DMFT.Mu 1.0", "DMFT.beta 20.0",
        "%block DMFT.Baths", "  -0.6", "  0.1", "  0.7", "%endblock DMFT.Baths",
        "%block DMFT.BathCouplings", "  0.3", "  0.0", "  0.4", "%endblock DMFT.BathCouplings",
        "DMFT.ContinuedFractionSteps 30", "DMFT.Nev 4", "DMFT.Nq 64", "DMFT.Nw 64",
        "DMFT.ScfTolerance 1d-12"])
    inp = pkg.configs.read_fdf(text)
    s = MultiStartSolver(oracle)
    hist = []
    out = pkg.dmft_loop(s, inp, nloop=1, callback=lambda i, r: hist.append(r), fit_starts=4)
    assert "fit_batch" in s.calls and "minimization" not in s.calls
    X0 = s.starts
    assert X0.shape[0] == 4 and np.all(X0[:, X0[0] == 0] == 0)     # zeros stay zero
    assert not np.array_equal(X0[0], X0[2])
    assert hist[0]["chi2"] == s.F[s.ST == 0].min()                  # the stopped start is skipped
    assert out["iterations"] == 1
