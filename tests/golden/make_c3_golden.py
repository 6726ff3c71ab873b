"""Generate tests/golden/c3_oracle.npz: the oracle's FP64 results on the full
C3 sector (3 orbitals x 3 bath levels, Nup = Ndn = 6, D = 853,776).

The oracle (oracle/, the C restatement of the reference) runs on the host:
  * ed_solve (ed_solver.F90:28-105) with nev = 6: kept eigenvalues and
    Boltzmann weights;
  * ed_calc_green_ftn (ed_green.F90:60-185) with the configuration's 150
    Lanczos steps over 1024 Matsubara frequencies at beta = 200: G(i w_n);
  * lanczos_iteration (ed_lanczos.F90:14-68), 150 steps from the seeded start
    vector numpy.random.default_rng(START_SEED).standard_normal(D): a, b,
    nstep_calc.
Run from the repository root:  python tests/golden/make_c3_golden.py
(about 10 minutes on 8 cores).  Only the tests read the output.
"""
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

NEV = 6
START_SEED = 20


def main():
    import __graft_entry__ as g
    O = g.load_oracle()
    cfg = g.load_package().configs.config("C3")
    ek, vk = cfg.model()
    m = O.Model(cfg.norb, cfg.nbath, cfg.U, cfg.J, ek, vk)
    sectors = cfg.sectors
    om = cfg.omega()
    t0 = time.time()
    states, vecs = O.ed_solve(m, sectors, NEV, cfg.beta)
    print(f"ed_solve: {len(states)} kept states, E0 = {states[0]['val']:.12f} ({time.time() - t0:.0f} s)",
          flush=True)
    _, vals, _ = O.sector_eigs(m, sectors[0][1], sectors[0][0] - sectors[0][1], NEV, want_vectors=False)
    t0 = time.time()
    Gr = O.ed_calc_green_ftn(m, sectors, states, vecs, cfg.nstep, om)
    print(f"green: ({time.time() - t0:.0f} s)", flush=True)
    nup = sectors[0][1]
    b = O.Basis(cfg.nsite, nup, sectors[0][0] - nup)
    v0 = np.random.default_rng(START_SEED).standard_normal(b.ntot)
    t0 = time.time()
    nc, a, bb = O.lanczos_iteration(m, b, v0, cfg.nstep)
    print(f"lanczos: nstep_calc = {nc} ({time.time() - t0:.0f} s)", flush=True)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "c3_oracle.npz")
    np.savez_compressed(out, nev=NEV, start_seed=START_SEED, eigvals=vals,
                        state_val=np.array([s["val"] for s in states]),
                        state_prob=np.array([s["prob"] for s in states]),
                        state_level=np.array([s["level"] for s in states]),
                        omega=om, Gr=Gr, lz_nstep_calc=nc, lz_a=a, lz_b=bb)
    print("wrote", out)


if __name__ == "__main__":
    main()
