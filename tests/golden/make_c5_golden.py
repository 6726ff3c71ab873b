"""Generate tests/golden/c5_oracle.npz: the oracle's frprmn on every start of
the C5 bath fit (3 orbitals x 4 bath levels, 512 w_n at beta = 200, 256
random starts; mo-dmft_gb300/configs.py fit_config(seed=4)).

For each start the oracle (oracle/, the C restatement of frprmn.f90 driven as
minimization() drives it, func.f90:144-163, FTOL 1e-7) returns the final
parameters, chi^2, the CG iteration count and the status (0, or the code for
the reference's own limits: frprmn itmax 20000, brent ITMAX 100).
Run from the repository root:  python tests/golden/make_c5_golden.py
(a few minutes on 8 cores).  Only the tests read the output.
"""
import multiprocessing as mp
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)


def _fit(b):
    import __graft_entry__ as g
    O = g.load_oracle()
    P = g.load_package().configs.fit_config(seed=4, nbatch=256)
    norb, nbath = P["norb"], P["nbath"]
    t0 = time.perf_counter()
    x, f, it, rc = O.frprmn(P["X0"][b], norb + nbath, P["omega"], P["dev"], nbath, norb)
    return b, x, f, it, rc, time.perf_counter() - t0


def main():
    import __graft_entry__ as g
    P = g.load_package().configs.fit_config(seed=4, nbatch=256)
    nb, nx = P["X0"].shape
    X = np.zeros((nb, nx))
    fret, secs = np.zeros(nb), np.zeros(nb)
    it, st = np.zeros(nb, dtype=np.int32), np.zeros(nb, dtype=np.int32)
    t0 = time.time()
    with mp.get_context("spawn").Pool(os.cpu_count()) as pool:
        for b, x, f, i, rc, s in pool.imap_unordered(_fit, range(nb)):
            X[b], fret[b], it[b], st[b], secs[b] = x, f, i, rc, s
    print(f"{nb} fits in {time.time() - t0:.0f} s; {int((st != 0).sum())} stopped by a limit; "
          f"median {np.median(it):.0f} iterations, {np.median(secs):.2f} s per fit")
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "c5_oracle.npz")
    np.savez_compressed(out, X=X, fret=fret, iter=it, status=st, seconds=secs)
    print("wrote", out)


if __name__ == "__main__":
    main()
