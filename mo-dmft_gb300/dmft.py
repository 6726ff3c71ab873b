"""The reference's DMFT self-consistency loop (main.f90:40-160) on one GPU.

Every step is a call of the C-ABI through EDSolver, in the reference's
order:

  ed_read_options / ed_set_band_structure / ed_green_init  (initial D_ev = calc_dev)
  loop:  ed_solve -> ed_calc_green_ftn -> ed_delta_new -> n_from_gksum
         -> ev_to_x -> minimization -> x_to_ev -> scf_diff -> calc_dev
  Sigma = i w_n - D_ev - 1/Gr

The input is the dict configs.read_fdf returns (the reference's FDF labels).
One GPU holds every Matsubara frequency, so the MPI gathers and broadcasts of
the reference are identities here.
"""
from __future__ import annotations

import time

import numpy as np

from .ed import EDError, EDSolver, ev_to_x, matsubara, x_to_ev


def dmft_loop(solver: EDSolver, inp: dict, nloop: int | None = None, precision: str = "fp32",
              green_fp64: bool = False, callback=None, trace: list | None = None, fit_starts: int = 1) -> dict:
    """Run the DMFT loop of main.f90 with the parameters of an FDF input.

    solver: an open EDSolver (its options, model, sectors and omega are set here).
    inp: configs.read_fdf output.  nloop overrides DMFT.MaxIterations.
    callback(iteration, record) is called after every iteration with its record
    (scf_diff, chi^2, CG iterations, occupations, nev_calc, seconds).
    fit_starts: 1 (default) is the reference's single minimization from the
    current bath, which STOPs the run (EDError, MO_ED_ERR_FIT) when frprmn
    exceeds its iteration limit.  fit_starts > 1 fits the current bath and
    fit_starts - 1 seeded perturbations of it (every parameter scaled by
    1 + 0.05 N(0, 1), so zero couplings stay zero) in one batched device fit
    (mo_ed_fit_batch) and takes the lowest chi^2 of the fits that end within
    frprmn's limits; the run STOPs only when none does.
    trace: a list that receives, per iteration, the iteration's starting bath
    (ek, vk, ef), the D_ev it starts from, Gr, Gksum, the new D_ev of
    delta_new and the fitted parameters x (copies).

    Returns dict(converged, iterations, history, Gr, D_ev, Gksum, Sigma, ek, vk, ef, nocc, omega)."""
    norb, nbath = inp["DMFT.Norbs"], inp["DMFT.Nbaths"]
    nsite = norb + nbath
    beta, mu = inp["DMFT.beta"], inp["DMFT.Mu"]
    nw, nq = inp["DMFT.Nw"], inp["DMFT.Nq"]
    nloop = inp["DMFT.MaxIterations"] if nloop is None else nloop
    scf_tol = inp["DMFT.ScfTolerance"]
    U, J = inp["DMFT.U"], inp["DMFT.J"]
    ek = np.zeros(nsite)
    ek[norb:] = inp["eps_bath"]
    vk = np.array(inp["vk"], dtype=np.float64).reshape(norb, nbath)
    solver.set_options(precision=precision, green_fp64=green_fp64, nstep=inp["DMFT.ContinuedFractionSteps"],
                       nev=inp["DMFT.Nev"], beta=beta)
    # ed_hamiltonian_init / ed_set_band_structure: ek(1:norb) = ef = band average
    solver.set_model(norb, nbath, U, J, ek, vk)
    ef = solver.set_band_structure(nq)
    ek[:norb] = ef
    # ed_green_init: omega_n and D_ev = calc_dev
    omega = matsubara(nw, beta)
    solver.set_omega(omega)
    solver.set_sectors([n for n, _ in inp["sectors"]], [u for _, u in inp["sectors"]])
    D_ev = solver.calc_dev(norb, nsite, omega, ek, vk, ef)
    Gr_prev = np.zeros((norb, nw), dtype=np.complex128)
    nx = nbath + nbath * norb + norb
    history, converged, iloop = [], False, 0
    Gr = Gksum = nocc = None
    while not converged and iloop < nloop:
        t0 = time.perf_counter()
        if trace is not None:
            step = dict(ek=ek.copy(), vk=vk.copy(), ef=np.array(ef, dtype=np.float64), D_ev_in=D_ev.copy())
        solver.set_model(norb, nbath, U, J, ek, vk)
        states = solver.ed_solve()
        Gr = solver.ed_calc_green_ftn()
        D_ev, Gksum = solver.delta_new(Gr, D_ev, mu)
        nocc = solver.n_from_gksum(Gksum, beta)
        x = ev_to_x(ek, vk, ef, nsite, nbath)
        if fit_starts <= 1:
            x, fret, it = solver.minimization(x, nw, nsite, nx, omega, D_ev, nbath, norb)
        else:
            rng = np.random.default_rng(1000 + iloop)
            X0 = np.repeat(x[None, :], fit_starts, axis=0)
            X0[1:] *= 1.0 + 0.05 * rng.standard_normal((fit_starts - 1, nx))
            X, F, IT, ST = solver.fit_batch(X0, omega, D_ev, nbath, norb)
            ok = np.flatnonzero(ST == 0)
            if ok.size == 0:
                raise EDError(6, "frprmn: iteration limit exceeded from every start")
            k = ok[np.argmin(F[ok])]
            x, fret, it = X[k], float(F[k]), int(IT[k])
        if trace is not None:
            step.update(Gr=Gr.copy(), Gksum=np.array(Gksum), D_ev=D_ev.copy(), x=np.array(x))
            trace.append(step)
        ef, ek, vk = x_to_ev(x, nsite, nbath, norb)
        # scf_diff (main.f90:95-101): mean over orbitals of sum_w |Gr_prev - Gr| / float(Nw)
        tol = float(np.sum(np.abs(Gr_prev - Gr).sum(axis=1) / float(np.float32(nw))) / norb)
        Gr_prev = Gr.copy()
        D_ev = solver.calc_dev(norb, nsite, omega, ek, vk, ef)
        converged = tol < scf_tol
        rec = dict(iteration=iloop, scf_diff=tol, chi2=fret, cg_iterations=it, nocc=nocc.tolist(),
                   nev_calc=len(states), seconds=time.perf_counter() - t0)
        history.append(rec)
        if callback is not None:
            callback(iloop, rec)
        iloop += 1
    # self-energy (main.f90:145-150); CMPLX(0, omega) rounds omega to default REAL
    sigma = 1j * omega.astype(np.float32).astype(np.float64)[None, :] - D_ev - 1.0 / Gr
    return dict(converged=converged, iterations=iloop, history=history, Gr=Gr, D_ev=D_ev, Gksum=Gksum,
                Sigma=sigma, ek=ek, vk=vk, ef=ef, nocc=nocc, omega=omega)
