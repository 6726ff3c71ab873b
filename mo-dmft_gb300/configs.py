"""Synthetic impurity models of the five benchmark configurations.

No dataset is involved: every input is drawn from numpy.random.default_rng(seed)
in the order bath energies eps_k, then couplings V (row-major [orbital][bath
level of that orbital]).  "k bath levels per orbital" is the reference's shared
bath list (ed_config.f90:97-114) with Nbath = norb*k and a block-diagonal V
(orbital a couples to levels a*k .. a*k+k-1).

The impurity level ek(1:norb) is the particle-hole symmetric value
-mu_ph = -(U + (norb-1)(2U' - J))/2 with U' = U - 2J, so the half-filled
sectors named by the configurations hold the ground state (the reference
starts from the band average and lets the bath fit move it,
ed_hamiltonian.F90:53-56, func.f90:199-202).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class ImpurityConfig:
    name: str
    norb: int
    nper: int                 # bath levels per orbital
    U: float
    J: float
    beta: float
    nw: int
    nstep: int
    seed: int
    eps_range: tuple
    v_range: tuple
    sectors: list = field(default_factory=list)   # (nelec, nup)

    @property
    def nbath(self):
        return self.norb * self.nper

    @property
    def nsite(self):
        return self.norb + self.nbath

    def mu_ph(self):
        Up = self.U - 2 * self.J
        return 0.5 * (self.U + (self.norb - 1) * (2 * Up - self.J))

    def model(self):
        """(ek[nsite], vk[norb, nbath]) for this configuration."""
        rng = np.random.default_rng(self.seed)
        eps = rng.uniform(self.eps_range[0], self.eps_range[1], self.nbath)
        v = rng.uniform(self.v_range[0], self.v_range[1], (self.norb, self.nper))
        vk = np.zeros((self.norb, self.nbath))
        for a in range(self.norb):
            vk[a, a * self.nper:(a + 1) * self.nper] = v[a]
        ek = np.concatenate([np.full(self.norb, -self.mu_ph()), eps])
        return ek, vk

    def omega(self):
        return (2.0 * np.arange(self.nw) + 1.0) * np.pi / self.beta


def all_sectors(nsite):
    return [(nu + nd, nu) for nu in range(nsite + 1) for nd in range(nsite + 1)]


def config(name: str) -> ImpurityConfig:
    """C1..C4 impurity configurations."""
    if name == "C1":   # single band, 4 bath levels, all sectors, U=2, mu=U/2, beta=50
        c = ImpurityConfig("C1", 1, 4, 2.0, 0.0, 50.0, 1024, 100, 0, (-1.0, 1.0), (0.1, 0.5))
        c.sectors = all_sectors(c.nsite)
        return c
    if name == "C2":   # 2-orbital Kanamori, 3 bath levels per orbital, all sectors
        c = ImpurityConfig("C2", 2, 3, 4.0, 1.0, 100.0, 2048, 100, 1, (-2.0, 2.0), (0.1, 0.6))
        c.sectors = all_sectors(c.nsite)
        return c
    if name == "C3":   # 3 orbitals x 3 bath levels, sector (6,6), 150 steps
        c = ImpurityConfig("C3", 3, 3, 3.0, 0.5, 200.0, 1024, 150, 2, (-1.0, 1.0), (0.1, 0.5))
        c.sectors = [(12, 6)]
        return c
    if name == "C4":   # 3 orbitals x 4 bath levels, ground sector (7,8), 4096 w
        c = ImpurityConfig("C4", 3, 4, 3.0, 0.5, 200.0, 4096, 100, 3, (-1.0, 1.0), (0.1, 0.5))
        c.sectors = [(15, 7)]
        return c
    raise KeyError(name)


def fit_config(seed=4, nbatch=256, noise=1e-4):
    """C5: 3 orbitals x 4 bath levels, 512 w at beta=200, target Delta from a
    hidden bath (eps ~ U[-2,2], V ~ U[0.1,0.6]) plus complex Gaussian noise,
    and nbatch random initial parameter sets.  Returns a dict."""
    norb, nper, nw, beta = 3, 4, 512, 200.0
    nbath = norb * nper
    rng = np.random.default_rng(seed)
    eps = rng.uniform(-2.0, 2.0, nbath)
    v = rng.uniform(0.1, 0.6, (norb, nper))
    vk = np.zeros((norb, nbath))
    for a in range(norb):
        vk[a, a * nper:(a + 1) * nper] = v[a]
    ef = rng.uniform(-0.5, 0.5, norb)
    omega = (2.0 * np.arange(nw) + 1.0) * np.pi / beta
    z = 1j * omega[None, :, None] - eps[None, None, :]
    dev = (vk[:, None, :] ** 2 / z).sum(-1) + ef[:, None]
    dev = dev + noise * (rng.standard_normal(dev.shape) + 1j * rng.standard_normal(dev.shape))
    nx = nbath + nbath * norb + norb
    X0 = np.zeros((nbatch, nx))
    for b in range(nbatch):
        e0 = rng.uniform(-2.0, 2.0, nbath)
        v0 = rng.uniform(0.1, 0.6, (norb, nper))
        vk0 = np.zeros((norb, nbath))
        for a in range(norb):
            vk0[a, a * nper:(a + 1) * nper] = v0[a]
        f0 = rng.uniform(-0.5, 0.5, norb)
        X0[b, :nbath] = e0
        X0[b, nbath:nbath + nbath * norb] = vk0.ravel()   # x = [eps, V(1,:), ..., V(norb,:), ef]
        X0[b, nbath + nbath * norb:] = f0
    return dict(norb=norb, nbath=nbath, nw=nw, beta=beta, omega=omega, dev=dev, X0=X0,
                hidden=dict(eps=eps, vk=vk, ef=ef))
