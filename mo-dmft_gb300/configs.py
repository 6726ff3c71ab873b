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


# ---------------------------------------------------------------------------
# FDF input files (ed_config.f90:43-126)
# ---------------------------------------------------------------------------
# Labels the reference reads, with its defaults.  FDF compares labels without
# case and without '.', '_' and '-'.
FDF_DEFAULTS = {
    "DMFT.Norbs": 2, "DMFT.Nbaths": 2, "DMFT.Nsectors": 2, "DMFT.U": 1.0, "DMFT.J": 0.3,
    "DMFT.Mu": 1.0, "DMFT.beta": 100.0, "DMFT.small": 0.05, "DMFT.ContinuedFractionSteps": 50,
    "DMFT.MaxIterations": 100, "DMFT.ScfTolerance": 1e-4, "DMFT.Nev": 30, "DMFT.Nq": 10000,
    "DMFT.Nw": 2000,
}


def _fdf_key(label):
    return "".join(ch for ch in label.lower() if ch not in "._-")


def read_fdf(path_or_text):
    """Parse an FDF input with the reference's DMFT labels.

    Returns a dict with every scalar of ed_config.f90:52-126 (the reference's
    defaults where a label is absent), "sectors" [(nelec, nup)] from
    %block DMFT.Sectors, "eps_bath" (nbath) from DMFT.Baths and "vk"
    (norb, nbath) from DMFT.BathCouplings (one line per bath level, one column
    per orbital).  Lines after the first Nsectors / Nbaths of a block are
    ignored, as the reference's loops stop there."""
    text = path_or_text
    if "\n" not in text and not text.lstrip().startswith("DMFT"):
        with open(path_or_text) as f:
            text = f.read()
    scal, blocks, cur = {}, {}, None
    for raw in text.splitlines():
        line = raw.split("#", 1)[0].strip()
        if not line:
            continue
        words = line.split()
        if words[0].lower() == "%block":
            cur = _fdf_key(words[1])
            blocks[cur] = []
            continue
        if words[0].lower() == "%endblock":
            cur = None
            continue
        if cur is not None:
            blocks[cur].append(words)
        elif len(words) >= 2:
            scal[_fdf_key(words[0])] = words[1]
    out = {}
    for label, dflt in FDF_DEFAULTS.items():
        v = scal.get(_fdf_key(label))
        if v is None:
            out[label] = dflt
        else:
            v = v.replace("d", "e").replace("D", "e")
            out[label] = int(v) if isinstance(dflt, int) else float(v)
    norb, nbath, nsec = out["DMFT.Norbs"], out["DMFT.Nbaths"], out["DMFT.Nsectors"]
    sec = blocks.get(_fdf_key("DMFT.Sectors"), [])[:nsec]
    out["sectors"] = [(int(w[0]), int(w[1])) for w in sec]
    baths = blocks.get(_fdf_key("DMFT.Baths"), [])[:nbath]
    out["eps_bath"] = np.array([float(w[0].replace("d", "e").replace("D", "e")) for w in baths])
    cpl = blocks.get(_fdf_key("DMFT.BathCouplings"), [])[:nbath]
    vk = np.zeros((norb, nbath))
    for i, w in enumerate(cpl):
        for j in range(norb):
            vk[j, i] = float(w[j].replace("d", "e").replace("D", "e"))
    out["vk"] = vk
    return out


def write_fdf(cfg: ImpurityConfig, path, nev=30, nq=10000, mu=None, small=0.05, nloop=100, scf_tol=1e-4):
    """Write a configuration as an FDF input the reference reads
    (ed_config.f90:52-126).  The reference takes the impurity levels from the
    band structure (ed_hamiltonian.F90:53-56), not from the input, so ek(1:norb)
    of cfg.model() is not written."""
    ek, vk = cfg.model()
    lines = [
        f"DMFT.Norbs {cfg.norb}", f"DMFT.Nbaths {cfg.nbath}", f"DMFT.Nsectors {len(cfg.sectors)}",
        "%block DMFT.Sectors", *[f"  {n} {u}" for n, u in cfg.sectors], "%endblock DMFT.Sectors",
        f"DMFT.U {cfg.U!r}", f"DMFT.J {cfg.J!r}", f"DMFT.Mu {float(cfg.mu_ph() if mu is None else mu)!r}",
        f"DMFT.beta {cfg.beta!r}",
        "%block DMFT.Baths", *[f"  {float(e)!r}" for e in ek[cfg.norb:]], "%endblock DMFT.Baths",
        "%block DMFT.BathCouplings", *["  " + " ".join(repr(float(v)) for v in vk[:, i]) for i in range(cfg.nbath)],
        "%endblock DMFT.BathCouplings",
        f"DMFT.small {small!r}", f"DMFT.ContinuedFractionSteps {cfg.nstep}", f"DMFT.MaxIterations {nloop}",
        f"DMFT.ScfTolerance {scf_tol!r}", f"DMFT.Nev {nev}", f"DMFT.Nq {nq}", f"DMFT.Nw {cfg.nw}",
    ]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
