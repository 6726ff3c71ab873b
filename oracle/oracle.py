"""Python face of the CPU oracle (TEST INFRASTRUCTURE ONLY).

This module is the parity reference for the CUDA solver and the "port" CPU baseline of
``bench.py``.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` may import it; the product library never does.

It wraps ``oracle/lib/libedoracle.so`` (the C restatement in ``ed_oracle.c``,
built by ``oracle/Makefile``) and adds, in numpy:

* ``jw_sector_H`` -- an independent Jordan-Wigner construction of the sector
  Hamiltonian from explicit fermion-operator matrices, used to pin the C
  restatement's term coefficients and fermion signs;
* ``ed_solve`` -- ed_solver.F90:28-105 with the PARPACK ``diag`` (not part of
  the reference sources) replaced by dense ``numpy.linalg.eigh`` for small
  sectors and by ``scipy.sparse.linalg.eigsh`` (ARPACK, which='SA') on the
  restated ``multiply_H`` otherwise;
* ``ed_calc_green_ftn`` -- ed_green.F90:60-185 on top of the restated
  ``apply_c``, ``lanczos_iteration`` and continued fraction.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "lib", "libedoracle.so")
_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class _Model(C.Structure):
    _fields_ = [("norb", C.c_int), ("nbath", C.c_int), ("nsite", C.c_int),
                ("U", C.c_double), ("Jex", C.c_double),
                ("ek", _dp), ("vk", _dp)]


class _Basis(C.Structure):
    _fields_ = [("nsite", C.c_int), ("ne_up", C.c_int), ("ne_down", C.c_int),
                ("nup", C.c_int), ("ndown", C.c_int), ("ntot", C.c_int64),
                ("up", _ip), ("down", _ip), ("idx_up", _ip), ("idx_down", _ip)]


def build():
    """Compile the C restatement with its Makefile (gcc, portable flags)."""
    import subprocess
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        L.or_icom.restype = C.c_int
        L.or_icom.argtypes = [C.c_int, C.c_int]
        L.or_generate_basis.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(_Basis)]
        L.or_free_basis.argtypes = [C.POINTER(_Basis)]
        L.or_basis_get.restype = C.c_uint32
        L.or_basis_get.argtypes = [C.POINTER(_Basis), C.c_int64]
        L.or_basis_idx.restype = C.c_int64
        L.or_basis_idx.argtypes = [C.POINTER(_Basis), C.c_uint32]
        for f in ("or_number_op", "or_destruction_op", "or_creation_op"):
            getattr(L, f).restype = C.c_int
            getattr(L, f).argtypes = [C.c_uint32, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_uint32)]
        L.or_multiply_H.argtypes = [C.POINTER(_Model), C.POINTER(_Basis), _dp, _dp]
        L.or_multiply_H_omp.argtypes = [C.POINTER(_Model), C.POINTER(_Basis), _dp, _dp, C.c_int]
        L.or_multiply_H_rows.argtypes = [C.POINTER(_Model), C.POINTER(_Basis), _dp, _dp, C.c_int64,
                                         C.c_int64, C.c_int]
        L.or_dense_H.argtypes = [C.POINTER(_Model), C.POINTER(_Basis), _dp]
        L.or_apply_c.argtypes = [C.POINTER(_Model), C.POINTER(_Basis), _dp, C.c_int, C.c_int,
                                 C.c_int, C.POINTER(_Basis), C.POINTER(_dp)]
        L.or_lanczos_iteration.restype = C.c_int
        L.or_lanczos_iteration.argtypes = [C.POINTER(_Model), C.POINTER(_Basis), _dp, C.c_int,
                                           _dp, _dp, C.c_int]
        L.or_green_cf.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, _dp, _dp,
                                  C.c_int, _dp, _dp]
        L.or_boltzmann_factor.argtypes = [_dp, C.c_int, C.c_double, _dp]
        L.or_sort.argtypes = [C.c_int, _dp, _ip]
        L.or_ev_to_x.argtypes = [_dp, _dp, _dp, C.c_int, C.c_int, C.c_int, _dp]
        L.or_x_to_ev.argtypes = [_dp, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp]
        L.or_func.restype = C.c_double
        L.or_func.argtypes = [_dp, C.c_int, C.c_int, C.c_int, _dp, _dp, C.c_int, C.c_int]
        L.or_dfunc.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_int, _dp, _dp, C.c_int, C.c_int]
        L.or_frprmn.restype = C.c_int
        L.or_frprmn.argtypes = [_dp, C.c_int, C.c_double, _ip, _dp, C.c_int, C.c_int, C.c_int,
                                _dp, _dp, C.c_int, C.c_int]
        L.or_calc_dev.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp]
        L.or_set_band_structure.restype = C.c_int
        L.or_set_band_structure.argtypes = [C.c_int, C.c_int, _dp, _dp]
        L.or_delta_new.argtypes = [C.c_int, C.c_int, C.c_int, _dp, C.c_double, _dp, _dp, _dp]
        L.or_n_from_gksum.argtypes = [C.c_int, C.c_int, _dp, C.c_double, _dp]
        L.or_dos.argtypes = [C.c_int, C.c_int, _ip, _dp, _dp, _ip, _ip, _ip, _dp, C.c_int, C.c_int, _dp,
                             C.c_double, C.c_int, _dp]
        L.or_func_calls.restype = C.c_int64
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


@dataclass
class Model:
    """ed_config.f90:11-36 globals for one impurity model.

    ``vk`` has shape (norb, nbath): vk[iorb, ibath] = Fortran vk(iorb+1, norb+ibath+1).
    """
    norb: int
    nbath: int
    U: float
    J: float
    ek: np.ndarray          # (nsite,)
    vk: np.ndarray          # (norb, nbath)
    _keep: list = field(default_factory=list, repr=False)

    @property
    def nsite(self):
        return self.norb + self.nbath

    def c(self):
        ek = np.ascontiguousarray(self.ek, dtype=np.float64)
        vkf = np.asfortranarray(np.asarray(self.vk, dtype=np.float64).reshape(self.norb, self.nbath))
        vk = np.ascontiguousarray(vkf.ravel(order="F"))
        self._keep = [ek, vk]
        return _Model(self.norb, self.nbath, self.nsite, float(self.U), float(self.J), _d(ek), _d(vk))


class Basis:
    """type(basis_t) of ed_basis.F90:10-30 (one rank)."""

    def __init__(self, nsite, ne_up, ne_down):
        self.c = _Basis()
        rc = lib().or_generate_basis(nsite, ne_up, ne_down, C.byref(self.c))
        if rc:
            lib().or_free_basis(C.byref(self.c))
            raise ValueError(f"invalid sector ({ne_up},{ne_down}) for nsite={nsite}")
        self.nsite, self.ne_up, self.ne_down = nsite, ne_up, ne_down
        self.nup, self.ndown, self.ntot = self.c.nup, self.c.ndown, self.c.ntot
        self.up = np.ctypeslib.as_array(self.c.up, (self.nup,)).copy()
        self.down = np.ctypeslib.as_array(self.c.down, (self.ndown,)).copy()
        self.idx_up = np.ctypeslib.as_array(self.c.idx_up, (1 << nsite,)).copy()
        self.idx_down = np.ctypeslib.as_array(self.c.idx_down, (1 << nsite,)).copy()

    def get(self, idx):
        return lib().or_basis_get(C.byref(self.c), idx)

    def idx(self, state):
        return lib().or_basis_idx(C.byref(self.c), state)

    def __del__(self):
        try:
            lib().or_free_basis(C.byref(self.c))
        except Exception:
            pass


def icom(n, m):
    return lib().or_icom(n, m)


def multiply_H(model: Model, basis: Basis, A, nthreads=0):
    A = np.ascontiguousarray(A, dtype=np.float64)
    B = np.empty_like(A)
    m = model.c()
    lib().or_multiply_H_omp(C.byref(m), C.byref(basis.c), _d(A), _d(B), nthreads)
    return B


def multiply_H_rows(model: Model, basis: Basis, A, B, row0, row1, nthreads=0):
    """B[row0:row1] = (H*A)[row0:row1] (in place)."""
    m = model.c()
    lib().or_multiply_H_rows(C.byref(m), C.byref(basis.c), _d(A), _d(B), row0, row1, nthreads)


def dense_H(model: Model, basis: Basis):
    n = basis.ntot
    H = np.empty((n, n), dtype=np.float64)
    m = model.c()
    lib().or_dense_H(C.byref(m), C.byref(basis.c), _d(H))
    return H


def apply_c(model: Model, basis: Basis, vec, pm, iorb, ispin):
    """Returns (basis_out, vec_out); raises ValueError if the target sector is empty."""
    nu, nd = basis.ne_up, basis.ne_down
    d = 1 if pm == 1 else -1
    if ispin == 1:
        nu += d
    else:
        nd += d
    out = Basis(basis.nsite, nu, nd)
    vec = np.ascontiguousarray(vec, dtype=np.float64)
    m = model.c()
    bo = _Basis()
    p = _dp()
    rc = lib().or_apply_c(C.byref(m), C.byref(basis.c), _d(vec), pm, iorb, ispin, C.byref(bo), C.byref(p))
    if rc:
        raise ValueError("apply_c: invalid target sector")
    v = np.ctypeslib.as_array(p, (bo.ntot,)).copy()
    lib().or_free_basis(C.byref(bo))
    C.CDLL(None).free(p)
    return out, v


def lanczos_iteration(model: Model, basis: Basis, vec, nstep, nthreads=0):
    """ed_lanczos.F90:14-68.  Returns (nstep_calc, a[0:nstep], b[0:nstep])."""
    a = np.zeros(nstep + 1)
    b = np.zeros(nstep + 1)
    vec = np.ascontiguousarray(vec, dtype=np.float64)
    m = model.c()
    n = lib().or_lanczos_iteration(C.byref(m), C.byref(basis.c), _d(vec), nstep, _d(a), _d(b), nthreads)
    return n, a, b


def green_cf(sgn, eigval, pev, factor, nstep_calc, a, b, omega, gr):
    """ed_green.F90:160-168 (sgn=+1) / 176-184 (sgn=-1); gr (complex128, nw) updated in place."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    omega = np.ascontiguousarray(omega, dtype=np.float64)
    g = np.ascontiguousarray(gr, dtype=np.complex128).view(np.float64)
    lib().or_green_cf(sgn, eigval, pev, factor, nstep_calc, _d(a), _d(b), len(omega), _d(omega), _d(g))
    gr[:] = g.view(np.complex128)


def boltzmann_factor(elv, beta):
    elv = np.ascontiguousarray(elv, dtype=np.float64)
    p = np.empty_like(elv)
    lib().or_boltzmann_factor(_d(elv), len(elv), beta, _d(p))
    return p


def sort(arr):
    """func.f90:301-353; returns 1-based index array."""
    arr = np.ascontiguousarray(arr, dtype=np.float64)
    ind = np.zeros(len(arr), dtype=np.int32)
    lib().or_sort(len(arr), _d(arr), _i(ind))
    return ind


def ev_to_x(ek, vk, ef, ns, nbath):
    norb = ns - nbath
    nxsize = nbath + nbath * norb + norb
    x = np.zeros(nxsize)
    vkf = np.ascontiguousarray(np.asarray(vk, dtype=np.float64).reshape(norb, nbath).ravel(order="F"))
    lib().or_ev_to_x(_d(np.ascontiguousarray(ek, dtype=np.float64)), _d(vkf),
                     _d(np.ascontiguousarray(ef, dtype=np.float64)), ns, nbath, nxsize, _d(x))
    return x


def x_to_ev(x, ns, nbath, norb):
    x = np.ascontiguousarray(x, dtype=np.float64)
    ef = np.zeros(norb)
    ek = np.zeros(ns)
    vkf = np.zeros(norb * nbath)
    lib().or_x_to_ev(_d(x), len(x), ns, nbath, norb, _d(ef), _d(ek), _d(vkf))
    return ef, ek, vkf.reshape(nbath, norb).T.copy()


def _dev_arg(dev):
    """D_ev as Fortran (norb, nw) complex -> interleaved float64 buffer."""
    dev = np.asarray(dev, dtype=np.complex128)
    return np.ascontiguousarray(dev.T).view(np.float64).ravel()


def func(x, ns, omega, dev, nbath, norb):
    x = np.ascontiguousarray(x, dtype=np.float64)
    om = np.ascontiguousarray(omega, dtype=np.float64)
    dv = _dev_arg(dev)
    return lib().or_func(_d(x), ns, len(om), len(x), _d(om), _d(dv), nbath, norb)


def dfunc(x, ns, omega, dev, nbath, norb):
    x = np.ascontiguousarray(x, dtype=np.float64)
    p = np.zeros_like(x)
    om = np.ascontiguousarray(omega, dtype=np.float64)
    dv = _dev_arg(dev)
    lib().or_dfunc(_d(x), _d(p), len(om), ns, len(x), _d(om), _d(dv), nbath, norb)
    return p


def frprmn(x, ns, omega, dev, nbath, norb, ftol=1.0e-7):
    """frprmn.f90 driven as minimization() does (func.f90:144-163).

    Returns (x_min, fret, iter, status)."""
    p = np.array(x, dtype=np.float64)
    om = np.ascontiguousarray(omega, dtype=np.float64)
    dv = _dev_arg(dev)
    it = C.c_int(0)
    fret = C.c_double(0.0)
    rc = lib().or_frprmn(_d(p), len(p), ftol, C.byref(it), C.byref(fret), len(p), len(om), ns,
                         _d(om), _d(dv), nbath, norb)
    return p, fret.value, it.value, rc


def calc_dev(norb, nsite, omega, ek, vk, ef):
    om = np.ascontiguousarray(omega, dtype=np.float64)
    vkf = np.ascontiguousarray(np.asarray(vk, dtype=np.float64).reshape(norb, nsite - norb).ravel(order="F"))
    out = np.zeros(2 * norb * len(om))
    lib().or_calc_dev(norb, nsite, len(om), _d(om), _d(np.ascontiguousarray(ek, dtype=np.float64)),
                      _d(vkf), _d(np.ascontiguousarray(ef, dtype=np.float64)), _d(out))
    return out.view(np.complex128).reshape(len(om), norb).T.copy()


def set_band_structure(norb, nq):
    """ed_hamiltonian.F90:29-85 -> (hk[nq], ef[norb])."""
    hk, ef = np.zeros(nq), np.zeros(norb)
    if lib().or_set_band_structure(norb, nq, _d(hk), _d(ef)) != 0:
        raise ValueError("Nq is not a square")
    return hk, ef


def delta_new(hk, rmu, gr, dev):
    """ed_green.F90:187-214: gr, dev complex (norb, nw) -> (new dev, gksum)."""
    norb, nw = gr.shape
    g = np.ascontiguousarray(np.asarray(gr, np.complex128).T).view(np.float64).ravel()
    d = np.ascontiguousarray(np.asarray(dev, np.complex128).T).view(np.float64).ravel().copy()
    gk = np.zeros_like(d)
    lib().or_delta_new(norb, nw, len(hk), _d(np.ascontiguousarray(hk, np.float64)), rmu, _d(g), _d(d), _d(gk))
    back = lambda a: a.view(np.complex128).reshape(nw, norb).T.copy()
    return back(d), back(gk)


def n_from_gksum(gksum, beta):
    """ed_green.F90:227-253: occupations from Gksum (complex (norb, nw))."""
    norb, nw = gksum.shape
    g = np.ascontiguousarray(np.asarray(gksum, np.complex128).T).view(np.float64).ravel()
    out = np.zeros(norb)
    lib().or_n_from_gksum(norb, nw, _d(g), beta, _d(out))
    return out


def dos(norb, records, omega_real, small, weighted=False):
    """dos.f90:1-106 over apbpanbn.dat records: list of dicts with iorb (1-based),
    ev, prob, even, np, nn (-1: no run), ap, bp, an, bn -> A (norb, nw)."""
    n = len(records)
    ld = max(max(r["np"], r["nn"]) for r in records) + 1 if n else 1
    ab = np.zeros((max(n, 1), 4, ld))
    for i, r in enumerate(records):
        ab[i, 0, :r["np"] + 1] = r["ap"][:r["np"] + 1]
        ab[i, 1, :r["np"] + 1] = r["bp"][:r["np"] + 1]
        ab[i, 2, :r["nn"] + 1] = r["an"][:r["nn"] + 1]
        ab[i, 3, :r["nn"] + 1] = r["bn"][:r["nn"] + 1]   # nstep_calc -1: no run
    ii = lambda k: np.ascontiguousarray([int(r[k]) for r in records] or [0], np.int32)
    dd = lambda k: np.ascontiguousarray([float(r[k]) for r in records] or [0.0], np.float64)
    om = np.ascontiguousarray(omega_real, np.float64)
    out = np.zeros(norb * len(om))
    lib().or_dos(norb, n, _i(ii("iorb")), _d(dd("ev")), _d(dd("prob")), _i(ii("even")), _i(ii("np")),
                 _i(ii("nn")), _d(np.ascontiguousarray(ab.ravel())), ld, len(om), _d(om), small, int(weighted),
                 _d(out))
    return out.reshape(len(om), norb).T.copy()


def matsubara(nw, beta):
    """ed_green.F90:41-52 on one rank."""
    return (2.0 * np.arange(nw, dtype=np.float64) + 1.0) * np.pi / beta


# ---------------------------------------------------------------------------
# Independent Jordan-Wigner construction (pins the C restatement's signs)
# ---------------------------------------------------------------------------
def jw_sector_H(model: Model, ne_up, ne_down):
    """Sector Hamiltonian built from explicit fermion matrices.

    Spin-orbital (site s, spin sp) is mode q = (sp-1)*nsite + s-1 (bit q of the
    state word), and c_q|n> carries (-1)^(number of occupied modes below q) --
    the convention of ed_operators.F90:63-66,292-348.  The operator terms are
    those of ed_hamiltonian.F90:88-191 written as products of these matrices.
    """
    ns = model.nsite
    nmodes = 2 * ns
    basis = Basis(ns, ne_up, ne_down)
    states = np.array([basis.get(i + 1) for i in range(basis.ntot)], dtype=np.int64)
    pos = {int(s): i for i, s in enumerate(states)}
    n = basis.ntot

    def cop(q, dag):
        """matrix of c_q (dag=False) or c_q^dagger restricted to all 2^nmodes states (sparse dict)."""
        def act(s):
            occ = (s >> q) & 1
            if dag and occ:
                return None
            if not dag and not occ:
                return None
            sign = -1 if bin(s & ((1 << q) - 1)).count("1") % 2 else 1
            return s ^ (1 << q), sign
        return act

    def apply_ops(ops, s):
        """ops applied right to left (ops[-1] first) to |s>."""
        sign = 1
        for q, dag in reversed(ops):
            r = cop(q, dag)(s)
            if r is None:
                return None
            s, sg = r
            sign *= sg
        return s, sign

    def mode(site, spin):
        return (spin - 1) * ns + site - 1

    H = np.zeros((n, n))

    def add_term(coef, ops):
        for j, s in enumerate(states):
            r = apply_ops(ops, int(s))
            if r is None:
                continue
            t, sg = r
            H[pos[t], j] += coef * sg

    norb, nbath = model.norb, model.nbath
    U, J = model.U, model.J
    for spin in (1, 2):
        for site in range(1, ns + 1):
            add_term(model.ek[site - 1], [(mode(site, spin), True), (mode(site, spin), False)])
    for i in range(1, norb + 1):
        add_term(U, [(mode(i, 1), True), (mode(i, 1), False), (mode(i, 2), True), (mode(i, 2), False)])
    for i in range(1, norb + 1):
        for j in range(i + 1, norb + 1):
            for si in (1, 2):
                for sj in (1, 2):
                    coef = U - 3 * J if si == sj else U - 2 * J
                    add_term(coef, [(mode(i, si), True), (mode(i, si), False),
                                    (mode(j, sj), True), (mode(j, sj), False)])
    for spin in (1, 2):
        for i in range(1, norb + 1):
            for k in range(1, nbath + 1):
                v = model.vk[i - 1, k - 1]
                add_term(v, [(mode(i, spin), True), (mode(norb + k, spin), False)])
                add_term(v, [(mode(norb + k, spin), True), (mode(i, spin), False)])
    for i in range(1, norb + 1):
        for j in range(1, norb + 1):
            if i == j:
                continue
            # -J c+_{i up} c_{i dn} c+_{j dn} c_{j up}   (ed_operators.F90:183-215)
            add_term(-J, [(mode(i, 1), True), (mode(i, 2), False), (mode(j, 2), True), (mode(j, 1), False)])
            # -J c+_{i up} c+_{i dn} c_{j up} c_{j dn}   (ed_operators.F90:236-268)
            add_term(-J, [(mode(i, 1), True), (mode(i, 2), True), (mode(j, 1), False), (mode(j, 2), False)])
    return H


# ---------------------------------------------------------------------------
# ed_solve / ed_calc_green_ftn restated on top of the C pieces
# ---------------------------------------------------------------------------
def sector_eigs(model: Model, ne_up, ne_down, nev, dense_max=2500, want_vectors=True):
    """diag() stand-in: nev lowest eigenpairs (ed_solver.F90:107-191).

    Dense eigh for ntot <= dense_max (the regime where PARPACK cannot run,
    nev >= ntot), scipy ARPACK eigsh(which='SA') on the restated multiply_H
    otherwise.  Missing eigenvalues are reported as +huge, as diag() does
    for unconverged ones (ed_solver.F90:185-189)."""
    basis = Basis(model.nsite, ne_up, ne_down)
    n = basis.ntot
    vals = np.full(nev, np.finfo(np.float64).max)
    vecs = np.zeros((n, nev)) if want_vectors else None
    if n <= dense_max:
        H = dense_H(model, basis)
        w, V = np.linalg.eigh(0.5 * (H + H.T))
        k = min(nev, n)
        vals[:k] = w[:k]
        if want_vectors:
            vecs[:, :k] = V[:, :k]
    else:
        from scipy.sparse.linalg import LinearOperator, eigsh
        op = LinearOperator((n, n), matvec=lambda x: multiply_H(model, basis, x), dtype=np.float64)
        k = min(nev, n - 1)
        w, V = eigsh(op, k=k, which="SA", ncv=min(n, max(2 * k + 1, 20)), tol=0,
                     v0=np.ones(n) / np.sqrt(n))
        order = np.argsort(w)
        vals[:k] = w[order]
        if want_vectors:
            vecs[:, :k] = V[:, order]
    return basis, vals, vecs


PROB_THRESHOLD = 0.001  # ed_solver.F90:14


def ed_solve(model: Model, sectors, nev, beta):
    """ed_solver.F90:28-105.  sectors: list of (nelec, nup).  Returns a list of
    dicts {val, prob, sector (1-based), level (1-based)} and the per-sector
    eigenvectors."""
    nsector = len(sectors)
    eig_all = np.zeros(nev * nsector)
    vecs = []
    for isec, (nelec, nup) in enumerate(sectors):
        _, vals, V = sector_eigs(model, nup, nelec - nup, nev)
        eig_all[isec * nev:(isec + 1) * nev] = vals
        vecs.append(V)
    ind = sort(eig_all)
    pev = boltzmann_factor(eig_all, beta)
    nev_calc = sum(1 for i in range(nev) if pev[ind[i] - 1] > PROB_THRESHOLD)
    out = []
    Z = 0.0
    for i in range(nev_calc):
        k = ind[i] - 1
        out.append(dict(val=eig_all[k], prob=pev[k], sector=k // nev + 1, level=k % nev + 1))
        Z += pev[k]
    for e in out:
        e["prob"] /= Z
    return out, vecs


def green_diag(model, basis, eigvec, eigval, pev, factor, iorb, ispin, nstep, omega, gr):
    """ed_green.F90:136-185 for one (state, orbital, spin); gr updated in place.

    Returns (nstep_calcp, nstep_calcn, ap, bp, an, bn)."""
    res = []
    try:
        bo, v = apply_c(model, basis, eigvec, 1, iorb, ispin)
        np_, ap, bp = lanczos_iteration(model, bo, v, nstep)
        normsq = float(np.dot(v, v))
        bp[0] = normsq
        green_cf(+1, eigval, pev, factor, np_, ap, bp, omega, gr)
    except ValueError:
        normsq, np_, ap, bp = 0.0, 0, np.zeros(nstep + 1), np.zeros(nstep + 1)
    res += [np_, ap, bp]
    try:
        bo, v = apply_c(model, basis, eigvec, 2, iorb, ispin)
        nn, an, bn = lanczos_iteration(model, bo, v, nstep)
        bn[0] = 1.0 - normsq
        green_cf(-1, eigval, pev, factor, nn, an, bn, omega, gr)
    except ValueError:
        nn, an, bn = 0, np.zeros(nstep + 1), np.zeros(nstep + 1)
    return res[0], nn, res[1], res[2], an, bn


def ed_calc_green_ftn(model, sectors, states, vecs, nstep, omega):
    """ed_green.F90:60-134.  Returns Gr (norb, nw) complex."""
    nw = len(omega)
    Gr = np.zeros((model.norb, nw), dtype=np.complex128)
    for st in states:
        nelec, nup = sectors[st["sector"] - 1]
        nd = nelec - nup
        factor = 1.0 if nd == nup else 0.5
        basis = Basis(model.nsite, nup, nd)
        vec = vecs[st["sector"] - 1][:, st["level"] - 1]
        spins = (1,) if nd == nup else (1, 2)
        for ispin in spins:
            for iorb in range(1, model.norb + 1):
                g = Gr[iorb - 1]
                green_diag(model, basis, vec, st["val"], st["prob"], factor, iorb, ispin, nstep, omega, g)
                Gr[iorb - 1] = g
    return Gr
