"""Host-side mirror of the MO-DMFT ED / bath-fit interface over the C-ABI.

Every method maps to one entry point of ``include/mo_ed.h`` and keeps the
name and argument meaning of the reference routine it replaces:

=====================  ===============================================
reference routine      here
=====================  ===============================================
generate_basis         ``EDSolver.generate_basis`` (ed_basis.F90:35)
ed_basis_get / _idx    ``EDSolver.ed_basis_get`` / ``ed_basis_idx``
multiply_H             ``EDSolver.multiply_H`` (ed_hamiltonian.F90:88)
apply_c                ``EDSolver.apply_c`` (ed_operators.F90:10)
lanczos_iteration      ``EDSolver.lanczos_iteration`` (ed_lanczos.F90:14)
diag                   ``EDSolver.diag`` (ed_solver.F90:107)
ed_solve               ``EDSolver.ed_solve`` (ed_solver.F90:28)
ed_calc_green_ftn      ``EDSolver.ed_calc_green_ftn`` (ed_green.F90:60)
FUNC / dfunc           ``EDSolver.FUNC`` / ``EDSolver.dfunc`` (func.f90:1,47)
minimization/frprmn    ``EDSolver.minimization`` (func.f90:144)
calc_dev               ``EDSolver.calc_dev`` (ed_green.F90:260)
ev_to_x / x_to_ev      module functions (func.f90:165,193)
=====================  ===============================================

The reference stops the program (``die`` / ``STOP``) on errors; here every
nonzero status raises :class:`EDError` with the library's message.  There is
no CPU fallback: without the built library or a CUDA device the solver
cannot be constructed.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libmoed.so")

OK, ERR_ARG, ERR_SECTOR, ERR_CUDA, ERR_NOMEM, ERR_NOCONV, ERR_FIT, ERR_STATE, ERR_CAPACITY = range(9)
FP64, FP32 = 0, 1

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)
_llp = C.POINTER(C.c_longlong)
_up = C.POINTER(C.c_uint)


class Options(C.Structure):
    """mo_ed_options (include/mo_ed.h)."""
    _fields_ = [("nstep", C.c_int), ("nev", C.c_int), ("beta", C.c_double), ("precision", C.c_int),
                ("fortran_cmplx", C.c_int), ("gs_ncv", C.c_int), ("gs_maxcycles", C.c_int),
                ("gs_tol", C.c_double), ("green_reorth", C.c_int),
                ("green_fp64", C.c_int), ("solve_threads", C.c_int), ("fit_quantum", C.c_int),
                ("reserved", C.c_int * 5)]


class EDError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"mo_ed error {code}: {msg}")
        self.code = code


_lib = None

# every symbol declared in include/mo_ed.h: (name, restype, argtypes)
SIGNATURES = [
    ("mo_ed_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_void_p]),
    ("mo_ed_destroy", C.c_int, [C.c_void_p]),
    ("mo_ed_last_error", C.c_char_p, [C.c_void_p]),
    ("mo_ed_version", C.c_char_p, []),
    ("mo_ed_default_options", C.c_int, [C.POINTER(Options)]),
    ("mo_ed_set_options", C.c_int, [C.c_void_p, C.POINTER(Options)]),
    ("mo_ed_set_model", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double, _dp, _dp]),
    ("mo_ed_set_sectors", C.c_int, [C.c_void_p, C.c_int, _ip, _ip]),
    ("mo_ed_set_omega", C.c_int, [C.c_void_p, C.c_int, _dp]),
    ("mo_ed_icom", C.c_longlong, [C.c_int, C.c_int]),
    ("mo_ed_sector_dims", C.c_int, [C.c_void_p, C.c_int, C.c_int, _ip, _ip, _llp]),
    ("mo_ed_vector_layout", C.c_int, [C.c_void_p, C.c_int, C.c_int, _ip, _llp]),
    ("mo_ed_generate_basis", C.c_int, [C.c_void_p, C.c_int, C.c_int, _ip, _ip, _ip, _ip]),
    ("mo_ed_basis_get", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_longlong, _llp, _up]),
    ("mo_ed_basis_idx", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_longlong, _up, _llp]),
    ("mo_ed_multiply_h", C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _dp]),
    ("mo_ed_multiply_h_f32", C.c_int, [C.c_void_p, C.c_int, C.c_int, _fp, _fp]),
    ("mo_ed_multiply_h_dev", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    ("mo_ed_multiply_h_mixed_dev", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    ("mo_ed_hv_tuning", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, _ip, _ip,
                                  C.POINTER(C.c_float), _ip]),
    ("mo_ed_hv_set_variant", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]),
    ("mo_ed_apply_c", C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, C.c_int, C.c_int, C.c_int, _dp,
                                C.c_longlong, _llp]),
    ("mo_ed_lanczos_iteration", C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _ip, _dp, _dp]),
    ("mo_ed_lanczos_iteration_noalloc", C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _ip, _dp, _dp]),
    ("mo_ed_diag", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, _dp, _dp]),
    ("mo_ed_diag_stats", C.c_int, [C.c_void_p, _ip, _llp, _dp, _dp]),
    ("mo_ed_green_stats", C.c_int, [C.c_void_p, _dp]),
    ("mo_ed_set_band_structure", C.c_int, [C.c_void_p, C.c_int, _dp]),
    ("mo_ed_delta_new", C.c_int, [C.c_void_p, C.c_int, C.c_double, _dp, _dp, _dp]),
    ("mo_ed_n_from_gksum", C.c_int, [C.c_void_p, C.c_int, _dp, C.c_double, _dp]),
    ("mo_ed_dos", C.c_int, [C.c_void_p, C.c_int, _dp, C.c_double, C.c_int, _dp]),
    ("mo_ed_export_eigvec", C.c_int, [C.c_void_p, C.c_char_p]),
    ("mo_ed_import_eigvec", C.c_int, [C.c_void_p, C.c_char_p, _ip]),
    ("mo_ed_write_apbpanbn", C.c_int, [C.c_void_p, C.c_char_p]),
    ("mo_ed_read_apbpanbn", C.c_int, [C.c_void_p, C.c_char_p, _ip]),
    ("mo_ed_solve", C.c_int, [C.c_void_p, _ip, _dp, _dp, _ip, _ip, C.c_int]),
    ("mo_ed_calc_green_ftn", C.c_int, [C.c_void_p, _dp]),
    ("mo_ed_green_coeffs", C.c_int, [C.c_void_p, _ip, _ip, _dp, C.c_int]),
    ("mo_ed_func", C.c_int, [C.c_void_p, _dp, C.c_int, C.c_int, C.c_int, _dp, _dp, C.c_int, C.c_int, _dp]),
    ("mo_ed_dfunc", C.c_int, [C.c_void_p, _dp, _dp, C.c_int, C.c_int, C.c_int, _dp, _dp, C.c_int, C.c_int]),
    ("mo_ed_minimization", C.c_int, [C.c_void_p, _dp, C.c_int, C.c_int, C.c_int, _dp, _dp, C.c_int, C.c_int,
                                     _dp, _ip]),
    ("mo_ed_fit_batch", C.c_int, [C.c_void_p, C.c_int, _dp, C.c_int, C.c_int, C.c_int, _dp, _dp, C.c_int,
                                  C.c_int, C.c_double, _dp, _ip, _ip]),
    ("mo_ed_fit_stats", C.c_int, [C.c_void_p, _llp, _ip]),
    ("mo_ed_chi2_grad_dev", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p,
                                      C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    ("mo_ed_calc_dev", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp]),
    ("mo_ed_ev_to_x", C.c_int, [_dp, _dp, _dp, C.c_int, C.c_int, C.c_int, _dp]),
    ("mo_ed_x_to_ev", C.c_int, [_dp, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp]),
    ("mo_ed_kernel_launches", C.c_longlong, [C.c_void_p]),
]


def lib():
    """Load the in-tree library (built by build.py); fails loudly if absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _vk_f(vk, norb, nbath):
    """(norb, nbath) array -> Fortran vk(norb, norb+1:nsite) column-major buffer."""
    vk = np.asarray(vk, dtype=np.float64).reshape(norb, nbath)
    return np.ascontiguousarray(vk.ravel(order="F"))


def _dev_f(D_ev):
    """D_ev (norb, nw) complex -> interleaved Fortran-order buffer."""
    D_ev = np.asarray(D_ev, dtype=np.complex128)
    return np.ascontiguousarray(D_ev.T).view(np.float64).ravel()


def icom(n, m):
    """iCom (ed_utils.f90:54-69)."""
    return int(lib().mo_ed_icom(n, m))


def ev_to_x(ek, vk, ef, ns, nbath):
    """ev_to_x (func.f90:165-191); vk as (norb, nbath)."""
    norb = ns - nbath
    nx = nbath + nbath * norb + norb
    x = np.zeros(nx)
    rc = lib().mo_ed_ev_to_x(_d(_f64(ek)), _d(_vk_f(vk, norb, nbath)), _d(_f64(ef)), ns, nbath, nx, _d(x))
    if rc:
        raise EDError(rc, "ev_to_x: bad dimensions")
    return x


def x_to_ev(x, ns, nbath, norb):
    """x_to_ev (func.f90:193-216); returns (ef, ek, vk[norb, nbath])."""
    x = _f64(x)
    ef, ek, vk = np.zeros(norb), np.zeros(ns), np.zeros(norb * nbath)
    rc = lib().mo_ed_x_to_ev(_d(x), len(x), ns, nbath, norb, _d(ef), _d(ek), _d(vk))
    if rc:
        raise EDError(rc, "x_to_ev: bad dimensions")
    return ef, ek, vk.reshape(nbath, norb).T.copy()


class EDSolver:
    """One solver context (one GPU, one stream): the ed_config globals plus
    the device-resident sector tables and eigenvectors."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self._ctx = C.c_void_p()
        rc = lib().mo_ed_create(C.byref(self._ctx), device, C.c_void_p(stream or 0))
        if rc:
            raise EDError(rc, "mo_ed_create failed (no usable CUDA device?)")
        self.opt = Options()
        lib().mo_ed_default_options(C.byref(self.opt))
        self.norb = self.nbath = self.nsite = 0
        self.nw = 0

    # ---- plumbing -------------------------------------------------------
    def close(self):
        if self._ctx:
            lib().mo_ed_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc):
        if rc:
            msg = lib().mo_ed_last_error(self._ctx)
            raise EDError(rc, msg.decode() if msg else "")

    @property
    def kernel_launches(self):
        return int(lib().mo_ed_kernel_launches(self._ctx))

    # ---- configuration (ed_config.f90) ------------------------------------
    def set_options(self, **kw):
        for k, v in kw.items():
            if k == "precision" and isinstance(v, str):
                v = {"fp32": FP32, "fp64": FP64}[v.lower()]
            if k in ("fortran_cmplx", "green_reorth", "green_fp64"):
                v = int(bool(v))
            setattr(self.opt, k, v)
        self._chk(lib().mo_ed_set_options(self._ctx, C.byref(self.opt)))

    def set_model(self, norb, nbath, U, J, ek, vk):
        ek = _f64(ek)
        self._chk(lib().mo_ed_set_model(self._ctx, norb, nbath, float(U), float(J), _d(ek),
                                        _d(_vk_f(vk, norb, nbath))))
        self.norb, self.nbath, self.nsite = norb, nbath, norb + nbath

    def set_sectors(self, nelec, nup):
        ne = np.ascontiguousarray(nelec, dtype=np.int32)
        nu = np.ascontiguousarray(nup, dtype=np.int32)
        self._chk(lib().mo_ed_set_sectors(self._ctx, len(ne), ne.ctypes.data_as(_ip), nu.ctypes.data_as(_ip)))
        self.sectors = list(zip(ne.tolist(), nu.tolist()))

    def set_omega(self, omega):
        om = _f64(omega)
        self._chk(lib().mo_ed_set_omega(self._ctx, len(om), _d(om)))
        self.omega = om
        self.nw = len(om)

    # ---- basis (ed_basis.F90) ----------------------------------------------
    def sector_dims(self, ne_up, ne_down):
        a, b, n = C.c_int(), C.c_int(), C.c_longlong()
        self._chk(lib().mo_ed_sector_dims(self._ctx, ne_up, ne_down, C.byref(a), C.byref(b), C.byref(n)))
        return a.value, b.value, n.value

    def vector_layout(self, ne_up, ne_down):
        """(ld, nelem) of the device layout: ndown rows of stride ld (zero pads)."""
        ld, n = C.c_int(), C.c_longlong()
        self._chk(lib().mo_ed_vector_layout(self._ctx, ne_up, ne_down, C.byref(ld), C.byref(n)))
        return ld.value, n.value

    def generate_basis(self, ne_up, ne_down):
        nup, ndn, _ = self.sector_dims(ne_up, ne_down)
        nw = 1 << self.nsite
        up, dn = np.zeros(nup, np.int32), np.zeros(ndn, np.int32)
        iu, idn = np.zeros(nw, np.int32), np.zeros(nw, np.int32)
        self._chk(lib().mo_ed_generate_basis(self._ctx, ne_up, ne_down, up.ctypes.data_as(_ip),
                                             dn.ctypes.data_as(_ip), iu.ctypes.data_as(_ip),
                                             idn.ctypes.data_as(_ip)))
        return dict(nup=nup, ndown=ndn, ntot=nup * ndn, up=up, down=dn, idx_up=iu, idx_down=idn)

    def ed_basis_get(self, ne_up, ne_down, idx):
        idx = np.ascontiguousarray(idx, dtype=np.int64)
        out = np.zeros(len(idx), np.uint32)
        self._chk(lib().mo_ed_basis_get(self._ctx, ne_up, ne_down, len(idx), idx.ctypes.data_as(_llp),
                                        out.ctypes.data_as(_up)))
        return out

    def ed_basis_idx(self, ne_up, ne_down, state):
        st = np.ascontiguousarray(state, dtype=np.uint32)
        out = np.zeros(len(st), np.int64)
        self._chk(lib().mo_ed_basis_idx(self._ctx, ne_up, ne_down, len(st), st.ctypes.data_as(_up),
                                        out.ctypes.data_as(_llp)))
        return out

    # ---- H*v (ed_hamiltonian.F90:88) ---------------------------------------
    def multiply_H(self, ne_up, ne_down, A):
        """B = H*A; FP64 path for float64 input, FP32 path for float32 input."""
        A = np.asarray(A)
        if A.dtype == np.float32:
            A = np.ascontiguousarray(A)
            B = np.empty_like(A)
            self._chk(lib().mo_ed_multiply_h_f32(self._ctx, ne_up, ne_down, A.ctypes.data_as(_fp),
                                                 B.ctypes.data_as(_fp)))
            return B
        A = _f64(A)
        B = np.empty_like(A)
        self._chk(lib().mo_ed_multiply_h(self._ctx, ne_up, ne_down, _d(A), _d(B)))
        return B

    def multiply_H_dev(self, ne_up, ne_down, dA, dB, dtype=FP32):
        """Device pointers (ints) in the device layout (vector_layout); no synchronization."""
        self._chk(lib().mo_ed_multiply_h_dev(self._ctx, ne_up, ne_down, dtype, C.c_void_p(dA), C.c_void_p(dB)))

    def multiply_H_mixed_dev(self, ne_up, ne_down, dA, dB):
        self._chk(lib().mo_ed_multiply_h_mixed_dev(self._ctx, ne_up, ne_down, C.c_void_p(dA), C.c_void_p(dB)))

    def hv_set_variant(self, ne_up, ne_down, variant, dtype=FP32):
        """Pin the H*v tile-shape variant (index of hv_tuning's list)."""
        self._chk(lib().mo_ed_hv_set_variant(self._ctx, ne_up, ne_down, dtype, variant))

    def hv_tuning(self, ne_up, ne_down, dtype=FP32):
        """Autotuner record: list of ((R, threads, CTAs/SM, kernel), ms) and the chosen index;
        kernel 0 k_hv, 1 k_hv_async, 2 / 3 split (k_hv_down on 128- / 64-byte slices + k_hv_async)."""
        cap = 16
        nv, ch = C.c_int(), C.c_int()
        shape = np.zeros(4 * cap, np.int32)
        ms = np.zeros(cap, np.float32)
        self._chk(lib().mo_ed_hv_tuning(self._ctx, ne_up, ne_down, dtype, cap, C.byref(nv),
                                        shape.ctypes.data_as(_ip), ms.ctypes.data_as(C.POINTER(C.c_float)),
                                        C.byref(ch)))
        return [(tuple(int(v) for v in shape[4 * i:4 * i + 4]), float(ms[i])) for i in range(nv.value)], ch.value

    # ---- apply_c (ed_operators.F90:10) --------------------------------------
    def apply_c(self, ne_up, ne_down, vec, pm, iorb, ispin):
        d = 1 if pm == 1 else -1
        tu = ne_up + (d if ispin == 1 else 0)
        td = ne_down + (d if ispin == 2 else 0)
        _, _, n = self.sector_dims(tu, td)
        out = np.zeros(n)
        nout = C.c_longlong()
        self._chk(lib().mo_ed_apply_c(self._ctx, ne_up, ne_down, _d(_f64(vec)), pm, iorb, ispin, _d(out), n,
                                      C.byref(nout)))
        return (tu, td), out

    # ---- Lanczos / eigensolver --------------------------------------------
    def lanczos_iteration(self, ne_up, ne_down, vec):
        """ed_lanczos.F90:14 -> (nstep_calc, a[0:nstep], b[0:nstep])."""
        n = self.opt.nstep
        a, b = np.zeros(n + 1), np.zeros(n + 1)
        nc = C.c_int()
        self._chk(lib().mo_ed_lanczos_iteration(self._ctx, ne_up, ne_down, _d(_f64(vec)), C.byref(nc), _d(a), _d(b)))
        return nc.value, a, b

    def lanczos_iteration_noalloc(self, ne_up, ne_down, vec):
        """lanczos_iteration on the library's fixed device region (no device
        allocation; the sector must be prepared by an earlier call)."""
        n = self.opt.nstep
        a, b = np.zeros(n + 1), np.zeros(n + 1)
        nc = C.c_int()
        self._chk(lib().mo_ed_lanczos_iteration_noalloc(self._ctx, ne_up, ne_down, _d(_f64(vec)), C.byref(nc),
                                                        _d(a), _d(b)))
        return nc.value, a, b

    def diag(self, ne_up, ne_down, nev, vectors=True):
        """ed_solver.F90:107 -> (eigval[nev], eigvec[ntot, nev] or None)."""
        _, _, n = self.sector_dims(ne_up, ne_down)
        ev = np.zeros(nev)
        vec = np.zeros((nev, n)) if vectors else None
        self._chk(lib().mo_ed_diag(self._ctx, ne_up, ne_down, nev, _d(ev),
                                   _d(vec) if vectors else _dp()))
        return ev, (vec.T.copy() if vectors else None)

    def diag_stats(self):
        """(cycles, matvecs, residual estimate, FP64 true residual) of the last eigensolve."""
        c, m, a, b = C.c_int(), C.c_longlong(), C.c_double(), C.c_double()
        self._chk(lib().mo_ed_diag_stats(self._ctx, C.byref(c), C.byref(m), C.byref(a), C.byref(b)))
        return dict(cycles=c.value, matvecs=m.value, res_est=a.value, res_true=b.value)

    def green_stats(self):
        """Largest Ritz residual of the FP64 eigenvector refinement of the last
        ed_calc_green_ftn (green_fp64 over FP32 eigenvectors; 0 if none ran)."""
        r = C.c_double()
        self._chk(lib().mo_ed_green_stats(self._ctx, C.byref(r)))
        return r.value

    def ed_solve(self):
        """ed_solver.F90:28 -> list of eigval_t dicts (val, prob, sector, level; 1-based)."""
        cap = self.opt.nev
        val, prob = np.zeros(cap), np.zeros(cap)
        sec, lev = np.zeros(cap, np.int32), np.zeros(cap, np.int32)
        nc = C.c_int()
        self._chk(lib().mo_ed_solve(self._ctx, C.byref(nc), _d(val), _d(prob), sec.ctypes.data_as(_ip),
                                    lev.ctypes.data_as(_ip), cap))
        return [dict(val=val[i], prob=prob[i], sector=int(sec[i]), level=int(lev[i])) for i in range(nc.value)]

    def ed_calc_green_ftn(self):
        """ed_green.F90:60 -> Gr (norb, nw) complex128."""
        g = np.zeros(2 * self.norb * self.nw)
        self._chk(lib().mo_ed_calc_green_ftn(self._ctx, _d(g)))
        return g.view(np.complex128).reshape(self.nw, self.norb).T.copy()

    def green_coeffs(self):
        """apbpanbn.dat content of the last Green's function: list of records."""
        nrec = C.c_int()
        self._chk(lib().mo_ed_green_coeffs(self._ctx, C.byref(nrec), _ip(), _dp(), 0))
        n, ld = nrec.value, self.opt.nstep + 1
        nsc = np.zeros(2 * max(n, 1), np.int32)
        ab = np.zeros(4 * ld * max(n, 1))
        self._chk(lib().mo_ed_green_coeffs(self._ctx, C.byref(nrec), nsc.ctypes.data_as(_ip), _d(ab), n))
        ab = ab.reshape(-1, 4, ld)
        return [dict(np=int(nsc[2 * r]), nn=int(nsc[2 * r + 1]), ap=ab[r, 0], bp=ab[r, 1], an=ab[r, 2],
                     bn=ab[r, 3]) for r in range(n)]

    # ---- DMFT self-consistency and spectra (ed_green.F90:187-253, dos.f90) --
    def set_band_structure(self, nq):
        """ed_hamiltonian.F90:29-85 -> ef (norb); the band stays on the device."""
        ef = np.zeros(self.norb)
        self._chk(lib().mo_ed_set_band_structure(self._ctx, nq, _d(ef)))
        return ef

    def delta_new(self, Gr, D_ev, rmu):
        """ed_green.F90:187-214 -> (new D_ev, Gksum), complex (norb, nw)."""
        norb, nw = Gr.shape
        g = np.ascontiguousarray(np.asarray(Gr, np.complex128).T).view(np.float64).ravel()
        d = np.ascontiguousarray(np.asarray(D_ev, np.complex128).T).view(np.float64).ravel().copy()
        k = np.zeros_like(d)
        self._chk(lib().mo_ed_delta_new(self._ctx, nw, float(rmu), _d(g), _d(d), _d(k)))
        back = lambda a: a.view(np.complex128).reshape(nw, norb).T.copy()
        return back(d), back(k)

    def n_from_gksum(self, Gksum, beta):
        """ed_green.F90:227-253 -> nocc (norb)."""
        norb, nw = Gksum.shape
        g = np.ascontiguousarray(np.asarray(Gksum, np.complex128).T).view(np.float64).ravel()
        out = np.zeros(norb)
        self._chk(lib().mo_ed_n_from_gksum(self._ctx, nw, _d(g), float(beta), _d(out)))
        return out

    def dos(self, omega_real, small, weighted=False):
        """dos.f90:1-106 from the last Green's function's records -> A (norb, nw)."""
        om = _f64(omega_real)
        out = np.zeros(self.norb * len(om))
        self._chk(lib().mo_ed_dos(self._ctx, len(om), _d(om), float(small), int(bool(weighted)), _d(out)))
        return out.reshape(len(om), self.norb).T.copy()

    # ---- files (ed_io.F90, apbpanbn.dat) ----------------------------------
    def export_eigvec(self, directory=""):
        """ed_io.F90 export_eigval / export_eigvec of the kept states."""
        self._chk(lib().mo_ed_export_eigvec(self._ctx, os.fsencode(directory)))

    def import_eigvec(self, directory=""):
        """Kept states from eigenvalues.dat + eigvec files -> nev_calc."""
        n = C.c_int()
        self._chk(lib().mo_ed_import_eigvec(self._ctx, os.fsencode(directory), C.byref(n)))
        return n.value

    def write_apbpanbn(self, path):
        self._chk(lib().mo_ed_write_apbpanbn(self._ctx, os.fsencode(path)))

    def read_apbpanbn(self, path):
        n = C.c_int()
        self._chk(lib().mo_ed_read_apbpanbn(self._ctx, os.fsencode(path), C.byref(n)))
        return n.value

    # ---- bath fit (func.f90, frprmn.f90) ---------------------------------
    def FUNC(self, x, Ns, nwloc, nxsize, omega, D_ev, Nbath, Norb):
        f = C.c_double()
        self._chk(lib().mo_ed_func(self._ctx, _d(_f64(x)), Ns, nwloc, nxsize, _d(_f64(omega)), _d(_dev_f(D_ev)),
                                   Nbath, Norb, C.byref(f)))
        return f.value

    def dfunc(self, x, nwloc, Ns, nxsize, omega, D_ev, Nbath, Norb):
        p = np.zeros(nxsize)
        self._chk(lib().mo_ed_dfunc(self._ctx, _d(_f64(x)), _d(p), nwloc, Ns, nxsize, _d(_f64(omega)),
                                    _d(_dev_f(D_ev)), Nbath, Norb))
        return p

    def minimization(self, x, nwloc, Ns, nxsize, omega, D_ev, Nbath, Norb):
        """func.f90:144 -> (x_min, fret, iter)."""
        x = np.array(x, dtype=np.float64)
        fret, it = C.c_double(), C.c_int()
        self._chk(lib().mo_ed_minimization(self._ctx, _d(x), nwloc, Ns, nxsize, _d(_f64(omega)), _d(_dev_f(D_ev)),
                                           Nbath, Norb, C.byref(fret), C.byref(it)))
        return x, fret.value, it.value

    def fit_batch(self, X, omega, D_ev, Nbath, Norb, ftol=1.0e-7):
        """Many fits (rows of X) in one launch -> (X_min, fret, iter, status);
        each row's result equals that of the same fit run alone."""
        X = np.array(X, dtype=np.float64, order="C")
        nb, nx = X.shape
        fret, it, st = np.zeros(nb), np.zeros(nb, np.int32), np.zeros(nb, np.int32)
        om = _f64(omega)
        self._chk(lib().mo_ed_fit_batch(self._ctx, nb, _d(X), len(om), Nbath + Norb, nx, _d(om), _d(_dev_f(D_ev)),
                                        Nbath, Norb, ftol, _d(fret), it.ctypes.data_as(_ip), st.ctypes.data_as(_ip)))
        return X, fret, it, st

    def fit_stats(self):
        """Suspensions (a fit giving up its cluster to a waiting fit) and
        clusters launched, of the last fit_batch / minimization."""
        n, c = C.c_longlong(), C.c_int()
        self._chk(lib().mo_ed_fit_stats(self._ctx, C.byref(n), C.byref(c)))
        return dict(suspensions=n.value, clusters=c.value)

    def chi2_grad_dev(self, nbatch, dx, nwloc, nxsize, domega, ddev, Nbath, Norb, df, dg):
        self._chk(lib().mo_ed_chi2_grad_dev(self._ctx, nbatch, C.c_void_p(dx), nwloc, Nbath + Norb, nxsize,
                                            C.c_void_p(domega), C.c_void_p(ddev), Nbath, Norb, C.c_void_p(df),
                                            C.c_void_p(dg)))

    def calc_dev(self, norb, nsite, omega, ek, vk, ef):
        om = _f64(omega)
        out = np.zeros(2 * norb * len(om))
        self._chk(lib().mo_ed_calc_dev(self._ctx, norb, nsite, len(om), _d(om), _d(_f64(ek)),
                                       _d(_vk_f(vk, norb, nsite - norb)), _d(_f64(ef)), _d(out)))
        return out.view(np.complex128).reshape(len(om), norb).T.copy()


def matsubara(nw, beta):
    """omega(i) = (2(i-1)+1) pi / beta (ed_green.F90:41-52, one rank)."""
    return (2.0 * np.arange(nw, dtype=np.float64) + 1.0) * np.pi / beta
