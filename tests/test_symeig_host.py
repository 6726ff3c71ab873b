"""The host eigensolver of the eigensolver's projected (Rayleigh-Ritz) problem
(mo-dmft_gb300/csrc/symeig.h: Householder tridiagonalisation + implicit QR
with the Wilkinson shift) against numpy.linalg.eigh: random symmetric
matrices, the thick-restart shape (diagonal kept block, arrow, tridiagonal
tail), degenerate spectra and the zero matrix, n = 1 .. 65 (kMaxNcv is 64)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = r"""
#include <vector>
#include "symeig.h"
extern "C" int sym_eig_c(int n, const double *a, double *w, double *z)
{
    std::vector<double> A(a, a + (size_t)n * n);
    return moed::sym_eig(n, A, w, z) ? 0 : 1;
}
"""


@pytest.fixture(scope="module")
def symeig(tmp_path_factory):
    d = tmp_path_factory.mktemp("symeig")
    src, lib = d / "shim.cpp", d / "libsymeig.so"
    src.write_text(SHIM)
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", os.path.join(ROOT, "mo-dmft_gb300", "csrc"),
                    "-o", str(lib), str(src)], check=True)
    L = C.CDLL(str(lib))
    dp = C.POINTER(C.c_double)

    def run(A):
        n = A.shape[0]
        a = np.ascontiguousarray(A, dtype=np.float64)
        w, z = np.zeros(n), np.zeros(n * n)
        assert L.sym_eig_c(n, a.ctypes.data_as(dp), w.ctypes.data_as(dp), z.ctypes.data_as(dp)) == 0
        return w, z.reshape(n, n).T          # columns are the eigenvectors
    return run


def check(run, A, tol=1e-13):
    w, Z = run(A)
    n = A.shape[0]
    sc = max(1.0, np.abs(A).max())
    assert np.all(np.diff(w) >= 0)
    assert np.abs(w - np.linalg.eigvalsh(A)).max() <= tol * sc * max(1, n)
    assert np.abs(A @ Z - Z * w).max() <= tol * sc * max(1, n)
    assert np.abs(Z.T @ Z - np.eye(n)).max() <= 1e-13 * max(1, n)


def test_random_symmetric(symeig):
    rng = np.random.default_rng(0)
    for n in range(1, 66):
        M = rng.standard_normal((n, n))
        check(symeig, M + M.T)


def test_thick_restart_shape_and_degenerate(symeig):
    rng = np.random.default_rng(1)
    for n in (2, 7, 20, 40, 64):
        k = n // 3
        T = np.zeros((n, n))
        T[np.arange(k), np.arange(k)] = np.sort(rng.standard_normal(k))
        for j in range(k, n):
            T[j, j] = rng.standard_normal()
            if j + 1 < n:
                T[j + 1, j] = T[j, j + 1] = abs(rng.standard_normal())
        if k < n:
            T[k, :k] = T[:k, k] = 1e-3 * rng.standard_normal(k)
        check(symeig, T)
        D = np.diag(np.repeat(rng.standard_normal((n + 2) // 3), 3)[:n])
        Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        check(symeig, 37.0 * Q @ D @ Q.T)
        check(symeig, np.zeros((n, n)))
