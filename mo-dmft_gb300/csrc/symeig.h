// symeig.h -- eigenvalues and eigenvectors of a small dense symmetric matrix
// on the host: the projected (Rayleigh-Ritz) problem of the thick-restart
// Lanczos, m <= kMaxNcv.  The reference's eigensolver (PARPACK) also solves
// its projected problem on the host (LAPACK); on GB300 a one-CTA FP64
// Jacobi of an m = 40 matrix takes ~1.4 ms per call, the host a few tens of
// microseconds.
//
// Method (Golub & Van Loan, Matrix Computations, 4th ed., 8.3):
//   1. Householder reduction to tridiagonal form, T = Q^T A Q, with Q
//      accumulated;
//   2. implicit symmetric QR steps with the Wilkinson shift on T, chasing the
//      bulge with Givens rotations that are accumulated into Q, deflating
//      off-diagonal entries below eps (|d_i| + |d_i+1|);
//   3. eigenpairs sorted by ascending eigenvalue.
#pragma once

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

namespace moed {

// a: n x n symmetric, row-major (only read).  w[n]: ascending eigenvalues.
// z[n * n]: column j (z[j * n + i], i = 0..n-1) is the unit eigenvector of
// w[j].  Returns false if the QR iteration did not converge.
inline bool sym_eig(int n, const std::vector<double> &a, double *w, double *z)
{
    if (n <= 0) return true;
    std::vector<double> A(a.begin(), a.begin() + (size_t)n * n);
    std::vector<double> Q((size_t)n * n, 0.0);   // row-major, Q[r * n + c]
    for (int i = 0; i < n; ++i) Q[(size_t)i * n + i] = 1.0;
    std::vector<double> v(n), p(n);
    // 1. Householder: zero column k below the subdiagonal, k = 0 .. n-3
    for (int k = 0; k + 2 < n; ++k) {
        double s2 = 0.0;
        for (int i = k + 1; i < n; ++i) s2 += A[(size_t)i * n + k] * A[(size_t)i * n + k];
        const double tail = s2 - A[(size_t)(k + 1) * n + k] * A[(size_t)(k + 1) * n + k];
        if (tail == 0.0) continue;                        // already tridiagonal in this column
        const double x0 = A[(size_t)(k + 1) * n + k];
        const double alpha = x0 >= 0.0 ? -std::sqrt(s2) : std::sqrt(s2);
        for (int i = 0; i < n; ++i) v[i] = 0.0;
        for (int i = k + 1; i < n; ++i) v[i] = A[(size_t)i * n + k];
        v[k + 1] = x0 - alpha;
        double vv = 0.0;
        for (int i = k + 1; i < n; ++i) vv += v[i] * v[i];
        if (vv == 0.0) continue;
        const double beta = 2.0 / vv;                     // H = I - beta v v^T
        // H A H on the trailing block: A - v q^T - q v^T, p = beta A v,
        // q = p - (beta v^T p / 2) v
        double vp = 0.0;
        for (int i = k + 1; i < n; ++i) {
            double t = 0.0;
            for (int j = k + 1; j < n; ++j) t += A[(size_t)i * n + j] * v[j];
            p[i] = beta * t;
            vp += v[i] * p[i];
        }
        const double K = 0.5 * beta * vp;
        for (int i = k + 1; i < n; ++i) p[i] -= K * v[i];
        for (int i = k + 1; i < n; ++i)
            for (int j = k + 1; j < n; ++j) A[(size_t)i * n + j] -= v[i] * p[j] + p[i] * v[j];
        A[(size_t)(k + 1) * n + k] = A[(size_t)k * n + k + 1] = alpha;
        for (int i = k + 2; i < n; ++i) A[(size_t)i * n + k] = A[(size_t)k * n + i] = 0.0;
        // Q <- Q H
        for (int r = 0; r < n; ++r) {
            double t = 0.0;
            for (int j = k + 1; j < n; ++j) t += Q[(size_t)r * n + j] * v[j];
            t *= beta;
            for (int j = k + 1; j < n; ++j) Q[(size_t)r * n + j] -= t * v[j];
        }
    }
    std::vector<double> d(n), e(n, 0.0);                  // e[i] = T(i+1, i)
    for (int i = 0; i < n; ++i) d[i] = A[(size_t)i * n + i];
    for (int i = 0; i + 1 < n; ++i) e[i] = A[(size_t)(i + 1) * n + i];
    // 2. implicit QR with the Wilkinson shift, deflating from the bottom
    const double eps = 2.220446049250313e-16;
    int hi = n - 1, iters = 0;
    while (hi > 0) {
        if (std::fabs(e[hi - 1]) <= eps * (std::fabs(d[hi - 1]) + std::fabs(d[hi]))) {
            e[hi - 1] = 0.0;
            --hi;
            continue;
        }
        if (++iters > 60 * n) return false;
        int lo = hi - 1;
        while (lo > 0 && std::fabs(e[lo - 1]) > eps * (std::fabs(d[lo - 1]) + std::fabs(d[lo]))) --lo;
        // shift: the eigenvalue of the trailing 2 x 2 closer to d[hi]
        const double delta = 0.5 * (d[hi - 1] - d[hi]), b = e[hi - 1];
        const double mu = delta == 0.0 ? d[hi] - std::fabs(b)
                                       : d[hi] - b * b / (delta + std::copysign(std::hypot(delta, b), delta));
        double x = d[lo] - mu, y = e[lo];
        for (int k = lo; k < hi; ++k) {
            // rotation R = [c s; -s c] on rows / columns k, k+1 that zeroes y
            // (the shifted first column, then the bulge at (k+1, k-1))
            const double r = std::hypot(x, y);
            const double c = r == 0.0 ? 1.0 : x / r, s = r == 0.0 ? 0.0 : y / r;
            if (k > lo) e[k - 1] = r;
            const double dk = d[k], dk1 = d[k + 1], ek = e[k];
            d[k] = c * c * dk + 2.0 * c * s * ek + s * s * dk1;
            d[k + 1] = s * s * dk - 2.0 * c * s * ek + c * c * dk1;
            e[k] = c * s * (dk1 - dk) + (c * c - s * s) * ek;
            if (k + 1 < hi) {
                y = s * e[k + 1];                          // the bulge at (k+2, k)
                e[k + 1] *= c;
                x = e[k];
            }
            for (int rr = 0; rr < n; ++rr) {               // Q <- Q R^T
                const double qk = Q[(size_t)rr * n + k], qk1 = Q[(size_t)rr * n + k + 1];
                Q[(size_t)rr * n + k] = c * qk + s * qk1;
                Q[(size_t)rr * n + k + 1] = -s * qk + c * qk1;
            }
        }
    }
    // 3. ascending order
    std::vector<int> ord(n);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int i, int j) { return d[i] < d[j]; });
    for (int j = 0; j < n; ++j) {
        w[j] = d[ord[j]];
        for (int i = 0; i < n; ++i) z[(size_t)j * n + i] = Q[(size_t)i * n + ord[j]];
    }
    return true;
}

}  // namespace moed
