// Small dense solves with the semantics of the reference's solve_N (host + device).
//
// solve_n reproduces common/math/wrapper/wrapper.cpp:90-198 (used by
// common/math/math_tools.py:132-158): an LDL^T factorisation with symmetric pivoting, every
// pivot raised to at least 1e-8, the system rebuilt from the factors and solved.  It is the
// regularised solve of the ADMM local steps and of the a.so-compatible solve_N exports.
#pragma once

#include "common.cuh"

namespace fipc {

constexpr int PD_LD = 12;   // row stride of the matrices handled here (n <= 12)

// In-place LDL^T with symmetric diagonal pivoting on a (n x n, stride PD_LD, lower triangle
// read): step k brings to position k the remaining row whose ORIGINAL diagonal entry has the
// largest magnitude (the first of equal ones), the pivot order of the reference's Eigen LDLT
// (its choice looks at the input's diagonal, not at the updated Schur complement).  perm[k] =
// the row swapped with k at step k.  On return the strict lower triangle holds L (unit
// diagonal) and the diagonal holds D, both in the permuted order.  A zero pivot leaves its
// column of L at zero.
FIPC_HD void ldlt_pivoted(int n, double* a, int* perm) {
#define A_(i, j) a[(i) * PD_LD + (j)]
    double dg[PD_LD];
    for (int i = 0; i < n; ++i) {
        dg[i] = A_(i, i);
        for (int j = i + 1; j < n; ++j) A_(i, j) = A_(j, i);   // keep a full symmetric copy
    }
    for (int k = 0; k < n; ++k) {
        int p = k;
        for (int i = k + 1; i < n; ++i)
            if (fabs(dg[i]) > fabs(dg[p])) p = i;
        perm[k] = p;
        if (p != k) {
            const double t = dg[k];
            dg[k] = dg[p];
            dg[p] = t;
            for (int j = 0; j < n; ++j) {
                const double u = A_(k, j);
                A_(k, j) = A_(p, j);
                A_(p, j) = u;
            }
            for (int i = 0; i < n; ++i) {
                const double u = A_(i, k);
                A_(i, k) = A_(i, p);
                A_(i, p) = u;
            }
        }
        const double d = A_(k, k);
        if (d == 0.0) {
            for (int i = k + 1; i < n; ++i) A_(i, k) = A_(k, i) = 0.0;
            continue;
        }
        for (int i = k + 1; i < n; ++i) {
            const double lik = A_(i, k) / d;
            for (int j = k + 1; j <= i; ++j) A_(i, j) -= lik * A_(j, k);
            for (int j = k + 1; j <= i; ++j) A_(j, i) = A_(i, j);
        }
        for (int i = k + 1; i < n; ++i) {
            A_(i, k) /= d;
            A_(k, i) = A_(i, k);
        }
    }
#undef A_
}

// x = A^+ b from the factorisation above (pseudo-inverse of D: zero pivots give zero)
FIPC_HD void ldlt_solve(int n, const double* f, const int* perm, const double* b, double* x) {
    double y[PD_LD];
    for (int i = 0; i < n; ++i) y[i] = b[i];
    for (int k = 0; k < n; ++k)
        if (perm[k] != k) {
            const double t = y[k];
            y[k] = y[perm[k]];
            y[perm[k]] = t;
        }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < i; ++j) y[i] -= f[i * PD_LD + j] * y[j];
    for (int i = 0; i < n; ++i) y[i] = f[i * PD_LD + i] != 0.0 ? y[i] / f[i * PD_LD + i] : 0.0;
    for (int i = n - 1; i >= 0; --i)
        for (int j = i + 1; j < n; ++j) y[i] -= f[j * PD_LD + i] * y[j];
    for (int k = n - 1; k >= 0; --k)
        if (perm[k] != k) {
            const double t = y[k];
            y[k] = y[perm[k]];
            y[perm[k]] = t;
        }
    for (int i = 0; i < n; ++i) x[i] = y[i];
}

// solve_N of wrapper.cpp:90-198: factor A = P^T L D L^T P, raise every pivot of D to at least
// 1e-8, rebuild F = L D L^T (in the pivoted order, as the reference rebuilds it from the factors
// alone) and solve F x = rhs.  When no pivoting happens F is A with its pivots clamped.
FIPC_HD void solve_n(int n, const double* in, const double* rhs, double* out) {
    double a[PD_LD * PD_LD], f[PD_LD * PD_LD], x[PD_LD];
    int perm[PD_LD];
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) a[i * PD_LD + j] = in[i * n + j];
    ldlt_pivoted(n, a, perm);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j <= i; ++j) {
            double s = 0.0;
            for (int k = 0; k <= j; ++k) {
                const double lik = k == i ? 1.0 : a[i * PD_LD + k];
                const double ljk = k == j ? 1.0 : a[j * PD_LD + k];
                s += lik * fmax(a[k * PD_LD + k], 1e-8) * ljk;
            }
            f[i * PD_LD + j] = f[j * PD_LD + i] = s;
        }
    ldlt_pivoted(n, f, perm);
    ldlt_solve(n, f, perm, rhs, x);
    for (int i = 0; i < n; ++i) out[i] = x[i];
}

}  // namespace fipc
