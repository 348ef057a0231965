// Small dense symmetric eigen-solvers in FP64 (host + device).
//
//  * sym_eig: Householder reduction to tridiagonal form followed by the implicit-shift QL
//    iteration (the EISPACK tred2/tql2 method, as described in Numerical Recipes 11.2-11.3),
//    for n <= 9.  Used for the PSD projection of the reduced barrier Hessians.
//  * psd_project: the PSD projection of common/math/wrapper/UTILS.h:8-25 (makePD): when the
//    smallest eigenvalue is >= 0 the matrix is returned unchanged, otherwise every negative
//    eigenvalue is clamped to zero.  Implemented as M - sum_{lambda<0} lambda v v^T.
#pragma once

#include "common.cuh"

namespace fipc {

constexpr int EIG_LD = 9;  // row stride of the matrices handled here

// a: n x n symmetric (row-major, stride LD, n <= LD).  On return a holds the orthonormal
// eigenvectors in its columns and d the eigenvalues (ascending).  Returns 0 on success,
// 1 if the QL iteration did not converge within its iteration limit.
template <int LD>
FIPC_HD int sym_eig_ld(int n, double* a, double* d) {
    double e[LD];
#define A_(i, j) a[(i) * LD + (j)]
    // --- Householder tridiagonalisation, accumulating the orthogonal transform in a
    for (int i = n - 1; i > 0; --i) {
        const int l = i - 1;
        double h = 0.0, scale = 0.0;
        if (l > 0) {
            for (int k = 0; k <= l; ++k) scale += fabs(A_(i, k));
            if (scale == 0.0) {
                e[i] = A_(i, l);
            } else {
                for (int k = 0; k <= l; ++k) {
                    A_(i, k) /= scale;
                    h += A_(i, k) * A_(i, k);
                }
                double f = A_(i, l);
                double g = f >= 0.0 ? -sqrt(h) : sqrt(h);
                e[i] = scale * g;
                h -= f * g;
                A_(i, l) = f - g;
                f = 0.0;
                for (int j = 0; j <= l; ++j) {
                    A_(j, i) = A_(i, j) / h;
                    g = 0.0;
                    for (int k = 0; k <= j; ++k) g += A_(j, k) * A_(i, k);
                    for (int k = j + 1; k <= l; ++k) g += A_(k, j) * A_(i, k);
                    e[j] = g / h;
                    f += e[j] * A_(i, j);
                }
                const double hh = f / (h + h);
                for (int j = 0; j <= l; ++j) {
                    f = A_(i, j);
                    e[j] = g = e[j] - hh * f;
                    for (int k = 0; k <= j; ++k) A_(j, k) -= (f * e[k] + g * A_(i, k));
                }
            }
        } else {
            e[i] = A_(i, l);
        }
        d[i] = h;
    }
    d[0] = 0.0;
    e[0] = 0.0;
    for (int i = 0; i < n; ++i) {
        const int l = i - 1;
        if (d[i] != 0.0) {
            for (int j = 0; j <= l; ++j) {
                double g = 0.0;
                for (int k = 0; k <= l; ++k) g += A_(i, k) * A_(k, j);
                for (int k = 0; k <= l; ++k) A_(k, j) -= g * A_(k, i);
            }
        }
        d[i] = A_(i, i);
        A_(i, i) = 1.0;
        for (int j = 0; j <= l; ++j) A_(j, i) = A_(i, j) = 0.0;
    }
    // --- implicit-shift QL on the tridiagonal (d, e), rotating the eigenvector columns
    for (int i = 1; i < n; ++i) e[i - 1] = e[i];
    e[n - 1] = 0.0;
    int status = 0;
    for (int l = 0; l < n; ++l) {
        int iter = 0, m;
        do {
            for (m = l; m < n - 1; ++m) {
                const double dd = fabs(d[m]) + fabs(d[m + 1]);
                if (fabs(e[m]) <= 2.220446049250313e-16 * dd) break;
            }
            if (m != l) {
                if (iter++ == 64) { status = 1; break; }
                double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
                double r = sqrt(g * g + 1.0);
                g = d[m] - d[l] + e[l] / (g + (g >= 0.0 ? r : -r));
                double s = 1.0, c = 1.0, p = 0.0;
                int i;
                for (i = m - 1; i >= l; --i) {
                    double f = s * e[i];
                    const double b = c * e[i];
                    r = sqrt(f * f + g * g);
                    e[i + 1] = r;
                    if (r == 0.0) {
                        d[i + 1] -= p;
                        e[m] = 0.0;
                        break;
                    }
                    s = f / r;
                    c = g / r;
                    g = d[i + 1] - p;
                    r = (d[i] - g) * s + 2.0 * c * b;
                    p = s * r;
                    d[i + 1] = g + p;
                    g = c * r - b;
                    for (int k = 0; k < n; ++k) {
                        f = A_(k, i + 1);
                        A_(k, i + 1) = s * A_(k, i) + c * f;
                        A_(k, i) = c * A_(k, i) - s * f;
                    }
                }
                if (r == 0.0 && i >= l) continue;
                d[l] -= p;
                e[l] = g;
                e[m] = 0.0;
            }
        } while (m != l);
    }
    // --- ascending order (selection sort carrying the eigenvector columns)
    for (int i = 0; i < n - 1; ++i) {
        int k = i;
        for (int j = i + 1; j < n; ++j)
            if (d[j] < d[k]) k = j;
        if (k != i) {
            const double t = d[i];
            d[i] = d[k];
            d[k] = t;
            for (int r = 0; r < n; ++r) {
                const double tv = A_(r, i);
                A_(r, i) = A_(r, k);
                A_(r, k) = tv;
            }
        }
    }
#undef A_
    return status;
}

FIPC_HD int sym_eig(int n, double* a, double* d) { return sym_eig_ld<EIG_LD>(n, a, d); }

// M (n x n, stride LD) <- its PSD projection; returns the sym_eig status.
template <int LD>
FIPC_HD int psd_project_ld(int n, double* M) {
    double Q[LD * LD], lam[LD];
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) Q[i * LD + j] = M[i * LD + j];
    const int st = sym_eig_ld<LD>(n, Q, lam);
    if (lam[0] >= 0.0) return st;
    for (int k = 0; k < n && lam[k] < 0.0; ++k) {
        const double l = lam[k];
        for (int i = 0; i < n; ++i) {
            const double li = l * Q[i * LD + k];
            for (int j = 0; j < n; ++j) M[i * LD + j] -= li * Q[j * LD + k];
        }
    }
    return st;
}

FIPC_HD int psd_project(int n, double* M) { return psd_project_ld<EIG_LD>(n, M); }

// 3x3 symmetric eigen-decomposition by cyclic Jacobi rotations (a: stride 3, destroyed;
// v: eigenvectors in columns; w: eigenvalues, ascending).
FIPC_HD void sym_eig3(double* a, double* w, double* v) {
    for (int i = 0; i < 9; ++i) v[i] = (i % 4 == 0) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 12; ++sweep) {
        const double off = a[1] * a[1] + a[2] * a[2] + a[5] * a[5];
        const double dia = a[0] * a[0] + a[4] * a[4] + a[8] * a[8];
        if (off <= 1e-34 * dia || off == 0.0) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                const double apq = a[p * 3 + q];
                if (apq == 0.0) continue;
                const double theta = (a[q * 3 + q] - a[p * 3 + p]) / (2.0 * apq);
                const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; ++k) {
                    const double akp = a[k * 3 + p], akq = a[k * 3 + q];
                    a[k * 3 + p] = c * akp - s * akq;
                    a[k * 3 + q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; ++k) {
                    const double apk = a[p * 3 + k], aqk = a[q * 3 + k];
                    a[p * 3 + k] = c * apk - s * aqk;
                    a[q * 3 + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; ++k) {
                    const double vkp = v[k * 3 + p], vkq = v[k * 3 + q];
                    v[k * 3 + p] = c * vkp - s * vkq;
                    v[k * 3 + q] = s * vkp + c * vkq;
                }
            }
    }
    w[0] = a[0];
    w[1] = a[4];
    w[2] = a[8];
    for (int i = 0; i < 2; ++i) {
        int k = i;
        for (int j = i + 1; j < 3; ++j)
            if (w[j] < w[k]) k = j;
        if (k != i) {
            const double t = w[i];
            w[i] = w[k];
            w[k] = t;
            for (int r = 0; r < 3; ++r) {
                const double tv = v[r * 3 + i];
                v[r * 3 + i] = v[r * 3 + k];
                v[r * 3 + k] = tv;
            }
        }
    }
}

// 3x3 PSD projection (makePD for n = 3), stride 3.  A matrix whose leading principal minors
// are all positive (Sylvester's criterion) is positive definite and returned unchanged without
// the eigen-solve, as makePD returns it when its smallest eigenvalue is >= 0.
FIPC_HD void psd_project3(double* M) {
    {
        const double m1 = M[0], m2 = M[0] * M[4] - M[1] * M[3];
        const double m3 = M[0] * (M[4] * M[8] - M[5] * M[7]) - M[1] * (M[3] * M[8] - M[5] * M[6]) + M[2] * (M[3] * M[7] - M[4] * M[6]);
        if (m1 > 0.0 && m2 > 0.0 && m3 > 0.0) return;
    }
    double a[9], w[3], v[9];
    for (int i = 0; i < 9; ++i) a[i] = M[i];
    sym_eig3(a, w, v);
    if (w[0] >= 0.0) return;
    for (int k = 0; k < 3 && w[k] < 0.0; ++k)
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) M[i * 3 + j] -= w[k] * v[i * 3 + k] * v[j * 3 + k];
}

}  // namespace fipc
