// IPC barrier energy, gradient and PSD-projected Hessian per constraint row (host + device).
//
// Restates common/math/ipc.py:30-329 (PP/PE/PT/EE/EEM/PPM/PEM _energy, _g_and_H) with the
// distances of common/math/distance.py (PP_3D_E 955, PE_3D_E 684, PT_3D_E 976, EE_3D_E 192,
// EECN2_E 1345), the barrier of distance.py:22-44 and the mollifier of distance.py:1625-1673.
//
// Derivatives are hand-derived in translation-free reduced coordinates y = C x:
//   PT  (p,t0,t1,t2):    r = p-t0,  e1 = t1-t0, e2 = t2-t0,   d = (r.(e1 x e2))^2 / |e1 x e2|^2
//   EE* (a0,a1,b0,b1):   r = b0-a0, e1 = a1-a0, e2 = b1-b0,   d as above (EEM), |r|^2 (PPM),
//                        |r x e2|^2/|e2|^2 (PEM); the mollifier variable is |e1 x e2|^2
//   PE  (p,e0,e1):       q = e0-p,  e = e1-e0,                d = |q x e|^2 / |e|^2
//   PP  (a,b):           r = a-b,                             d = |r|^2
// Every energy is translation invariant, so the x-space Hessian H = C^T H_y C has the three
// rigid translations in its null space and H = Q M Q^T with Q the orthonormal (Helmert) basis
// of zero-sum vertex combinations and M = (CQ)^T H_y (CQ).  The PSD projection of the
// reference's n x n matrix (n = 12, 9, 6) therefore equals Q proj(M) Q^T with M of size
// 9, 6, 3: the projection runs on the reduced matrix.
#pragma once

#include "common.cuh"
#include "eig.cuh"

namespace fipc {

// ---------------------------------------------------------------- barrier scalar function
FIPC_HD double barrier_E(double d, double dh2, double k) {
    return d < dh2 ? -k * (d - dh2) * (d - dh2) * log(d / dh2) : 0.0;
}
FIPC_HD double barrier_g(double d, double dh2, double k) {
    const double t2 = d - dh2;
    return d < dh2 ? k * (t2 * log(d / dh2) * -2.0 - (t2 * t2) / d) : 0.0;
}
FIPC_HD double barrier_H(double d, double dh2, double k) {
    const double t2 = d - dh2;
    return d < dh2 ? k * ((log(d / dh2) * -2.0 - t2 * 4.0 / d) + 1.0 / (d * d) * (t2 * t2)) : 0.0;
}

// ---------------------------------------------------------------- reduced-space helpers
// 9-dim y = (y0, y1, y2) blocks of 3; gradients g[9]; Hessians H[9*9] row-major.
FIPC_HD void put3(double* g, int blk, v3 a, double s) {
    g[3 * blk + 0] += s * a.x;
    g[3 * blk + 1] += s * a.y;
    g[3 * blk + 2] += s * a.z;
}
// H[blk_i][blk_j] += s * (a b^T)
FIPC_HD void put_outer(double* H, int bi, int bj, v3 a, v3 b, double s) {
    const double A[3] = {a.x, a.y, a.z}, B[3] = {b.x, b.y, b.z};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) H[(3 * bi + i) * 9 + 3 * bj + j] += s * A[i] * B[j];
}
FIPC_HD void put_ident(double* H, int bi, int bj, double s) {
    for (int i = 0; i < 3; ++i) H[(3 * bi + i) * 9 + 3 * bj + i] += s;
}
// H[bi][bj] += s [a]_x  (skew matrix with [a]_x b = a x b), and the transposed block
FIPC_HD void put_skew_pair(double* H, int bi, int bj, v3 a, double s) {
    const double S[9] = {0, -a.z, a.y, a.z, 0, -a.x, -a.y, a.x, 0};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            H[(3 * bi + i) * 9 + 3 * bj + j] += s * S[i * 3 + j];
            H[(3 * bj + j) * 9 + 3 * bi + i] += s * S[i * 3 + j];
        }
}
FIPC_HD void sym_outer(double* H, const double* a, const double* b, double s, int n) {
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) H[i * 9 + j] += s * (a[i] * b[j] + b[i] * a[j]);
}

// Value, gradient and Hessian of N = |u x w|^2 in blocks (bu, bw) of a 9-dim space.
FIPC_HD double cross_norm2(v3 u, v3 w, int bu, int bw, double* g, double* H) {
    const v3 c = cross(u, w);
    put3(g, bu, cross(w, c), 2.0);   // dN/du = 2 w x c
    put3(g, bw, cross(c, u), 2.0);   // dN/dw = 2 c x u
    const double uu = sq(u), ww = sq(w), uw = dot(u, w);
    put_ident(H, bu, bu, 2.0 * ww);
    put_outer(H, bu, bu, w, w, -2.0);
    put_ident(H, bw, bw, 2.0 * uu);
    put_outer(H, bw, bw, u, u, -2.0);
    // [u][w] block: 2 (u w^T - (u.w) I - [c]_x); [w][u] its transpose
    put_outer(H, bu, bw, u, w, 2.0);
    put_outer(H, bw, bu, w, u, 2.0);
    put_ident(H, bu, bw, -2.0 * uw);
    put_ident(H, bw, bu, -2.0 * uw);
    put_skew_pair(H, bu, bw, c, -2.0);
    return sq(c);
}

// squared point-plane style distance d = s^2 / D, s = r.(e1 x e2), D = |e1 x e2|^2 in blocks
// (0,1,2) = (r,e1,e2).  Also returns D with its gradient/Hessian (the mollifier variable).
FIPC_HD double triple_dist(v3 r, v3 e1, v3 e2, double* g, double* H, double* Dv, double* Dg, double* DH) {
    for (int i = 0; i < 9; ++i) Dg[i] = 0.0;
    for (int i = 0; i < 81; ++i) DH[i] = 0.0;
    const double D = cross_norm2(e1, e2, 1, 2, Dg, DH);
    const v3 n = cross(e1, e2);
    const double s = dot(r, n);
    double sg[9] = {0};
    put3(sg, 0, n, 1.0);
    put3(sg, 1, cross(e2, r), 1.0);
    put3(sg, 2, cross(r, e1), 1.0);
    const double iD = 1.0 / D, d = s * s * iD;
    for (int i = 0; i < 9; ++i) g[i] = 2.0 * s * iD * sg[i] - d * iD * Dg[i];
    for (int i = 0; i < 81; ++i) H[i] = -d * iD * DH[i];
    // s Hessian: [r][e1] = -[e2]_x, [r][e2] = [e1]_x, [e1][e2] = -[r]_x (plus transposes)
    const double k = 2.0 * s * iD;
    put_skew_pair(H, 0, 1, e2, -k);
    put_skew_pair(H, 0, 2, e1, k);
    put_skew_pair(H, 1, 2, r, -k);
    for (int i = 0; i < 9; ++i)
        for (int j = 0; j < 9; ++j)
            H[i * 9 + j] += 2.0 * iD * sg[i] * sg[j] + 2.0 * d * iD * iD * Dg[i] * Dg[j]
                            - 2.0 * s * iD * iD * (sg[i] * Dg[j] + Dg[i] * sg[j]);
    *Dv = D;
    return d;
}

// squared point-line distance d = |q x e|^2 / |e|^2 in blocks (bq, be)
FIPC_HD double line_dist(v3 q, v3 e, int bq, int be, double* g, double* H) {
    double Ng[9] = {0}, NH[81] = {0};
    const double N = cross_norm2(q, e, bq, be, Ng, NH);
    const double L = sq(e), iL = 1.0 / L, d = N * iL;
    double Lg[9] = {0};
    put3(Lg, be, e, 2.0);
    for (int i = 0; i < 9; ++i) g[i] = Ng[i] * iL - d * iL * Lg[i];
    for (int i = 0; i < 81; ++i) H[i] = NH[i] * iL;
    put_ident(H, be, be, -2.0 * d * iL);
    for (int i = 0; i < 9; ++i)
        for (int j = 0; j < 9; ++j)
            H[i * 9 + j] += -iL * iL * (Ng[i] * Lg[j] + Lg[i] * Ng[j]) + 2.0 * N * iL * iL * iL * Lg[i] * Lg[j];
    return d;
}

// ---------------------------------------------------------------- per-row evaluation
// Reduced-coordinate maps C[k][v] (rows: y blocks, columns: vertices of the row)
struct RowMap {
    int nv, ny;          // vertices, reduced blocks
    double C[3][4];
};
FIPC_HD RowMap row_map(int type) {
    RowMap m{};
    if (type == T_PP) {
        m.nv = 2; m.ny = 1;
        m.C[0][0] = 1; m.C[0][1] = -1;
    } else if (type == T_PE) {
        m.nv = 3; m.ny = 2;
        m.C[0][0] = -1; m.C[0][1] = 1;                 // q = e0 - p
        m.C[1][1] = -1; m.C[1][2] = 1;                 // e = e1 - e0
    } else if (type == T_PT) {
        m.nv = 4; m.ny = 3;
        m.C[0][0] = 1; m.C[0][1] = -1;                 // r = p - t0
        m.C[1][1] = -1; m.C[1][2] = 1;                 // e1 = t1 - t0
        m.C[2][1] = -1; m.C[2][3] = 1;                 // e2 = t2 - t0
    } else {
        m.nv = 4; m.ny = 3;
        m.C[0][0] = -1; m.C[0][2] = 1;                 // r = b0 - a0
        m.C[1][0] = -1; m.C[1][1] = 1;                 // e1 = a1 - a0
        m.C[2][2] = -1; m.C[2][3] = 1;                 // e2 = b1 - b0
    }
    return m;
}

// Orthonormal basis of zero-sum combinations of nv vertices (Helmert), Qb[v][a], a < nv-1
FIPC_HD double helmert(int nv, int v, int a) {
    // column a: (1, .., 1, -(a+1), 0, ..) / sqrt((a+1)(a+2)) with a+1 ones
    const double s = 1.0 / sqrt((double)((a + 1) * (a + 2)));
    if (v <= a) return s;
    if (v == a + 1) return -(double)(a + 1) * s;
    (void)nv;
    return 0.0;
}

// Energy (E), gradient (g, 12 = 3*nv used) and projected Hessian in 3x3 vertex blocks
// (Hb[(v*4+w)*9 + i*3+j] for v,w < nv) of one constraint row.  X: the row's vertices
// (nv used), X0: rest positions of the four EE-type vertices (mollified types only).
// want: 0 energy only, 1 energy + gradient + projected Hessian, 2 energy + gradient + the
// Hessian without the projection.  Returns the eigen-solver status.
FIPC_HD int barrier_row(int type, const v3* X, const v3* X0, double dh2, double kappa, int want,
                        double* E, double* g, double* Hb) {
    const RowMap m = row_map(type);
    v3 y[3];
    for (int k = 0; k < m.ny; ++k) {
        v3 s = mk(0, 0, 0);
        for (int v = 0; v < m.nv; ++v)
            if (m.C[k][v] != 0.0) s = s + m.C[k][v] * X[v];
        y[k] = s;
    }
    double fg[9] = {0}, fH[81] = {0};
    double Dv = 0.0, Dg[9] = {0}, DH[81] = {0};
    double f;
    // distance (f) and, for EE-type rows, the mollifier variable D = |e1 x e2|^2
    if (type == T_PP || type == T_PPM) {
        f = sq(y[0]);
        put3(fg, 0, y[0], 2.0);
        put_ident(fH, 0, 0, 2.0);
        if (type == T_PPM) Dv = cross_norm2(y[1], y[2], 1, 2, Dg, DH);
    } else if (type == T_PE) {
        f = line_dist(y[0], y[1], 0, 1, fg, fH);
    } else if (type == T_PEM) {
        f = line_dist(y[0], y[2], 0, 2, fg, fH);
        Dv = cross_norm2(y[1], y[2], 1, 2, Dg, DH);
    } else {
        f = triple_dist(y[0], y[1], y[2], fg, fH, &Dv, Dg, DH);
    }
    const double b = barrier_E(f, dh2, kappa);
    double mval = 1.0, m1 = 0.0, m2 = 0.0;
    if (type >= T_EEM) {
        // mollifier threshold on the rest shape (distance.py:1671-1673) and EEM_E/g/H
        const double eps = 1.0e-3 * sq(X0[0] - X0[1]) * sq(X0[2] - X0[3]);
        if (Dv < eps) {
            const double q = Dv / eps;
            mval = (-q + 2.0) * q;
            m1 = 2.0 * (1.0 / eps) * (-(1.0 / eps) * Dv + 1.0);
            m2 = -2.0 / (eps * eps);
        }
    }
    *E = b * mval;
    if (!want) return 0;
    const double b1 = barrier_g(f, dh2, kappa), b2 = barrier_H(f, dh2, kappa);
    const int n = 3 * m.ny;
    double gy[9], Hy[81];
    for (int i = 0; i < n; ++i) gy[i] = mval * b1 * fg[i] + b * m1 * Dg[i];
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            Hy[i * 9 + j] = mval * (b2 * fg[i] * fg[j] + b1 * fH[i * 9 + j])
                            + b1 * m1 * (fg[i] * Dg[j] + Dg[i] * fg[j])
                            + b * (m2 * Dg[i] * Dg[j] + m1 * DH[i * 9 + j]);
    // x-space gradient g = C^T gy
    for (int v = 0; v < m.nv; ++v)
        for (int c = 0; c < 3; ++c) {
            double s = 0.0;
            for (int k = 0; k < m.ny; ++k) s += m.C[k][v] * gy[3 * k + c];
            g[3 * v + c] = s;
        }
    // K = C Q (ny x ny coefficient matrix), M = K^T Hy K (blockwise, 3x3 identity factor)
    const int na = m.nv - 1;   // == ny
    double K[3][3];
    for (int k = 0; k < m.ny; ++k)
        for (int a = 0; a < na; ++a) {
            double s = 0.0;
            for (int v = 0; v < m.nv; ++v) s += m.C[k][v] * helmert(m.nv, v, a);
            K[k][a] = s;
        }
    double M[81];
    for (int a = 0; a < na; ++a)
        for (int bb = 0; bb < na; ++bb)
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    double s = 0.0;
                    for (int k = 0; k < m.ny; ++k)
                        for (int l = 0; l < m.ny; ++l) s += K[k][a] * K[l][bb] * Hy[(3 * k + i) * 9 + 3 * l + j];
                    M[(3 * a + i) * 9 + 3 * bb + j] = s;
                }
    int st = 0;
    if (want == 2) {
        // no projection
    } else if (n == 3) {
        double M3[9];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) M3[i * 3 + j] = M[i * 9 + j];
        psd_project3(M3);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) M[i * 9 + j] = M3[i * 3 + j];
    } else {
        st = psd_project(n, M);
    }
    // H = Q proj(M) Q^T in 3x3 vertex blocks
    for (int v = 0; v < m.nv; ++v)
        for (int w = 0; w < m.nv; ++w)
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    double s = 0.0;
                    for (int a = 0; a < na; ++a) {
                        const double qa = helmert(m.nv, v, a);
                        if (qa == 0.0) continue;
                        for (int bb = 0; bb < na; ++bb) s += qa * helmert(m.nv, w, bb) * M[(3 * a + i) * 9 + 3 * bb + j];
                    }
                    Hb[(v * 4 + w) * 9 + i * 3 + j] = s;
                }
    return st;
}

}  // namespace fipc
