// 2D element and contact math of the reference's 2D path (host + device).
//
//   * fixed-corotated triangle: energy, first Piola stress and the projected dP/dF of
//     common/physics/fixed_corotated.py (2D branches), assembled into the element gradient and
//     Hessian as compute_elasticity does for dim 2 (projects/FastIPC/NEWTON_IPC.py:577-624);
//   * the 2x2 SVD in the convention of the reference's svd_2 (rotations U and V,
//     s0 >= |s1|, s1 < 0 exactly when det F < 0), written from the closed form of a 2x2 matrix
//     as a scaled rotation plus a scaled reflection;
//   * point-edge continuous collision detection, common/math/ipc.py:415-481;
//   * point_inside_triangle, common/math/ipc.py:502-509.
// The 2D barrier rows reuse barrier.cuh on positions with z = 0: the 3D point-point and
// point-edge distances of planar points are the 2D ones, and their Hessians have zero z rows.
#pragma once

#include "barrier.cuh"
#include "common.cuh"
#include "nh.cuh"

namespace fipc {

// F (row-major 2x2) = U diag(s) V^T
FIPC_HD void svd2(const double* F, double* U, double* s, double* V) {
    const double E = 0.5 * (F[0] + F[3]), Fm = 0.5 * (F[0] - F[3]);
    const double G = 0.5 * (F[2] + F[1]), H = 0.5 * (F[2] - F[1]);
    const double Q = sqrt(E * E + H * H), R = sqrt(Fm * Fm + G * G);
    s[0] = Q + R;
    s[1] = Q - R;
    const double a1 = atan2(G, Fm), a2 = atan2(H, E);
    const double ph = 0.5 * (a2 + a1), th = 0.5 * (a2 - a1);
    const double cp = cos(ph), sp = sin(ph), ct = cos(th), st = sin(th);
    U[0] = cp;
    U[1] = -sp;
    U[2] = sp;
    U[3] = cp;
    // V = rotation by -th
    V[0] = ct;
    V[1] = st;
    V[2] = -st;
    V[3] = ct;
}

// fixed_corotated.py elasticity_energy, dim 2
FIPC_HD double fc2_psi(const double* s, double la, double mu) {
    const double a = s[0] - 1.0, b = s[1] - 1.0, p = s[0] * s[1] - 1.0;
    return mu * (a * a + b * b) + la / 2 * p * p;
}

FIPC_HD double fc2_psi_F(const double* F, double la, double mu) {
    double U[4], s[2], V[4];
    svd2(F, U, s, V);
    return fc2_psi(s, la, mu);
}

// P (row-major) and dPdF [4][4] (index j*2+i for F_ij, as the reference orders it) of the
// fixed-corotated energy, the sigma Hessian and the twist block made PSD by make_pd
FIPC_HD void fc2_P_dPdF(const double* F, double la, double mu, double* P, double* dPdF) {
    double U[4], s[2], V[4];
    svd2(F, U, s, V);
    const double J = F[0] * F[3] - F[1] * F[2];
    const double R[4] = {U[0] * V[0] + U[1] * V[1], U[0] * V[2] + U[1] * V[3], U[2] * V[0] + U[3] * V[1],
                         U[2] * V[2] + U[3] * V[3]};
    const double cof[4] = {F[3], -F[2], -F[1], F[0]};
    for (int k = 0; k < 4; ++k) P[k] = 2 * mu * (F[k] - R[k]) + la * (J - 1) * cof[k];
    const double pm1 = s[0] * s[1] - 1.0;
    const double g0 = 2 * mu * (s[0] - 1) + s[1] * la * pm1, g1 = 2 * mu * (s[1] - 1) + s[0] * la * pm1;
    double Hs[4] = {2 * mu + la * s[1] * s[1], la * (pm1 + s[1] * s[0]), la * (pm1 + s[1] * s[0]), 2 * mu + la * s[0] * s[0]};
    make_pd2(Hs);
    const double left = mu - la / 2 * pm1;
    double sum = s[0] + s[1];
    sum = sum > 0.000001 ? sum : 0.000001;
    const double right = (g0 + g1) / (2 * sum);
    double B[4] = {left + right, left - right, left - right, left + right};
    make_pd2(B);
    // basis e_p = vec(u_a v_b^T), p = 2a+b; M couples (00,11) through Hs and (01,10) through B
    double e[4][4];
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int i = 0; i < 2; ++i)
                for (int j = 0; j < 2; ++j) e[2 * a + b][j * 2 + i] = U[i * 2 + a] * V[j * 2 + b];
    const double M[4][4] = {{Hs[0], 0, 0, Hs[1]}, {0, B[0], B[1], 0}, {0, B[2], B[3], 0}, {Hs[2], 0, 0, Hs[3]}};
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            double acc = 0.0;
            for (int p = 0; p < 4; ++p)
                for (int q = 0; q < 4; ++q)
                    if (M[p][q] != 0.0) acc += M[p][q] * e[p][r] * e[q][c];
            dPdF[r * 4 + c] = acc;
        }
}

// One triangle (compute_elasticity, dim 2): F = Ds IB, Ds = [x1-x0, x2-x0].  g [6] and the 3x3
// vertex blocks of the 6x6 Hessian, H [9][4] (block a*3+b, entries d*2+e), of w psi(F);
// returns w psi(F).
FIPC_HD double fc2_element(const double* X /*[3][2]*/, const double* IB, double la, double mu, double w, double* g, double* H) {
    const double Ds[4] = {X[2] - X[0], X[4] - X[0], X[3] - X[1], X[5] - X[1]};
    const double F[4] = {Ds[0] * IB[0] + Ds[1] * IB[2], Ds[0] * IB[1] + Ds[1] * IB[3], Ds[2] * IB[0] + Ds[3] * IB[2],
                         Ds[2] * IB[1] + Ds[3] * IB[3]};
    double P[4], dPdF[16];
    fc2_P_dPdF(F, la, mu, P, dPdF);
    // dF_ij / dx_{a,d} = delta_id D[a][j]
    const double D[3][2] = {{-IB[0] - IB[2], -IB[1] - IB[3]}, {IB[0], IB[1]}, {IB[2], IB[3]}};
    for (int a = 0; a < 3; ++a)
        for (int d = 0; d < 2; ++d) g[a * 2 + d] = w * (P[d * 2 + 0] * D[a][0] + P[d * 2 + 1] * D[a][1]);
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            for (int d = 0; d < 2; ++d)
                for (int e2 = 0; e2 < 2; ++e2) {
                    double acc = 0.0;
                    for (int j = 0; j < 2; ++j)
                        for (int s2 = 0; s2 < 2; ++s2) acc += dPdF[(j * 2 + d) * 4 + s2 * 2 + e2] * D[a][j] * D[b][s2];
                    H[(a * 3 + b) * 4 + d * 2 + e2] = w * acc;
                }
    return w * fc2_psi_F(F, la, mu);
}

// ---------------------------------------------------------------- 2D contact primitives
FIPC_HD double pp2_dist2(const double* a, const double* b) {
    const double dx = a[0] - b[0], dy = a[1] - b[1];
    return dx * dx + dy * dy;
}
// PE_2D_E (common/math/distance.py:68-71)
FIPC_HD double pe2_dist2(const double* p, const double* e0, const double* e1) {
    const double ex = e1[0] - e0[0], ey = e1[1] - e0[1];
    const double num = ey * p[0] - ex * p[1] + e1[0] * e0[1] - e1[1] * e0[0];
    return num * num / (ex * ex + ey * ey);
}
// PE_type (distance.py:1757-1768): 0 nearest e0, 1 nearest e1, 2 interior
FIPC_HD int pe2_type(const double* p, const double* e0, const double* e1) {
    const double ex = e1[0] - e0[0], ey = e1[1] - e0[1];
    const double ratio = (ex * (p[0] - e0[0]) + ey * (p[1] - e0[1])) / (ex * ex + ey * ey);
    return ratio < 0 ? 0 : (ratio > 1 ? 1 : 2);
}
FIPC_HD double pe2_dist2_typed(const double* p, const double* e0, const double* e1, int c) {
    return c == 0 ? pp2_dist2(p, e0) : (c == 1 ? pp2_dist2(p, e1) : pe2_dist2(p, e0, e1));
}

// point_edge_ccd_broadphase / moving_point_edge_ccd_broadphase (ipc.py:367-381)
FIPC_HD bool pe2_broad(const double* x0, const double* x1, const double* x2, double dhat) {
    for (int k = 0; k < 2; ++k) {
        const double lo = fmin(x1[k], x2[k]), hi = fmax(x1[k], x2[k]);
        if (!(x0[k] < hi + dhat && lo - dhat < x0[k])) return false;
    }
    return true;
}
FIPC_HD bool pe2_moving_broad(const double* x0, const double* x1, const double* x2, const double* d0, const double* d1,
                              const double* d2, double dhat) {
    for (int k = 0; k < 2; ++k) {
        const double p1 = x0[k] + d0[k];
        const double lp = fmin(x0[k], p1), hp = fmax(x0[k], p1);
        const double a1 = x1[k] + d1[k], b1 = x2[k] + d2[k];
        const double le = fmin(fmin(x1[k], x2[k]), fmin(a1, b1)), he = fmax(fmax(x1[k], x2[k]), fmax(a1, b1));
        if (!(lp < he + dhat && le - dhat < hp)) return false;
    }
    return true;
}

// check_overlap (ipc.py:415-421): the contact point at time root lies on the edge
FIPC_HD bool pe2_overlap(const double* x0, const double* x1, const double* x2, const double* d0, const double* d1,
                         const double* d2, double root) {
    const double p0x = x0[0] + d0[0] * root, p0y = x0[1] + d0[1] * root;
    const double e0x = x1[0] + d1[0] * root, e0y = x1[1] + d1[1] * root;
    const double e1x = x2[0] + d2[0] * root, e1y = x2[1] + d2[1] * root;
    const double ex = e1x - e0x, ey = e1y - e0y;
    const double ratio = (ex * (p0x - e0x) + ey * (p0y - e0y)) / (ex * ex + ey * ey);
    return 0 <= ratio && ratio <= 1;
}

// point_edge_ccd_impl (ipc.py:423-470): the earliest root in (0, 1] of the collinearity
// quadratic a t^2 + b t + c whose contact point lies on the edge, times (1 - eta)
FIPC_HD double pe2_ccd_impl(const double* x0, const double* x1, const double* x2, const double* d0, const double* d1,
                            const double* d2, double eta) {
    double toc = 1.0;
    const double a = d0[0] * (d2[1] - d1[1]) + d0[1] * (d1[0] - d2[0]) + d2[0] * d1[1] - d2[1] * d1[0];
    const double b = x0[0] * (d2[1] - d1[1]) + d0[0] * (x2[1] - x1[1]) + d0[1] * (x1[0] - x2[0]) + x0[1] * (d1[0] - d2[0]) +
                     d1[1] * x2[0] + d2[0] * x1[1] - d1[0] * x2[1] - d2[1] * x1[0];
    const double c = x0[0] * (x2[1] - x1[1]) + x0[1] * (x1[0] - x2[0]) + x2[0] * x1[1] - x2[1] * x1[0];
    auto take = [&](double root) {
        if (root > 0 && root <= 1 && pe2_overlap(x0, x1, x2, d0, d1, d2, root)) toc = fmin(toc, root * (1 - eta));
    };
    if (a == 0 && b == 0 && c == 0) {
        // collinear throughout: the point can only reach an endpoint
        for (int k = 0; k < 2; ++k) {
            const double* xe = k == 0 ? x1 : x2;
            const double* de = k == 0 ? d1 : d2;
            const double rx = x0[0] - xe[0], ry = x0[1] - xe[1], vx = d0[0] - de[0], vy = d0[1] - de[1];
            if (rx * vx + ry * vy < 0) {
                const double root = sqrt((rx * rx + ry * ry) / (vx * vx + vy * vy));
                if (root > 0 && root <= 1) toc = fmin(toc, root * (1 - eta));
            }
        }
    } else if (a == 0) {
        if (b != 0) take(-c / b);
    } else {
        const double delta = b * b - 4 * a * c;
        if (delta == 0) {
            take(-b / (2 * a));
        } else if (delta > 0) {
            const double sq = sqrt(delta);
            if (b > 0) {
                take((-b - sq) / (2 * a));
                take(2 * c / (-b - sq));
            } else {
                take(2 * c / (-b + sq));
                take((-b + sq) / (2 * a));
            }
        }
    }
    return toc;
}

// point_edge_ccd (ipc.py:472-481): additive lower bound first, the exact test when it is < 1
FIPC_HD double pe2_ccd(const double* x0, const double* x1, const double* x2, const double* d0, const double* d1,
                       const double* d2, double eta) {
    const double dist2 = pe2_dist2_typed(x0, x1, x2, pe2_type(x0, x1, x2));
    const double m0 = d0[0] * d0[0] + d0[1] * d0[1], m1 = d1[0] * d1[0] + d1[1] * d1[1], m2 = d2[0] * d2[0] + d2[1] * d2[1];
    const double mx = fmax(fmax(m0, m1), m2);
    double toc = 1.0;
    if (mx > 0) {
        const double lb = (1 - eta) * sqrt(dist2) / (2 * sqrt(mx));
        if (lb <= 1) {
            toc = pe2_ccd_impl(x0, x1, x2, d0, d1, d2, eta);
            toc = fmax(toc, lb);
        }
    }
    return toc;
}

// PP_g_and_H / PE_g_and_H for 2D points (common/math/ipc.py:67-136): type 0 PP (2 vertices),
// 1 PE (3).  X [nv][2]; g [2 nv]; H [nv*nv][4] (2x2 vertex blocks v*nv+w, entries d*2+e).
// The points are lifted to z = 0 and the 3D rows of barrier.cuh evaluated: the planar
// distances equal the 2D ones, and the z rows and columns of the Hessians are zero.
FIPC_HD int barrier_row_2d(int type, const double* X, double dh2, double kappa, int want, double* E, double* g, double* H) {
    const int nv = type == 0 ? 2 : 3;
    v3 P[4], P0[4];
    for (int k = 0; k < 4; ++k) {
        const int v = k < nv ? k : 0;
        P[k] = mk(X[2 * v], X[2 * v + 1], 0.0);
        P0[k] = mk(0, 0, 0);
    }
    double gg[12], hb[144];
    const int st = barrier_row(type == 0 ? T_PP : T_PE, P, P0, dh2, kappa, want, E, gg, hb);
    if (!want) return st;
    for (int v = 0; v < nv; ++v)
        for (int d = 0; d < 2; ++d) g[2 * v + d] = gg[3 * v + d];
    for (int v = 0; v < nv; ++v)
        for (int w = 0; w < nv; ++w)
            for (int d = 0; d < 2; ++d)
                for (int f = 0; f < 2; ++f) H[4 * (v * nv + w) + 2 * d + f] = hb[(v * 4 + w) * 9 + 3 * d + f];
    return st;
}

// point_inside_triangle (ipc.py:502-509), inclusive of the boundary
FIPC_HD bool point_in_tri2(const double* P, const double* A, const double* B, const double* C) {
    const double d1 = (P[0] - B[0]) * (A[1] - B[1]) - (P[1] - B[1]) * (A[0] - B[0]);
    const double d2 = (P[0] - C[0]) * (B[1] - C[1]) - (P[1] - C[1]) * (B[0] - C[0]);
    const double d3 = (P[0] - A[0]) * (C[1] - A[1]) - (P[1] - A[1]) * (C[0] - A[0]);
    const bool neg = d1 < 0 || d2 < 0 || d3 < 0;
    const bool pos = d1 > 0 || d2 > 0 || d3 > 0;
    return !(neg && pos);
}

}  // namespace fipc
