// Neo-Hookean tet element: energy, gradient and PSD-projected Hessian (host + device).
//
// Restates common/physics/neo_hookean.py (psi(sigma) 6-16, d psi/d sigma 20-34, its Hessian
// 38-58, P(F) 62-67, projected dP/dF 71-131) and the element assembly of
// projects/FastIPC/NEWTON_IPC.py:568-691 (F = Ds Dm^-1, scaled by dt^2 * vol0).
//
// dP/dF is never formed.  In the basis D_ab = u_a v_b^T (U, V from the SVD of F) it is the
// block matrix M of the reference: the projected 3x3 sigma-Hessian on {D_00, D_11, D_22} and
// one make_pd-ed 2x2 block per pair (a, b) on {D_ab, D_ba}.  With z_b = B^T-image of v_b
// (z_b[0] = -sum_m (Dm^-1 V)[m][b], z_b[m+1] = (Dm^-1 V)[m][b]) the 3x3 block (v, w) of the
// 12x12 element Hessian is U C(v,w) U^T with C_ac = sum_{b,d} M[ab][cd] z_b[v] z_d[w]; M has
// 21 nonzeros, so each block costs two 3x3 products.
#pragma once

#include "common.cuh"
#include "eig.cuh"

namespace fipc {

// make_pd of common/math/math_tools.py:40-64 on [[a, b], [c, d]] (row-major)
FIPC_HD void make_pd2(double* Mx) {
    const double a = Mx[0], b = (Mx[1] + Mx[2]) / 2.0, d = Mx[3];
    const double b2 = b * b, D = a * d - b2, T2 = (a + d) / 2.0;
    const double sq_ = sqrt(T2 * T2 - D);
    const double L2 = T2 - sq_;
    if (L2 < 0.0) {
        const double L1 = T2 + sq_;
        if (L1 <= 0.0) {
            Mx[0] = Mx[1] = Mx[2] = Mx[3] = 0.0;
        } else if (b2 == 0.0) {
            Mx[0] = L1;
            Mx[1] = Mx[2] = Mx[3] = 0.0;
        } else {
            const double L1md = L1 - d, r = L1md / L1;
            Mx[0] = r * L1md;
            Mx[1] = b * r;
            Mx[2] = b * r;
            Mx[3] = b2 / L1;
        }
    }
}

FIPC_HD double det3(const double* F) {
    return F[0] * (F[4] * F[8] - F[5] * F[7]) - F[1] * (F[3] * F[8] - F[5] * F[6]) + F[2] * (F[3] * F[7] - F[4] * F[6]);
}

// Rotation-variant SVD by one-sided Jacobi (Hestenes) on the columns of F:
// F = U diag(s) V^T, det U = det V = +1, s descending in magnitude, s[2] < 0 iff det F < 0.
FIPC_HD void svd3(const double* F, double* U, double* s, double* V) {
    double B[9];
    for (int i = 0; i < 9; ++i) {
        B[i] = F[i];
        V[i] = (i % 4 == 0) ? 1.0 : 0.0;
    }
    for (int sweep = 0; sweep < 10; ++sweep) {
        bool rotated = false;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                double al = 0, be = 0, ga = 0;
                for (int r = 0; r < 3; ++r) {
                    al += B[r * 3 + p] * B[r * 3 + p];
                    be += B[r * 3 + q] * B[r * 3 + q];
                    ga += B[r * 3 + p] * B[r * 3 + q];
                }
                if (fabs(ga) <= 1e-15 * sqrt(al * be) || ga == 0.0) continue;
                rotated = true;
                const double zeta = (be - al) / (2.0 * ga);
                const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                const double c = 1.0 / sqrt(1.0 + t * t), sn = c * t;
                for (int r = 0; r < 3; ++r) {
                    const double bp = B[r * 3 + p], bq = B[r * 3 + q];
                    B[r * 3 + p] = c * bp - sn * bq;
                    B[r * 3 + q] = sn * bp + c * bq;
                    const double vp = V[r * 3 + p], vq = V[r * 3 + q];
                    V[r * 3 + p] = c * vp - sn * vq;
                    V[r * 3 + q] = sn * vp + c * vq;
                }
            }
        if (!rotated) break;
    }
    double nrm[3];
    for (int c = 0; c < 3; ++c) nrm[c] = sqrt(B[c] * B[c] + B[3 + c] * B[3 + c] + B[6 + c] * B[6 + c]);
    // descending order
    int o[3] = {0, 1, 2};
    for (int i = 0; i < 2; ++i)
        for (int j = i + 1; j < 3; ++j)
            if (nrm[o[j]] > nrm[o[i]]) { const int t = o[i]; o[i] = o[j]; o[j] = t; }
    double Vs[9], Bs[9];
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) {
            Vs[r * 3 + c] = V[r * 3 + o[c]];
            Bs[r * 3 + c] = B[r * 3 + o[c]];
        }
    if (det3(Vs) < 0.0)
        for (int r = 0; r < 3; ++r) { Vs[r * 3 + 2] = -Vs[r * 3 + 2]; Bs[r * 3 + 2] = -Bs[r * 3 + 2]; }
    for (int i = 0; i < 9; ++i) V[i] = Vs[i];
    // u0, u1 from the two largest columns, u2 = u0 x u1; s_i = u_i . b_i
    const v3 b0 = mk(Bs[0], Bs[3], Bs[6]), b1 = mk(Bs[1], Bs[4], Bs[7]), b2 = mk(Bs[2], Bs[5], Bs[8]);
    const double n0 = sqrt(sq(b0));
    const v3 u0 = (1.0 / n0) * b0;
    v3 u1 = b1 - dot(u0, b1) * u0;
    u1 = (1.0 / sqrt(sq(u1))) * u1;
    const v3 u2 = cross(u0, u1);
    U[0] = u0.x; U[3] = u0.y; U[6] = u0.z;
    U[1] = u1.x; U[4] = u1.y; U[7] = u1.z;
    U[2] = u2.x; U[5] = u2.y; U[8] = u2.z;
    s[0] = dot(u0, b0);
    s[1] = dot(u1, b1);
    s[2] = dot(u2, b2);
}

// psi(sigma) (neo_hookean.py:6-16)
FIPC_HD double nh_psi_sigma(const double* s, double la, double mu) {
    const double s2 = s[0] * s[0] + s[1] * s[1] + s[2] * s[2], lp = log(s[0] * s[1] * s[2]);
    return mu / 2.0 * (s2 - 3) - (mu - la / 2.0 * lp) * lp;
}

// psi from F directly: sum sigma^2 = |F|^2 and prod sigma = det F (energy-only paths)
FIPC_HD double nh_psi_F(const double* F, double la, double mu) {
    double s2 = 0.0;
    for (int i = 0; i < 9; ++i) s2 += F[i] * F[i];
    const double lp = log(det3(F));
    return mu / 2.0 * (s2 - 3) - (mu - la / 2.0 * lp) * lp;
}

// deformation gradient F = Ds Dm^-1 (row-major)
FIPC_HD void deformation_gradient(const v3* X, const double* IB, double* F) {
    const v3 d1 = X[1] - X[0], d2 = X[2] - X[0], d3 = X[3] - X[0];
    const double Ds[9] = {d1.x, d2.x, d3.x, d1.y, d2.y, d3.y, d1.z, d2.z, d3.z};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            F[i * 3 + j] = Ds[i * 3 + 0] * IB[0 * 3 + j] + Ds[i * 3 + 1] * IB[1 * 3 + j] + Ds[i * 3 + 2] * IB[2 * 3 + j];
}

// Element energy (returned), gradient g[12] and the 10 upper 3x3 blocks of the Hessian
// Hu[blk*9 + i*3 + j], blk enumerating (v, w) with v <= w in row order
// (0,0)(0,1)(0,2)(0,3)(1,1)(1,2)(1,3)(2,2)(2,3)(3,3).  w = dt^2 * vol0.
FIPC_HD double nh_element(const v3* X, const double* IB, double la, double mu, double wgt, double* g, double* Hu) {
    double F[9], U[9], s[3], V[9];
    deformation_gradient(X, IB, F);
    svd3(F, U, s, V);
    const double psi = nh_psi_sigma(s, la, mu) * wgt;
    // P(F) = mu F + (la ln J - mu) F^-T  (neo_hookean.py:62-67)
    {
        const double J = det3(F), sc = (la * log(J) - mu) / J;
        const double C[9] = {F[4] * F[8] - F[5] * F[7], F[5] * F[6] - F[3] * F[8], F[3] * F[7] - F[4] * F[6],
                             F[2] * F[7] - F[1] * F[8], F[0] * F[8] - F[2] * F[6], F[1] * F[6] - F[0] * F[7],
                             F[1] * F[5] - F[2] * F[4], F[2] * F[3] - F[0] * F[5], F[0] * F[4] - F[1] * F[3]};
        double P[9];
        for (int i = 0; i < 9; ++i) P[i] = (mu * F[i] + sc * C[i]) * wgt;
        // g_{m+1, i} = sum_j IB[m][j] P[i][j], g_0 = -sum_m
        for (int i = 0; i < 3; ++i) {
            double acc = 0.0;
            for (int mm = 0; mm < 3; ++mm) {
                const double r = IB[mm * 3 + 0] * P[i * 3 + 0] + IB[mm * 3 + 1] * P[i * 3 + 1] + IB[mm * 3 + 2] * P[i * 3 + 2];
                g[(mm + 1) * 3 + i] = r;
                acc += r;
            }
            g[i] = -acc;
        }
    }
    // sigma-space gradient / projected Hessian and the three 2x2 blocks (neo_hookean.py:75-98)
    const double lp = log(s[0] * s[1] * s[2]);
    const double inv[3] = {1.0 / s[0], 1.0 / s[1], 1.0 / s[2]};
    double gs[3], Hs[9];
    for (int i = 0; i < 3; ++i) {
        gs[i] = mu * (s[i] - inv[i]) + la * inv[i] * lp;
        const double i2 = inv[i] * inv[i];
        Hs[i * 4] = mu * (1.0 + i2) - la * i2 * (lp - 1.0);
    }
    Hs[1] = Hs[3] = la * inv[0] * inv[1];
    Hs[5] = Hs[7] = la * inv[1] * inv[2];
    Hs[2] = Hs[6] = la * inv[0] * inv[2];
    psd_project3(Hs);
    const double middle = mu - la * lp;
    double Bk[3][4];
    const int pa[3] = {0, 1, 2}, pb[3] = {1, 2, 0};
    for (int k = 0; k < 3; ++k) {
        const int i = pa[k], j = pb[k];
        const double left = (mu + middle * inv[i] * inv[j]) / 2.0;
        double right = gs[i] + gs[j];
        const double ss = fmax(s[i] + s[j], 0.000001);
        right /= (2 * ss);
        Bk[k][0] = left + right;
        Bk[k][1] = left - right;
        Bk[k][2] = left - right;
        Bk[k][3] = left + right;
        // its eigenvalues are 2 left and 2 right: with both clearly positive make_pd leaves the
        // block unchanged, so its square root is skipped
        if (!(left > 1e-8 * fabs(right) && right > 1e-8 * fabs(left))) make_pd2(Bk[k]);
    }
    // the weight dt^2 vol0 folded into the sigma-space coefficients once
    for (int i = 0; i < 9; ++i) Hs[i] *= wgt;
    for (int k = 0; k < 3; ++k)
        for (int i = 0; i < 4; ++i) Bk[k][i] *= wgt;
    // z_b over the 4 vertices
    double z[3][4];
    for (int b = 0; b < 3; ++b) {
        double acc = 0.0;
        for (int mm = 0; mm < 3; ++mm) {
            const double zz = IB[mm * 3 + 0] * V[0 * 3 + b] + IB[mm * 3 + 1] * V[1 * 3 + b] + IB[mm * 3 + 2] * V[2 * 3 + b];
            z[b][mm + 1] = zz;
            acc += zz;
        }
        z[b][0] = -acc;
    }
    // Blocks (v, w) with 1 <= v <= w <= 3 directly: U C U^T with C built from z_b[v] z_d[w].  The
    // Hessian is bilinear in (z[.][v], z[.][w]) and z[.][0] = -(z[.][1] + z[.][2] + z[.][3]), so
    // the blocks of vertex 0 follow by sums: H(0,w) = -sum_{v>=1} H(v,w) with H(v,w) = H(w,v)^T,
    // and H(0,0) = -sum_{w>=1} H(0,w)^T.
#pragma unroll
    for (int v = 1; v < 4; ++v)
#pragma unroll
        for (int w = v; w < 4; ++w) {
            double Z[3][3];  // Z[b][d] = z_b[v] z_d[w]
            for (int b = 0; b < 3; ++b)
                for (int d = 0; d < 3; ++d) Z[b][d] = z[b][v] * z[d][w];
            double C[9];
            // Bk[0]: pair (0,1); Bk[1]: pair (1,2); Bk[2]: pair (2,0)   (row-major 2x2)
            C[0 * 3 + 0] = Hs[0] * Z[0][0] + Bk[0][0] * Z[1][1] + Bk[2][3] * Z[2][2];
            C[1 * 3 + 1] = Hs[4] * Z[1][1] + Bk[0][3] * Z[0][0] + Bk[1][0] * Z[2][2];
            C[2 * 3 + 2] = Hs[8] * Z[2][2] + Bk[1][3] * Z[1][1] + Bk[2][0] * Z[0][0];
            C[0 * 3 + 1] = Hs[1] * Z[0][1] + Bk[0][1] * Z[1][0];
            C[1 * 3 + 0] = Hs[3] * Z[1][0] + Bk[0][2] * Z[0][1];
            C[1 * 3 + 2] = Hs[5] * Z[1][2] + Bk[1][1] * Z[2][1];
            C[2 * 3 + 1] = Hs[7] * Z[2][1] + Bk[1][2] * Z[1][2];
            C[0 * 3 + 2] = Hs[2] * Z[0][2] + Bk[2][2] * Z[2][0];
            C[2 * 3 + 0] = Hs[6] * Z[2][0] + Bk[2][1] * Z[0][2];
            double T[9];
            for (int i = 0; i < 3; ++i)
                for (int c = 0; c < 3; ++c) T[i * 3 + c] = U[i * 3 + 0] * C[0 * 3 + c] + U[i * 3 + 1] * C[1 * 3 + c] + U[i * 3 + 2] * C[2 * 3 + c];
            // Hu block of (v, w), v <= w: (1,1) 4, (1,2) 5, (1,3) 6, (2,2) 7, (2,3) 8, (3,3) 9
            double* out = Hu + 9 * (v == 1 ? 3 + w : (v == 2 ? 5 + w : 9));
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j)
                    out[i * 3 + j] = T[i * 3 + 0] * U[j * 3 + 0] + T[i * 3 + 1] * U[j * 3 + 1] + T[i * 3 + 2] * U[j * 3 + 2];
        }
    // H(0,w), w = 1..3 (blocks 1..3) and H(0,0) (block 0)
    const double* H11 = Hu + 36;
    const double* H12 = Hu + 45;
    const double* H13 = Hu + 54;
    const double* H22 = Hu + 63;
    const double* H23 = Hu + 72;
    const double* H33 = Hu + 81;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const int ij = i * 3 + j, ji = j * 3 + i;
            Hu[9 + ij] = -(H11[ij] + H12[ji] + H13[ji]);
            Hu[18 + ij] = -(H12[ij] + H22[ij] + H23[ji]);
            Hu[27 + ij] = -(H13[ij] + H23[ij] + H33[ij]);
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const int ji = j * 3 + i;
            Hu[i * 3 + j] = -(Hu[9 + ji] + Hu[18 + ji] + Hu[27 + ji]);
        }
    return psi;
}

}  // namespace fipc
