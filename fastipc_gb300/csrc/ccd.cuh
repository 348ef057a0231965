// Continuous collision detection for the line-search filter (host + device).
//
// Restates the reference's CCD exactly in structure:
//  * the step clamp and early-out of common/math/wrapper/wrapper.cpp:254-328: with
//    d0 = current squared distance, the additive lower bound (1 - eta) sqrt(d0) / (|dp| + max|dt|)
//    is the time before which the distance cannot drop below eta sqrt(d0); if it is >= 1 the
//    pair is skipped (toc = 1), otherwise the exact interval test runs and its result is
//    clamped from below by the bound;
//  * the EVCTCD interval test (common/math/wrapper/EVCTCD/CTCD.cpp:92-472): time intervals on
//    which the coplanarity/distance polynomial (degree 6) and the barycentric/side polynomials
//    (degrees 3-4) have the required sign are intersected; the earliest common start is the
//    time of impact.
// Root isolation differs from the reference (Jenkins-Traub): real roots in [0, 1] come from
// bracketing by the derivative's roots (recursively, iteratively here) and bisection.  Only
// roots in [0, 1] shape the clamped intervals the reference builds, so the interval sets agree.
//
// Also the tet inversion-free step (common/math/math_tools.py:161-181, wrapper.cpp:200-252):
// smallest positive real root of det(Ds + t dDs) by Cardano with complex arithmetic.
#pragma once

#include "common.cuh"

namespace fipc {

struct Ivl {
    double l, u;
};

FIPC_HD double horner(const double* op, int n, double t) {
    double f = op[0];
    for (int i = 1; i <= n; ++i) {
        f *= t;
        f += op[i];
    }
    return f;
}

// real roots in [0,1] of op (degree n <= 6, op[0] != 0), ascending; returns the count
FIPC_HD int roots01(const double* op, int n, double* out) {
    // derivative chain: level k holds the (n-k)-th derivative, degree k
    double der[7][7];
    for (int i = 0; i <= n; ++i) der[n][i] = op[i];
    for (int k = n; k > 1; --k)
        for (int i = 0; i < k; ++i) der[k - 1][i] = der[k][i] * (k - i);
    double rts[8];
    int nr = 0;
    {   // degree 1
        const double r = -der[1][1] / der[1][0];
        if (r >= 0.0 && r <= 1.0) rts[nr++] = r;
    }
    for (int k = 2; k <= n; ++k) {
        double crit[9];
        int nc = 0;
        crit[nc++] = 0.0;
        for (int i = 0; i < nr; ++i)
            if (rts[i] > 0.0 && rts[i] < 1.0) crit[nc++] = rts[i];
        crit[nc++] = 1.0;
        const double* p = der[k];
        double nx[8];
        int m = 0;
        for (int i = 0; i + 1 < nc; ++i) {
            double a = crit[i], b = crit[i + 1];
            double fa = horner(p, k, a);
            const double fb = horner(p, k, b);
            if (fa == 0.0) {
                if (m == 0 || nx[m - 1] != a) nx[m++] = a;
                continue;
            }
            if (fb == 0.0 || (fa < 0.0) == (fb < 0.0)) continue;
            // p is monotone on [a, b] (its ends are consecutive critical points), so the root is
            // unique there: safeguarded Newton (p and p' by one Horner pass), the bracket
            // shrinking at every step and a bisection step whenever Newton would leave it; stops
            // once a step moves t by at most 1e-16 (the roots are interval ends in [0, 1]) or
            // the bracket cannot be split further
            double t = 0.5 * (a + b);
            for (int it = 0; it < 128; ++it) {
                double f = p[0], df = 0.0;
                for (int q = 1; q <= k; ++q) {
                    df = df * t + f;
                    f = f * t + p[q];
                }
                if (f == 0.0) {
                    a = b = t;
                    break;
                }
                if ((f < 0.0) == (fa < 0.0)) {
                    a = t;
                    fa = f;
                } else {
                    b = t;
                }
                double tn = df != 0.0 ? t - f / df : 0.5 * (a + b);
                if (!(tn > a && tn < b)) tn = 0.5 * (a + b);
                if (tn <= a || tn >= b || fabs(tn - t) <= 1e-16) {
                    t = tn > a && tn < b ? tn : t;
                    break;
                }
                t = tn;
            }
            nx[m++] = (a == b) ? a : t;
        }
        if (horner(p, k, 1.0) == 0.0 && (m == 0 || nx[m - 1] != 1.0)) nx[m++] = 1.0;
        nr = m;
        for (int i = 0; i < m; ++i) rts[i] = nx[i];
    }
    for (int i = 0; i < nr; ++i) out[i] = rts[i];
    return nr;
}

FIPC_HD void check_interval(double t1, double t2, const double* op, int deg, Ivl* iv, int* niv, bool pos) {
    t1 = fmin(1.0, fmax(0.0, t1));
    t2 = fmin(1.0, fmax(0.0, t2));
    const double f = horner(op, deg, (t2 + t1) / 2);
    if ((pos && f >= 0) || (!pos && f <= 0)) {
        iv[*niv].l = t1;
        iv[*niv].u = t2;
        (*niv)++;
    }
}

FIPC_HD bool could_have_roots(const double* op, int deg, bool pos) {
    double r = 0;
    if ((pos && op[0] > 0) || (!pos && op[0] < 0)) r = op[0];
    for (int i = 1; i < deg; ++i)
        if ((pos && op[i] > 0) || (!pos && op[i] < 0)) r += op[i];
    r += op[deg];
    return !((pos && r < 0) || (!pos && r > 0));
}

FIPC_HD int quad_roots(double a, double b, double c, double* t0, double* t1) {
    const double sign = b < 0 ? -1.0 : 1.0;
    const double D = b * b - 4 * a * c;
    if (D >= 0) {
        const double q = -0.5 * (b + sign * sqrt(D));
        *t0 = q / a;
        *t1 = c / q;
        if (*t0 > *t1) { const double t = *t0; *t0 = *t1; *t1 = t; }
        return 2;
    }
    return 0;
}

// CTCD.cpp:92-163 (intervals in [0,1] where op has the sign `pos`); op is modified
FIPC_HD void find_intervals(double* op, int n, Ivl* iv, int* niv, bool pos) {
    *niv = 0;
    double maxval = 0;
    for (int i = 0; i <= n; ++i) maxval = fmax(maxval, fabs(op[i]));
    if (maxval != 0)
        for (int i = 0; i <= n; ++i) op[i] /= maxval;
    int rd = n;
    for (int i = 0; i < n; ++i) {
        if (op[i] == 0) rd--;
        else break;
    }
    if (rd < n)
        for (int i = 0; i <= rd; ++i) op[i] = op[i + n - rd];
    double tm[8];
    int roots = 0;
    if (rd > 2) {
        if (!could_have_roots(op, rd, pos)) return;
        roots = roots01(op, rd, tm);
    } else if (rd == 2) {
        roots = quad_roots(op[0], op[1], op[2], &tm[0], &tm[1]);
    } else if (rd == 1) {
        tm[0] = -op[1] / op[0];
        roots = 1;
    } else {
        if ((!pos && op[0] <= 0) || (pos && op[0] >= 0)) {
            iv[0].l = 0;
            iv[0].u = 1.0;
            *niv = 1;
        }
        return;
    }
    if (roots > 0) {
        for (int i = 1; i < roots; ++i)
            for (int j = i; j > 0 && tm[j] < tm[j - 1]; --j) { const double t = tm[j]; tm[j] = tm[j - 1]; tm[j - 1] = t; }
        if (tm[0] >= 0) check_interval(0, tm[0], op, rd, iv, niv, pos);
        for (int i = 0; i < roots - 1; ++i)
            if (!((tm[i] < 0 && tm[i + 1] < 0) || (tm[i] > 1.0 && tm[i + 1] > 1.0))) check_interval(tm[i], tm[i + 1], op, rd, iv, niv, pos);
        if (tm[roots - 1] <= 1.0) check_interval(tm[roots - 1], 1.0, op, rd, iv, niv, pos);
    } else {
        check_interval(0.0, 1.0, op, rd, iv, niv, pos);
    }
}

FIPC_HD double triple3(v3 a, v3 b, v3 c) { return dot(a, cross(b, c)); }

FIPC_HD void bary_poly(v3 x10, v3 x20, v3 x30, v3 v10, v3 v20, v3 v30, Ivl* iv, int* niv) {
    const double A = dot(x10, x10), B = 2 * dot(x10, v10), C = dot(v10, v10);
    const double D = dot(x20, x10), E = dot(x20, v10) + dot(v20, x10), F = dot(v20, v10);
    const double G = dot(x30, x20), H = dot(x30, v20) + dot(v30, x20), I = dot(v30, v20);
    const double J = dot(x30, x10), K = dot(x30, v10) + dot(v30, x10), L = dot(v30, v10);
    double op[5];
    op[0] = F * L - C * I;
    op[1] = F * K + E * L - C * H - B * I;
    op[2] = F * J + D * L + E * K - C * G - A * I - B * H;
    op[3] = D * K + E * J - A * H - B * G;
    op[4] = D * J - A * G;
    find_intervals(op, 4, iv, niv, true);
}

FIPC_HD void plane_poly(v3 x10, v3 x20, v3 x30, v3 v10, v3 v20, v3 v30, Ivl* iv, int* niv) {
    double op[4];
    op[0] = triple3(v10, v20, v30);
    op[1] = triple3(x10, v20, v30) + triple3(v10, x20, v30) + triple3(v10, v20, x30);
    op[2] = triple3(x10, x20, v30) + triple3(x10, v20, x30) + triple3(v10, x20, x30);
    op[3] = triple3(x10, x20, x30);
    find_intervals(op, 3, iv, niv, true);
}

FIPC_HD void distance_poly(v3 x10, v3 x20, v3 x30, v3 v10, v3 v20, v3 v30, double minD2, Ivl* iv, int* niv) {
    const double A = triple3(v10, v20, v30);
    const double B = triple3(x10, v20, v30) + triple3(v10, x20, v30) + triple3(v10, v20, x30);
    const double C = triple3(x10, x20, v30) + triple3(x10, v20, x30) + triple3(v10, x20, x30);
    const double D = triple3(x10, x20, x30);
    const v3 E = cross(x20, x30), F = cross(x20, v30) + cross(v20, x30), G = cross(v20, v30);
    double op[7];
    op[0] = A * A;
    op[1] = 2 * A * B;
    op[2] = B * B + 2 * A * C - dot(G, G) * minD2;
    op[3] = 2 * A * D + 2 * B * C - 2 * dot(G, F) * minD2;
    op[4] = 2 * B * D + C * C - (2 * dot(G, E) + dot(F, F)) * minD2;
    op[5] = 2 * C * D - 2 * dot(F, E) * minD2;
    op[6] = D * D - dot(E, E) * minD2;
    find_intervals(op, 6, iv, niv, false);
}

FIPC_HD bool overlap_all(const Ivl* v, int n) {
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j)
            if (v[i].l > v[j].u || v[j].l > v[i].u) return false;
    return true;
}
FIPC_HD Ivl intersect_all(const Ivl* v, int n) {
    Ivl r{0.0, 1.0};
    for (int i = 0; i < n; ++i) {
        r.l = fmax(v[i].l, r.l);
        r.u = fmin(v[i].u, r.u);
    }
    return r;
}

// CTCD.cpp:383-472
FIPC_HD bool vertex_face_ctcd(v3 q0s, v3 q1s, v3 q2s, v3 q3s, v3 q0e, v3 q1e, v3 q2e, v3 q3e, double eta, double* t) {
    const double minD = eta * eta;
    const v3 v0 = q0e - q0s, v1 = q1e - q1s, v2 = q2e - q2s, v3_ = q3e - q3s;
    Ivl cp[8], e1[8], e2[8], e3[8];
    int ncp, ne1, ne2, ne3;
    plane_poly(q0s - q1s, cross(q3s - q1s, q2s - q1s), q3s - q1s, v0 - v1, cross(v3_ - v1, v2 - v1), v3_ - v1, e1, &ne1);
    if (!ne1) return false;
    plane_poly(q0s - q2s, cross(q1s - q2s, q3s - q2s), q1s - q2s, v0 - v2, cross(v1 - v2, v3_ - v2), v1 - v2, e2, &ne2);
    if (!ne2) return false;
    plane_poly(q0s - q3s, cross(q2s - q3s, q1s - q3s), q2s - q3s, v0 - v3_, cross(v2 - v3_, v1 - v3_), v2 - v3_, e3, &ne3);
    if (!ne3) return false;
    distance_poly(q0s - q1s, q2s - q1s, q3s - q1s, v0 - v1, v2 - v1, v3_ - v1, minD, cp, &ncp);
    if (!ncp) return false;
    bool col = false;
    double mint = 1.0;
    for (int i = 0; i < ncp; ++i)
        for (int j = 0; j < ne1; ++j)
            for (int k = 0; k < ne2; ++k)
                for (int l = 0; l < ne3; ++l) {
                    const Ivl s[4] = {cp[i], e1[j], e2[k], e3[l]};
                    if (overlap_all(s, 4)) {
                        mint = fmin(intersect_all(s, 4).l, mint);
                        col = true;
                    }
                }
    if (col) *t = mint;
    return col;
}

// CTCD.cpp:245-381
FIPC_HD bool edge_edge_ctcd(v3 q0s, v3 p0s, v3 q1s, v3 p1s, v3 q0e, v3 p0e, v3 q1e, v3 p1e, double eta, double* t) {
    const double minD = eta * eta;
    Ivl raw[8], cp[8], par[8], a0[8], a1[8], b0[8], b1[8];
    int nraw, ncp = 0, npar = 0, na0, na1, nb0, nb1;
    const v3 vp0 = p0e - p0s, vp1 = p1e - p1s, vq0 = q0e - q0s, vq1 = q1e - q1s;
    distance_poly(p0s - p1s, p0s - q0s, p1s - q1s, vp0 - vp1, vp0 - vq0, vp1 - vq1, minD, raw, &nraw);
    for (int i = 0; i < nraw; ++i) {
        const double midt = (raw[i].u + raw[i].l) / 2;
        const v3 x10 = (q0s - p0s) + midt * (vq0 - vp0), x20 = (q1s - p1s) + midt * (vq1 - vp1);
        if (sqrt(sq(cross(x10, x20))) < 1e-8) par[npar++] = raw[i];
        else cp[ncp++] = raw[i];
    }
    if (!ncp) return false;
    v3 x10 = p1s - q1s, v10 = vp1 - vq1;
    bary_poly(x10, p0s - q0s, q0s - q1s, v10, vp0 - vq0, vq0 - vq1, a0, &na0);
    if (!na0) return false;
    bary_poly(x10, q0s - p0s, p0s - q1s, v10, vq0 - vp0, vp0 - vq1, a1, &na1);
    if (!na1) return false;
    x10 = p0s - q0s;
    v10 = vp0 - vq0;
    bary_poly(x10, p1s - q1s, q1s - q0s, v10, vp1 - vq1, vq1 - vq0, b0, &nb0);
    if (!nb0) return false;
    bary_poly(x10, q1s - p1s, p1s - q0s, v10, vq1 - vp1, vp1 - vq0, b1, &nb1);
    if (!nb1) return false;
    bool col = false;
    double mint = 1.0;
    for (int i = 0; i < ncp; ++i)
        for (int j = 0; j < na0; ++j)
            for (int k = 0; k < na1; ++k)
                for (int l = 0; l < nb0; ++l)
                    for (int m = 0; m < nb1; ++m) {
                        const Ivl s[5] = {cp[i], a0[j], a1[k], b0[l], b1[m]};
                        if (!overlap_all(s, 5)) continue;
                        const Ivl is = intersect_all(s, 5);
                        bool skip = false;
                        for (int p = 0; p < npar; ++p) {
                            const Ivl pc[2] = {is, par[p]};
                            if (overlap_all(pc, 2)) { skip = true; break; }
                        }
                        if (!skip) {
                            mint = fmin(mint, is.l);
                            col = true;
                        }
                    }
    if (col) *t = mint;
    return col;
}

// The additive lower bound of wrapper.cpp:254-328: lb = (1 - eta) sqrt(dist2) / maxDisp is the
// time before which the distance cannot drop below eta sqrt(dist2).  False when the pair's toc is
// 1 without the exact test (no motion, or lb >= 1); else *lb holds the bound.
FIPC_HD bool pt_needs_exact(v3 dp, v3 dt0, v3 dt1, v3 dt2, double eta, double dist2, double* lb) {
    const double maxDisp = sqrt(sq(dp)) + sqrt(fmax(fmax(sq(dt0), sq(dt1)), sq(dt2)));
    if (maxDisp == 0) return false;
    *lb = (1 - eta) * sqrt(dist2) / maxDisp;
    return *lb < 1;
}
FIPC_HD bool ee_needs_exact(v3 da0, v3 da1, v3 db0, v3 db1, double eta, double dist2, double* lb) {
    const double maxDisp = sqrt(fmax(sq(da0), sq(da1))) + sqrt(fmax(sq(db0), sq(db1)));
    if (maxDisp == 0) return false;
    *lb = (1 - eta) * sqrt(dist2) / maxDisp;
    return *lb < 1;
}

// the exact interval test, its toc clamped from below by lb (1 when no collision)
FIPC_HD double pt_ccd_exact(v3 p, v3 t0, v3 t1, v3 t2, v3 dp, v3 dt0, v3 dt1, v3 dt2, double eta, double dist2, double lb) {
    double toc = 1.0;
    if (vertex_face_ctcd(p, t0, t1, t2, p + dp, t0 + dt0, t1 + dt1, t2 + dt2, eta * sqrt(dist2), &toc))
        if (toc < lb) toc = lb;
    return toc;
}
FIPC_HD double ee_ccd_exact(v3 a0, v3 a1, v3 b0, v3 b1, v3 da0, v3 da1, v3 db0, v3 db1, double eta, double dist2, double lb) {
    double toc = 1.0;
    if (edge_edge_ctcd(a0, a1, b0, b1, a0 + da0, a1 + da1, b0 + db0, b1 + db1, eta * sqrt(dist2), &toc))
        if (toc < lb) toc = lb;
    return toc;
}

// additive lower bound + exact test for a point-triangle pair (wrapper.cpp:254-290)
FIPC_HD double pt_ccd(v3 p, v3 t0, v3 t1, v3 t2, v3 dp, v3 dt0, v3 dt1, v3 dt2, double eta, double dist2) {
    double lb;
    if (!pt_needs_exact(dp, dt0, dt1, dt2, eta, dist2, &lb)) return 1.0;
    return pt_ccd_exact(p, t0, t1, t2, dp, dt0, dt1, dt2, eta, dist2, lb);
}

// additive lower bound + exact test for an edge-edge pair (wrapper.cpp:292-328)
FIPC_HD double ee_ccd(v3 a0, v3 a1, v3 b0, v3 b1, v3 da0, v3 da1, v3 db0, v3 db1, double eta, double dist2) {
    double lb;
    if (!ee_needs_exact(da0, da1, db0, db1, eta, dist2, &lb)) return 1.0;
    return ee_ccd_exact(a0, a1, b0, b1, da0, da1, db0, db1, eta, dist2, lb);
}

// ---------------------------------------------------------------- inversion-free step
struct cplx {
    double re, im;
};
FIPC_HD cplx cadd(cplx a, cplx b) { return cplx{a.re + b.re, a.im + b.im}; }
FIPC_HD cplx csub(cplx a, cplx b) { return cplx{a.re - b.re, a.im - b.im}; }
FIPC_HD cplx cmul(cplx a, cplx b) { return cplx{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
FIPC_HD cplx cdiv(cplx a, cplx b) {
    const double d = b.re * b.re + b.im * b.im;
    return cplx{(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
}
FIPC_HD cplx cscale(cplx a, double s) { return cplx{a.re * s, a.im * s}; }
FIPC_HD double cabs_(cplx a) { return sqrt(a.re * a.re + a.im * a.im); }
// principal square root
FIPC_HD cplx csqrt_(cplx z) {
    const double r = cabs_(z);
    if (r == 0.0) return cplx{0.0, 0.0};
    const double re = sqrt(0.5 * (r + fabs(z.re)));
    if (z.re >= 0.0) return cplx{re, z.im / (2.0 * re)};
    return cplx{fabs(z.im) / (2.0 * re), z.im >= 0.0 ? re : -re};
}
// principal z^(1/3) = |z|^(1/3) exp(i arg(z) / 3)
FIPC_HD cplx ccbrt_(cplx z) {
    const double r = cabs_(z);
    if (r == 0.0) return cplx{0.0, 0.0};
    const double m = pow(r, 1.0 / 3.0), th = atan2(z.im, z.re) / 3.0;
    return cplx{m * cos(th), m * sin(th)};
}

FIPC_HD double quad_root_pos(double a, double b, double c, double tol) {
    double t;
    if (fabs(a) <= tol) t = -c / b;
    else {
        const double desc = b * b - 4 * a * c;
        if (desc > 0) {
            t = (-b - sqrt(desc)) / (2 * a);
            if (t < 0) t = (-b + sqrt(desc)) / (2 * a);
        } else t = -1;
    }
    return t;
}

// smallest positive real root of a t^3 + b t^2 + c t + d, or a negative value (wrapper.cpp:220-252)
FIPC_HD double cubic_root_pos(double a, double b, double c, double d, double tol) {
    if (fabs(a) <= tol) return quad_root_pos(b, c, d, tol);
    double t = -1;
    const cplx d0{b * b - 3 * a * c, 0.0};
    const cplx d1{2 * b * b * b - 9 * a * b * c + 27 * a * a * d, 0.0};
    const cplx disc = csub(cmul(d1, d1), cscale(cmul(cmul(d0, d0), d0), 4.0));
    cplx C = ccbrt_(cscale(cadd(d1, csqrt_(disc)), 0.5));
    if (cabs_(C) == 0.0) C = ccbrt_(cscale(csub(d1, csqrt_(disc)), 0.5));
    const double s3 = sqrt(3.0);
    const cplx u2{-0.5, 0.5 * s3}, u3{-0.5, -0.5 * s3};
    const double den = -3.0 * a;
    const cplx bb{b, 0.0};
    const cplx t1 = cscale(cadd(cadd(bb, C), cdiv(d0, C)), 1.0 / den);
    const cplx u2C = cmul(u2, C), u3C = cmul(u3, C);
    const cplx t2 = cscale(cadd(cadd(bb, u2C), cdiv(d0, u2C)), 1.0 / den);
    const cplx t3 = cscale(cadd(cadd(bb, u3C), cdiv(d0, u3C)), 1.0 / den);
    if (fabs(t1.im) < tol && t1.re > 0) t = t1.re;
    if (fabs(t2.im) < tol && t2.re > 0 && (t2.re < t || t < 0)) t = t2.re;
    if (fabs(t3.im) < tol && t3.re > 0 && (t3.re < t || t < 0)) t = t3.re;
    return t;
}

// coefficients of det(Ds + t dDs) = a t^3 + b t^2 + c t + d (6 x the tet's volume along the step)
FIPC_HD void inversion_cubic(const v3* X, const v3* P, double* k) {
    const v3 v01 = X[1] - X[0], v02 = X[2] - X[0], v03 = X[3] - X[0];
    const v3 p01 = P[1] - P[0], p02 = P[2] - P[0], p03 = P[3] - P[0];
    const v3 pp = cross(p01, p02);
    const v3 mix = cross(v01, p02) + cross(p01, v02);
    const v3 vv = cross(v01, v02);
    k[0] = dot(p03, pp);
    k[1] = dot(v03, pp) + dot(p03, mix);
    k[2] = dot(p03, vv) + dot(v03, mix);
    k[3] = dot(v03, vv);
}

// largest step keeping the tet's orientation, scaled by (1 - eta); 1 if none (math_tools.py:161-181)
FIPC_HD double inversion_free_step(const v3* X, const v3* P, double eta) {
    double k[4];
    inversion_cubic(X, P, k);
    const double r = cubic_root_pos(k[0], k[1], k[2], k[3], 1e-8);
    return r < 0.0 ? 1.0 : r * (1.0 - eta);
}

// Early-out of the step filter for tets whose result is provably >= 1, a no-op in the minimum
// over all of them (the filter's minimum starts at 1).
// A tet whose volume polynomial stays above d / 2 on [0, T], T = 2 / (1 - eta), because
// |c| T + |b| T^2 + |a| T^3 <= d / 2, has no root below T: inversion_free_step returns 1 (no
// positive root) or (1 - eta) r >= 2.
FIPC_HD bool inversion_cannot_flip(const v3* X, const v3* P, double eta) {
    if (!(eta < 1.0)) return false;
    double k[4];
    inversion_cubic(X, P, k);
    if (!(k[3] > 0.0)) return false;
    const double T = 2.0 / (1.0 - eta);
    return ((fabs(k[0]) * T + fabs(k[1])) * T + fabs(k[2])) * T <= 0.5 * k[3];
}

}  // namespace fipc
