// Feature classification, squared distances and the predicates of the broad phase
// (host + device).  Restates common/math/distance.py (PT_type 1676, EE_type 1706,
// PT_dist2 1771, EE_dist2 1791, the *_3D_E distances) and common/math/ipc.py
// (broad-phase AABB tests 332-379, segment_intersect_triangle 511-526).
#pragma once

#include "common.cuh"

namespace fipc {

FIPC_HD double d_PP(v3 a, v3 b) { return sq(a - b); }
FIPC_HD double d_PE(v3 p, v3 e0, v3 e1) { return sq(cross(e0 - p, e1 - p)) / sq(e1 - e0); }
FIPC_HD double d_PT(v3 p, v3 t0, v3 t1, v3 t2) {
    const v3 n = cross(t1 - t0, t2 - t0);
    const double s = dot(p - t0, n);
    return s * s / sq(n);
}
FIPC_HD double d_EE(v3 a0, v3 a1, v3 b0, v3 b1) {
    const v3 n = cross(a1 - a0, b1 - b0);
    const double s = dot(b0 - a0, n);
    return s * s / sq(n);
}
FIPC_HD double d_EECN2(v3 a0, v3 a1, v3 b0, v3 b1) { return sq(cross(a1 - a0, b1 - b0)); }
FIPC_HD double m_threshold(v3 a0, v3 a1, v3 b0, v3 b1) { return 1.0e-3 * sq(a0 - a1) * sq(b0 - b1); }

// parameters of p against edge (o, o+e) in the triangle plane with normal nrm:
// solve (B B^T) x = B (p - o) with B rows e and e x nrm  (distance.py:1678-1680)
FIPC_HD void pt_param(v3 p, v3 o, v3 e, v3 nrm, double* prm) {
    const v3 b1 = cross(e, nrm), q = p - o;
    const double a00 = dot(e, e), a01 = dot(e, b1), a11 = dot(b1, b1);
    const double r0 = dot(e, q), r1 = dot(b1, q);
    const double inv = 1.0 / (a00 * a11 - a01 * a01);
    prm[0] = inv * (a11 * r0 - a01 * r1);
    prm[1] = inv * (-a01 * r0 + a00 * r1);
}

// 0,1,2: closest to t0,t1,t2; 3,4,5: edges t0t1, t1t2, t2t0; 6: interior
FIPC_HD int pt_type(v3 p, v3 t0, v3 t1, v3 t2) {
    const v3 n = cross(t1 - t0, t2 - t0);
    double p0[2], p1[2], p2[2];
    pt_param(p, t0, t1 - t0, n, p0);
    if (0.0 < p0[0] && p0[0] < 1.0 && 0.0 <= p0[1]) return 3;
    pt_param(p, t1, t2 - t1, n, p1);
    if (0.0 < p1[0] && p1[0] < 1.0 && 0.0 <= p1[1]) return 4;
    pt_param(p, t2, t0 - t2, n, p2);
    if (0.0 < p2[0] && p2[0] < 1.0 && 0.0 < p2[1]) return 5;
    if (p0[0] <= 0.0 && p2[0] >= 1.0) return 0;
    if (p1[0] <= 0.0 && p0[0] >= 1.0) return 1;
    if (p2[0] <= 0.0 && p1[0] >= 1.0) return 2;
    return 6;
}

// 0..8 as distance.py:1706-1754
FIPC_HD int ee_type(v3 a0, v3 a1, v3 b0, v3 b1) {
    const v3 u = a1 - a0, v = b1 - b0, w = a0 - b0;
    const double a = dot(u, u), b = dot(u, v), c = dot(v, v), d = dot(u, w), e = dot(v, w);
    const double D = a * c - b * b;
    double tD = D, tN = 0.0;
    const double sN = b * e - c * d;
    int cs = 8;
    if (sN <= 0.0) { tN = e; tD = c; cs = 2; }
    else if (sN >= D) { tN = e + b; tD = c; cs = 5; }
    else {
        tN = a * e - b * d;
        const v3 uv = cross(u, v);
        if (0.0 < tN && tN < tD && (dot(uv, w) == 0.0 || dot(uv, uv) < 1.0e-20 * a * c)) {
            if (sN < D / 2) { tN = e; tD = c; cs = 2; }
            else { tN = e + b; tD = c; cs = 5; }
        }
    }
    if (tN <= 0.0) {
        if (-d <= 0.0) cs = 0;
        else if (-d >= a) cs = 3;
        else cs = 6;
    } else if (tN >= tD) {
        if (-d + b <= 0.0) cs = 1;
        else if (-d + b >= a) cs = 4;
        else cs = 7;
    }
    return cs;
}

FIPC_HD double pt_dist2(v3 p, v3 t0, v3 t1, v3 t2) {
    switch (pt_type(p, t0, t1, t2)) {
        case 0: return d_PP(p, t0);
        case 1: return d_PP(p, t1);
        case 2: return d_PP(p, t2);
        case 3: return d_PE(p, t0, t1);
        case 4: return d_PE(p, t1, t2);
        case 5: return d_PE(p, t2, t0);
        default: return d_PT(p, t0, t1, t2);
    }
}
FIPC_HD double ee_dist2(v3 a0, v3 a1, v3 b0, v3 b1) {
    switch (ee_type(a0, a1, b0, b1)) {
        case 0: return d_PP(a0, b0);
        case 1: return d_PP(a0, b1);
        case 2: return d_PE(a0, b0, b1);
        case 3: return d_PP(a1, b0);
        case 4: return d_PP(a1, b1);
        case 5: return d_PE(a1, b0, b1);
        case 6: return d_PE(b0, a0, a1);
        case 7: return d_PE(b1, a0, a1);
        default: return d_EE(a0, a1, b0, b1);
    }
}

// ipc.py:332-336 (point vs triangle box, +-dHat)
FIPC_HD bool pt_aabb(v3 p, v3 t0, v3 t1, v3 t2, double dh) {
    const v3 mn = vmin(vmin(t0, t1), t2), mx = vmax(vmax(t0, t1), t2);
    return p.x < mx.x + dh && p.y < mx.y + dh && p.z < mx.z + dh && mn.x - dh < p.x && mn.y - dh < p.y && mn.z - dh < p.z;
}
// ipc.py:348-354
FIPC_HD bool ee_aabb(v3 a0, v3 a1, v3 b0, v3 b1, double dh) {
    const v3 mxa = vmax(a0, a1), mna = vmin(a0, a1), mxb = vmax(b0, b1), mnb = vmin(b0, b1);
    return mna.x < mxb.x + dh && mna.y < mxb.y + dh && mna.z < mxb.z + dh && mnb.x - dh < mxa.x && mnb.y - dh < mxa.y &&
           mnb.z - dh < mxa.z;
}
// ipc.py:339-345 (moving point vs moving triangle)
FIPC_HD bool pt_aabb_moving(v3 p, v3 t0, v3 t1, v3 t2, v3 dp, v3 dt0, v3 dt1, v3 dt2, double dh) {
    const v3 maxp = vmax(p, p + dp), minp = vmin(p, p + dp);
    const v3 maxt = vmax(vmax(t0, t0 + dt0), vmax(vmax(t1, t1 + dt1), vmax(t2, t2 + dt2)));
    const v3 mint = vmin(vmin(t0, t0 + dt0), vmin(vmin(t1, t1 + dt1), vmin(t2, t2 + dt2)));
    return minp.x < maxt.x + dh && minp.y < maxt.y + dh && minp.z < maxt.z + dh && mint.x - dh < maxp.x && mint.y - dh < maxp.y &&
           mint.z - dh < maxp.z;
}
// ipc.py:357-363
FIPC_HD bool ee_aabb_moving(v3 a0, v3 a1, v3 b0, v3 b1, v3 da0, v3 da1, v3 db0, v3 db1, double dh) {
    const v3 mxa = vmax(vmax(a0, a0 + da0), vmax(a1, a1 + da1)), mna = vmin(vmin(a0, a0 + da0), vmin(a1, a1 + da1));
    const v3 mxb = vmax(vmax(b0, b0 + db0), vmax(b1, b1 + db1)), mnb = vmin(vmin(b0, b0 + db0), vmin(b1, b1 + db1));
    return mna.x < mxb.x + dh && mna.y < mxb.y + dh && mna.z < mxb.z + dh && mnb.x - dh < mxa.x && mnb.y - dh < mxa.y &&
           mnb.z - dh < mxa.z;
}

// one-sided segment/triangle intersection (ipc.py:511-526)
FIPC_HD bool seg_tri(v3 P, v3 Q, v3 A, v3 B, v3 C) {
    const double RLen = sqrt(sq(Q - P));
    const v3 D = Q - P, R = mk(D.x / RLen, D.y / RLen, D.z / RLen);
    const v3 E1 = B - A, E2 = C - A, N = cross(E1, E2);
    const double det = -dot(R, N), invdet = 1.0 / det;
    const v3 AO = P - A, DAO = cross(AO, R);
    const double u = dot(E2, DAO) * invdet, v = -dot(E1, DAO) * invdet, t = dot(AO, N) * invdet;
    return det >= 1e-12 && t >= 0.0 && u >= 0.0 && v >= 0.0 && (u + v) <= 1.0 && t <= RLen;
}

}  // namespace fipc
