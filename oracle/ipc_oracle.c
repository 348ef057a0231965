/*
 * CPU oracle for the FastIPC Newton inner loop — TEST INFRASTRUCTURE, NOT PRODUCT.
 *
 * A plain-C restatement of the reference's per-element and per-constraint arithmetic, used
 * only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker.
 * Every function names the reference source it restates (paths relative to the FastIPC
 * checkout).  It is pinned against golden vectors produced by the reference's own code
 * (the .npz files under tests/golden, made by tests/golden/gen_golden.py).
 *
 * Methods are deliberately different from the GPU product so that agreement means something:
 *   - distances, barrier and mollifier derivatives: second-order forward-mode automatic
 *     differentiation ("jets") of the energy expressions (the reference uses generated
 *     closed forms, the GPU hand-derived reduced-coordinate forms);
 *   - PSD projection: cyclic Jacobi eigen-decomposition of the full n x n matrix (the
 *     reference uses Eigen's tridiagonal QR, the GPU a reduced 9x9 / 6x6 / 3x3 problem);
 *   - 3x3 SVD: Jacobi on F^T F;
 *   - CCD: the EVCTCD interval algorithm with real roots isolated by derivative bracketing
 *     and bisection (the reference uses Jenkins–Traub).
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXV 12

/* ------------------------------------------------------------------------------------------
 * second-order forward-mode AD over up to 12 variables
 * ---------------------------------------------------------------------------------------- */
typedef struct {
    double v;
    double g[MAXV];
    double h[MAXV * MAXV];
} jet;

static _Thread_local int JN = 12; /* active variable count (set per evaluation) */

static void j_const(jet* r, double c) { memset(r, 0, sizeof(jet)); r->v = c; }
static void j_var(jet* r, int i, double c) { j_const(r, c); r->g[i] = 1.0; }

static void j_add(jet* r, const jet* a, const jet* b) {
    r->v = a->v + b->v;
    for (int i = 0; i < JN; ++i) r->g[i] = a->g[i] + b->g[i];
    for (int i = 0; i < JN; ++i)
        for (int k = 0; k < JN; ++k) r->h[i * MAXV + k] = a->h[i * MAXV + k] + b->h[i * MAXV + k];
}
static void j_sub(jet* r, const jet* a, const jet* b) {
    r->v = a->v - b->v;
    for (int i = 0; i < JN; ++i) r->g[i] = a->g[i] - b->g[i];
    for (int i = 0; i < JN; ++i)
        for (int k = 0; k < JN; ++k) r->h[i * MAXV + k] = a->h[i * MAXV + k] - b->h[i * MAXV + k];
}
static void j_mul(jet* r, const jet* a, const jet* b) {
    jet t;
    t.v = a->v * b->v;
    for (int i = 0; i < JN; ++i) t.g[i] = a->v * b->g[i] + b->v * a->g[i];
    for (int i = 0; i < JN; ++i)
        for (int k = 0; k < JN; ++k)
            t.h[i * MAXV + k] = a->v * b->h[i * MAXV + k] + b->v * a->h[i * MAXV + k] + a->g[i] * b->g[k] + b->g[i] * a->g[k];
    *r = t;
}
/* r = f(a) given f, f', f'' at a->v (chain rule) */
static void j_fn(jet* r, const jet* a, double f, double f1, double f2) {
    jet t;
    t.v = f;
    for (int i = 0; i < JN; ++i) t.g[i] = f1 * a->g[i];
    for (int i = 0; i < JN; ++i)
        for (int k = 0; k < JN; ++k) t.h[i * MAXV + k] = f2 * a->g[i] * a->g[k] + f1 * a->h[i * MAXV + k];
    *r = t;
}
static void j_div(jet* r, const jet* a, const jet* b) {
    jet inv;
    double x = b->v;
    j_fn(&inv, b, 1.0 / x, -1.0 / (x * x), 2.0 / (x * x * x));
    j_mul(r, a, &inv);
}
typedef struct { jet c[3]; } jvec;
static void jv_sub(jvec* r, const jvec* a, const jvec* b) { for (int d = 0; d < 3; ++d) j_sub(&r->c[d], &a->c[d], &b->c[d]); }
static void jv_dot(jet* r, const jvec* a, const jvec* b) {
    jet t;
    j_mul(r, &a->c[0], &b->c[0]);
    j_mul(&t, &a->c[1], &b->c[1]); j_add(r, r, &t);
    j_mul(&t, &a->c[2], &b->c[2]); j_add(r, r, &t);
}
static void jv_cross(jvec* r, const jvec* a, const jvec* b) {
    jet t1, t2;
    jvec o;
    j_mul(&t1, &a->c[1], &b->c[2]); j_mul(&t2, &a->c[2], &b->c[1]); j_sub(&o.c[0], &t1, &t2);
    j_mul(&t1, &a->c[2], &b->c[0]); j_mul(&t2, &a->c[0], &b->c[2]); j_sub(&o.c[1], &t1, &t2);
    j_mul(&t1, &a->c[0], &b->c[1]); j_mul(&t2, &a->c[1], &b->c[0]); j_sub(&o.c[2], &t1, &t2);
    *r = o;
}
static void jv_load(jvec* r, const double* x, int vidx) {
    for (int d = 0; d < 3; ++d) j_var(&r->c[d], 3 * vidx + d, x[3 * vidx + d]);
}

/* squared distances, common/math/distance.py: PP_3D_E 955, PE_3D_E 684, PT_3D_E 976,
 * EE_3D_E 192, EECN2_E 1345; vertices are variable blocks ia, ib, ... */
static void j_PP(jet* r, const jvec* a, const jvec* b) { jvec d; jv_sub(&d, a, b); jv_dot(r, &d, &d); }
static void j_PE(jet* r, const jvec* p, const jvec* e0, const jvec* e1) {
    jvec u, w, c, e; jet n, dd;
    jv_sub(&u, e0, p); jv_sub(&w, e1, p); jv_cross(&c, &u, &w); jv_dot(&n, &c, &c);
    jv_sub(&e, e1, e0); jv_dot(&dd, &e, &e); j_div(r, &n, &dd);
}
static void j_PT(jet* r, const jvec* p, const jvec* t0, const jvec* t1, const jvec* t2) {
    jvec e1, e2, n, q; jet s, s2, nn;
    jv_sub(&e1, t1, t0); jv_sub(&e2, t2, t0); jv_cross(&n, &e1, &e2); jv_sub(&q, p, t0);
    jv_dot(&s, &q, &n); j_mul(&s2, &s, &s); jv_dot(&nn, &n, &n); j_div(r, &s2, &nn);
}
static void j_EE(jet* r, const jvec* a0, const jvec* a1, const jvec* b0, const jvec* b1) {
    jvec u, v, n, q; jet s, s2, nn;
    jv_sub(&u, a1, a0); jv_sub(&v, b1, b0); jv_cross(&n, &u, &v); jv_sub(&q, b0, a0);
    jv_dot(&s, &q, &n); j_mul(&s2, &s, &s); jv_dot(&nn, &n, &n); j_div(r, &s2, &nn);
}
static void j_EECN2(jet* r, const jvec* a0, const jvec* a1, const jvec* b0, const jvec* b1) {
    jvec u, v, n;
    jv_sub(&u, a1, a0); jv_sub(&v, b1, b0); jv_cross(&n, &u, &v); jv_dot(r, &n, &n);
}

/* barrier b(d) and derivatives, distance.py:22-44 (d is a squared distance) */
static double bar_E(double d, double dh2, double k) {
    return d < dh2 ? -k * (d - dh2) * (d - dh2) * log(d / dh2) : 0.0;
}
static double bar_g(double d, double dh2, double k) {
    double t2 = d - dh2;
    return d < dh2 ? k * (t2 * log(d / dh2) * -2.0 - (t2 * t2) / d) : 0.0;
}
static double bar_H(double d, double dh2, double k) {
    double t2 = d - dh2;
    return d < dh2 ? k * ((log(d / dh2) * -2.0 - t2 * 4.0 / d) + 1.0 / (d * d) * (t2 * t2)) : 0.0;
}

void oracle_barrier_scalar(int n, const double* d, double dh2, double k, double* E, double* g, double* H) {
    for (int i = 0; i < n; ++i) { E[i] = bar_E(d[i], dh2, k); g[i] = bar_g(d[i], dh2, k); H[i] = bar_H(d[i], dh2, k); }
}

/* ------------------------------------------------------------------------------------------
 * symmetric eigen-decomposition (cyclic Jacobi) and PSD projection
 * restates UTILS.h:8-25 makePD (Eigen SelfAdjointEigenSolver; eigenvalues ascending; if the
 * smallest is >= 0 the matrix is returned unchanged, otherwise leading negative eigenvalues
 * are set to zero and V diag V^T is rebuilt)
 * ---------------------------------------------------------------------------------------- */
static void jacobi_eig(int n, const double* Ain, double* w, double* V) {
    double A[MAXV * MAXV];
    memcpy(A, Ain, sizeof(double) * n * MAXV);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) V[i * MAXV + j] = (i == j);
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0, tot = 0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) { double a = A[i * MAXV + j] * A[i * MAXV + j]; tot += a; if (i != j) off += a; }
        if (off <= 1e-36 * tot || off == 0) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                double apq = A[p * MAXV + q];
                if (apq == 0) continue;
                double app = A[p * MAXV + p], aqq = A[q * MAXV + q];
                double theta = (aqq - app) / (2 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1));
                double c = 1 / sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < n; ++k) {
                    double akp = A[k * MAXV + p], akq = A[k * MAXV + q];
                    A[k * MAXV + p] = c * akp - s * akq;
                    A[k * MAXV + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    double apk = A[p * MAXV + k], aqk = A[q * MAXV + k];
                    A[p * MAXV + k] = c * apk - s * aqk;
                    A[q * MAXV + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    double vkp = V[k * MAXV + p], vkq = V[k * MAXV + q];
                    V[k * MAXV + p] = c * vkp - s * vkq;
                    V[k * MAXV + q] = s * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < n; ++i) w[i] = A[i * MAXV + i];
    /* sort ascending (selection) with eigenvector columns */
    for (int i = 0; i < n; ++i) {
        int m = i;
        for (int j = i + 1; j < n; ++j) if (w[j] < w[m]) m = j;
        if (m != i) {
            double t = w[i]; w[i] = w[m]; w[m] = t;
            for (int k = 0; k < n; ++k) { double tv = V[k * MAXV + i]; V[k * MAXV + i] = V[k * MAXV + m]; V[k * MAXV + m] = tv; }
        }
    }
}

/* in/out n x n row-major with row stride MAXV */
static void project_pd_inplace(int n, double* A) {
    double w[MAXV], V[MAXV * MAXV];
    jacobi_eig(n, A, w, V);
    if (w[0] >= 0) return;
    for (int i = 0; i < n; ++i) { if (w[i] < 0) w[i] = 0; else break; }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            double s = 0;
            for (int k = 0; k < n; ++k) s += V[i * MAXV + k] * w[k] * V[j * MAXV + k];
            A[i * MAXV + j] = s;
        }
}

/* batched projection, dense n x n row-major in and out (for unit tests) */
void oracle_project_pd(int count, int n, const double* in, double* out) {
    for (int c = 0; c < count; ++c) {
        double A[MAXV * MAXV];
        for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) A[i * MAXV + j] = in[(size_t)c * n * n + i * n + j];
        project_pd_inplace(n, A);
        for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) out[(size_t)c * n * n + i * n + j] = A[i * MAXV + j];
    }
}

/* ------------------------------------------------------------------------------------------
 * per-constraint barrier energy, gradient and projected Hessian
 * restates common/math/ipc.py:30-329 (PP/PE/PT/EE/EEM/PPM/PEM _energy and _g_and_H) with the
 * mollifier of distance.py:1625-1673
 * types: 0 PP(p0,p1) 6 dof; 1 PE(p,e0,e1) 9; 2 PT(p,t0,t1,t2) 12; 3 EE(a0,a1,b0,b1) 12;
 *        4 EEM, 5 PPM, 6 PEM (a0,a1,b0,b1 with rest positions X0) 12
 * ---------------------------------------------------------------------------------------- */
static const int TYPE_NV[7] = {2, 3, 4, 4, 4, 4, 4};

static double m_threshold(const double* a0, const double* a1, const double* b0, const double* b1) {
    double da = 0, db = 0;
    for (int d = 0; d < 3; ++d) { da += (a0[d] - a1[d]) * (a0[d] - a1[d]); db += (b0[d] - b1[d]) * (b0[d] - b1[d]); }
    return 1.0e-3 * da * db;
}

/* X: nv*3 positions of the row's vertices (in row order), X0 their rest positions.
 * energy only if want_derivs == 0.  Returns dof count. */
static int barrier_eval(int type, const double* X, const double* X0, double dh2, double kappa,
                        int want_derivs, double* E, double* g, double* H) {
    int nv = TYPE_NV[type];
    JN = want_derivs ? 3 * nv : 0;
    jvec P[4];
    for (int k = 0; k < nv; ++k) jv_load(&P[k], X, k);
    jet d;
    switch (type) {
        case 0: j_PP(&d, &P[0], &P[1]); break;
        case 1: j_PE(&d, &P[0], &P[1], &P[2]); break;
        case 2: j_PT(&d, &P[0], &P[1], &P[2], &P[3]); break;
        case 3: j_EE(&d, &P[0], &P[1], &P[2], &P[3]); break;
        case 4: j_EE(&d, &P[0], &P[1], &P[2], &P[3]); break;
        case 5: j_PP(&d, &P[0], &P[2]); break;
        default: j_PE(&d, &P[0], &P[2], &P[3]); break;
    }
    jet b;
    j_fn(&b, &d, bar_E(d.v, dh2, kappa), bar_g(d.v, dh2, kappa), bar_H(d.v, dh2, kappa));
    if (type >= 4) {
        double eps = m_threshold(X0, X0 + 3, X0 + 6, X0 + 9);
        jet c, m;
        j_EECN2(&c, &P[0], &P[1], &P[2], &P[3]);
        if (c.v < eps) {
            /* EEM_E/g/H, distance.py:1625-1639 */
            double q = c.v / eps;
            j_fn(&m, &c, (-q + 2.0) * q, 2.0 * (1.0 / eps) * (-(1.0 / eps) * c.v + 1.0), -2.0 / (eps * eps));
        } else {
            j_const(&m, 1.0);
        }
        j_mul(&b, &b, &m);
    }
    *E = b.v;
    if (!want_derivs) return 3 * nv;
    int n = 3 * nv;
    double A[MAXV * MAXV];
    for (int i = 0; i < n; ++i) {
        g[i] = b.g[i];
        for (int j = 0; j < n; ++j) A[i * MAXV + j] = b.h[i * MAXV + j];
    }
    project_pd_inplace(n, A);
    for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) H[i * n + j] = A[i * MAXV + j];
    return n;
}

/* batched: rows [count x 4] vertex ids (unused trailing ids ignored), x/x0 [V x 3].
 * g_out [count x 12], H_out [count x 144] (leading n entries / n x n block used), E_out [count] */
void oracle_barrier_rows(int type, int count, const int* rows, const double* x, const double* x0,
                         double dh2, double kappa, double* E_out, double* g_out, double* H_out) {
    int nv = TYPE_NV[type];
    #pragma omp parallel for schedule(dynamic, 64)
    for (int r = 0; r < count; ++r) {
        double X[12], X0[12];
        for (int k = 0; k < 4; ++k)
            for (int d = 0; d < 3; ++d) {
                int v = k < nv || type >= 4 ? rows[r * 4 + k] : rows[r * 4];
                X[3 * k + d] = x[3 * v + d];
                X0[3 * k + d] = x0 ? x0[3 * v + d] : 0.0;
            }
        double e;
        if (g_out) barrier_eval(type, X, X0, dh2, kappa, 1, &e, g_out + (size_t)r * 12, H_out + (size_t)r * 144);
        else barrier_eval(type, X, X0, dh2, kappa, 0, &e, 0, 0);
        E_out[r] = e;
    }
}

/* raw squared distance and its derivatives (unprojected), for pinning against distance.py */
void oracle_distance(int kind, int count, const double* pts, double* E, double* g, double* H) {
    /* kind: 0 PP, 1 PE, 2 PT, 3 EE, 4 EECN2 ; pts [count x 4 x 3] */
    static const int nvk[5] = {2, 3, 4, 4, 4};
    for (int c = 0; c < count; ++c) {
        int nv = nvk[kind];
        JN = 3 * nv;
        jvec P[4];
        for (int k = 0; k < nv; ++k) jv_load(&P[k], pts + (size_t)c * 12, k);
        jet d;
        if (kind == 0) j_PP(&d, &P[0], &P[1]);
        else if (kind == 1) j_PE(&d, &P[0], &P[1], &P[2]);
        else if (kind == 2) j_PT(&d, &P[0], &P[1], &P[2], &P[3]);
        else if (kind == 3) j_EE(&d, &P[0], &P[1], &P[2], &P[3]);
        else j_EECN2(&d, &P[0], &P[1], &P[2], &P[3]);
        int n = 3 * nv;
        E[c] = d.v;
        for (int i = 0; i < n; ++i) { g[(size_t)c * 12 + i] = d.g[i]; for (int j = 0; j < n; ++j) H[(size_t)c * 144 + i * n + j] = d.h[i * MAXV + j]; }
    }
}

/* mollifier M(x) with threshold eps (distance.py:1642-1668) */
void oracle_mollifier(int count, const double* pts, const double* eps, double* E, double* g, double* H) {
    for (int c = 0; c < count; ++c) {
        JN = 12;
        jvec P[4];
        for (int k = 0; k < 4; ++k) jv_load(&P[k], pts + (size_t)c * 12, k);
        jet cn, m;
        j_EECN2(&cn, &P[0], &P[1], &P[2], &P[3]);
        double e = eps[c];
        if (cn.v < e) { double q = cn.v / e; j_fn(&m, &cn, (-q + 2.0) * q, 2.0 * (1.0 / e) * (-(1.0 / e) * cn.v + 1.0), -2.0 / (e * e)); }
        else j_const(&m, 1.0);
        E[c] = m.v;
        for (int i = 0; i < 12; ++i) { g[(size_t)c * 12 + i] = m.g[i]; for (int j = 0; j < 12; ++j) H[(size_t)c * 144 + i * 12 + j] = m.h[i * MAXV + j]; }
    }
}

/* ------------------------------------------------------------------------------------------
 * feature classification, distance.py:1676-1823
 * ---------------------------------------------------------------------------------------- */
static double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static void sub3(double* r, const double* a, const double* b) { r[0] = a[0] - b[0]; r[1] = a[1] - b[1]; r[2] = a[2] - b[2]; }
static void cross3(double* r, const double* a, const double* b) {
    double t0 = a[1] * b[2] - a[2] * b[1], t1 = a[2] * b[0] - a[0] * b[2], t2 = a[0] * b[1] - a[1] * b[0];
    r[0] = t0; r[1] = t1; r[2] = t2;
}

/* projection parameters of p onto the edge (o -> o+e) and its in-plane normal direction
 * (basis rows e and e x n; (B B^T)^-1 B (p - o)), distance.py:1678-1680 */
static void pt_param(const double* p, const double* o, const double* e, const double* nrm, double* prm) {
    double b1[3], q[3];
    cross3(b1, e, nrm);
    sub3(q, p, o);
    double a00 = dot3(e, e), a01 = dot3(e, b1), a11 = dot3(b1, b1);
    double r0 = dot3(e, q), r1 = dot3(b1, q);
    double inv = 1.0 / (a00 * a11 - a01 * a01);
    prm[0] = inv * (a11 * r0 - a01 * r1);
    prm[1] = inv * (-a01 * r0 + a00 * r1);
}

int oracle_pt_type(const double* p, const double* t0, const double* t1, const double* t2) {
    double e0[3], e1[3], e2[3], n[3], tmp[3], p0[2], p1[2], p2[2];
    sub3(e0, t1, t0); sub3(tmp, t2, t0); cross3(n, e0, tmp);
    pt_param(p, t0, e0, n, p0);
    if (0.0 < p0[0] && p0[0] < 1.0 && 0.0 <= p0[1]) return 3;
    sub3(e1, t2, t1);
    pt_param(p, t1, e1, n, p1);
    if (0.0 < p1[0] && p1[0] < 1.0 && 0.0 <= p1[1]) return 4;
    sub3(e2, t0, t2);
    pt_param(p, t2, e2, n, p2);
    if (0.0 < p2[0] && p2[0] < 1.0 && 0.0 < p2[1]) return 5;
    if (p0[0] <= 0.0 && p2[0] >= 1.0) return 0;
    if (p1[0] <= 0.0 && p0[0] >= 1.0) return 1;
    if (p2[0] <= 0.0 && p1[0] >= 1.0) return 2;
    return 6;
}

int oracle_ee_type(const double* a0, const double* a1, const double* b0, const double* b1) {
    double u[3], v[3], w[3], uv[3];
    sub3(u, a1, a0); sub3(v, b1, b0); sub3(w, a0, b0);
    double a = dot3(u, u), b = dot3(u, v), c = dot3(v, v), d = dot3(u, w), e = dot3(v, w);
    double D = a * c - b * b, tD = D, sN = b * e - c * d, tN = 0.0;
    int cs = 8;
    if (sN <= 0.0) { tN = e; tD = c; cs = 2; }
    else if (sN >= D) { tN = e + b; tD = c; cs = 5; }
    else {
        tN = a * e - b * d;
        cross3(uv, u, v);
        if (0.0 < tN && tN < tD && (dot3(uv, w) == 0.0 || dot3(uv, uv) < 1.0e-20 * a * c)) {
            if (sN < D / 2) { tN = e; tD = c; cs = 2; }
            else { tN = e + b; tD = c; cs = 5; }
        }
    }
    if (tN <= 0.0) { if (-d <= 0.0) cs = 0; else if (-d >= a) cs = 3; else cs = 6; }
    else if (tN >= tD) { if (-d + b <= 0.0) cs = 1; else if (-d + b >= a) cs = 4; else cs = 7; }
    return cs;
}

int oracle_pe_type(const double* p, const double* e0, const double* e1) {
    double e[3], q[3];
    sub3(e, e1, e0); sub3(q, p, e0);
    double ratio = dot3(e, q) / dot3(e, e);
    return ratio < 0 ? 0 : (ratio > 1 ? 1 : 2);
}

static double d_PP(const double* a, const double* b) { double d[3]; sub3(d, a, b); return dot3(d, d); }
static double d_PE(const double* p, const double* e0, const double* e1) {
    double u[3], w[3], c[3], e[3];
    sub3(u, e0, p); sub3(w, e1, p); cross3(c, u, w); sub3(e, e1, e0);
    return dot3(c, c) / dot3(e, e);
}
static double d_PT(const double* p, const double* t0, const double* t1, const double* t2) {
    double e1[3], e2[3], n[3], q[3];
    sub3(e1, t1, t0); sub3(e2, t2, t0); cross3(n, e1, e2); sub3(q, p, t0);
    double s = dot3(q, n);
    return s * s / dot3(n, n);
}
static double d_EE(const double* a0, const double* a1, const double* b0, const double* b1) {
    double u[3], v[3], n[3], q[3];
    sub3(u, a1, a0); sub3(v, b1, b0); cross3(n, u, v); sub3(q, b0, a0);
    double s = dot3(q, n);
    return s * s / dot3(n, n);
}
static double d_EECN2(const double* a0, const double* a1, const double* b0, const double* b1) {
    double u[3], v[3], n[3];
    sub3(u, a1, a0); sub3(v, b1, b0); cross3(n, u, v);
    return dot3(n, n);
}

/* PT_dist2 / EE_dist2, distance.py:1771-1813 */
static double pt_dist2(const double* p, const double* t0, const double* t1, const double* t2) {
    switch (oracle_pt_type(p, t0, t1, t2)) {
        case 0: return d_PP(p, t0);
        case 1: return d_PP(p, t1);
        case 2: return d_PP(p, t2);
        case 3: return d_PE(p, t0, t1);
        case 4: return d_PE(p, t1, t2);
        case 5: return d_PE(p, t2, t0);
        default: return d_PT(p, t0, t1, t2);
    }
}
static double ee_dist2(const double* a0, const double* a1, const double* b0, const double* b1) {
    switch (oracle_ee_type(a0, a1, b0, b1)) {
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

void oracle_types(int count, const double* pts, int* pt, int* ee, int* pe) {
    for (int c = 0; c < count; ++c) {
        const double* q = pts + (size_t)c * 12;
        pt[c] = oracle_pt_type(q, q + 3, q + 6, q + 9);
        ee[c] = oracle_ee_type(q, q + 3, q + 6, q + 9);
        pe[c] = oracle_pe_type(q, q + 3, q + 6);
    }
}

/* ------------------------------------------------------------------------------------------
 * Neo-Hookean, common/physics/neo_hookean.py; 2x2 make_pd, common/math/math_tools.py:40-64
 * ---------------------------------------------------------------------------------------- */
static void make_pd2(double* M /* a b; c d row-major */) {
    double a = M[0], b = (M[1] + M[2]) / 2.0, d = M[3];
    double b2 = b * b, D = a * d - b2, T_div_2 = (a + d) / 2.0;
    double sq = sqrt(T_div_2 * T_div_2 - D);
    double L2 = T_div_2 - sq;
    if (L2 < 0.0) {
        double L1 = T_div_2 + sq;
        if (L1 <= 0.0) { M[0] = M[1] = M[2] = M[3] = 0.0; }
        else if (b2 == 0.0) { M[0] = L1; M[1] = M[2] = M[3] = 0.0; }
        else {
            double L1md = L1 - d, r = L1md / L1;
            M[0] = r * L1md; M[1] = b * r; M[2] = b * r; M[3] = b2 / L1;
        }
    }
}

void oracle_make_pd2(int count, const double* in, double* out) {
    for (int c = 0; c < count; ++c) { memcpy(out + 4 * c, in + 4 * c, 32); make_pd2(out + 4 * c); }
}

static double det3(const double* F) {
    return F[0] * (F[4] * F[8] - F[5] * F[7]) - F[1] * (F[3] * F[8] - F[5] * F[6]) + F[2] * (F[3] * F[7] - F[4] * F[6]);
}
static void inv3(const double* A, double* R) {
    double c00 = A[4] * A[8] - A[5] * A[7], c01 = A[5] * A[6] - A[3] * A[8], c02 = A[3] * A[7] - A[4] * A[6];
    double det = A[0] * c00 + A[1] * c01 + A[2] * c02, id = 1.0 / det;
    R[0] = c00 * id; R[1] = (A[2] * A[7] - A[1] * A[8]) * id; R[2] = (A[1] * A[5] - A[2] * A[4]) * id;
    R[3] = c01 * id; R[4] = (A[0] * A[8] - A[2] * A[6]) * id; R[5] = (A[2] * A[3] - A[0] * A[5]) * id;
    R[6] = c02 * id; R[7] = (A[1] * A[6] - A[0] * A[7]) * id; R[8] = (A[0] * A[4] - A[1] * A[3]) * id;
}

/* rotation-variant SVD F = U diag(s) V^T (det U = det V = 1) via Jacobi on F^T F */
void oracle_svd3(const double* F, double* U, double* s, double* V) {
    double A[MAXV * MAXV] = {0}, w[MAXV], Q[MAXV * MAXV];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) { double t = 0; for (int k = 0; k < 3; ++k) t += F[k * 3 + i] * F[k * 3 + j]; A[i * MAXV + j] = t; }
    jacobi_eig(3, A, w, Q);
    /* descending singular values */
    int ord[3] = {2, 1, 0};
    for (int c = 0; c < 3; ++c) for (int r = 0; r < 3; ++r) V[r * 3 + c] = Q[r * MAXV + ord[c]];
    double dv = det3(V);
    if (dv < 0) for (int r = 0; r < 3; ++r) V[r * 3 + 2] = -V[r * 3 + 2];
    double u0[3], u1[3], u2[3];
    for (int r = 0; r < 3; ++r) { u0[r] = F[r * 3 + 0] * V[0] + F[r * 3 + 1] * V[3] + F[r * 3 + 2] * V[6]; }
    for (int r = 0; r < 3; ++r) { u1[r] = F[r * 3 + 0] * V[1] + F[r * 3 + 1] * V[4] + F[r * 3 + 2] * V[7]; }
    double n0 = sqrt(dot3(u0, u0));
    for (int r = 0; r < 3; ++r) u0[r] /= n0;
    double pr = dot3(u0, u1);
    for (int r = 0; r < 3; ++r) u1[r] -= pr * u0[r];
    double n1 = sqrt(dot3(u1, u1));
    for (int r = 0; r < 3; ++r) u1[r] /= n1;
    cross3(u2, u0, u1);
    for (int r = 0; r < 3; ++r) { U[r * 3 + 0] = u0[r]; U[r * 3 + 1] = u1[r]; U[r * 3 + 2] = u2[r]; }
    /* s_i = u_i^T F v_i (the last one carries the sign of det F) */
    for (int c = 0; c < 3; ++c) {
        double t = 0;
        for (int r = 0; r < 3; ++r) for (int k = 0; k < 3; ++k) t += U[r * 3 + c] * F[r * 3 + k] * V[k * 3 + c];
        s[c] = t;
    }
}

/* neo_hookean.py:6-58 */
static double nh_psi(const double* s, double la, double mu) {
    double s2 = s[0] * s[0] + s[1] * s[1] + s[2] * s[2], lp = log(s[0] * s[1] * s[2]);
    return mu / 2.0 * (s2 - 3) - (mu - la / 2.0 * lp) * lp;
}
static void nh_grad(const double* s, double la, double mu, double* g) {
    double lp = log(s[0] * s[1] * s[2]);
    for (int i = 0; i < 3; ++i) { double inv = 1.0 / s[i]; g[i] = mu * (s[i] - inv) + la * inv * lp; }
}
static void nh_hess(const double* s, double la, double mu, double* H /*3x3 stride MAXV*/) {
    double lp = log(s[0] * s[1] * s[2]);
    for (int i = 0; i < 3; ++i) {
        double i2 = 1.0 / s[i] / s[i];
        H[i * MAXV + i] = mu * (1.0 + i2) - la * i2 * (lp - 1.0);
    }
    H[0 * MAXV + 1] = H[1 * MAXV + 0] = la / s[0] / s[1];
    H[1 * MAXV + 2] = H[2 * MAXV + 1] = la / s[1] / s[2];
    H[0 * MAXV + 2] = H[2 * MAXV + 0] = la / s[0] / s[2];
}

/* first Piola P(F) (neo_hookean.py:62-67); F, P row-major 3x3 */
static void nh_P(const double* F, double la, double mu, double* P) {
    double J = det3(F), lJ = log(J), scale = la * lJ - mu;
    double C[9] = {F[4] * F[8] - F[5] * F[7], F[5] * F[6] - F[3] * F[8], F[3] * F[7] - F[4] * F[6],
                   F[2] * F[7] - F[1] * F[8], F[0] * F[8] - F[2] * F[6], F[1] * F[6] - F[0] * F[7],
                   F[1] * F[5] - F[2] * F[4], F[2] * F[3] - F[0] * F[5], F[0] * F[4] - F[1] * F[3]};
    for (int i = 0; i < 9; ++i) P[i] = mu * F[i] + scale * (C[i] / J);
}

/* projected dP/dF (neo_hookean.py:71-131) as 9x9 with flat index ij = col*3 + row */
static void nh_dPdF(const double* F, double la, double mu, double* dP) {
    double U[9], s[3], V[9];
    oracle_svd3(F, U, s, V);
    double g[3], Hs[MAXV * MAXV] = {0};
    nh_grad(s, la, mu, g);
    nh_hess(s, la, mu, Hs);
    project_pd_inplace(3, Hs);
    double middle = mu - la * log(s[0] * s[1] * s[2]);
    double Bm[3][4];
    int pr[3][2] = {{0, 1}, {1, 2}, {2, 0}};
    for (int k = 0; k < 3; ++k) {
        int i = pr[k][0], j = pr[k][1];
        double left = (mu + middle / s[i] / s[j]) / 2.0;
        double right = g[i] + g[j];
        double ss = s[i] + s[j];
        if (ss < 0.000001) ss = 0.000001;
        right /= (2 * ss);
        double B[4] = {left + right, left - right, left - right, left + right};
        make_pd2(B);
        memcpy(Bm[k], B, sizeof(B));
    }
    /* M in the basis D_ab = u_a v_b^T, k = 3a + b */
    double M[81] = {0};
    int sc[3] = {0, 4, 8};
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) M[sc[i] * 9 + sc[j]] = Hs[i * MAXV + j];
    M[1 * 9 + 1] = Bm[0][0]; M[1 * 9 + 3] = Bm[0][1]; M[3 * 9 + 1] = Bm[0][2]; M[3 * 9 + 3] = Bm[0][3];
    M[5 * 9 + 5] = Bm[1][0]; M[5 * 9 + 7] = Bm[1][1]; M[7 * 9 + 5] = Bm[1][2]; M[7 * 9 + 7] = Bm[1][3];
    M[2 * 9 + 2] = Bm[2][3]; M[2 * 9 + 6] = Bm[2][2]; M[6 * 9 + 2] = Bm[2][1]; M[6 * 9 + 6] = Bm[2][0];
    /* basis vectors: d_k[col*3 + row] = U[row][a] V[col][b] */
    double Dk[9][9];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            for (int col = 0; col < 3; ++col)
                for (int row = 0; row < 3; ++row) Dk[3 * a + b][col * 3 + row] = U[row * 3 + a] * V[col * 3 + b];
    for (int x = 0; x < 9; ++x)
        for (int y = 0; y < 9; ++y) {
            double t = 0;
            for (int k = 0; k < 9; ++k)
                for (int l = 0; l < 9; ++l)
                    if (M[k * 9 + l] != 0.0) t += M[k * 9 + l] * Dk[k][x] * Dk[l][y];
            dP[x * 9 + y] = t;
        }
}

void oracle_nh_material(int count, const double* F, double la, double mu, double* psi, double* P, double* dPdF) {
    for (int c = 0; c < count; ++c) {
        const double* f = F + 9 * c;
        double U[9], s[3], V[9];
        oracle_svd3(f, U, s, V);
        psi[c] = nh_psi(s, la, mu);
        nh_P(f, la, mu, P + 9 * c);
        nh_dPdF(f, la, mu, dPdF + 81 * c);
    }
}

/* per-tet element: energy, gradient (12) and Hessian (144) of dt^2 * vol0 * psi(F), F = Ds Dm^-1;
 * restates NEWTON_IPC.py:568-691 (3D branch) and compute_energy :521-525.
 * Dm [T x 9] row-major rest shape matrices (columns x1-x0, x2-x0, x3-x0). */
void oracle_elasticity(int T, const int* tets, const double* x, const double* Dm, const double* la,
                       const double* mu, double dt, double* E_out, double* g_out, double* H_out) {
    #pragma omp parallel for schedule(static)
    for (int e = 0; e < T; ++e) {
        const int* t = tets + 4 * e;
        double Ds[9], IB[9], F[9];
        for (int i = 0; i < 3; ++i)
            for (int m = 0; m < 3; ++m) Ds[i * 3 + m] = x[3 * t[m + 1] + i] - x[3 * t[0] + i];
        inv3(Dm + 9 * e, IB);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) F[i * 3 + j] = Ds[i * 3 + 0] * IB[0 * 3 + j] + Ds[i * 3 + 1] * IB[1 * 3 + j] + Ds[i * 3 + 2] * IB[2 * 3 + j];
        double vol0 = det3(Dm + 9 * e) / 6.0, w = dt * dt * vol0;
        double U[9], s[3], V[9];
        oracle_svd3(F, U, s, V);
        E_out[e] = nh_psi(s, la[e], mu[e]) * w;
        if (!g_out) continue;
        double P[9], dP[81];
        nh_P(F, la[e], mu[e], P);
        nh_dPdF(F, la[e], mu[e], dP);
        /* B: d vec(F)[col*3+row] / d x_{v}[row]  = IB[v-1][col] (v >= 1), vertex 0: -sum */
        double Bm[9][12];
        memset(Bm, 0, sizeof(Bm));
        for (int col = 0; col < 3; ++col)
            for (int row = 0; row < 3; ++row) {
                double s0 = 0;
                for (int m = 0; m < 3; ++m) { Bm[col * 3 + row][(m + 1) * 3 + row] = IB[m * 3 + col]; s0 += IB[m * 3 + col]; }
                Bm[col * 3 + row][row] = -s0;
            }
        double vP[9];
        for (int col = 0; col < 3; ++col) for (int row = 0; row < 3; ++row) vP[col * 3 + row] = P[row * 3 + col];
        for (int a = 0; a < 12; ++a) {
            double t = 0;
            for (int k = 0; k < 9; ++k) t += Bm[k][a] * vP[k];
            g_out[(size_t)e * 12 + a] = t * w;
        }
        double BtD[12][9];
        for (int a = 0; a < 12; ++a)
            for (int l = 0; l < 9; ++l) { double t = 0; for (int k = 0; k < 9; ++k) t += Bm[k][a] * dP[k * 9 + l]; BtD[a][l] = t; }
        for (int a = 0; a < 12; ++a)
            for (int b = 0; b < 12; ++b) { double t = 0; for (int l = 0; l < 9; ++l) t += BtD[a][l] * Bm[l][b]; H_out[(size_t)e * 144 + a * 12 + b] = t * w; }
    }
}

/* ------------------------------------------------------------------------------------------
 * inversion-free step: math_tools.py:161-181 + wrapper.cpp:200-252 (Cardano, complex)
 * ---------------------------------------------------------------------------------------- */
static double quad_root(double a, double b, double c, double tol) {
    double t;
    if (fabs(a) <= tol) t = -c / b;
    else {
        double desc = b * b - 4 * a * c;
        if (desc > 0) { t = (-b - sqrt(desc)) / (2 * a); if (t < 0) t = (-b + sqrt(desc)) / (2 * a); }
        else t = -1;
    }
    return t;
}
static double cubic_root(double a, double b, double c, double d, double tol) {
    double t = -1;
    if (fabs(a) <= tol) return quad_root(b, c, d, tol);
    double complex d0 = b * b - 3 * a * c;
    double complex d1 = 2 * b * b * b - 9 * a * b * c + 27 * a * a * d;
    double complex C = cpow((d1 + csqrt(d1 * d1 - 4.0 * d0 * d0 * d0)) / 2.0, 1.0 / 3.0);
    if (cabs(C) == 0.0) C = cpow((d1 - csqrt(d1 * d1 - 4.0 * d0 * d0 * d0)) / 2.0, 1.0 / 3.0);
    double complex u2 = (-1.0 + sqrt(3.0) * I) / 2.0, u3 = (-1.0 - sqrt(3.0) * I) / 2.0;
    double complex t1 = (b + C + d0 / C) / (-3.0 * a);
    double complex t2 = (b + u2 * C + d0 / (u2 * C)) / (-3.0 * a);
    double complex t3 = (b + u3 * C + d0 / (u3 * C)) / (-3.0 * a);
    if (fabs(cimag(t1)) < tol && creal(t1) > 0) t = creal(t1);
    if (fabs(cimag(t2)) < tol && creal(t2) > 0 && (creal(t2) < t || t < 0)) t = creal(t2);
    if (fabs(cimag(t3)) < tol && creal(t3) > 0 && (creal(t3) < t || t < 0)) t = creal(t3);
    return t;
}
static double inversion_free_step(const double* xs, const double* ps, double eta) {
    double v1[3], v2[3], v3[3], p1[3], p2[3], p3[3];
    sub3(v1, xs + 3, xs); sub3(v2, xs + 6, xs); sub3(v3, xs + 9, xs);
    sub3(p1, ps + 3, ps); sub3(p2, ps + 6, ps); sub3(p3, ps + 9, ps);
    double pp[3], t1[3], t2[3], mix[3], vv[3];
    cross3(pp, p1, p2);
    cross3(t1, v1, p2); cross3(t2, p1, v2);
    for (int d = 0; d < 3; ++d) mix[d] = t1[d] + t2[d];
    cross3(vv, v1, v2);
    double a = dot3(p3, pp), b = dot3(v3, pp) + dot3(p3, mix), c = dot3(p3, vv) + dot3(v3, mix), d = dot3(v3, vv);
    double r = cubic_root(a, b, c, d, 1e-8);
    return r < 0.0 ? 1.0 : r * (1.0 - eta);
}
void oracle_inversion_free(int count, const double* xs, const double* ps, double eta, double* out) {
    for (int c = 0; c < count; ++c) out[c] = inversion_free_step(xs + 12 * c, ps + 12 * c, eta);
}

/* ------------------------------------------------------------------------------------------
 * CCD: EVCTCD (common/math/wrapper/EVCTCD/CTCD.cpp) + the wrapper's step clamp
 * (wrapper.cpp:254-328).  Real roots in [0, 1] by derivative bracketing + bisection.
 * ---------------------------------------------------------------------------------------- */
typedef struct { double l, u; } tivl;

static double horner(const double* op, int n, double t) { double f = op[0]; for (int i = 1; i <= n; ++i) { f *= t; f += op[i]; } return f; }

/* real roots of op (degree n, op[0] leading, nonzero) inside [0,1], ascending: the critical
 * points (roots of the derivative, recursively) split [0,1] into monotone pieces; a piece
 * with a strict sign change holds exactly one root, found by bisection to full precision */
static int roots01(const double* op, int n, double* out) {
    if (n == 1) { double r = -op[1] / op[0]; if (r >= 0 && r <= 1) { out[0] = r; return 1; } return 0; }
    double dp[7], crit[8], cr[6];
    for (int i = 0; i < n; ++i) dp[i] = op[i] * (n - i);
    int nc = 0, k = roots01(dp, n - 1, cr);
    crit[nc++] = 0.0;
    for (int i = 0; i < k; ++i) if (cr[i] > 0.0 && cr[i] < 1.0) crit[nc++] = cr[i];
    crit[nc++] = 1.0;
    int m = 0;
    for (int i = 0; i + 1 < nc; ++i) {
        double a = crit[i], b = crit[i + 1];
        double fa = horner(op, n, a), fb = horner(op, n, b);
        if (fa == 0.0) { if (m == 0 || out[m - 1] != a) out[m++] = a; continue; }
        if (fb == 0.0 || (fa < 0) == (fb < 0)) continue;
        for (int it = 0; it < 200; ++it) {
            double mid = 0.5 * (a + b);
            if (mid <= a || mid >= b) break;
            double fm = horner(op, n, mid);
            if (fm == 0.0) { a = b = mid; break; }
            if ((fm < 0) == (fa < 0)) { a = mid; fa = fm; } else b = mid;
        }
        out[m++] = 0.5 * (a + b);
    }
    if (horner(op, n, 1.0) == 0.0 && (m == 0 || out[m - 1] != 1.0)) out[m++] = 1.0;
    return m;
}

static void check_interval(double t1, double t2, const double* op, int deg, tivl* iv, int* niv, int pos) {
    t1 = t1 > 0.0 ? t1 : 0.0; t2 = t2 > 0.0 ? t2 : 0.0;
    t1 = t1 < 1.0 ? t1 : 1.0; t2 = t2 < 1.0 ? t2 : 1.0;
    double f = horner(op, deg, (t2 + t1) / 2);
    if ((pos && f >= 0) || (!pos && f <= 0)) { iv[*niv].l = t1; iv[*niv].u = t2; (*niv)++; }
}
static int could_have_roots(const double* op, int deg, int pos) {
    double r = 0;
    if ((pos && op[0] > 0) || (!pos && op[0] < 0)) r = op[0];
    for (int i = 1; i < deg; ++i) { r *= 1.0; if ((pos && op[i] > 0) || (!pos && op[i] < 0)) r += op[i]; }
    r *= 1.0; r += op[deg];
    return !((pos && r < 0) || (!pos && r > 0));
}
static int quad_roots(double a, double b, double c, double* t0, double* t1) {
    int sign = b < 0 ? -1 : 1;
    double D = b * b - 4 * a * c;
    if (D >= 0) {
        double q = -0.5 * (b + sign * sqrt(D));
        *t0 = q / a; *t1 = c / q;
        if (*t0 > *t1) { double t = *t0; *t0 = *t1; *t1 = t; }
        return 2;
    }
    return 0;
}
static void find_intervals(double* op, int n, tivl* iv, int* niv, int pos) {
    *niv = 0;
    double maxval = 0;
    for (int i = 0; i <= n; ++i) maxval = fmax(maxval, fabs(op[i]));
    if (maxval != 0) for (int i = 0; i <= n; ++i) op[i] /= maxval;
    int rd = n;
    for (int i = 0; i < n; ++i) { if (op[i] == 0) rd--; else break; }
    if (rd < n) for (int i = 0; i <= rd; ++i) op[i] = op[i + n - rd];
    double tm[8];
    int roots = 0;
    if (rd > 2) {
        if (!could_have_roots(op, rd, pos)) return;
        roots = roots01(op, rd, tm);
    } else if (rd == 2) {
        roots = quad_roots(op[0], op[1], op[2], &tm[0], &tm[1]);
    } else if (rd == 1) {
        tm[0] = -op[1] / op[0]; roots = 1;
    } else {
        if ((!pos && op[0] <= 0) || (pos && op[0] >= 0)) { iv[0].l = 0; iv[0].u = 1.0; *niv = 1; }
        return;
    }
    if (roots > 0) {
        for (int i = 1; i < roots; ++i) for (int j = i; j > 0 && tm[j] < tm[j - 1]; --j) { double t = tm[j]; tm[j] = tm[j - 1]; tm[j - 1] = t; }
        if (tm[0] >= 0) check_interval(0, tm[0], op, rd, iv, niv, pos);
        for (int i = 0; i < roots - 1; ++i)
            if (!((tm[i] < 0 && tm[i + 1] < 0) || (tm[i] > 1.0 && tm[i + 1] > 1.0))) check_interval(tm[i], tm[i + 1], op, rd, iv, niv, pos);
        if (tm[roots - 1] <= 1.0) check_interval(tm[roots - 1], 1.0, op, rd, iv, niv, pos);
    } else {
        check_interval(0.0, 1.0, op, rd, iv, niv, pos);
    }
}

static void bary_poly(const double* x10, const double* x20, const double* x30, const double* v10, const double* v20,
                      const double* v30, tivl* iv, int* niv) {
    double A = dot3(x10, x10), B = 2 * dot3(x10, v10), C = dot3(v10, v10);
    double D = dot3(x20, x10), E = dot3(x20, v10) + dot3(v20, x10), F = dot3(v20, v10);
    double G = dot3(x30, x20), H = dot3(x30, v20) + dot3(v30, x20), I_ = dot3(v30, v20);
    double J = dot3(x30, x10), K = dot3(x30, v10) + dot3(v30, x10), L = dot3(v30, v10);
    double op[5];
    op[0] = F * L - C * I_;
    op[1] = F * K + E * L - C * H - B * I_;
    op[2] = F * J + D * L + E * K - C * G - A * I_ - B * H;
    op[3] = D * K + E * J - A * H - B * G;
    op[4] = D * J - A * G;
    find_intervals(op, 4, iv, niv, 1);
}
static double triple(const double* a, const double* b, const double* c) { double t[3]; cross3(t, b, c); return dot3(a, t); }
static void plane_poly(const double* x10, const double* x20, const double* x30, const double* v10, const double* v20,
                       const double* v30, tivl* iv, int* niv) {
    double op[4];
    op[0] = triple(v10, v20, v30);
    op[1] = triple(x10, v20, v30) + triple(v10, x20, v30) + triple(v10, v20, x30);
    op[2] = triple(x10, x20, v30) + triple(x10, v20, x30) + triple(v10, x20, x30);
    op[3] = triple(x10, x20, x30);
    find_intervals(op, 3, iv, niv, 1);
}
static void distance_poly(const double* x10, const double* x20, const double* x30, const double* v10, const double* v20,
                          const double* v30, double minD2, tivl* iv, int* niv) {
    double A = triple(v10, v20, v30);
    double B = triple(x10, v20, v30) + triple(v10, x20, v30) + triple(v10, v20, x30);
    double C = triple(x10, x20, v30) + triple(x10, v20, x30) + triple(v10, x20, x30);
    double D = triple(x10, x20, x30);
    double E[3], F[3], G[3], t1[3], t2[3];
    cross3(E, x20, x30);
    cross3(t1, x20, v30); cross3(t2, v20, x30);
    for (int d = 0; d < 3; ++d) F[d] = t1[d] + t2[d];
    cross3(G, v20, v30);
    double op[7];
    op[0] = A * A;
    op[1] = 2 * A * B;
    op[2] = B * B + 2 * A * C - dot3(G, G) * minD2;
    op[3] = 2 * A * D + 2 * B * C - 2 * dot3(G, F) * minD2;
    op[4] = 2 * B * D + C * C - (2 * dot3(G, E) + dot3(F, F)) * minD2;
    op[5] = 2 * C * D - 2 * dot3(F, E) * minD2;
    op[6] = D * D - dot3(E, E) * minD2;
    find_intervals(op, 6, iv, niv, 0);
}
static int overlap_all(const tivl* v, int n) {
    for (int i = 0; i < n; ++i) for (int j = i + 1; j < n; ++j) if (v[i].l > v[j].u || v[j].l > v[i].u) return 0;
    return 1;
}
static tivl intersect_all(const tivl* v, int n) {
    tivl r = {0.0, 1.0};
    for (int i = 0; i < n; ++i) { r.l = fmax(v[i].l, r.l); r.u = fmin(v[i].u, r.u); }
    return r;
}

/* CTCD.cpp:383-472 */
static int vertex_face_ctcd(const double* q0s, const double* q1s, const double* q2s, const double* q3s,
                            const double* q0e, const double* q1e, const double* q2e, const double* q3e, double eta, double* t) {
    double minD = eta * eta;
    double v0[3], v1[3], v2[3], v3[3];
    sub3(v0, q0e, q0s); sub3(v1, q1e, q1s); sub3(v2, q2e, q2s); sub3(v3, q3e, q3s);
    tivl cp[8], e1[8], e2[8], e3[8];
    int ncp, ne1, ne2, ne3;
    double x10[3], v10[3], x20[3], v20[3], x30[3], v30[3], a[3], b[3];
    sub3(x10, q0s, q1s); sub3(v10, v0, v1);
    sub3(a, q3s, q1s); sub3(b, q2s, q1s); cross3(x20, a, b);
    sub3(a, v3, v1); sub3(b, v2, v1); cross3(v20, a, b);
    sub3(x30, q3s, q1s); sub3(v30, v3, v1);
    plane_poly(x10, x20, x30, v10, v20, v30, e1, &ne1);
    if (!ne1) return 0;
    sub3(x10, q0s, q2s); sub3(v10, v0, v2);
    sub3(a, q1s, q2s); sub3(b, q3s, q2s); cross3(x20, a, b);
    sub3(a, v1, v2); sub3(b, v3, v2); cross3(v20, a, b);
    sub3(x30, q1s, q2s); sub3(v30, v1, v2);
    plane_poly(x10, x20, x30, v10, v20, v30, e2, &ne2);
    if (!ne2) return 0;
    sub3(x10, q0s, q3s); sub3(v10, v0, v3);
    sub3(a, q2s, q3s); sub3(b, q1s, q3s); cross3(x20, a, b);
    sub3(a, v2, v3); sub3(b, v1, v3); cross3(v20, a, b);
    sub3(x30, q2s, q3s); sub3(v30, v2, v3);
    plane_poly(x10, x20, x30, v10, v20, v30, e3, &ne3);
    if (!ne3) return 0;
    sub3(x10, q0s, q1s); sub3(x20, q2s, q1s); sub3(x30, q3s, q1s);
    sub3(v10, v0, v1); sub3(v20, v2, v1); sub3(v30, v3, v1);
    distance_poly(x10, x20, x30, v10, v20, v30, minD, cp, &ncp);
    if (!ncp) return 0;
    int col = 0;
    double mint = 1.0;
    for (int i = 0; i < ncp; ++i) for (int j = 0; j < ne1; ++j) for (int k = 0; k < ne2; ++k) for (int l = 0; l < ne3; ++l) {
        tivl s[4] = {cp[i], e1[j], e2[k], e3[l]};
        if (overlap_all(s, 4)) { mint = fmin(intersect_all(s, 4).l, mint); col = 1; }
    }
    if (col) *t = mint;
    return col;
}

/* CTCD.cpp:245-381 */
static int edge_edge_ctcd(const double* q0s, const double* p0s, const double* q1s, const double* p1s,
                          const double* q0e, const double* p0e, const double* q1e, const double* p1e, double eta, double* t) {
    double minD = eta * eta;
    tivl raw[8], cp[8], par[8], a0[8], a1[8], b0[8], b1[8];
    int nraw, ncp = 0, npar = 0, na0, na1, nb0, nb1;
    double x10[3], x20[3], x30[3], vp0[3], vp1[3], vq0[3], vq1[3], v10[3], v20[3], v30[3];
    sub3(x10, p0s, p1s); sub3(x20, p0s, q0s); sub3(x30, p1s, q1s);
    sub3(vp0, p0e, p0s); sub3(vp1, p1e, p1s); sub3(vq0, q0e, q0s); sub3(vq1, q1e, q1s);
    sub3(v10, vp0, vp1); sub3(v20, vp0, vq0); sub3(v30, vp1, vq1);
    distance_poly(x10, x20, x30, v10, v20, v30, minD, raw, &nraw);
    for (int i = 0; i < nraw; ++i) {
        double midt = (raw[i].u + raw[i].l) / 2, c[3];
        for (int d = 0; d < 3; ++d) { x10[d] = (q0s[d] - p0s[d]) + midt * (vq0[d] - vp0[d]); x20[d] = (q1s[d] - p1s[d]) + midt * (vq1[d] - vp1[d]); }
        cross3(c, x10, x20);
        if (sqrt(dot3(c, c)) < 1e-8) par[npar++] = raw[i]; else cp[ncp++] = raw[i];
    }
    if (!ncp) return 0;
    sub3(x10, p1s, q1s); sub3(v10, vp1, vq1);
    sub3(x20, p0s, q0s); sub3(v20, vp0, vq0);
    sub3(x30, q0s, q1s); sub3(v30, vq0, vq1);
    bary_poly(x10, x20, x30, v10, v20, v30, a0, &na0);
    if (!na0) return 0;
    sub3(x20, q0s, p0s); sub3(v20, vq0, vp0);
    sub3(x30, p0s, q1s); sub3(v30, vp0, vq1);
    bary_poly(x10, x20, x30, v10, v20, v30, a1, &na1);
    if (!na1) return 0;
    sub3(x10, p0s, q0s); sub3(v10, vp0, vq0);
    sub3(x20, p1s, q1s); sub3(v20, vp1, vq1);
    sub3(x30, q1s, q0s); sub3(v30, vq1, vq0);
    bary_poly(x10, x20, x30, v10, v20, v30, b0, &nb0);
    if (!nb0) return 0;
    sub3(x20, q1s, p1s); sub3(v20, vq1, vp1);
    sub3(x30, p1s, q0s); sub3(v30, vp1, vq0);
    bary_poly(x10, x20, x30, v10, v20, v30, b1, &nb1);
    if (!nb1) return 0;
    int col = 0;
    double mint = 1.0;
    for (int i = 0; i < ncp; ++i) for (int j = 0; j < na0; ++j) for (int k = 0; k < na1; ++k)
        for (int l = 0; l < nb0; ++l) for (int m = 0; m < nb1; ++m) {
            tivl s[5] = {cp[i], a0[j], a1[k], b0[l], b1[m]};
            if (overlap_all(s, 5)) {
                tivl is = intersect_all(s, 5);
                int skip = 0;
                for (int p = 0; p < npar; ++p) { tivl pc[2] = {is, par[p]}; if (overlap_all(pc, 2)) { skip = 1; break; } }
                if (!skip) { mint = fmin(mint, is.l); col = 1; }
            }
        }
    if (col) *t = mint;
    return col;
}

/* wrapper.cpp:254-290 */
static double pt_ccd(const double* p, const double* t0, const double* t1, const double* t2, const double* dp, const double* dt0,
                     const double* dt1, const double* dt2, double eta, double dist2) {
    double toc = 1.0;
    double m = fmax(fmax(dot3(dt0, dt0), dot3(dt1, dt1)), dot3(dt2, dt2));
    double maxDisp = sqrt(dot3(dp, dp)) + sqrt(m);
    if (maxDisp != 0) {
        double lb = (1 - eta) * sqrt(dist2) / maxDisp;
        if (lb < 1) {
            double pe[3], a[3], b[3], c[3];
            for (int d = 0; d < 3; ++d) { pe[d] = p[d] + dp[d]; a[d] = t0[d] + dt0[d]; b[d] = t1[d] + dt1[d]; c[d] = t2[d] + dt2[d]; }
            if (vertex_face_ctcd(p, t0, t1, t2, pe, a, b, c, eta * sqrt(dist2), &toc)) { if (toc < lb) toc = lb; }
        }
    }
    return toc;
}
/* wrapper.cpp:292-328 */
static double ee_ccd(const double* a0, const double* a1, const double* b0, const double* b1, const double* da0, const double* da1,
                     const double* db0, const double* db1, double eta, double dist2) {
    double toc = 1.0;
    double maxDisp = sqrt(fmax(dot3(da0, da0), dot3(da1, da1))) + sqrt(fmax(dot3(db0, db0), dot3(db1, db1)));
    if (maxDisp != 0) {
        double lb = (1 - eta) * sqrt(dist2) / maxDisp;
        if (lb < 1) {
            double e0[3], e1[3], e2[3], e3[3];
            for (int d = 0; d < 3; ++d) { e0[d] = a0[d] + da0[d]; e1[d] = a1[d] + da1[d]; e2[d] = b0[d] + db0[d]; e3[d] = b1[d] + db1[d]; }
            if (edge_edge_ctcd(a0, a1, b0, b1, e0, e1, e2, e3, eta * sqrt(dist2), &toc)) { if (toc < lb) toc = lb; }
        }
    }
    return toc;
}

/* batched CCD on explicit primitives: x [count x 4 x 3], p [count x 4 x 3]; dist2 computed
 * from the current feature type as NEWTON_IPC.py:404 / :438 do */
void oracle_ccd(int kind, int count, const double* x, const double* p, double eta, double* toc) {
    for (int c = 0; c < count; ++c) {
        const double* q = x + 12 * c;
        const double* d = p + 12 * c;
        if (kind == 0) toc[c] = pt_ccd(q, q + 3, q + 6, q + 9, d, d + 3, d + 6, d + 9, eta, pt_dist2(q, q + 3, q + 6, q + 9));
        else toc[c] = ee_ccd(q, q + 3, q + 6, q + 9, d, d + 3, d + 6, d + 9, eta, ee_dist2(q, q + 3, q + 6, q + 9));
    }
}

/* ipc.py:511-526 */
static int seg_tri(const double* P, const double* Q, const double* A, const double* B, const double* C) {
    double R[3], E1[3], E2[3], N[3], AO[3], DAO[3];
    sub3(R, Q, P);
    double RLen = sqrt(dot3(R, R));
    for (int d = 0; d < 3; ++d) R[d] /= RLen;
    sub3(E1, B, A); sub3(E2, C, A); cross3(N, E1, E2);
    double det = -dot3(R, N), invdet = 1.0 / det;
    sub3(AO, P, A); cross3(DAO, AO, R);
    double u = dot3(E2, DAO) * invdet, v = -dot3(E1, DAO) * invdet, t = dot3(AO, N) * invdet;
    return det >= 1e-12 && t >= 0.0 && u >= 0.0 && v >= 0.0 && (u + v) <= 1.0 && t <= RLen;
}
void oracle_seg_tri(int count, const double* pts, int* hit) {
    for (int c = 0; c < count; ++c) { const double* q = pts + 15 * c; hit[c] = seg_tri(q, q + 3, q + 6, q + 9, q + 12); }
}

/* ------------------------------------------------------------------------------------------
 * uniform-grid broad phase with the reference's exact predicates
 * ---------------------------------------------------------------------------------------- */
typedef struct { uint64_t key; int id; } cellent;
static int cmp_cell(const void* a, const void* b) {
    const cellent* x = a; const cellent* y = b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return x->id - y->id;
}
static uint64_t cell_key(long i, long j, long k) {
    return ((uint64_t)(i + (1 << 20)) << 42) | ((uint64_t)(j + (1 << 20)) << 21) | (uint64_t)(k + (1 << 20));
}
typedef struct { cellent* e; long n, cap; } grid_t;
static void grid_add(grid_t* g, const double* lo, const double* hi, double inv_dx, int id) {
    long l[3], u[3];
    for (int d = 0; d < 3; ++d) { l[d] = (long)floor(lo[d] * inv_dx); u[d] = (long)floor(hi[d] * inv_dx); }
    for (long i = l[0]; i <= u[0]; ++i) for (long j = l[1]; j <= u[1]; ++j) for (long k = l[2]; k <= u[2]; ++k) {
        if (g->n == g->cap) { g->cap = g->cap ? 2 * g->cap : 1024; g->e = realloc(g->e, g->cap * sizeof(cellent)); }
        g->e[g->n].key = cell_key(i, j, k); g->e[g->n].id = id; g->n++;
    }
}
static long grid_lower(const grid_t* g, uint64_t key) {
    long lo = 0, hi = g->n;
    while (lo < hi) { long m = (lo + hi) / 2; if (g->e[m].key < key) lo = m + 1; else hi = m; }
    return lo;
}

typedef struct { int* r; long n, cap; int w; } rowbuf;
static void rb_push(rowbuf* b, int a0, int a1, int a2, int a3) {
    if (b->n == b->cap) { b->cap = b->cap ? 2 * b->cap : 256; b->r = realloc(b->r, b->cap * 4 * sizeof(int)); }
    int* q = b->r + 4 * b->n;
    q[0] = a0; q[1] = a1; q[2] = a2; q[3] = a3;
    b->n++;
}
static int g_w;
static int cmp_row(const void* a, const void* b) {
    const int* x = a; const int* y = b;
    for (int i = 0; i < g_w; ++i) if (x[i] != y[i]) return x[i] < y[i] ? -1 : 1;
    return 0;
}

/* NEWTON_IPC.py:181-212 */
static void attempt_pt(const double* x, double dh, double dh2, int p, int t0, int t1, int t2, rowbuf* rb) {
    if (p == t0 || p == t1 || p == t2) return;
    const double *P = x + 3 * p, *A = x + 3 * t0, *B = x + 3 * t1, *C = x + 3 * t2;
    for (int d = 0; d < 3; ++d) {
        double mn = fmin(fmin(A[d], B[d]), C[d]), mx = fmax(fmax(A[d], B[d]), C[d]);
        if (!(P[d] < mx + dh && mn - dh < P[d])) return;
    }
    switch (oracle_pt_type(P, A, B, C)) {
        case 0: if (d_PP(P, A) < dh2) rb_push(&rb[0], p, t0, 0, 0); break;
        case 1: if (d_PP(P, B) < dh2) rb_push(&rb[0], p, t1, 0, 0); break;
        case 2: if (d_PP(P, C) < dh2) rb_push(&rb[0], p, t2, 0, 0); break;
        case 3: if (d_PE(P, A, B) < dh2) rb_push(&rb[1], p, t0, t1, 0); break;
        case 4: if (d_PE(P, B, C) < dh2) rb_push(&rb[1], p, t1, t2, 0); break;
        case 5: if (d_PE(P, C, A) < dh2) rb_push(&rb[1], p, t2, t0, 0); break;
        default: if (d_PT(P, A, B, C) < dh2) rb_push(&rb[2], p, t0, t1, t2); break;
    }
}
/* NEWTON_IPC.py:235-312 ; list order PP PE PT EE EEM PPM PEM */
static void attempt_ee(const double* x, const double* x0, double dh, double dh2, int a0, int a1, int b0, int b1, rowbuf* rb) {
    if (a0 == b0 || a0 == b1 || a1 == b0 || a1 == b1) return;
    const double *A0 = x + 3 * a0, *A1 = x + 3 * a1, *B0 = x + 3 * b0, *B1 = x + 3 * b1;
    for (int d = 0; d < 3; ++d) {
        double mxa = fmax(A0[d], A1[d]), mna = fmin(A0[d], A1[d]), mxb = fmax(B0[d], B1[d]), mnb = fmin(B0[d], B1[d]);
        if (!(mna < mxb + dh && mnb - dh < mxa)) return;
    }
    double ecn = d_EECN2(A0, A1, B0, B1);
    double eps = m_threshold(x0 + 3 * a0, x0 + 3 * a1, x0 + 3 * b0, x0 + 3 * b1);
    int m = ecn < eps;
    switch (oracle_ee_type(A0, A1, B0, B1)) {
        case 0: if (d_PP(A0, B0) < dh2) { if (m) rb_push(&rb[5], a0, a1, b0, b1); else rb_push(&rb[0], a0, b0, 0, 0); } break;
        case 1: if (d_PP(A0, B1) < dh2) { if (m) rb_push(&rb[5], a0, a1, b1, b0); else rb_push(&rb[0], a0, b1, 0, 0); } break;
        case 2: if (d_PE(A0, B0, B1) < dh2) { if (m) rb_push(&rb[6], a0, a1, b0, b1); else rb_push(&rb[1], a0, b0, b1, 0); } break;
        case 3: if (d_PP(A1, B0) < dh2) { if (m) rb_push(&rb[5], a1, a0, b0, b1); else rb_push(&rb[0], a1, b0, 0, 0); } break;
        case 4: if (d_PP(A1, B1) < dh2) { if (m) rb_push(&rb[5], a1, a0, b1, b0); else rb_push(&rb[0], a1, b1, 0, 0); } break;
        case 5: if (d_PE(A1, B0, B1) < dh2) { if (m) rb_push(&rb[6], a1, a0, b0, b1); else rb_push(&rb[1], a1, b0, b1, 0); } break;
        case 6: if (d_PE(B0, A0, A1) < dh2) { if (m) rb_push(&rb[6], b0, b1, a0, a1); else rb_push(&rb[1], b0, a0, a1, 0); } break;
        case 7: if (d_PE(B1, A0, A1) < dh2) { if (m) rb_push(&rb[6], b1, b0, a0, a1); else rb_push(&rb[1], b1, a0, a1, 0); } break;
        default: if (d_EE(A0, A1, B0, B1) < dh2) { if (m) rb_push(&rb[4], a0, a1, b0, b1); else rb_push(&rb[3], a0, a1, b0, b1); } break;
    }
}

static const int ROW_W[7] = {2, 3, 4, 4, 4, 4, 4};
static rowbuf g_rows[7];

/* find_constraints (NEWTON_IPC.py:213-357): rows are sorted and deduplicated per list like
 * np.unique(axis=0).  Returns the counts in counts[7]; fetch rows with oracle_get_rows. */
void oracle_find_constraints(int nV, const double* x, const double* x0, int nbp, const int* bp, int nbe, const int* be,
                             int nbt, const int* bt, double dh2, double inv_dx, int* counts) {
    double dh = sqrt(dh2);
    for (int k = 0; k < 7; ++k) g_rows[k].n = 0;
    /* point-triangle: points hashed by [p - dh, p + dh], triangles query their bbox cells */
    grid_t g = {0};
    for (int i = 0; i < nbp; ++i) {
        const double* P = x + 3 * bp[i];
        double lo[3], hi[3];
        for (int d = 0; d < 3; ++d) { lo[d] = P[d] - dh; hi[d] = P[d] + dh; }
        grid_add(&g, lo, hi, inv_dx, i);
    }
    qsort(g.e, g.n, sizeof(cellent), cmp_cell);
    for (int i = 0; i < nbt; ++i) {
        int t0 = bt[3 * i], t1 = bt[3 * i + 1], t2 = bt[3 * i + 2];
        long l[3], u[3];
        for (int d = 0; d < 3; ++d) {
            double mn = fmin(fmin(x[3 * t0 + d], x[3 * t1 + d]), x[3 * t2 + d]);
            double mx = fmax(fmax(x[3 * t0 + d], x[3 * t1 + d]), x[3 * t2 + d]);
            l[d] = (long)floor(mn * inv_dx); u[d] = (long)floor(mx * inv_dx);
        }
        for (long a = l[0]; a <= u[0]; ++a) for (long b = l[1]; b <= u[1]; ++b) for (long c = l[2]; c <= u[2]; ++c) {
            uint64_t key = cell_key(a, b, c);
            for (long s = grid_lower(&g, key); s < g.n && g.e[s].key == key; ++s) attempt_pt(x, dh, dh2, bp[g.e[s].id], t0, t1, t2, g_rows);
        }
    }
    /* edge-edge: edges hashed by bbox, queried by bbox +- dh, pairs i < j */
    g.n = 0;
    for (int i = 0; i < nbe; ++i) {
        const double *A = x + 3 * be[2 * i], *B = x + 3 * be[2 * i + 1];
        double lo[3], hi[3];
        for (int d = 0; d < 3; ++d) { lo[d] = fmin(A[d], B[d]); hi[d] = fmax(A[d], B[d]); }
        grid_add(&g, lo, hi, inv_dx, i);
    }
    qsort(g.e, g.n, sizeof(cellent), cmp_cell);
    for (int i = 0; i < nbe; ++i) {
        int a0 = be[2 * i], a1 = be[2 * i + 1];
        long l[3], u[3];
        for (int d = 0; d < 3; ++d) {
            l[d] = (long)floor((fmin(x[3 * a0 + d], x[3 * a1 + d]) - dh) * inv_dx);
            u[d] = (long)floor((fmax(x[3 * a0 + d], x[3 * a1 + d]) + dh) * inv_dx);
        }
        for (long a = l[0]; a <= u[0]; ++a) for (long b = l[1]; b <= u[1]; ++b) for (long c = l[2]; c <= u[2]; ++c) {
            uint64_t key = cell_key(a, b, c);
            for (long s = grid_lower(&g, key); s < g.n && g.e[s].key == key; ++s) {
                int j = g.e[s].id;
                if (i < j) attempt_ee(x, x0, dh, dh2, a0, a1, be[2 * j], be[2 * j + 1], g_rows);
            }
        }
    }
    free(g.e);
    for (int k = 0; k < 7; ++k) {
        rowbuf* b = &g_rows[k];
        g_w = ROW_W[k];
        /* compact to width w for the lexicographic sort on the first w entries */
        if (b->n > 1) qsort(b->r, b->n, 4 * sizeof(int), cmp_row);
        long m = 0;
        for (long i = 0; i < b->n; ++i) {
            if (m > 0 && cmp_row(b->r + 4 * (m - 1), b->r + 4 * i) == 0) continue;
            memmove(b->r + 4 * m, b->r + 4 * i, 4 * sizeof(int));
            m++;
        }
        b->n = m;
        counts[k] = (int)m;
    }
}
void oracle_get_rows(int type, int* out) {
    rowbuf* b = &g_rows[type];
    for (long i = 0; i < b->n; ++i) for (int k = 0; k < 4; ++k) out[4 * i + k] = b->r[4 * i + k];
}

/* CCD step filter over all surface pairs (NEWTON_IPC.py:377-453, 456-468) */
double oracle_ccd_step(int nV, const double* x, const double* p, int nbp, const int* bp, int nbe, const int* be, int nbt,
                       const int* bt, int T, const int* tets, double dh2, double inv_dx, double eta, int with_inversion) {
    double dh = sqrt(dh2), alpha = 1.0;
    grid_t g = {0};
    for (int i = 0; i < nbp; ++i) {
        const double *P = x + 3 * bp[i], *D = p + 3 * bp[i];
        double lo[3], hi[3];
        for (int d = 0; d < 3; ++d) { lo[d] = fmin(P[d], P[d] + D[d]) - dh; hi[d] = fmax(P[d], P[d] + D[d]) + dh; }
        grid_add(&g, lo, hi, inv_dx, i);
    }
    qsort(g.e, g.n, sizeof(cellent), cmp_cell);
    for (int i = 0; i < nbt; ++i) {
        int t[3] = {bt[3 * i], bt[3 * i + 1], bt[3 * i + 2]};
        long l[3], u[3];
        for (int d = 0; d < 3; ++d) {
            double mn = 1e300, mx = -1e300;
            for (int k = 0; k < 3; ++k) { double a = x[3 * t[k] + d], b = a + p[3 * t[k] + d]; mn = fmin(mn, fmin(a, b)); mx = fmax(mx, fmax(a, b)); }
            l[d] = (long)floor(mn * inv_dx); u[d] = (long)floor(mx * inv_dx);
        }
        for (long a = l[0]; a <= u[0]; ++a) for (long b = l[1]; b <= u[1]; ++b) for (long c = l[2]; c <= u[2]; ++c) {
            uint64_t key = cell_key(a, b, c);
            for (long s = grid_lower(&g, key); s < g.n && g.e[s].key == key; ++s) {
                int pp = bp[g.e[s].id];
                if (pp == t[0] || pp == t[1] || pp == t[2]) continue;
                double q[12], dq[12];
                int vs[4] = {pp, t[0], t[1], t[2]};
                for (int k = 0; k < 4; ++k) for (int d = 0; d < 3; ++d) { q[3 * k + d] = x[3 * vs[k] + d]; dq[3 * k + d] = p[3 * vs[k] + d]; }
                int ok = 1;
                for (int d = 0; d < 3 && ok; ++d) {
                    double maxp = fmax(q[d], q[d] + dq[d]), minp = fmin(q[d], q[d] + dq[d]);
                    double maxt = -1e300, mint = 1e300;
                    for (int k = 1; k < 4; ++k) { maxt = fmax(maxt, fmax(q[3 * k + d], q[3 * k + d] + dq[3 * k + d])); mint = fmin(mint, fmin(q[3 * k + d], q[3 * k + d] + dq[3 * k + d])); }
                    ok = minp < maxt + dh && mint - dh < maxp;
                }
                if (!ok) continue;
                double toc;
                oracle_ccd(0, 1, q, dq, eta, &toc);
                alpha = fmin(alpha, toc);
            }
        }
    }
    g.n = 0;
    for (int i = 0; i < nbe; ++i) {
        int e[2] = {be[2 * i], be[2 * i + 1]};
        double lo[3], hi[3];
        for (int d = 0; d < 3; ++d) {
            lo[d] = 1e300; hi[d] = -1e300;
            for (int k = 0; k < 2; ++k) { double a = x[3 * e[k] + d], b = a + p[3 * e[k] + d]; lo[d] = fmin(lo[d], fmin(a, b)); hi[d] = fmax(hi[d], fmax(a, b)); }
        }
        grid_add(&g, lo, hi, inv_dx, i);
    }
    qsort(g.e, g.n, sizeof(cellent), cmp_cell);
    for (int i = 0; i < nbe; ++i) {
        int e[2] = {be[2 * i], be[2 * i + 1]};
        long l[3], u[3];
        for (int d = 0; d < 3; ++d) {
            double mn = 1e300, mx = -1e300;
            for (int k = 0; k < 2; ++k) { double a = x[3 * e[k] + d], b = a + p[3 * e[k] + d]; mn = fmin(mn, fmin(a, b)); mx = fmax(mx, fmax(a, b)); }
            l[d] = (long)floor((mn - dh) * inv_dx); u[d] = (long)floor((mx + dh) * inv_dx);
        }
        for (long a = l[0]; a <= u[0]; ++a) for (long b = l[1]; b <= u[1]; ++b) for (long c = l[2]; c <= u[2]; ++c) {
            uint64_t key = cell_key(a, b, c);
            for (long s = grid_lower(&g, key); s < g.n && g.e[s].key == key; ++s) {
                int j = g.e[s].id;
                int b0 = be[2 * j], b1 = be[2 * j + 1];
                if (!(i < j && e[0] != b0 && e[0] != b1 && e[1] != b0 && e[1] != b1)) continue;
                double q[12], dq[12];
                int vs[4] = {e[0], e[1], b0, b1};
                for (int k = 0; k < 4; ++k) for (int d = 0; d < 3; ++d) { q[3 * k + d] = x[3 * vs[k] + d]; dq[3 * k + d] = p[3 * vs[k] + d]; }
                int ok = 1;
                for (int d = 0; d < 3 && ok; ++d) {
                    double mxa = fmax(fmax(q[d], q[d] + dq[d]), fmax(q[3 + d], q[3 + d] + dq[3 + d]));
                    double mna = fmin(fmin(q[d], q[d] + dq[d]), fmin(q[3 + d], q[3 + d] + dq[3 + d]));
                    double mxb = fmax(fmax(q[6 + d], q[6 + d] + dq[6 + d]), fmax(q[9 + d], q[9 + d] + dq[9 + d]));
                    double mnb = fmin(fmin(q[6 + d], q[6 + d] + dq[6 + d]), fmin(q[9 + d], q[9 + d] + dq[9 + d]));
                    ok = mna < mxb + dh && mnb - dh < mxa;
                }
                if (!ok) continue;
                double toc;
                oracle_ccd(1, 1, q, dq, eta, &toc);
                alpha = fmin(alpha, toc);
            }
        }
    }
    free(g.e);
    if (with_inversion) {
        for (int e = 0; e < T; ++e) {
            double xs[12], ps[12];
            for (int k = 0; k < 4; ++k) for (int d = 0; d < 3; ++d) { xs[3 * k + d] = x[3 * tets[4 * e + k] + d]; ps[3 * k + d] = p[3 * tets[4 * e + k] + d]; }
            alpha = fmin(alpha, inversion_free_step(xs, ps, eta));
        }
    }
    return alpha;
}

/* check_collision_3d (NEWTON_IPC.py:855-880) */
int oracle_check_collision(const double* x, int nbe, const int* be, int nbt, const int* bt, double dh2, double inv_dx) {
    double dh = sqrt(dh2);
    grid_t g = {0};
    for (int i = 0; i < nbe; ++i) {
        const double *A = x + 3 * be[2 * i], *B = x + 3 * be[2 * i + 1];
        double lo[3], hi[3];
        for (int d = 0; d < 3; ++d) { lo[d] = fmin(A[d], B[d]) - dh; hi[d] = fmax(A[d], B[d]) + dh; }
        grid_add(&g, lo, hi, inv_dx, i);
    }
    qsort(g.e, g.n, sizeof(cellent), cmp_cell);
    int res = 0;
    for (int i = 0; i < nbt && !res; ++i) {
        int t0 = bt[3 * i], t1 = bt[3 * i + 1], t2 = bt[3 * i + 2];
        long l[3], u[3];
        for (int d = 0; d < 3; ++d) {
            double mn = fmin(fmin(x[3 * t0 + d], x[3 * t1 + d]), x[3 * t2 + d]);
            double mx = fmax(fmax(x[3 * t0 + d], x[3 * t1 + d]), x[3 * t2 + d]);
            l[d] = (long)floor(mn * inv_dx); u[d] = (long)floor(mx * inv_dx);
        }
        for (long a = l[0]; a <= u[0] && !res; ++a) for (long b = l[1]; b <= u[1] && !res; ++b) for (long c = l[2]; c <= u[2] && !res; ++c) {
            uint64_t key = cell_key(a, b, c);
            for (long s = grid_lower(&g, key); s < g.n && g.e[s].key == key; ++s) {
                int j = g.e[s].id, a0 = be[2 * j], a1 = be[2 * j + 1];
                if (a0 != t0 && a0 != t1 && a0 != t2 && a1 != t0 && a1 != t1 && a1 != t2)
                    if (seg_tri(x + 3 * a0, x + 3 * a1, x + 3 * t0, x + 3 * t1, x + 3 * t2)) { res = 1; break; }
            }
        }
    }
    free(g.e);
    return res;
}

/* ------------------------------------------------------------------------------------------
 * energy and system assembly (NEWTON_IPC.py:514-555, 558-567, 736-747)
 * ---------------------------------------------------------------------------------------- */
/* total incremental potential: inertia + elasticity + barrier over the given rows */
double oracle_energy(int nV, const double* x, const double* xt, const double* m, int T, const int* tets, const double* Dm,
                     const double* la, const double* mu, double dt, const double* x0, const int* counts,
                     const int* rows_all, double dh2, double kappa) {
    /* rows_all: the 7 lists back to back ([counts[k] x 4] each, list order PP..PEM) */
    double e = 0;
    for (int i = 0; i < nV; ++i) {
        double s = 0;
        for (int d = 0; d < 3; ++d) s += (x[3 * i + d] - xt[3 * i + d]) * (x[3 * i + d] - xt[3 * i + d]);
        e += 0.5 * m[i] * s;
    }
    double* Ee = malloc(sizeof(double) * (T > 0 ? T : 1));
    oracle_elasticity(T, tets, x, Dm, la, mu, dt, Ee, 0, 0);
    for (int i = 0; i < T; ++i) e += Ee[i];
    free(Ee);
    long off = 0;
    for (int k = 0; k < 7; ++k) {
        const int* rows = rows_all + 4 * off;
        off += counts[k];
        if (!counts[k]) continue;
        double* Eb = malloc(sizeof(double) * counts[k]);
        oracle_barrier_rows(k, counts[k], rows, x, x0, dh2, kappa, Eb, 0, 0);
        for (int i = 0; i < counts[k]; ++i) e += Eb[i];
        free(Eb);
    }
    return e;
}

/* block-Jacobi preconditioned CG on a CSR matrix with Dirichlet rows/cols projected out
 * (the CPU stand-in for the direct solve at sizes where a factorisation is impractical) */
int oracle_pcg(int n, const long* indptr, const int* indices, const double* data, const double* b, const unsigned char* fixed,
               double rtol, int maxit, double* x) {
    double *r = calloc(n, 8), *z = calloc(n, 8), *p = calloc(n, 8), *Ap = calloc(n, 8), *Minv = calloc((size_t)n / 3 * 9, 8);
    for (int i = 0; i < n / 3; ++i) {
        double B[9] = {0};
        for (int a = 0; a < 3; ++a) {
            int row = 3 * i + a;
            for (long k = indptr[row]; k < indptr[row + 1]; ++k) { int c = indices[k]; if (c / 3 == i) B[a * 3 + c % 3] = data[k]; }
        }
        if (fixed[i]) { memset(B, 0, sizeof(B)); B[0] = B[4] = B[8] = 1; }
        inv3(B, Minv + 9 * i);
    }
    for (int i = 0; i < n; ++i) { x[i] = 0; r[i] = fixed[i / 3] ? 0 : b[i]; }
    double rz = 0, r0 = 0;
    for (int i = 0; i < n / 3; ++i) for (int a = 0; a < 3; ++a) {
        double s = 0; for (int c = 0; c < 3; ++c) s += Minv[9 * i + 3 * a + c] * r[3 * i + c];
        z[3 * i + a] = s;
    }
    for (int i = 0; i < n; ++i) { p[i] = z[i]; rz += r[i] * z[i]; r0 += r[i] * r[i]; }
    r0 = sqrt(r0);
    int it;
    for (it = 0; it < maxit; ++it) {
        double rn = 0;
        for (int i = 0; i < n; ++i) rn += r[i] * r[i];
        if (sqrt(rn) <= rtol * r0 || r0 == 0) break;
        #pragma omp parallel for schedule(static)
        for (int row = 0; row < n; ++row) {
            double s = 0;
            if (!fixed[row / 3]) for (long k = indptr[row]; k < indptr[row + 1]; ++k) { int c = indices[k]; if (!fixed[c / 3]) s += data[k] * p[c]; }
            Ap[row] = s;
        }
        double pAp = 0;
        for (int i = 0; i < n; ++i) pAp += p[i] * Ap[i];
        double alpha = rz / pAp;
        for (int i = 0; i < n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * Ap[i]; }
        for (int i = 0; i < n / 3; ++i) for (int a = 0; a < 3; ++a) {
            double s = 0; for (int c = 0; c < 3; ++c) s += Minv[9 * i + 3 * a + c] * r[3 * i + c];
            z[3 * i + a] = fixed[i] ? 0 : s;
        }
        double rz2 = 0;
        for (int i = 0; i < n; ++i) rz2 += r[i] * z[i];
        double beta = rz2 / rz;
        rz = rz2;
        for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    }
    free(r); free(z); free(p); free(Ap); free(Minv);
    return it;
}

int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------------------------
 * block-sparse (3x3) assembly and PCG for large scenes (the timed CPU baseline)
 * ---------------------------------------------------------------------------------------- */
/* val[pos16[e*16 + a*4 + b]] += block (a, b) of the element Hessian H[e] (12x12 row-major) */
void oracle_bsr_accumulate(int T, const long long* pos16, const double* H, double* val) {
    for (int e = 0; e < T; ++e)
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) {
                double* dst = val + 9 * pos16[16 * (long long)e + a * 4 + b];
                const double* src = H + 144 * (long long)e;
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) dst[i * 3 + j] += src[(3 * a + i) * 12 + 3 * b + j];
            }
}

/* y = A p over the rows of a 3x3 block-sparse matrix (rows of fixed vertices are zero) */
static void bsr_spmv(int nV, const long long* rp, const int* ci, const double* va, const unsigned char* fixed, const double* p,
                     double* y, int accumulate) {
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < nV; ++i) {
        double s0 = 0, s1 = 0, s2 = 0;
        if (!fixed[i])
            for (long long k = rp[i]; k < rp[i + 1]; ++k) {
                const int j = ci[k];
                if (fixed[j]) continue;
                const double* B = va + 9 * k;
                s0 += B[0] * p[3 * j] + B[1] * p[3 * j + 1] + B[2] * p[3 * j + 2];
                s1 += B[3] * p[3 * j] + B[4] * p[3 * j + 1] + B[5] * p[3 * j + 2];
                s2 += B[6] * p[3 * j] + B[7] * p[3 * j + 1] + B[8] * p[3 * j + 2];
            }
        if (accumulate) { y[3 * i] += s0; y[3 * i + 1] += s1; y[3 * i + 2] += s2; }
        else { y[3 * i] = s0; y[3 * i + 1] = s1; y[3 * i + 2] = s2; }
    }
}

static double pdot(long long n, const double* a, const double* b) {
    double s = 0;
    #pragma omp parallel for reduction(+ : s) schedule(static)
    for (long long i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

int oracle_bsr_pcg_guess(int nV, const long long* rp, const int* ci, const double* va, const long long* crp, const int* cci,
                         const double* cva, const long long* diag_pos, const double* b, const unsigned char* fixed, double rtol,
                         int maxit, int use_guess, double* x);

/* block-Jacobi PCG on elastic (rp, ci, va) + contact (crp, cci, cva) block-sparse matrices;
 * diag_pos: position of each diagonal block in the elastic matrix.  Returns iterations. */
int oracle_bsr_pcg(int nV, const long long* rp, const int* ci, const double* va, const long long* crp, const int* cci,
                   const double* cva, const long long* diag_pos, const double* b, const unsigned char* fixed, double rtol, int maxit,
                   double* x) {
    return oracle_bsr_pcg_guess(nV, rp, ci, va, crp, cci, cva, diag_pos, b, fixed, rtol, maxit, 0, x);
}

/* as oracle_bsr_pcg, starting from x when use_guess != 0; the tolerance is relative to |b| */
int oracle_bsr_pcg_guess(int nV, const long long* rp, const int* ci, const double* va, const long long* crp, const int* cci,
                         const double* cva, const long long* diag_pos, const double* b, const unsigned char* fixed, double rtol,
                         int maxit, int use_guess, double* x) {
    const long long n = 3ll * nV;
    double *r = malloc(8 * n), *z = malloc(8 * n), *p = malloc(8 * n), *Ap = malloc(8 * n), *Mi = malloc(72 * (long long)nV);
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < nV; ++i) {
        double B[9];
        if (fixed[i]) { for (int k = 0; k < 9; ++k) B[k] = (k % 4 == 0); }
        else {
            for (int k = 0; k < 9; ++k) B[k] = va[9 * diag_pos[i] + k];
            for (long long k = crp[i]; k < crp[i + 1]; ++k)
                if (cci[k] == i) for (int q = 0; q < 9; ++q) B[q] += cva[9 * k + q];
        }
        inv3(B, Mi + 9 * i);
    }
    double bb = 0;
    for (int i = 0; i < nV; ++i)
        for (int d = 0; d < 3; ++d) if (!fixed[i]) bb += b[3 * i + d] * b[3 * i + d];
    if (!use_guess)
        for (long long i = 0; i < n; ++i) x[i] = 0.0;
    for (int i = 0; i < nV; ++i) if (fixed[i]) x[3 * i] = x[3 * i + 1] = x[3 * i + 2] = 0;
    bsr_spmv(nV, rp, ci, va, fixed, x, Ap, 0);
    bsr_spmv(nV, crp, cci, cva, fixed, x, Ap, 1);
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < nV; ++i)
        for (int d = 0; d < 3; ++d) r[3 * i + d] = fixed[i] ? 0 : b[3 * i + d] - Ap[3 * i + d];
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < nV; ++i)
        for (int d = 0; d < 3; ++d) {
            z[3 * i + d] = Mi[9 * i + 3 * d] * r[3 * i] + Mi[9 * i + 3 * d + 1] * r[3 * i + 1] + Mi[9 * i + 3 * d + 2] * r[3 * i + 2];
            p[3 * i + d] = z[3 * i + d];
        }
    double rz = pdot(n, r, z), rr0 = bb;
    int it = 0;
    for (; it < maxit; ++it) {
        const double rr = pdot(n, r, r);
        if (rr <= rtol * rtol * rr0 || rr0 == 0) break;
        bsr_spmv(nV, rp, ci, va, fixed, p, Ap, 0);
        bsr_spmv(nV, crp, cci, cva, fixed, p, Ap, 1);
        const double alpha = rz / pdot(n, p, Ap);
        #pragma omp parallel for schedule(static)
        for (long long i = 0; i < n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * Ap[i]; }
        #pragma omp parallel for schedule(static)
        for (int i = 0; i < nV; ++i)
            for (int d = 0; d < 3; ++d)
                z[3 * i + d] = Mi[9 * i + 3 * d] * r[3 * i] + Mi[9 * i + 3 * d + 1] * r[3 * i + 1] + Mi[9 * i + 3 * d + 2] * r[3 * i + 2];
        const double rz2 = pdot(n, r, z), beta = rz2 / rz;
        rz = rz2;
        #pragma omp parallel for schedule(static)
        for (long long i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    }
    free(r); free(z); free(p); free(Ap); free(Mi);
    return it;
}

/* ------------------------------------------------------------------------------------------
 * 2D path (NEWTON_IPC.py with dim == 2), for the 2D oracle's fast mode and the CPU baseline.
 * Methods differ from the GPU's: the 2x2 SVD comes from a Jacobi rotation of F^T F (the GPU
 * uses the closed form of a scaled rotation plus reflection); the element Hessian is the
 * reference's dP/dF mapped through the 4 x 6 derivative of F, as in the numpy oracle.
 * ---------------------------------------------------------------------------------------- */

/* F (row-major) = U diag(s) V^T with U, V rotations, s0 >= |s1|, s1 < 0 iff det F < 0 */
static void svd2_jacobi(const double* F, double* U, double* s, double* V) {
    const double a = F[0] * F[0] + F[2] * F[2], b = F[0] * F[1] + F[2] * F[3], d = F[1] * F[1] + F[3] * F[3];
    const double th = 0.5 * atan2(2.0 * b, a - d);   /* rotation that diagonalises F^T F, larger first */
    const double c = cos(th), sn = sin(th);
    V[0] = c; V[1] = -sn; V[2] = sn; V[3] = c;       /* columns v0 = (c, sn), v1 = (-sn, c) */
    const double f0x = F[0] * c + F[1] * sn, f0y = F[2] * c + F[3] * sn;          /* F v0 */
    const double f1x = -F[0] * sn + F[1] * c, f1y = -F[2] * sn + F[3] * c;        /* F v1 */
    double s0 = sqrt(f0x * f0x + f0y * f0y);
    double ux = 1.0, uy = 0.0;
    if (s0 > 0) { ux = f0x / s0; uy = f0y / s0; }
    U[0] = ux; U[1] = -uy; U[2] = uy; U[3] = ux;     /* u1 = (-uy, ux) */
    double s1 = -uy * f1x + ux * f1y;
    if (fabs(s1) > s0) {                            /* the rotation picked the smaller value first */
        /* swap the roles of v0 and v1 (v1 -> v0, -v0 -> v1 keeps V a rotation) */
        V[0] = -sn; V[1] = -c; V[2] = c; V[3] = -sn;
        const double g0x = f1x, g0y = f1y, g1x = -f0x, g1y = -f0y;
        s0 = sqrt(g0x * g0x + g0y * g0y);
        ux = 1.0; uy = 0.0;
        if (s0 > 0) { ux = g0x / s0; uy = g0y / s0; }
        U[0] = ux; U[1] = -uy; U[2] = uy; U[3] = ux;
        s1 = -uy * g1x + ux * g1y;
    }
    s[0] = s0;
    s[1] = s1;
}

/* fixed_corotated.py (dim 2): psi, P and the projected dPdF [j*2+i][s*2+r] */
static double fc2_energy(const double* s, double la, double mu) {
    const double a = s[0] - 1, b = s[1] - 1, p = s[0] * s[1] - 1;
    return mu * (a * a + b * b) + la / 2 * p * p;
}

static void fc2_P_dPdF_oracle(const double* F, double la, double mu, double* P, double* dPdF, double* psi) {
    double U[4], s[2], V[4];
    svd2_jacobi(F, U, s, V);
    *psi = fc2_energy(s, la, mu);
    const double J = F[0] * F[3] - F[1] * F[2];
    double R[4];
    for (int i = 0; i < 2; ++i)
        for (int k = 0; k < 2; ++k) R[2 * i + k] = U[2 * i] * V[2 * k] + U[2 * i + 1] * V[2 * k + 1];
    const double cof[4] = {F[3], -F[2], -F[1], F[0]};
    for (int k = 0; k < 4; ++k) P[k] = 2 * mu * (F[k] - R[k]) + la * (J - 1) * cof[k];
    const double pm1 = s[0] * s[1] - 1;
    const double g0 = 2 * mu * (s[0] - 1) + s[1] * la * pm1, g1 = 2 * mu * (s[1] - 1) + s[0] * la * pm1;
    double Hs[4] = {2 * mu + la * s[1] * s[1], la * (pm1 + s[1] * s[0]), la * (pm1 + s[1] * s[0]), 2 * mu + la * s[0] * s[0]};
    make_pd2(Hs);
    const double left = mu - la / 2 * pm1;
    const double sum = s[0] + s[1] > 0.000001 ? s[0] + s[1] : 0.000001;
    const double right = (g0 + g1) / (2 * sum);
    double B[4] = {left + right, left - right, left - right, left + right};
    make_pd2(B);
    double M[4][4];
    memset(M, 0, sizeof(M));
    M[0][0] = Hs[0]; M[0][3] = Hs[1]; M[3][0] = Hs[2]; M[3][3] = Hs[3];
    M[1][1] = B[0]; M[1][2] = B[1]; M[2][1] = B[2]; M[2][2] = B[3];
    /* the reference's eight-term sum: dPdF[ij][rs] = sum M[p][q] (u_a v_b^T)_ij (u_c v_d^T)_rs */
    for (int j = 0; j < 2; ++j)
        for (int i = 0; i < 2; ++i)
            for (int ss = 0; ss < 2; ++ss)
                for (int r = 0; r < 2; ++r) {
                    double acc = 0;
                    for (int p = 0; p < 4; ++p)
                        for (int q = 0; q < 4; ++q) {
                            if (M[p][q] == 0.0) continue;
                            const int a = p / 2, b = p % 2, cc = q / 2, dd = q % 2;
                            acc += M[p][q] * U[2 * i + a] * V[2 * j + b] * U[2 * r + cc] * V[2 * ss + dd];
                        }
                    dPdF[(j * 2 + i) * 4 + ss * 2 + r] = acc;
                }
}

/* compute_elasticity for dim 2 (NEWTON_IPC.py:568-624): E [T], g [T][6], H [T][6][6] of
 * dt^2 vol0 psi; IB [T][4] = restT^-1 row-major; any of E, g, H may be NULL */
void oracle2d_elements(int nT, const int* tris, const double* x, const double* IB, const double* vol, const double* la,
                       const double* mu, double dt, double* E, double* g, double* H) {
    #pragma omp parallel for schedule(static)
    for (int e = 0; e < nT; ++e) {
        const double* X0 = x + 2 * tris[3 * e];
        const double* X1 = x + 2 * tris[3 * e + 1];
        const double* X2 = x + 2 * tris[3 * e + 2];
        const double* ib = IB + 4 * e;
        const double Ds[4] = {X1[0] - X0[0], X2[0] - X0[0], X1[1] - X0[1], X2[1] - X0[1]};
        double F[4];
        for (int i = 0; i < 2; ++i)
            for (int k = 0; k < 2; ++k) F[2 * i + k] = Ds[2 * i] * ib[k] + Ds[2 * i + 1] * ib[2 + k];
        double P[4], dPdF[16], psi;
        fc2_P_dPdF_oracle(F, la[e], mu[e], P, dPdF, &psi);
        const double w = dt * dt * vol[e];
        if (E) E[e] = psi * w;
        /* G[ij][2a+d] = delta_id D[a][j] */
        const double D[3][2] = {{-ib[0] - ib[2], -ib[1] - ib[3]}, {ib[0], ib[1]}, {ib[2], ib[3]}};
        double G[4][6];
        memset(G, 0, sizeof(G));
        for (int j = 0; j < 2; ++j)
            for (int i = 0; i < 2; ++i)
                for (int a = 0; a < 3; ++a) G[j * 2 + i][2 * a + i] = D[a][j];
        if (g) {
            const double Pv[4] = {P[0], P[2], P[1], P[3]};   /* vec index j*2+i of P_ij */
            for (int n = 0; n < 6; ++n) {
                double acc = 0;
                for (int k = 0; k < 4; ++k) acc += Pv[k] * G[k][n];
                g[6 * e + n] = acc * w;
            }
        }
        if (H) {
            double T[4][6];
            for (int k = 0; k < 4; ++k)
                for (int m = 0; m < 6; ++m) {
                    double acc = 0;
                    for (int l = 0; l < 4; ++l) acc += dPdF[k * 4 + l] * G[l][m];
                    T[k][m] = acc;
                }
            for (int n = 0; n < 6; ++n)
                for (int m = 0; m < 6; ++m) {
                    double acc = 0;
                    for (int k = 0; k < 4; ++k) acc += G[k][n] * T[k][m];
                    H[36 * e + 6 * n + m] = acc * w;
                }
        }
    }
}

static double pe2_d2(const double* p, const double* e0, const double* e1) {
    const double ex = e1[0] - e0[0], ey = e1[1] - e0[1];
    const double num = ey * p[0] - ex * p[1] + e1[0] * e0[1] - e1[1] * e0[0];
    return num * num / (ex * ex + ey * ey);
}
static double pp2_d2(const double* a, const double* b) {
    return (a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]);
}
static int pe2_case(const double* p, const double* e0, const double* e1) {
    const double ex = e1[0] - e0[0], ey = e1[1] - e0[1];
    const double ratio = (ex * (p[0] - e0[0]) + ey * (p[1] - e0[1])) / (ex * ex + ey * ey);
    return ratio < 0 ? 0 : (ratio > 1 ? 1 : 2);
}

/* find_constraints_2D_PE (NEWTON_IPC.py:159-179): candidate rows in any order (the caller
 * sorts and de-duplicates them as np.unique does).  pp [cap][2], pe [cap][3]; returns the
 * counts in n_out[2] (they may exceed cap: then the caller grows and calls again). */
void oracle2d_find(int nBP, const int* bp, int nBE, const int* be, const double* x, double dhat2, int cap, int* pp, int* pe,
                   int* n_out) {
    const double dhat = sqrt(dhat2);
    int npp = 0, npe = 0;
    #pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < nBP; ++i) {
        const int p = bp[i];
        const double* xp = x + 2 * p;
        for (int j = 0; j < nBE; ++j) {
            const int e0 = be[2 * j], e1 = be[2 * j + 1];
            if (p == e0 || p == e1) continue;
            const double* x0 = x + 2 * e0;
            const double* x1 = x + 2 * e1;
            int inside = 1;
            for (int k = 0; k < 2; ++k) {
                const double lo = fmin(x0[k], x1[k]), hi = fmax(x0[k], x1[k]);
                if (!(xp[k] < hi + dhat && lo - dhat < xp[k])) inside = 0;
            }
            if (!inside) continue;
            const int c = pe2_case(xp, x0, x1);
            if (c < 2) {
                const int o = c == 0 ? e0 : e1;
                if (pp2_d2(xp, c == 0 ? x0 : x1) < dhat2) {
                    int slot;
                    #pragma omp atomic capture
                    slot = npp++;
                    if (slot < cap) { pp[2 * slot] = p < o ? p : o; pp[2 * slot + 1] = p < o ? o : p; }
                }
            } else if (pe2_d2(xp, x0, x1) < dhat2) {
                int slot;
                #pragma omp atomic capture
                slot = npe++;
                if (slot < cap) { pe[3 * slot] = p; pe[3 * slot + 1] = e0; pe[3 * slot + 2] = e1; }
            }
        }
    }
    n_out[0] = npp;
    n_out[1] = npe;
}

/* point_edge_ccd with its broad phase (common/math/ipc.py:374-481), restated */
static int pe2_overlap(const double* x0, const double* x1, const double* x2, const double* d0, const double* d1,
                       const double* d2, double t) {
    double p[2], a[2], b[2];
    for (int k = 0; k < 2; ++k) { p[k] = x0[k] + d0[k] * t; a[k] = x1[k] + d1[k] * t; b[k] = x2[k] + d2[k] * t; }
    const double ex = b[0] - a[0], ey = b[1] - a[1];
    const double ratio = (ex * (p[0] - a[0]) + ey * (p[1] - a[1])) / (ex * ex + ey * ey);
    return 0 <= ratio && ratio <= 1;
}
static double pe2_ccd_oracle(const double* x0, const double* x1, const double* x2, const double* d0, const double* d1,
                             const double* d2, double eta) {
    const int c = pe2_case(x0, x1, x2);
    const double dist2 = c == 0 ? pp2_d2(x0, x1) : (c == 1 ? pp2_d2(x0, x2) : pe2_d2(x0, x1, x2));
    const double m0 = d0[0] * d0[0] + d0[1] * d0[1], m1 = d1[0] * d1[0] + d1[1] * d1[1], m2 = d2[0] * d2[0] + d2[1] * d2[1];
    const double mx = fmax(fmax(m0, m1), m2);
    if (!(mx > 0)) return 1.0;
    const double lb = (1 - eta) * sqrt(dist2) / (2 * sqrt(mx));
    if (!(lb <= 1)) return 1.0;
    const double A = d0[0] * (d2[1] - d1[1]) + d0[1] * (d1[0] - d2[0]) + d2[0] * d1[1] - d2[1] * d1[0];
    const double Bq = x0[0] * (d2[1] - d1[1]) + d0[0] * (x2[1] - x1[1]) + d0[1] * (x1[0] - x2[0]) + x0[1] * (d1[0] - d2[0]) +
                      d1[1] * x2[0] + d2[0] * x1[1] - d1[0] * x2[1] - d2[1] * x1[0];
    const double C = x0[0] * (x2[1] - x1[1]) + x0[1] * (x1[0] - x2[0]) + x2[0] * x1[1] - x2[1] * x1[0];
    double toc = 1.0, roots[2];
    int nr = 0;
    if (A == 0 && Bq == 0 && C == 0) {
        const double* xe[2] = {x1, x2};
        const double* de[2] = {d1, d2};
        for (int k = 0; k < 2; ++k) {
            const double rx = x0[0] - xe[k][0], ry = x0[1] - xe[k][1], vx = d0[0] - de[k][0], vy = d0[1] - de[k][1];
            if (rx * vx + ry * vy < 0) {
                const double t = sqrt((rx * rx + ry * ry) / (vx * vx + vy * vy));
                if (t > 0 && t <= 1 && t * (1 - eta) < toc) toc = t * (1 - eta);
            }
        }
    } else if (A == 0) {
        if (Bq != 0) roots[nr++] = -C / Bq;
    } else {
        const double disc = Bq * Bq - 4 * A * C;
        if (disc == 0) {
            roots[nr++] = -Bq / (2 * A);
        } else if (disc > 0) {
            const double sq = sqrt(disc);
            if (Bq > 0) { roots[nr++] = (-Bq - sq) / (2 * A); roots[nr++] = 2 * C / (-Bq - sq); }
            else { roots[nr++] = 2 * C / (-Bq + sq); roots[nr++] = (-Bq + sq) / (2 * A); }
        }
    }
    for (int k = 0; k < nr; ++k)
        if (roots[k] > 0 && roots[k] <= 1 && pe2_overlap(x0, x1, x2, d0, d1, d2, roots[k]) && roots[k] * (1 - eta) < toc)
            toc = roots[k] * (1 - eta);
    return toc > lb ? toc : lb;
}

/* compute_filter_2D_PE (NEWTON_IPC.py:361-374): the smallest CCD step over all pairs */
double oracle2d_ccd_step(int nBP, const int* bp, int nBE, const int* be, const double* x, const double* p, double dhat2,
                         double eta) {
    const double dhat = sqrt(dhat2);
    double alpha = 1.0;
    #pragma omp parallel for schedule(dynamic, 16) reduction(min:alpha)
    for (int i = 0; i < nBP; ++i) {
        const int q = bp[i];
        const double* x0 = x + 2 * q;
        const double* d0 = p + 2 * q;
        for (int j = 0; j < nBE; ++j) {
            const int a = be[2 * j], b = be[2 * j + 1];
            if (q == a || q == b) continue;
            const double *x1 = x + 2 * a, *x2 = x + 2 * b, *d1 = p + 2 * a, *d2 = p + 2 * b;
            int ok = 1;
            for (int k = 0; k < 2; ++k) {
                const double lp = fmin(x0[k], x0[k] + d0[k]), hp = fmax(x0[k], x0[k] + d0[k]);
                const double le = fmin(fmin(x1[k], x2[k]), fmin(x1[k] + d1[k], x2[k] + d2[k]));
                const double he = fmax(fmax(x1[k], x2[k]), fmax(x1[k] + d1[k], x2[k] + d2[k]));
                if (!(lp < he + dhat && le - dhat < hp)) ok = 0;
            }
            if (!ok) continue;
            const double t = pe2_ccd_oracle(x0, x1, x2, d0, d1, d2, eta);
            if (t < alpha) alpha = t;
        }
    }
    return alpha;
}

/* check_collision_2D (NEWTON_IPC.py:843-854) with point_inside_triangle (ipc.py:502-509) */
int oracle2d_collision(int nBP, const int* bp, int nT, const int* tris, const double* x) {
    int hit = 0;
    #pragma omp parallel for schedule(dynamic, 16) reduction(|:hit)
    for (int i = 0; i < nBP; ++i) {
        const int q = bp[i];
        const double* P = x + 2 * q;
        for (int e = 0; e < nT && !hit; ++e) {
            const int a = tris[3 * e], b = tris[3 * e + 1], c = tris[3 * e + 2];
            if (q == a || q == b || q == c) continue;
            const double *A = x + 2 * a, *B = x + 2 * b, *C = x + 2 * c;
            const double d1 = (P[0] - B[0]) * (A[1] - B[1]) - (P[1] - B[1]) * (A[0] - B[0]);
            const double d2 = (P[0] - C[0]) * (B[1] - C[1]) - (P[1] - C[1]) * (B[0] - C[0]);
            const double d3 = (P[0] - A[0]) * (C[1] - A[1]) - (P[1] - A[1]) * (C[0] - A[0]);
            const int neg = d1 < 0 || d2 < 0 || d3 < 0, pos = d1 > 0 || d2 > 0 || d3 > 0;
            if (!(neg && pos)) hit = 1;
        }
    }
    return hit;
}
