// Host build of the product's device math headers (barrier.cuh, nh.cuh, ccd.cuh, eig.cuh)
// for CPU unit tests against the oracle.  Test infrastructure only.
#include <string.h>

#include "../../fastipc_gb300/csrc/barrier.cuh"
#include "../../fastipc_gb300/csrc/ccd.cuh"
#include "../../fastipc_gb300/csrc/geometry.cuh"
#include "../../fastipc_gb300/csrc/nh.cuh"

using namespace fipc;

extern "C" {

// rows [count x 4], x/x0 [V x 3]; E [count], g [count x 12], H [count x 144] (full 12x12,
// leading 3nv x 3nv block used)
void hc_barrier_rows(int type, int count, const int* rows, const double* x, const double* x0, double dh2, double kappa,
                     double* E, double* g, double* H) {
    for (int r = 0; r < count; ++r) {
        const int nv = type_nverts(type);
        v3 X[4], X0[4];
        for (int k = 0; k < 4; ++k) {
            const int v = rows[4 * r + (k < nv ? k : 0)];
            X[k] = load3(x, v);
            X0[k] = x0 ? load3(x0, v) : mk(0, 0, 0);
        }
        double gg[12] = {0}, Hb[16 * 9] = {0};
        barrier_row(type, X, X0, dh2, kappa, g != nullptr, &E[r], gg, Hb);
        if (!g) continue;
        const int n = 3 * nv;
        for (int i = 0; i < n; ++i) g[12 * r + i] = gg[i];
        for (int v = 0; v < nv; ++v)
            for (int w = 0; w < nv; ++w)
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) H[144 * r + (3 * v + i) * n + 3 * w + j] = Hb[(v * 4 + w) * 9 + i * 3 + j];
    }
}

// X [count x 12], IB [count x 9]; H full 12x12
void hc_nh_element(int count, const double* Xs, const double* IB, double la, double mu, double w, double* E, double* g,
                   double* H) {
    for (int c = 0; c < count; ++c) {
        v3 X[4];
        for (int k = 0; k < 4; ++k) X[k] = load3(Xs + 12 * c, k);
        double Hu[90];
        E[c] = nh_element(X, IB + 9 * c, la, mu, w, g + 12 * c, Hu);
        int blk = 0;
        for (int v = 0; v < 4; ++v)
            for (int ww = v; ww < 4; ++ww, ++blk)
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) {
                        H[144 * c + (3 * v + i) * 12 + 3 * ww + j] = Hu[blk * 9 + i * 3 + j];
                        H[144 * c + (3 * ww + j) * 12 + 3 * v + i] = Hu[blk * 9 + i * 3 + j];
                    }
    }
}

void hc_svd3(int count, const double* F, double* U, double* s, double* V) {
    for (int c = 0; c < count; ++c) svd3(F + 9 * c, U + 9 * c, s + 3 * c, V + 9 * c);
}

void hc_sym_eig(int count, int n, const double* A, double* w, double* Vout) {
    for (int c = 0; c < count; ++c) {
        double a[81];
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) a[i * 9 + j] = A[c * n * n + i * n + j];
        sym_eig(n, a, w + c * n);
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) Vout[c * n * n + i * n + j] = a[i * 9 + j];
    }
}

void hc_ccd(int kind, int count, const double* x, const double* p, double eta, double* toc) {
    for (int c = 0; c < count; ++c) {
        const double* q = x + 12 * c;
        const double* d = p + 12 * c;
        v3 Q[4], Dd[4];
        for (int k = 0; k < 4; ++k) { Q[k] = load3(q, k); Dd[k] = load3(d, k); }
        // current distance by feature type (NEWTON_IPC.py:404, :438)
        const double dist2 = kind == 0 ? pt_dist2(Q[0], Q[1], Q[2], Q[3]) : ee_dist2(Q[0], Q[1], Q[2], Q[3]);
        toc[c] = kind == 0 ? pt_ccd(Q[0], Q[1], Q[2], Q[3], Dd[0], Dd[1], Dd[2], Dd[3], eta, dist2)
                           : ee_ccd(Q[0], Q[1], Q[2], Q[3], Dd[0], Dd[1], Dd[2], Dd[3], eta, dist2);
    }
}

void hc_types(int count, const double* pts, int* pt, int* ee) {
    for (int c = 0; c < count; ++c) {
        v3 Q[4];
        for (int k = 0; k < 4; ++k) Q[k] = load3(pts + 12 * c, k);
        pt[c] = pt_type(Q[0], Q[1], Q[2], Q[3]);
        ee[c] = ee_type(Q[0], Q[1], Q[2], Q[3]);
    }
}

void hc_seg_tri(int count, const double* pts, int* hit) {
    for (int c = 0; c < count; ++c) {
        v3 Q[5];
        for (int k = 0; k < 5; ++k) Q[k] = load3(pts + 15 * c, k);
        hit[c] = seg_tri(Q[0], Q[1], Q[2], Q[3], Q[4]);
    }
}

// the step filter's early-out for tets (1: the tet is skipped)
void hc_inversion_skip(int count, const double* xs, const double* ps, double eta, int* skip) {
    for (int c = 0; c < count; ++c) {
        v3 X[4], P[4];
        for (int k = 0; k < 4; ++k) { X[k] = load3(xs + 12 * c, k); P[k] = load3(ps + 12 * c, k); }
        skip[c] = inversion_cannot_flip(X, P, eta);
    }
}

void hc_inversion(int count, const double* xs, const double* ps, double eta, double* out) {
    for (int c = 0; c < count; ++c) {
        v3 X[4], P[4];
        for (int k = 0; k < 4; ++k) { X[k] = load3(xs + 12 * c, k); P[k] = load3(ps + 12 * c, k); }
        out[c] = inversion_free_step(X, P, eta);
    }
}
}
