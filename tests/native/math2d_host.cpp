// Host build of the product's 2D device math (fc2d.cuh) for CPU unit tests against the 2D
// oracle.  Test infrastructure only.
#include "../../fastipc_gb300/csrc/fc2d.cuh"

using namespace fipc;

extern "C" {

// X [n][3][2], IB [n][4] -> E [n], g [n][6], H [n][9][4]
void h2_elements(int n, const double* X, const double* IB, const double* la, const double* mu, const double* w, double* E,
                 double* g, double* H) {
    for (int e = 0; e < n; ++e) E[e] = fc2_element(X + 6 * e, IB + 4 * e, la[e], mu[e], w[e], g + 6 * e, H + 36 * e);
}

// type 0 PP / 1 PE; X [n][3][2] -> E [n], g [n][6], H [n][36] (leading 4 nv^2 used)
void h2_barrier(int type, int n, const double* X, double dh2, double kappa, double* E, double* g, double* H) {
    for (int r = 0; r < n; ++r) barrier_row_2d(type, X + 6 * r, dh2, kappa, 1, E + r, g + 6 * r, H + 36 * r);
}

// xq, pq [n][3][2] -> toc [n]
void h2_ccd(int n, const double* xq, const double* pq, double eta, double* toc) {
    for (int c = 0; c < n; ++c) {
        const double* X = xq + 6 * c;
        const double* P = pq + 6 * c;
        toc[c] = pe2_ccd(X, X + 2, X + 4, P, P + 2, P + 4, eta);
    }
}

// pts [n][4][2] (P, A, B, C) -> inside [n]
void h2_in_tri(int n, const double* pts, int* out) {
    for (int c = 0; c < n; ++c) {
        const double* q = pts + 8 * c;
        out[c] = point_in_tri2(q, q + 2, q + 4, q + 6);
    }
}

void h2_svd2(int n, const double* F, double* U, double* s, double* V) {
    for (int k = 0; k < n; ++k) svd2(F + 4 * k, U + 4 * k, s + 2 * k, V + 4 * k);
}

}  // extern "C"
