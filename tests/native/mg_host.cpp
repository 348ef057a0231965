// Host restatement of the multigrid-preconditioned CG of the direction solve, driven by the
// product's own hierarchy set-up (fastipc_gb300/csrc/mg_plan.h): the same aggregation,
// patterns, contribution lists, prolongation algebra, damped block-Jacobi smoothing with
// power-iteration estimates and dense coarsest solve as the GPU kernels.  Test infrastructure
// only: it checks the set-up and the V-cycle on the CPU against a reference sparse solve.
#include <cmath>
#include <cstring>
#include <vector>

#include "../../fastipc_gb300/csrc/mg_plan.h"

using namespace fipc;

namespace {

using Vec = std::vector<double>;

// C (nr x nc, row-major) += P_i^T B P_j for a finer block B (bi x bj, row-major), where P of a
// vertex member (3 DOFs) is [I, -[d]x] and of a node member (6 DOFs) [[I, -[d]x], [0, I]]
void add_galerkin(double* C, const double* B, int bi, int bj, const double* di, const double* dj) {
    auto P = [](const double* d, int b, double* out) {   // b x 6, row-major
        for (int k = 0; k < 6 * b; ++k) out[k] = 0.0;
        const double S[9] = {0, -d[2], d[1], d[2], 0, -d[0], -d[1], d[0], 0};   // [d]x
        for (int r = 0; r < 3; ++r) {
            out[6 * r + r] = 1.0;
            for (int c = 0; c < 3; ++c) out[6 * r + 3 + c] = -S[3 * r + c];
        }
        if (b == 6)
            for (int r = 0; r < 3; ++r) out[6 * (3 + r) + 3 + r] = 1.0;
    };
    double Pi[36], Pj[36], BP[36];
    P(di, bi, Pi);
    P(dj, bj, Pj);
    for (int r = 0; r < bi; ++r)
        for (int c = 0; c < 6; ++c) {
            double s = 0.0;
            for (int k = 0; k < bj; ++k) s += B[r * bj + k] * Pj[6 * k + c];
            BP[6 * r + c] = s;
        }
    for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c) {
            double s = 0.0;
            for (int k = 0; k < bi; ++k) s += Pi[6 * k + r] * BP[6 * k + c];
            C[6 * r + c] += s;
        }
}

// in-place inverse of an SPD n x n matrix (Gauss-Jordan without pivoting)
void inv_spd(double* A, int n) {
    for (int k = 0; k < n; ++k) {
        const double p = A[k * n + k];
        const double ip = 1.0 / p;
        for (int j = 0; j < n; ++j) A[k * n + j] *= ip;
        A[k * n + k] = ip;
        for (int i = 0; i < n; ++i) {
            if (i == k) continue;
            const double f = A[i * n + k];
            if (f == 0.0) continue;
            for (int j = 0; j < n; ++j) A[i * n + j] -= f * A[k * n + j];
            A[i * n + k] = -f * ip;
        }
    }
}

struct Level {
    int n = 0, b = 3;                 // nodes, DOFs per node
    Vec S, C;                          // block values (b*b per block)
    Vec M;                             // block-Jacobi inverses (b*b per node)
    Vec d;                             // level >= 1: offsets of the finer nodes from their aggregate
    Vec cent;                          // level >= 1: aggregate centroids
    double omega = 1.0;
    Vec g, z, z2, t;
};

struct Solver {
    MgPlan P;
    std::vector<Level> L;
    const unsigned char* fixed;
    int nV;
    Vec dense;                         // coarsest inverse (n_c x n_c)

    void spmv(int l, const Vec& v, Vec& y) const {
        const Level& lv = L[l];
        const int b = lv.b;
        y.assign((size_t)lv.n * b, 0.0);
        for (int pass = 0; pass < 2; ++pass) {
            const MgPattern& pt = pass ? P.L[l].C : P.L[l].S;
            const Vec& val = pass ? lv.C : lv.S;
            if (pt.nnz() == 0) continue;
            for (int i = 0; i < lv.n; ++i) {
                if (l == 0 && fixed[i]) continue;
                for (int k = pt.rp[i]; k < pt.rp[i + 1]; ++k) {
                    const int j = pt.ci[k];
                    if (l == 0 && fixed[j]) continue;
                    for (int r = 0; r < b; ++r) {
                        double s = 0.0;
                        for (int c = 0; c < b; ++c) s += val[(size_t)b * b * k + b * r + c] * v[(size_t)b * j + c];
                        y[(size_t)b * i + r] += s;
                    }
                }
            }
        }
    }
    void apply_M(int l, const Vec& r, Vec& z, double w) const {
        const Level& lv = L[l];
        const int b = lv.b;
        z.assign((size_t)lv.n * b, 0.0);
        for (int i = 0; i < lv.n; ++i) {
            if (l == 0 && fixed[i]) continue;
            for (int p = 0; p < b; ++p) {
                double s = 0.0;
                for (int q = 0; q < b; ++q) s += lv.M[(size_t)b * b * i + b * p + q] * r[(size_t)b * i + q];
                z[(size_t)b * i + p] = w * s;
            }
        }
    }
    // restriction of the finer level's vector t (level l-1) into level l
    void restrict_(int l, const Vec& t, Vec& g) const {
        const Level& c = L[l];
        const int bf = L[l - 1].b;
        g.assign(6 * (size_t)c.n, 0.0);
        const MgLevelPlan& pl = P.L[l];
        for (int I = 0; I < c.n; ++I)
            for (int k = pl.mem_ptr[I]; k < pl.mem_ptr[I + 1]; ++k) {
                const int i = pl.mem[k];
                if (l == 1 && fixed[i]) continue;
                const double* d = &c.d[3 * (size_t)i];
                const double a0 = t[bf * (size_t)i], a1 = t[bf * (size_t)i + 1], a2 = t[bf * (size_t)i + 2];
                g[6 * I] += a0;
                g[6 * I + 1] += a1;
                g[6 * I + 2] += a2;
                g[6 * I + 3] += d[1] * a2 - d[2] * a1;
                g[6 * I + 4] += d[2] * a0 - d[0] * a2;
                g[6 * I + 5] += d[0] * a1 - d[1] * a0;
                if (bf == 6)
                    for (int q = 0; q < 3; ++q) g[6 * I + 3 + q] += t[6 * (size_t)i + 3 + q];
            }
    }
    // z_{l-1} += P y_l
    void prolong(int l, const Vec& y, Vec& z) const {
        const Level& c = L[l];
        const int bf = L[l - 1].b;
        for (int i = 0; i < L[l - 1].n; ++i) {
            if (l == 1 && fixed[i]) continue;
            const int I = P.L[l].agg_of[i];
            const double* d = &c.d[3 * (size_t)i];
            const double* Y = &y[6 * (size_t)I];
            z[bf * (size_t)i] += Y[0] + (Y[4] * d[2] - Y[5] * d[1]);
            z[bf * (size_t)i + 1] += Y[1] + (Y[5] * d[0] - Y[3] * d[2]);
            z[bf * (size_t)i + 2] += Y[2] + (Y[3] * d[1] - Y[4] * d[0]);
            if (bf == 6)
                for (int q = 0; q < 3; ++q) z[6 * (size_t)i + 3 + q] += Y[3 + q];
        }
    }
    // z = V(r) at level l (l = 0: r is the PCG residual)
    void vcycle(int l, const Vec& r, Vec& z) {
        Level& lv = L[l];
        if (l == P.levels - 1) {
            const int n = 6 * lv.n;
            z.assign(n, 0.0);
            for (int i = 0; i < n; ++i) {
                double s = 0.0;
                for (int j = 0; j < n; ++j) s += dense[(size_t)i * n + j] * r[j];
                z[i] = s;
            }
            return;
        }
        Vec Az, t, zc, z2;
        apply_M(l, r, z, lv.omega);
        spmv(l, z, Az);
        t.resize(r.size());
        for (size_t k = 0; k < r.size(); ++k) t[k] = r[k] - Az[k];
        Vec g;
        restrict_(l + 1, t, g);
        vcycle(l + 1, g, zc);
        prolong(l + 1, zc, z);
        spmv(l, z, Az);
        for (size_t k = 0; k < r.size(); ++k) t[k] = r[k] - Az[k];
        apply_M(l, t, z2, lv.omega);
        for (size_t k = 0; k < r.size(); ++k) z[k] += z2[k];
        if (l == 0)
            for (int i = 0; i < nV; ++i)
                if (fixed[i]) z[3 * i] = z[3 * i + 1] = z[3 * i + 2] = 0.0;
    }
};

double power_rho(const Solver& s, int l) {
    const Level& lv = s.L[l];
    const size_t n = (size_t)lv.n * lv.b;
    Vec v(n), y, z;
    for (size_t k = 0; k < n; ++k) v[k] = (double)((k * 2654435761ull) % 1000) / 1000.0 - 0.5;
    if (l == 0)
        for (int i = 0; i < s.nV; ++i)
            if (s.fixed[i]) v[3 * i] = v[3 * i + 1] = v[3 * i + 2] = 0.0;
    double rho = 0.0;
    for (int it = 0; it < 8; ++it) {
        double nv = 0.0;
        for (double q : v) nv += q * q;
        nv = std::sqrt(nv);
        for (double& q : v) q /= nv;
        s.spmv(l, v, y);
        s.apply_M(l, y, z, 1.0);
        double nz = 0.0;
        for (double q : z) nz += q * q;
        rho = std::sqrt(nz);
        v.swap(z);
    }
    return rho;
}

}  // namespace

extern "C" {

// info: [0] levels, [1 + l] nodes of level l, [1 + MG_MAX_LEVELS + l] static blocks of level l
void mg_host_plan(int nV, const double* x0, const int* rp, const int* ci, double h, double* info) {
    MgPlan P;
    mg_build(nV, x0, rp, ci, h, P);
    info[0] = P.levels;
    for (int l = 0; l < P.levels; ++l) {
        info[1 + l] = P.L[l].n;
        info[1 + MG_MAX_LEVELS + l] = P.L[l].S.nnz();
    }
}

// level-1 aggregates: rot[a] (1: rotations, 0: translations only) and member counts; returns
// the number of aggregates
int mg_host_level1(int nV, const double* x0, const int* rp, const int* ci, double h, int* rot, int* members) {
    MgPlan P;
    mg_build(nV, x0, rp, ci, h, P);
    if (P.levels < 2) return 0;
    const MgLevelPlan& c = P.L[1];
    for (int a = 0; a < c.n; ++a) {
        rot[a] = c.rot[a];
        members[a] = c.mem_ptr[a + 1] - c.mem_ptr[a];
    }
    return c.n;
}

// MG-preconditioned CG on the Dirichlet-edited block system (blocks row-major, vertex BSR);
// x: current positions (the rigid modes' offsets), x0: rest positions (the aggregation).
// Returns the iteration count (-1: no convergence); info[0..] = omega per level.
int mg_host_pcg(int nV, const int* rp, const int* ci, const double* ev, const int* crp, const int* cci, const double* cv,
                const unsigned char* fixed, const double* x, const double* x0, double h, const double* rhs, double rtol, int maxit,
                double* sol, double* info) {
    Solver s;
    s.fixed = fixed;
    s.nV = nV;
    mg_build(nV, x0, rp, ci, h, s.P);
    mg_contact(s.P, nV, crp, cci);
    const int NL = s.P.levels;
    s.L.resize(NL);
    s.L[0].n = nV;
    s.L[0].b = 3;
    s.L[0].S.assign(ev, ev + 9 * (size_t)rp[nV]);
    if (crp && crp[nV] > 0) s.L[0].C.assign(cv, cv + 9 * (size_t)crp[nV]);
    // centroids and offsets (current positions), Galerkin products
    for (int l = 1; l < NL; ++l) {
        Level& c = s.L[l];
        const Level& f = s.L[l - 1];
        const MgLevelPlan& pl = s.P.L[l];
        c.n = pl.n;
        c.b = 6;
        c.cent.assign(3 * (size_t)c.n, 0.0);
        const double* fp = l == 1 ? x : f.cent.data();
        for (int I = 0; I < c.n; ++I) {
            for (int k = pl.mem_ptr[I]; k < pl.mem_ptr[I + 1]; ++k)
                for (int q = 0; q < 3; ++q) c.cent[3 * I + q] += fp[3 * (size_t)pl.mem[k] + q];
            for (int q = 0; q < 3; ++q) c.cent[3 * I + q] /= (double)(pl.mem_ptr[I + 1] - pl.mem_ptr[I]);
        }
        c.d.assign(3 * (size_t)f.n, 0.0);
        for (int i = 0; i < f.n; ++i)
            if (pl.rot.empty() || pl.rot[pl.agg_of[i]])   // translation-only aggregates keep zero offsets
                for (int q = 0; q < 3; ++q) c.d[3 * i + q] = fp[3 * (size_t)i + q] - c.cent[3 * (size_t)pl.agg_of[i] + q];
        for (int pass = 0; pass < 2; ++pass) {
            const MgPattern& pt = pass ? pl.C : pl.S;
            Vec& out = pass ? c.C : c.S;
            const Vec& src = pass ? f.C : f.S;
            out.assign(36 * (size_t)pt.nnz(), 0.0);
            for (int b = 0; b < pt.nnz(); ++b)
                for (int q = pt.con_ptr[b]; q < pt.con_ptr[b + 1]; ++q) {
                    const int i = pt.src_row[q], j = pt.src_col[q];
                    if (l == 1 && (fixed[i] || fixed[j])) continue;
                    add_galerkin(&out[36 * (size_t)b], &src[(size_t)f.b * f.b * pt.src[q]], f.b, f.b, &c.d[3 * (size_t)i],
                                 &c.d[3 * (size_t)j]);
                }
        }
    }
    // block-Jacobi inverses (diagonal blocks of both patterns; identity at fixed vertices),
    // shifted by 1e-10 of the block's largest diagonal entry
    for (int l = 0; l < NL; ++l) {
        Level& lv = s.L[l];
        const int b = lv.b;
        lv.M.assign((size_t)b * b * lv.n, 0.0);
        for (int i = 0; i < lv.n; ++i) {
            double D[36] = {0};
            for (int pass = 0; pass < 2; ++pass) {
                const MgPattern& pt = pass ? s.P.L[l].C : s.P.L[l].S;
                const Vec& val = pass ? lv.C : lv.S;
                if (pt.nnz() == 0) continue;
                for (int k = pt.rp[i]; k < pt.rp[i + 1]; ++k)
                    if (pt.ci[k] == i)
                        for (int e = 0; e < b * b; ++e) D[e] += val[(size_t)b * b * k + e];
            }
            double mx = 0.0;
            for (int p = 0; p < b; ++p) mx = std::fmax(mx, D[p * b + p]);
            if ((l == 0 && fixed[i]) || !(mx > 0.0)) {
                for (int p = 0; p < b; ++p) D[p * b + p] = 1.0;
            } else {
                for (int p = 0; p < b; ++p) D[p * b + p] += 1e-10 * mx;
            }
            inv_spd(D, b);
            for (int e = 0; e < b * b; ++e) lv.M[(size_t)b * b * i + e] = D[e];
        }
    }
    // coarsest: dense, zero diagonals to one, then the inverse
    {
        const Level& c = s.L[NL - 1];
        const int n = 6 * c.n;
        s.dense.assign((size_t)n * n, 0.0);
        for (int pass = 0; pass < 2; ++pass) {
            const MgPattern& pt = pass ? s.P.L[NL - 1].C : s.P.L[NL - 1].S;
            const Vec& val = pass ? c.C : c.S;
            if (pt.nnz() == 0) continue;
            for (int I = 0; I < c.n; ++I)
                for (int k = pt.rp[I]; k < pt.rp[I + 1]; ++k)
                    for (int p = 0; p < 6; ++p)
                        for (int q = 0; q < 6; ++q) s.dense[(size_t)(6 * I + p) * n + 6 * pt.ci[k] + q] += val[36 * (size_t)k + 6 * p + q];
        }
        for (int k = 0; k < n; ++k) {
            double& dk = s.dense[(size_t)k * n + k];
            dk = dk > 0.0 ? dk * (1.0 + 1e-12) : 1.0;
        }
        inv_spd(s.dense.data(), n);
    }
    for (int l = 0; l < NL - 1; ++l) {
        s.L[l].omega = 4.0 / (3.0 * 1.05 * power_rho(s, l));
        info[l] = s.L[l].omega;
    }
    // PCG
    const size_t n = 3 * (size_t)nV;
    Vec xk(n, 0.0), r(rhs, rhs + n), z, p, Ap;
    for (int i = 0; i < nV; ++i)
        if (fixed[i]) r[3 * i] = r[3 * i + 1] = r[3 * i + 2] = 0.0;
    double bb = 0.0;
    for (double q : r) bb += q * q;
    s.vcycle(0, r, z);
    p = z;
    double rz = 0.0;
    for (size_t k = 0; k < n; ++k) rz += r[k] * z[k];
    int it = 0;
    for (; it < maxit; ++it) {
        double rr = 0.0;
        for (double q : r) rr += q * q;
        if (rr <= rtol * rtol * bb) break;
        s.spmv(0, p, Ap);
        double pAp = 0.0;
        for (size_t k = 0; k < n; ++k) pAp += p[k] * Ap[k];
        const double a = rz / pAp;
        for (size_t k = 0; k < n; ++k) {
            xk[k] += a * p[k];
            r[k] -= a * Ap[k];
        }
        s.vcycle(0, r, z);
        double rz2 = 0.0;
        for (size_t k = 0; k < n; ++k) rz2 += r[k] * z[k];
        const double beta = rz2 / rz;
        rz = rz2;
        for (size_t k = 0; k < n; ++k) p[k] = z[k] + beta * p[k];
    }
    for (size_t k = 0; k < n; ++k) sol[k] = xk[k];
    return it < maxit ? it : -1;
}

}  // extern "C"
