// Host-side set-up of the multigrid preconditioner of the PCG direction solve (geometric
// aggregation with rigid-body modes).
//
// Level 0 is the vertex level (3 DOFs per vertex, the Newton system's 3x3 blocks).  Level l+1
// aggregates the nodes of level l by boxes of side box_l (the first box three mesh cells, each
// further box twice the one before); the first level also by connected component of the mesh,
// so that no level-1 aggregate spans two bodies.  Every level >= 1 node carries six DOFs: the
// translation t and rotation w of its aggregate, prolongated to a member node at offset d from
// the aggregate's centroid as
//     vertex member:  u = t + w x d                  (3 x 6:  [I, -[d]x])
//     node member:    (t', w') = (t + w x d, w)       (6 x 6:  [[I, -[d]x], [0, I]])
// The coarse matrices are the Galerkin products A_{l+1} = P^T A_l P, built on the device every
// Newton iteration from the contribution lists made here: for every block (I, J) of level l+1's
// static pattern, the level-l blocks (i, j) with i in I and j in J.  Contact blocks, whose
// pattern changes every iteration, get their own per-level patterns and lists (mg_contact).
//
// Plain C++ (no CUDA types), so that the set-up compiles into the CPU tests.
#pragma once

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

namespace fipc {

constexpr int MG_MAX_LEVELS = 8;
constexpr int MG_COARSEST = 160;       // aggregate until at most this many nodes remain (the dense coarsest: <= 960 DOFs)

// a block pattern (CSR over nodes, both triangles) with its Galerkin contribution lists: block
// s of this pattern sums the source blocks src[con_ptr[s] .. con_ptr[s + 1]) of the finer level
// (positions in the finer level's pattern of the same kind), rows src_row and columns src_col
struct MgPattern {
    std::vector<int> rp, ci;
    std::vector<int> con_ptr, src, src_row, src_col;
    int nnz() const { return rp.empty() ? 0 : rp.back(); }
};

struct MgLevelPlan {
    int n = 0;                       // nodes of this level (level 0: vertices)
    std::vector<int> agg_of;         // [n_{l-1}] aggregate of each finer node (levels >= 1)
    std::vector<int> mem_ptr, mem;   // members of each node (finer-level ids, ascending)
    std::vector<unsigned char> rot;  // level 1: 1 = the node carries rotations, 0 = translations only
    MgPattern S;                     // static pattern (level 0: the system's elastic pattern)
    MgPattern C;                     // contact pattern (rebuilt by mg_contact)
};

struct MgPlan {
    int levels = 0;                  // number of levels (>= 2 when the hierarchy is in use)
    std::vector<MgLevelPlan> L;
};

namespace mg_detail {

// pattern of the aggregated level and its contribution lists from a finer pattern (rp, ci)
inline void galerkin_pattern(int n_fine, const int* rp, const int* ci, const std::vector<int>& agg_of, int n_coarse, MgPattern& out) {
    struct E {
        long long key;
        int src, r, c;
    };
    std::vector<E> e;
    e.reserve(rp ? (size_t)rp[n_fine] : 0);
    if (rp)
        for (int i = 0; i < n_fine; ++i)
            for (int k = rp[i]; k < rp[i + 1]; ++k) {
                const int j = ci[k];
                e.push_back({(long long)agg_of[i] * n_coarse + agg_of[j], k, i, j});
            }
    std::sort(e.begin(), e.end(), [](const E& a, const E& b) { return a.key < b.key || (a.key == b.key && a.src < b.src); });
    out.rp.assign(n_coarse + 1, 0);
    out.ci.clear();
    out.con_ptr.assign(1, 0);
    out.src.resize(e.size());
    out.src_row.resize(e.size());
    out.src_col.resize(e.size());
    for (size_t q = 0; q < e.size(); ++q) {
        if (q == 0 || e[q].key != e[q - 1].key) {
            const int I = (int)(e[q].key / n_coarse), J = (int)(e[q].key % n_coarse);
            out.ci.push_back(J);
            ++out.rp[I + 1];
            if (q) out.con_ptr.push_back((int)q);
        }
        out.src[q] = e[q].src;
        out.src_row[q] = e[q].r;
        out.src_col[q] = e[q].c;
    }
    if (!e.empty()) out.con_ptr.push_back((int)e.size());
    for (int I = 0; I < n_coarse; ++I) out.rp[I + 1] += out.rp[I];
}

}  // namespace mg_detail

// Builds the hierarchy from the rest positions x0 [nV][3], the static pattern (rp, ci) and the
// mesh cell size h (a typical edge length).  Stops when a level has at most MG_COARSEST nodes
// or after MG_MAX_LEVELS levels; a box that would remove fewer than 10% of the nodes is widened
// first.
inline void mg_build(int nV, const double* x0, const int* rp, const int* ci, double h, MgPlan& P) {
    P = MgPlan();
    // connected components of the static pattern (union-find)
    std::vector<int> comp(nV);
    std::iota(comp.begin(), comp.end(), 0);
    auto find = [&](int a) {
        while (comp[a] != a) a = comp[a] = comp[comp[a]];
        return a;
    };
    for (int i = 0; i < nV; ++i)
        for (int k = rp[i]; k < rp[i + 1]; ++k) {
            const int a = find(i), b = find(ci[k]);
            if (a != b) comp[std::max(a, b)] = std::min(a, b);
        }
    for (int i = 0; i < nV; ++i) comp[i] = find(i);
    MgLevelPlan l0;
    l0.n = nV;
    l0.S.rp.assign(rp, rp + nV + 1);
    l0.S.ci.assign(ci, ci + rp[nV]);
    P.L.push_back(std::move(l0));
    std::vector<double> pos(x0, x0 + 3 * (size_t)nV);   // node positions of the current level
    std::vector<int> ncomp = comp;                        // component of each node
    double lo[3] = {1e300, 1e300, 1e300};
    for (int i = 0; i < nV; ++i)
        for (int d = 0; d < 3; ++d) lo[d] = std::min(lo[d], x0[3 * i + d]);
    double box = 3.0 * h;
    while ((int)P.L.size() < MG_MAX_LEVELS && P.L.back().n > MG_COARSEST) {
        const MgLevelPlan& f = P.L.back();
        const int n = f.n;
        struct K {
            long long key;
            int comp, node;
        };
        std::vector<K> keys(n);
        // the first level keeps bodies apart; coarser levels group purely by box, so that the
        // hierarchy still shrinks when many separate bodies remain
        const bool by_body = P.L.size() == 1;
        for (int i = 0; i < n; ++i) {
            long long q[3];
            for (int d = 0; d < 3; ++d) q[d] = (long long)std::floor((pos[3 * i + d] - lo[d]) / box + 1e-9);
            keys[i] = {(q[0] * 1048576 + q[1]) * 1048576 + q[2], by_body ? ncomp[i] : 0, i};
        }
        std::sort(keys.begin(), keys.end(), [](const K& a, const K& b) {
            return a.comp < b.comp || (a.comp == b.comp && (a.key < b.key || (a.key == b.key && a.node < b.node)));
        });
        MgLevelPlan c;
        c.agg_of.assign(n, -1);
        int na = 0;
        for (int q = 0; q < n; ++q) {
            if (q == 0 || keys[q].comp != keys[q - 1].comp || keys[q].key != keys[q - 1].key) ++na;
            c.agg_of[keys[q].node] = na - 1;
        }
        if (10 * na > 9 * n) {   // under 10% fewer nodes: widen the box instead of adding a level
            box *= 2.0;
            if (box > 1e6 * h) break;
            continue;
        }
        c.n = na;
        c.mem_ptr.assign(na + 1, 0);
        for (int i = 0; i < n; ++i) ++c.mem_ptr[c.agg_of[i] + 1];
        for (int a = 0; a < na; ++a) c.mem_ptr[a + 1] += c.mem_ptr[a];
        c.mem.resize(n);
        {
            std::vector<int> fill(c.mem_ptr.begin(), c.mem_ptr.end() - 1);
            for (int i = 0; i < n; ++i) c.mem[fill[c.agg_of[i]]++] = i;
        }
        mg_detail::galerkin_pattern(n, f.S.rp.data(), f.S.ci.data(), c.agg_of, na, c.S);
        std::vector<double> cp(3 * (size_t)na, 0.0);
        std::vector<int> cc(na, 0);
        for (int a = 0; a < na; ++a) {
            for (int k = c.mem_ptr[a]; k < c.mem_ptr[a + 1]; ++k)
                for (int d = 0; d < 3; ++d) cp[3 * a + d] += pos[3 * c.mem[k] + d];
            for (int d = 0; d < 3; ++d) cp[3 * a + d] /= (double)(c.mem_ptr[a + 1] - c.mem_ptr[a]);
            cc[a] = ncomp[c.mem[c.mem_ptr[a]]];
        }
        // level 1: an aggregate of vertices on one line (one or two vertices, or collinear ones)
        // has a rank-deficient rotation block (the rotation about that line moves nothing); it
        // keeps its translations only, so that its rotation rows of every coarse matrix are
        // exactly zero instead of rounding noise
        if (P.L.size() == 1) {
            c.rot.assign(na, 1);
            for (int a = 0; a < na; ++a) {
                double far2 = 0.0, u[3] = {0.0, 0.0, 0.0};
                for (int k = c.mem_ptr[a]; k < c.mem_ptr[a + 1]; ++k) {
                    double dv[3], d2 = 0.0;
                    for (int q = 0; q < 3; ++q) {
                        dv[q] = pos[3 * c.mem[k] + q] - cp[3 * a + q];
                        d2 += dv[q] * dv[q];
                    }
                    if (d2 > far2) {
                        far2 = d2;
                        for (int q = 0; q < 3; ++q) u[q] = dv[q];
                    }
                }
                double perp2 = 0.0;
                if (far2 > 0.0)
                    for (int k = c.mem_ptr[a]; k < c.mem_ptr[a + 1]; ++k) {
                        double dv[3];
                        for (int q = 0; q < 3; ++q) dv[q] = pos[3 * c.mem[k] + q] - cp[3 * a + q];
                        const double x = dv[1] * u[2] - dv[2] * u[1], y = dv[2] * u[0] - dv[0] * u[2], z = dv[0] * u[1] - dv[1] * u[0];
                        perp2 = std::max(perp2, (x * x + y * y + z * z) / far2);   // squared distance from the line
                    }
                if (!(perp2 > 1e-12 * far2)) c.rot[a] = 0;
            }
        }
        pos.swap(cp);
        ncomp.swap(cc);
        P.L.push_back(std::move(c));
        box *= 2.0;
    }
    P.levels = (int)P.L.size();
}

// Per-level contact patterns from the system's contact block pattern (crp, cci over vertices;
// null or empty: no contact).  Level 0's contact pattern is the system's own.
inline void mg_contact(MgPlan& P, int nV, const int* crp, const int* cci) {
    MgLevelPlan& l0 = P.L[0];
    l0.C = MgPattern();
    if (crp && crp[nV] > 0) {
        l0.C.rp.assign(crp, crp + nV + 1);
        l0.C.ci.assign(cci, cci + crp[nV]);
    }
    for (int l = 1; l < P.levels; ++l) {
        const MgLevelPlan& f = P.L[l - 1];
        MgLevelPlan& c = P.L[l];
        c.C = MgPattern();
        if (f.C.nnz() == 0) continue;
        mg_detail::galerkin_pattern(f.n, f.C.rp.data(), f.C.ci.data(), c.agg_of, c.n, c.C);
    }
}

}  // namespace fipc
