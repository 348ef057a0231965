// Host-side analysis for the multifrontal Cholesky factorisation of the Newton system (the
// direct solve that stands in for the reference's CHOLMOD call, NEWTON_IPC.py:764-776).
//
// Everything here works on vertices: each vertex owns three consecutive DOFs, so every index
// below is a vertex and every matrix entry a 3x3 block.  Dirichlet vertices (fixed[v] != 0) have
// an identity row and column in the edited system, so they are left out: their solution is 0.
//
//  * Ordering: geometric nested dissection of the free vertices.  A set of more than LEAF
//    vertices is split at the median of its longest bounding-box axis; the vertices of the lower
//    half that have a neighbour in the upper half form the separator, which is ordered after both
//    halves.  Contact blocks are part of the adjacency, so the separators respect them.
//  * Assembly tree: one node per leaf set or separator, in postorder (children first).  The
//    pivots of a node are its vertices (consecutive positions in the ordering); its structure is
//    the set of later vertices coupled to its subtree, and its frontal matrix is dense over
//    [pivots, structure] (no amalgamation of the pivots' own sparsity: a separator's block is
//    dense).
//  * Numeric schedule: nodes are grouped by height (0 for nodes without children); all nodes of
//    one height are independent.  A front is factored in panels of MF_TILE scalar columns; the
//    task tables below list, per (height, panel), the fronts that have that panel and the
//    prefix sums of their row chunks (triangular solve) and of their trailing-update tiles.
//
// Plain C++ with no CUDA types, so that the same analysis compiles into the CPU tests.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace fipc {

// the entry e of a prefix array pre[0..n] (pre[0] = 0, non-decreasing) with pre[e] <= q <
// pre[e + 1], for q < pre[n]
FIPC_HD int mf_find(const long long* pre, int n, long long q) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pre[mid] <= q) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// lower-triangular tile number t -> (ti, tj) with ti >= tj and t = ti (ti + 1) / 2 + tj
FIPC_HD void mf_tile(long long t, int* ti, int* tj) {
    long long i = (long long)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (i * (i + 1) / 2 > t) --i;
    while ((i + 1) * (i + 2) / 2 <= t) ++i;
    *ti = (int)i;
    *tj = (int)(t - i * (i + 1) / 2);
}

constexpr int MF_TILE = 64;     // panel width and trailing-update tile (scalar rows / columns)
constexpr int MF_LEAF = 48;     // largest vertex set ordered without further dissection

struct MfPlan {
    int nV = 0, n_free = 0;
    std::vector<int> order;      // order[k]: the vertex at position k (free vertices only)
    std::vector<int> pos;        // pos[v]: position of vertex v, -1 for fixed vertices
    // nodes in postorder
    int n_nodes = 0, height_max = -1;
    std::vector<int> piv0, npiv;            // pivot positions [piv0, piv0 + npiv)
    std::vector<int> nvf;                   // front size in vertices (pivots + structure)
    std::vector<long long> fidx0;           // front f's vertex positions: fidx[fidx0[f] .. + nvf[f])
    std::vector<int> fidx;
    std::vector<int> parent, height;
    std::vector<int> child0, children;      // children of f: children[child0[f] .. child0[f+1])
    std::vector<long long> foff;            // front f: doubles [foff, foff + N^2), N = 3 nvf, column-major
    std::vector<long long> woff;            // front f's vector in the solve: [woff, woff + N)
    long long f_total = 0, w_total = 0;
    // extend-add: for child c of parent p, cmap[cmap0[c] + I] = index of the parent's front
    // vertex I in c's front, or -1 (I < nvf[p])
    std::vector<long long> cmap0;
    std::vector<int> cmap;
    // nodes of each height, and for each node its rank there: level_nodes[lvl0[h] .. lvl0[h+1])
    std::vector<int> lvl0, level_nodes;
    // per (height, panel) task table: fronts that have the panel, with prefix sums of their
    // row chunks (MF_TILE rows below the diagonal tile) and of their lower trailing tiles
    struct Panel {
        int height, k;                      // k: panel index (columns [k MF_TILE, ...))
        long long t0;                       // start of this panel's entries in the task arrays
        int n_fronts;
        long long n_chunks, n_tiles;
    };
    std::vector<Panel> panels;
    std::vector<int> task_front;            // [n_fronts] per panel
    std::vector<long long> task_chunk0;     // [n_fronts + 1] per panel (prefix of row chunks)
    std::vector<long long> task_tile0;      // [n_fronts + 1] per panel (prefix of trailing tiles)
    std::vector<long long> task_off;        // start of panel p's prefix arrays (n_fronts + 1 each)
    // the system's blocks: destination of block b's (0, 0) entry in the front buffer (-1: not
    // stored, an upper-triangle or Dirichlet block) and the leading dimension there
    std::vector<long long> e_dst, c_dst;
    std::vector<int> e_ld, c_ld;
    double flops = 0;                       // factorisation flops (dense fronts)
};

namespace mf_detail {

struct Builder {
    const std::vector<int>& adj0;
    const std::vector<int>& adj;
    const double* x;
    MfPlan& P;
    std::vector<int> stamp;
    int next_stamp = 1;
    int next_pos = 0;
    std::vector<std::vector<int>> kids;     // children per node during construction

    Builder(const std::vector<int>& a0, const std::vector<int>& a, const double* xx, MfPlan& p)
        : adj0(a0), adj(a), x(xx), P(p), stamp(p.nV, 0) {}

    int new_node(const int* v, int n, std::vector<int> ch) {
        const int id = P.n_nodes++;
        P.piv0.push_back(next_pos);
        P.npiv.push_back(n);
        for (int i = 0; i < n; ++i) {
            P.order[next_pos] = v[i];
            P.pos[v[i]] = next_pos++;
        }
        kids.push_back(std::move(ch));
        return id;
    }

    // nested dissection of v[0..n); returns the node id of the subtree's root (-1 if n == 0)
    int build(int* v, int n) {
        if (n == 0) return -1;
        if (n <= MF_LEAF) return new_node(v, n, {});
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (int i = 0; i < n; ++i)
            for (int d = 0; d < 3; ++d) {
                lo[d] = std::min(lo[d], x[3 * v[i] + d]);
                hi[d] = std::max(hi[d], x[3 * v[i] + d]);
            }
        int ax = 0;
        for (int d = 1; d < 3; ++d)
            if (hi[d] - lo[d] > hi[ax] - lo[ax]) ax = d;
        const int h = n / 2;
        std::nth_element(v, v + h, v + n, [&](int a, int b) {
            const double xa = x[3 * a + ax], xb = x[3 * b + ax];
            return xa < xb || (xa == xb && a < b);
        });
        const int s = next_stamp++;
        for (int i = h; i < n; ++i) stamp[v[i]] = s;
        // separator: lower-half vertices with an upper-half neighbour, moved to the end of the
        // lower half (stable order inside both parts)
        std::vector<int> keep, sep;
        keep.reserve(h);
        for (int i = 0; i < h; ++i) {
            const int a = v[i];
            bool cut = false;
            for (int k = adj0[a]; k < adj0[a + 1] && !cut; ++k) cut = stamp[adj[k]] == s;
            (cut ? sep : keep).push_back(a);
        }
        for (int i = h; i < n; ++i) stamp[v[i]] = 0;
        std::copy(keep.begin(), keep.end(), v);
        std::copy(sep.begin(), sep.end(), v + keep.size());
        const int nk = (int)keep.size();
        std::vector<int> ch;
        const int a = build(v, nk);
        if (a >= 0) ch.push_back(a);
        const int b = build(v + h, n - h);
        if (b >= 0) ch.push_back(b);
        return new_node(v + nk, (int)sep.size(), std::move(ch));
    }
};

inline long long tri_tiles(long long rows) {
    const long long t = (rows + MF_TILE - 1) / MF_TILE;
    return t * (t + 1) / 2;
}

}  // namespace mf_detail

// Builds the plan.  Patterns are block CSR over vertices (any order of columns inside a row;
// both triangles present): the elastic + inertia pattern (rp, ci) and the contact pattern (crp,
// cci, may be empty).  x: vertex positions [nV][3].  Returns 0, or 1 when the structure check
// fails (a coupling between sibling subtrees, which the dissection rules out).
inline int mf_analyse(int nV, const int* rp, const int* ci, const int* crp, const int* cci, const unsigned char* fixed,
                      const double* x, MfPlan& P) {
    P = MfPlan();
    P.nV = nV;
    P.pos.assign(nV, -1);
    // adjacency of the free vertices (union of both patterns, no self loops)
    std::vector<int> deg(nV + 1, 0);
    auto count = [&](const int* r, const int* c) {
        if (!r) return;
        for (int i = 0; i < nV; ++i) {
            if (fixed[i]) continue;
            for (int k = r[i]; k < r[i + 1]; ++k)
                if (c[k] != i && !fixed[c[k]]) ++deg[i + 1];
        }
    };
    count(rp, ci);
    count(crp, cci);
    std::vector<int> adj0(nV + 1, 0);
    for (int i = 0; i < nV; ++i) adj0[i + 1] = adj0[i] + deg[i + 1];
    std::vector<int> adj(adj0[nV]);
    {
        std::vector<int> fill(adj0.begin(), adj0.end() - 1);
        auto put = [&](const int* r, const int* c) {
            if (!r) return;
            for (int i = 0; i < nV; ++i) {
                if (fixed[i]) continue;
                for (int k = r[i]; k < r[i + 1]; ++k)
                    if (c[k] != i && !fixed[c[k]]) adj[fill[i]++] = c[k];
            }
        };
        put(rp, ci);
        put(crp, cci);
    }
    std::vector<int> verts;
    for (int i = 0; i < nV; ++i)
        if (!fixed[i]) verts.push_back(i);
    P.n_free = (int)verts.size();
    P.order.assign(P.n_free, -1);
    mf_detail::Builder B(adj0, adj, x, P);
    B.build(verts.data(), (int)verts.size());
    const int nn = P.n_nodes;
    P.parent.assign(nn, -1);
    P.child0.assign(nn + 1, 0);
    for (int f = 0; f < nn; ++f) P.child0[f + 1] = P.child0[f] + (int)B.kids[f].size();
    for (int f = 0; f < nn; ++f)
        for (int c : B.kids[f]) {
            P.children.push_back(c);
            P.parent[c] = f;
        }
    // structure, bottom-up (postorder ids: children have smaller ids)
    std::vector<std::vector<int>> st(nn);
    P.height.assign(nn, 0);
    P.nvf.assign(nn, 0);
    std::vector<int> mark(P.n_free, -1);
    for (int f = 0; f < nn; ++f) {
        const int e0 = P.piv0[f] + P.npiv[f];   // first position after the pivots
        std::vector<int>& s = st[f];
        for (int k = P.piv0[f]; k < e0; ++k) {
            const int v = P.order[k];
            for (int q = adj0[v]; q < adj0[v + 1]; ++q) {
                const int u = P.pos[adj[q]];
                if (u >= e0 && mark[u] != f) {
                    mark[u] = f;
                    s.push_back(u);
                }
            }
        }
        for (int q = P.child0[f]; q < P.child0[f + 1]; ++q) {
            const int c = P.children[q];
            P.height[f] = std::max(P.height[f], P.height[c] + 1);
            for (int u : st[c]) {
                if (u >= P.piv0[f] && u < e0) continue;
                if (u < e0) return 1;               // a sibling subtree: cannot happen
                if (mark[u] != f) {
                    mark[u] = f;
                    s.push_back(u);
                }
            }
        }
        std::sort(s.begin(), s.end());
        P.nvf[f] = P.npiv[f] + (int)s.size();
        P.height_max = std::max(P.height_max, P.height[f]);
    }
    // front vertex lists and buffer offsets
    P.fidx0.assign(nn + 1, 0);
    P.foff.assign(nn + 1, 0);
    P.woff.assign(nn + 1, 0);
    for (int f = 0; f < nn; ++f) {
        P.fidx0[f + 1] = P.fidx0[f] + P.nvf[f];
        const long long N = 3ll * P.nvf[f];
        // fronts start on 32-double (256-byte) boundaries
        P.foff[f + 1] = P.foff[f] + ((N * N + 31) / 32) * 32;
        P.woff[f + 1] = P.woff[f] + ((N + 31) / 32) * 32;
        const double p = 3.0 * P.npiv[f], m = N - p;
        P.flops += p * p * p / 3 + p * p * m + p * m * m;
    }
    P.f_total = P.foff[nn];
    P.w_total = P.woff[nn];
    P.fidx.resize(P.fidx0[nn]);
    for (int f = 0; f < nn; ++f) {
        int* o = P.fidx.data() + P.fidx0[f];
        for (int k = 0; k < P.npiv[f]; ++k) o[k] = P.piv0[f] + k;
        std::copy(st[f].begin(), st[f].end(), o + P.npiv[f]);
    }
    // extend-add maps (both lists ascending: merge)
    P.cmap0.assign(nn + 1, 0);
    for (int c = 0; c < nn; ++c) P.cmap0[c + 1] = P.cmap0[c] + (P.parent[c] >= 0 ? P.nvf[P.parent[c]] : 0);
    P.cmap.assign(P.cmap0[nn], -1);
    for (int c = 0; c < nn; ++c) {
        const int p = P.parent[c];
        if (p < 0) continue;
        const int* pf = P.fidx.data() + P.fidx0[p];
        const int* cf = P.fidx.data() + P.fidx0[c];
        int* m = P.cmap.data() + P.cmap0[c];
        int j = P.npiv[c];
        for (int I = 0; I < P.nvf[p] && j < P.nvf[c]; ++I) {
            while (j < P.nvf[c] && cf[j] < pf[I]) ++j;
            if (j < P.nvf[c] && cf[j] == pf[I]) m[I] = j;
        }
    }
    // nodes by height
    P.lvl0.assign(P.height_max + 2, 0);
    for (int f = 0; f < nn; ++f) ++P.lvl0[P.height[f] + 1];
    for (int h = 0; h <= P.height_max; ++h) P.lvl0[h + 1] += P.lvl0[h];
    P.level_nodes.assign(nn, 0);
    {
        std::vector<int> fill(P.lvl0.begin(), P.lvl0.end() - 1);
        for (int f = 0; f < nn; ++f) P.level_nodes[fill[P.height[f]]++] = f;
    }
    // panel task tables
    for (int h = 0; h <= P.height_max; ++h) {
        int maxp = 0;
        for (int q = P.lvl0[h]; q < P.lvl0[h + 1]; ++q) {
            const int f = P.level_nodes[q];
            maxp = std::max(maxp, (3 * P.npiv[f] + MF_TILE - 1) / MF_TILE);
        }
        for (int k = 0; k < maxp; ++k) {
            MfPlan::Panel pn{h, k, (long long)P.task_front.size(), 0, 0, 0};
            P.task_off.push_back((long long)P.task_chunk0.size());
            long long ch = 0, tl = 0;
            P.task_chunk0.push_back(0);
            P.task_tile0.push_back(0);
            for (int q = P.lvl0[h]; q < P.lvl0[h + 1]; ++q) {
                const int f = P.level_nodes[q];
                const int p = 3 * P.npiv[f], N = 3 * P.nvf[f];
                if (p <= k * MF_TILE) continue;
                const int kb = std::min(MF_TILE, p - k * MF_TILE);
                const long long below = N - (long long)k * MF_TILE - kb;
                ch += (below + MF_TILE - 1) / MF_TILE;
                tl += mf_detail::tri_tiles(below);
                P.task_front.push_back(f);
                P.task_chunk0.push_back(ch);
                P.task_tile0.push_back(tl);
                ++pn.n_fronts;
            }
            pn.n_chunks = ch;
            pn.n_tiles = tl;
            P.panels.push_back(pn);
        }
    }
    // scatter destinations of the system's blocks
    std::vector<int> node_of(P.n_free, -1);
    for (int f = 0; f < nn; ++f)
        for (int k = 0; k < P.npiv[f]; ++k) node_of[P.piv0[f] + k] = f;
    auto dst = [&](const int* r, const int* c, std::vector<long long>& d, std::vector<int>& ld) {
        if (!r) return 0;
        const long long nb = r[nV];
        d.assign(nb, -1);
        ld.assign(nb, 0);
        for (int i = 0; i < nV; ++i) {
            if (fixed[i]) continue;
            const int pi = P.pos[i];
            for (int k = r[i]; k < r[i + 1]; ++k) {
                const int j = c[k];
                if (fixed[j]) continue;
                const int pj = P.pos[j];
                if (pi < pj) continue;              // upper triangle: its transpose is stored
                const int f = node_of[pj];
                const int* fl = P.fidx.data() + P.fidx0[f];
                const int col = pj - P.piv0[f];
                int row;
                if (pi < P.piv0[f] + P.npiv[f]) {
                    row = pi - P.piv0[f];
                } else {
                    const int* e = std::lower_bound(fl + P.npiv[f], fl + P.nvf[f], pi);
                    if (e == fl + P.nvf[f] || *e != pi) return 1;
                    row = (int)(e - fl);
                }
                const long long N = 3ll * P.nvf[f];
                d[k] = P.foff[f] + 3ll * row + 3ll * col * N;
                ld[k] = (int)N;
            }
        }
        return 0;
    };
    if (dst(rp, ci, P.e_dst, P.e_ld)) return 1;
    if (dst(crp, cci, P.c_dst, P.c_ld)) return 1;
    return 0;
}

}  // namespace fipc
