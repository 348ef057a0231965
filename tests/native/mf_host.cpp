// Host restatement of the multifrontal direct solve's numeric phase, driven by the product's own
// analysis (fastipc_gb300/csrc/mf_plan.h) and task tables, one task at a time in the order the
// GPU launches them.  Test infrastructure only: it checks the plan (ordering, structures,
// extend-add maps, scatter destinations, task decoding) against a reference sparse solve on the
// CPU before any device run.
#include <cmath>
#include <cstdio>
#include <vector>

#include "../../fastipc_gb300/csrc/mf_plan.h"

using namespace fipc;

namespace {

struct Front {
    double* F;
    int N, P;
    double& at(int i, int j) { return F[i + (long long)j * N]; }
};

Front front(MfPlan& P, std::vector<double>& buf, int f) {
    return Front{buf.data() + P.foff[f], 3 * P.nvf[f], 3 * P.npiv[f]};
}

}  // namespace

extern "C" {

// The analysis alone: info[0..5] = nodes, front doubles, flops, max height, largest front
// (vertices), panels.  Returns 0 or 1 (analysis failed).
int mf_host_analyse(int nV, const int* rp, const int* ci, const int* crp, const int* cci, const unsigned char* fixed, const double* x,
                    double* info) {
    MfPlan P;
    if (mf_analyse(nV, rp, ci, crp, cci, fixed, x, P)) return 1;
    int big = 0;
    for (int f = 0; f < P.n_nodes; ++f) big = P.nvf[f] > big ? P.nvf[f] : big;
    info[0] = P.n_nodes;
    info[1] = (double)P.f_total;
    info[2] = P.flops;
    info[3] = P.height_max;
    info[4] = big;
    info[5] = (double)P.panels.size();
    return 0;
}

// Solves the Dirichlet-edited block system; blocks (rp, ci, ev) and (crp, cci, cv) in vertex
// BSR, values row-major per 3x3 block.  info[0..4]: nodes, front doubles, flops, max height,
// largest front (vertices).  Returns 0, 1 (analysis failed) or 2 (non-positive pivot).
int mf_host_solve(int nV, const int* rp, const int* ci, const double* ev, const int* crp, const int* cci, const double* cv,
                  const unsigned char* fixed, const double* x, const double* rhs, double* sol, double* info) {
    MfPlan P;
    if (mf_analyse(nV, rp, ci, crp, cci, fixed, x, P)) return 1;
    int big = 0;
    for (int f = 0; f < P.n_nodes; ++f) big = P.nvf[f] > big ? P.nvf[f] : big;
    info[0] = P.n_nodes;
    info[1] = (double)P.f_total;
    info[2] = P.flops;
    info[3] = P.height_max;
    info[4] = big;
    std::vector<double> buf(P.f_total, 0.0);
    // scatter: elastic blocks, then contact blocks added
    for (long long k = 0; k < (long long)P.e_dst.size(); ++k) {
        if (P.e_dst[k] < 0) continue;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) buf[P.e_dst[k] + a + (long long)b * P.e_ld[k]] = ev[9 * k + 3 * a + b];
    }
    for (long long k = 0; k < (long long)P.c_dst.size(); ++k) {
        if (P.c_dst[k] < 0) continue;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) buf[P.c_dst[k] + a + (long long)b * P.c_ld[k]] += cv[9 * k + 3 * a + b];
    }
    int bad = 0;
    size_t pn = 0;
    for (int h = 0; h <= P.height_max; ++h) {
        // extend-add (pull): every lower entry of each front gathers its children's updates in order
        for (int q = P.lvl0[h]; q < P.lvl0[h + 1]; ++q) {
            const int f = P.level_nodes[q];
            Front Fp = front(P, buf, f);
            for (int j = 0; j < Fp.N; ++j)
                for (int i = j; i < Fp.N; ++i) {
                    double v = 0.0;
                    for (int e = P.child0[f]; e < P.child0[f + 1]; ++e) {
                        const int c = P.children[e];
                        const int* m = P.cmap.data() + P.cmap0[c];
                        const int ci_ = m[i / 3], cj = m[j / 3];
                        if (ci_ < 0 || cj < 0) continue;
                        Front Fc = front(P, buf, c);
                        v += Fc.at(3 * ci_ + i % 3, 3 * cj + j % 3);
                    }
                    Fp.at(i, j) += v;
                }
        }
        // panels of this height, in order
        for (; pn < P.panels.size() && P.panels[pn].height == h; ++pn) {
            const MfPlan::Panel& pl = P.panels[pn];
            const long long* ch0 = P.task_chunk0.data() + P.task_off[pn];
            const long long* tl0 = P.task_tile0.data() + P.task_off[pn];
            // diagonal tiles
            for (int e = 0; e < pl.n_fronts; ++e) {
                Front Fr = front(P, buf, P.task_front[pl.t0 + e]);
                const int c0 = pl.k * MF_TILE, kb = std::min(MF_TILE, Fr.P - c0);
                for (int j = 0; j < kb; ++j) {
                    double d = Fr.at(c0 + j, c0 + j);
                    if (!(d > 0.0) || !std::isfinite(d)) {
                        bad = 1;
                        d = 1.0;
                    }
                    d = std::sqrt(d);
                    Fr.at(c0 + j, c0 + j) = d;
                    for (int i = j + 1; i < kb; ++i) Fr.at(c0 + i, c0 + j) /= d;
                    for (int l = j + 1; l < kb; ++l)
                        for (int i = l; i < kb; ++i) Fr.at(c0 + i, c0 + l) -= Fr.at(c0 + i, c0 + j) * Fr.at(c0 + l, c0 + j);
                }
            }
            // row chunks: X L^T = B, right-looking over the panel's columns
            for (long long t = 0; t < pl.n_chunks; ++t) {
                const int e = mf_find(ch0, pl.n_fronts + 1, t);
                Front Fr = front(P, buf, P.task_front[pl.t0 + e]);
                const int c0 = pl.k * MF_TILE, kb = std::min(MF_TILE, Fr.P - c0);
                const int r0 = c0 + kb + (int)(t - ch0[e]) * MF_TILE, r1 = std::min(r0 + MF_TILE, Fr.N);
                for (int j = 0; j < kb; ++j) {
                    const double d = Fr.at(c0 + j, c0 + j);
                    for (int r = r0; r < r1; ++r) Fr.at(r, c0 + j) /= d;
                    for (int l = j + 1; l < kb; ++l)
                        for (int r = r0; r < r1; ++r) Fr.at(r, c0 + l) -= Fr.at(r, c0 + j) * Fr.at(c0 + l, c0 + j);
                }
            }
            // trailing tiles: C -= A_i A_j^T over the panel's columns
            for (long long t = 0; t < pl.n_tiles; ++t) {
                const int e = mf_find(tl0, pl.n_fronts + 1, t);
                Front Fr = front(P, buf, P.task_front[pl.t0 + e]);
                const int c0 = pl.k * MF_TILE, kb = std::min(MF_TILE, Fr.P - c0), s0 = c0 + kb;
                int ti, tj;
                mf_tile(t - tl0[e], &ti, &tj);
                const int i0 = s0 + ti * MF_TILE, j0 = s0 + tj * MF_TILE;
                for (int j = j0; j < std::min(j0 + MF_TILE, Fr.N); ++j)
                    for (int i = i0; i < std::min(i0 + MF_TILE, Fr.N); ++i) {
                        double acc = 0.0;
                        for (int l = 0; l < kb; ++l) acc += Fr.at(i, c0 + l) * Fr.at(j, c0 + l);
                        Fr.at(i, j) -= acc;
                    }
            }
        }
    }
    // forward: w = L^-1 b through the tree; backward: x = L^-T w
    std::vector<double> w(P.w_total, 0.0);
    for (int h = 0; h <= P.height_max; ++h)
        for (int q = P.lvl0[h]; q < P.lvl0[h + 1]; ++q) {
            const int f = P.level_nodes[q];
            Front Fr = front(P, buf, f);
            double* wf = w.data() + P.woff[f];
            for (int i = 0; i < Fr.N; ++i) {
                const int I = i / 3;
                double v = I < P.npiv[f] ? rhs[3 * P.order[P.piv0[f] + I] + i % 3] : 0.0;
                for (int e = P.child0[f]; e < P.child0[f + 1]; ++e) {
                    const int c = P.children[e];
                    const int m = P.cmap[P.cmap0[c] + I];
                    if (m >= 0) v += w[P.woff[c] + 3 * m + i % 3];
                }
                wf[i] = v;
            }
            for (int j = 0; j < Fr.P; ++j) {
                wf[j] /= Fr.at(j, j);
                for (int i = j + 1; i < Fr.N; ++i) wf[i] -= Fr.at(i, j) * wf[j];
            }
        }
    for (int i = 0; i < 3 * nV; ++i) sol[i] = 0.0;
    for (int h = P.height_max; h >= 0; --h)
        for (int q = P.lvl0[h]; q < P.lvl0[h + 1]; ++q) {
            const int f = P.level_nodes[q];
            Front Fr = front(P, buf, f);
            double* wf = w.data() + P.woff[f];
            const int* fl = P.fidx.data() + P.fidx0[f];
            for (int i = Fr.P; i < Fr.N; ++i) wf[i] = sol[3 * P.order[fl[i / 3]] + i % 3];
            for (int j = 0; j < Fr.P; ++j)
                for (int i = Fr.P; i < Fr.N; ++i) wf[j] -= Fr.at(i, j) * wf[i];
            for (int j = Fr.P - 1; j >= 0; --j) {
                double v = wf[j];
                for (int i = j + 1; i < Fr.P; ++i) v -= Fr.at(i, j) * wf[i];
                wf[j] = v / Fr.at(j, j);
            }
            for (int j = 0; j < Fr.P; ++j) sol[3 * P.order[P.piv0[f] + j / 3] + j % 3] = wf[j];
        }
    return bad ? 2 : 0;
}

}  // extern "C"
