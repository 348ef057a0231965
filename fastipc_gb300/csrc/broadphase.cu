// Sort-based spatial hash and the three queries built on it: constraint finding
// (NEWTON_IPC.py:181-357), the CCD step filter (NEWTON_IPC.py:377-468) and the
// intersection check (NEWTON_IPC.py:855-886).
//
// The grid keeps the reference's box conventions, with the median boundary edge as its cell.
// The reference uses the mean; enumeration is complete for any cell size, so the lists are the
// same.  What the reference appends to its sparse grid becomes (cell key, id) pairs,
// radix-sorted by key; unique keys and run starts give each cell's id range, found through an
// open-addressing table.  A candidate pair whose two cell ranges overlap in several cells is
// examined only in the overlap's lowest cell (componentwise max of the two lower corners), so
// every pair is tested once without a hash set.  The narrow phase applies the reference's exact
// predicates; constraint rows are then sorted lexicographically and de-duplicated per list
// exactly like np.unique(axis=0) (NEWTON_IPC.py:348-356).
#include <cooperative_groups.h>
#include <cub/cub.cuh>
#include <cuda_runtime.h>

#include "ccd.cuh"
#include "ctx.cuh"
#include "geometry.cuh"

namespace fipc {

namespace cg = cooperative_groups;

struct C3 {
    long long x, y, z;
};

__device__ __forceinline__ C3 cell_of(v3 p, double inv_dx) {
    return C3{(long long)floor(p.x * inv_dx), (long long)floor(p.y * inv_dx), (long long)floor(p.z * inv_dx)};
}
__device__ __forceinline__ C3 cmax(C3 a, C3 b) { return C3{a.x > b.x ? a.x : b.x, a.y > b.y ? a.y : b.y, a.z > b.z ? a.z : b.z}; }
__device__ __forceinline__ unsigned long long gkey(const SceneGeo& g, int s, long long cx, long long cy, long long cz) {
    return g.vscene ? cell_key_scene(s, cx, cy, cz) : cell_key(cx, cy, cz);
}
// first vertex of stored primitive i (its scene)
__device__ __forceinline__ int prim_vertex(int mode, int i, const int* __restrict__ prim) {
    return (mode == 0 || mode == 2) ? prim[i] : prim[2 * i];
}

// Box modes of stored primitives:
//  0 point [p - dh, p + dh]               (find constraints, point-triangle)
//  1 edge  [min, max]                      (find constraints, edge-edge)
//  2 moving point [min(p, p+dp) - dh, max + dh]   (CCD point-triangle)
//  3 moving edge  [min over 4 ends, max]           (CCD edge-edge)
//  4 edge  [min - dh, max + dh]            (intersection check)
__device__ __forceinline__ void stored_box(int mode, int i, const int* __restrict__ prim, const double* __restrict__ x,
                                           const double* __restrict__ p, double dh, v3* lo, v3* hi) {
    if (mode == 0 || mode == 2) {
        const v3 a = ld3(x, prim[i]);
        v3 mn = a, mx = a;
        if (mode == 2) {
            const v3 b = a + ld3(p, prim[i]);
            mn = vmin(a, b);
            mx = vmax(a, b);
        }
        *lo = mn - mk(dh, dh, dh);
        *hi = mx + mk(dh, dh, dh);
    } else {
        const v3 a = ld3(x, prim[2 * i]), b = ld3(x, prim[2 * i + 1]);
        v3 mn = vmin(a, b), mx = vmax(a, b);
        if (mode == 3) {
            const v3 a2 = a + ld3(p, prim[2 * i]), b2 = b + ld3(p, prim[2 * i + 1]);
            mn = vmin(mn, vmin(a2, b2));
            mx = vmax(mx, vmax(a2, b2));
        }
        if (mode == 4) {
            mn = mn - mk(dh, dh, dh);
            mx = mx + mk(dh, dh, dh);
        }
        *lo = mn;
        *hi = mx;
    }
}

constexpr long long MAX_CELLS_PER_PRIM = 1ll << 22;

__global__ void k_cell_count(int mode, int n, const int* __restrict__ prim, const double* __restrict__ x,
                             const double* __restrict__ p, double dh, SceneGeo g, long long* __restrict__ cnt,
                             int* __restrict__ overflow) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double inv_dx = g.idx(g.scene(prim_vertex(mode, i, prim)));
    if (mode != 0 && mode != 2 && g.big_edge && g.big_edge[i]) {   // handled by the big-primitive pass
        cnt[i] = 0;
        return;
    }
    v3 lo, hi;
    stored_box(mode, i, prim, x, p, dh, &lo, &hi);
    const C3 a = cell_of(lo, inv_dx), b = cell_of(hi, inv_dx);
    long long c = (b.x - a.x + 1) * (b.y - a.y + 1) * (b.z - a.z + 1);
    if (!(c > 0 && c <= MAX_CELLS_PER_PRIM)) {
        atomicOr(overflow, 1);
        c = 0;
    }
    cnt[i] = c;
}

__global__ void k_cell_emit(int mode, int n, const int* __restrict__ prim, const double* __restrict__ x,
                            const double* __restrict__ p, double dh, SceneGeo g, const long long* __restrict__ off,
                            const long long* __restrict__ cnt, unsigned long long* __restrict__ keys, int* __restrict__ ids) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || cnt[i] == 0) return;
    const int sc = g.scene(prim_vertex(mode, i, prim));
    const double inv_dx = g.idx(sc);
    v3 lo, hi;
    stored_box(mode, i, prim, x, p, dh, &lo, &hi);
    const C3 a = cell_of(lo, inv_dx), b = cell_of(hi, inv_dx);
    long long o = off[i];
    for (long long cx = a.x; cx <= b.x; ++cx)
        for (long long cy = a.y; cy <= b.y; ++cy)
            for (long long cz = a.z; cz <= b.z; ++cz) {
                keys[o] = gkey(g, sc, cx, cy, cz);
                ids[o] = i;
                ++o;
            }
}

// Candidate records of the stored primitives, built with the grid, so that the query kernels
// reject most candidates without FP64 work (GB300 issues FP64 at a small fraction of its FP32
// rate):
//  * cell: cell_of(stored lower corner), the first-cell test of the queries' pair
//    de-duplication, computed with the same FP64 expression;
//  * box: an FP32 box rounded outward around the FP64 box that the query's own FP64 test
//    compares against: mode 0 the point; 1 and 3 the (moving) edge box +- dh (ee_aabb,
//    ee_aabb_moving); 2 the moving point's box (pt_aabb_moving); 4 the edge box +- dh (the
//    intersection check, whose segment-triangle test cannot hit a triangle whose box is dh
//    away).  A candidate whose FP32 box misses the query's FP32 box (also rounded outward)
//    fails the FP64 test too, so the lists, steps and flags are unchanged.
__device__ __forceinline__ float4 f32_lo(v3 a) {
    return make_float4(__double2float_rd(a.x), __double2float_rd(a.y), __double2float_rd(a.z), 0.f);
}
__device__ __forceinline__ float4 f32_hi(v3 a) {
    return make_float4(__double2float_ru(a.x), __double2float_ru(a.y), __double2float_ru(a.z), 0.f);
}
__device__ __forceinline__ bool f32_overlap(float4 alo, float4 ahi, float4 blo, float4 bhi) {
    return alo.x < bhi.x && alo.y < bhi.y && alo.z < bhi.z && blo.x < ahi.x && blo.y < ahi.y && blo.z < ahi.z;
}
__device__ __forceinline__ int clamp_cell(long long c) {
    return (int)(c < -(1ll << 30) ? -(1ll << 30) : (c > (1ll << 30) ? (1ll << 30) : c));
}

__global__ void k_cand_records(int mode, int n, const int* __restrict__ prim, const double* __restrict__ x,
                               const double* __restrict__ p, double dh, SceneGeo g, int4* __restrict__ cell,
                               float4* __restrict__ box) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double inv_dx = g.idx(g.scene(prim_vertex(mode, i, prim)));
    v3 lo, hi;
    stored_box(mode, i, prim, x, p, dh, &lo, &hi);
    const C3 c = cell_of(lo, inv_dx);
    cell[i] = make_int4(clamp_cell(c.x), clamp_cell(c.y), clamp_cell(c.z), 0);
    const v3 d = mk(dh, dh, dh);
    v3 blo = lo, bhi = hi;
    if (mode == 0) {                      // the point itself
        blo = ld3(x, prim[i]);
        bhi = blo;
    } else if (mode == 2) {               // the moving point's box, without dh
        const v3 a = ld3(x, prim[i]), b = a + ld3(p, prim[i]);
        blo = vmin(a, b);
        bhi = vmax(a, b);
    } else if (mode == 1 || mode == 3) {  // edge box +- dh, as ee_aabb(_moving) forms it
        blo = lo - d;
        bhi = hi + d;
    }
    box[2 * (size_t)i] = f32_lo(blo);
    box[2 * (size_t)i + 1] = f32_hi(bhi);
}

struct CandView {
    const int4* cell;
    const float4* box;
};

// Cell lookup of a built grid: an open-addressing table (linear probing, load factor <= 1/2)
// maps each occupied cell key to its run of ids, so a query cell costs one or two probes instead
// of a binary search over all keys.  The table holds exactly the sorted grid's runs; which slot a
// key lands in depends on insertion order, the run it maps to does not.
constexpr unsigned long long HASH_EMPTY = ~0ull;
__device__ __forceinline__ unsigned long long mix64(unsigned long long k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}
struct GridView {
    const unsigned long long* hk;   // table keys
    const int* hv;                  // table values: run index
    unsigned long long mask;        // table size - 1
    const int* us;                  // run starts
    const int* ids;                 // primitive ids by run
    // run index of key, or -1 (at most mask + 1 probes)
    __device__ __forceinline__ int find(unsigned long long key) const {
        unsigned long long h = mix64(key) & mask;
        for (unsigned long long n = 0; n <= mask; ++n) {
            const unsigned long long k = __ldg(hk + h);
            if (k == key) return __ldg(hv + h);
            if (k == HASH_EMPTY) return -1;
            h = (h + 1) & mask;
        }
        return -1;
    }
};

// insert the nu unique keys (nu read on the device); a full table is impossible at load <= 1/2
__global__ void k_hash_insert(const unsigned long long* __restrict__ ukeys, const int* __restrict__ nu_p, unsigned long long* __restrict__ hk,
                              int* __restrict__ hv, unsigned long long mask) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= *nu_p) return;
    const unsigned long long key = ukeys[u];
    unsigned long long h = mix64(key) & mask;
    for (unsigned long long n = 0; n <= mask; ++n) {
        const unsigned long long prev = atomicCAS(hk + h, HASH_EMPTY, key);
        if (prev == HASH_EMPTY || prev == key) {
            hv[h] = u;
            return;
        }
        h = (h + 1) & mask;
    }
}

// lanes per edge-edge constraint, edge-edge CCD and intersection query: a few lanes share each
// cell's candidates.  One thread per query leaves most lanes idle in the FP64 narrow phase; a
// whole warp repeats the cell walk in every lane while most cells hold a handful of candidates.
// The point-triangle queries, whose cells hold fewer candidates, keep one thread per query.
constexpr int QG = 8;

// ---------------------------------------------------------------- constraint rows
struct RowSink {
    int4* rows[N_TYPES];
    int* counts;   // [N_TYPES + 1]; the last entry is the overflow flag
    int cap;
};
// Warp-aggregated emission: the lanes that reach this call together are partitioned by target
// list; one lane of each partition reserves the partition's rows with a single atomicAdd and
// every lane writes its row at base + its rank.  The lists are sorted and de-duplicated
// afterwards, so the order of the rows within a list does not matter.
__device__ __forceinline__ void emit(const RowSink& s, int t, int a, int b, int c, int d) {
    const cg::coalesced_group active = cg::coalesced_threads();
    const cg::coalesced_group same = cg::labeled_partition(active, t);
    int base = 0;
    if (same.thread_rank() == 0) base = atomicAdd(&s.counts[t], (int)same.size());
    base = same.shfl(base, 0);
    const int k = base + (int)same.thread_rank();
    if (k < s.cap) s.rows[t][k] = make_int4(a, b, c, d);
    else atomicOr(&s.counts[N_TYPES], 1);
}

// attempt_PT, NEWTON_IPC.py:181-212
__device__ void attempt_pt(const double* __restrict__ x, double dh, double dh2, int p, int t0, int t1, int t2, const RowSink& s) {
    if (p == t0 || p == t1 || p == t2) return;
    const v3 P = ld3(x, p), A = ld3(x, t0), B = ld3(x, t1), C = ld3(x, t2);
    if (!pt_aabb(P, A, B, C, dh)) return;
    switch (pt_type(P, A, B, C)) {
        case 0: if (d_PP(P, A) < dh2) emit(s, T_PP, p, t0, 0, 0); break;
        case 1: if (d_PP(P, B) < dh2) emit(s, T_PP, p, t1, 0, 0); break;
        case 2: if (d_PP(P, C) < dh2) emit(s, T_PP, p, t2, 0, 0); break;
        case 3: if (d_PE(P, A, B) < dh2) emit(s, T_PE, p, t0, t1, 0); break;
        case 4: if (d_PE(P, B, C) < dh2) emit(s, T_PE, p, t1, t2, 0); break;
        case 5: if (d_PE(P, C, A) < dh2) emit(s, T_PE, p, t2, t0, 0); break;
        default: if (d_PT(P, A, B, C) < dh2) emit(s, T_PT, p, t0, t1, t2); break;
    }
}

// attempt_EE, NEWTON_IPC.py:235-312
__device__ void attempt_ee(const double* __restrict__ x, const double* __restrict__ x0, double dh, double dh2, int a0, int a1, int b0,
                           int b1, const RowSink& s) {
    if (a0 == b0 || a0 == b1 || a1 == b0 || a1 == b1) return;
    const v3 A0 = ld3(x, a0), A1 = ld3(x, a1), B0 = ld3(x, b0), B1 = ld3(x, b1);
    if (!ee_aabb(A0, A1, B0, B1, dh)) return;
    // feature pair and its distance first; the mollifier switch (EECN2 < eps_x on the rest
    // shape) is needed only for pairs within d-hat, which is what gets emitted
    int t;
    double d2;
    switch (t = ee_type(A0, A1, B0, B1)) {
        case 0: d2 = d_PP(A0, B0); break;
        case 1: d2 = d_PP(A0, B1); break;
        case 2: d2 = d_PE(A0, B0, B1); break;
        case 3: d2 = d_PP(A1, B0); break;
        case 4: d2 = d_PP(A1, B1); break;
        case 5: d2 = d_PE(A1, B0, B1); break;
        case 6: d2 = d_PE(B0, A0, A1); break;
        case 7: d2 = d_PE(B1, A0, A1); break;
        default: d2 = d_EE(A0, A1, B0, B1); break;
    }
    if (!(d2 < dh2)) return;
    const bool m = d_EECN2(A0, A1, B0, B1) < m_threshold(ld3(x0, a0), ld3(x0, a1), ld3(x0, b0), ld3(x0, b1));
    switch (t) {
        case 0: if (m) emit(s, T_PPM, a0, a1, b0, b1); else emit(s, T_PP, a0, b0, 0, 0); break;
        case 1: if (m) emit(s, T_PPM, a0, a1, b1, b0); else emit(s, T_PP, a0, b1, 0, 0); break;
        case 2: if (m) emit(s, T_PEM, a0, a1, b0, b1); else emit(s, T_PE, a0, b0, b1, 0); break;
        case 3: if (m) emit(s, T_PPM, a1, a0, b0, b1); else emit(s, T_PP, a1, b0, 0, 0); break;
        case 4: if (m) emit(s, T_PPM, a1, a0, b1, b0); else emit(s, T_PP, a1, b1, 0, 0); break;
        case 5: if (m) emit(s, T_PEM, a1, a0, b0, b1); else emit(s, T_PE, a1, b0, b1, 0); break;
        case 6: if (m) emit(s, T_PEM, b0, b1, a0, a1); else emit(s, T_PE, b0, a0, a1, 0); break;
        case 7: if (m) emit(s, T_PEM, b1, b0, a0, a1); else emit(s, T_PE, b1, a0, a1, 0); break;
        default: if (m) emit(s, T_EEM, a0, a1, b0, b1); else emit(s, T_EE, a0, a1, b0, b1); break;
    }
}

// one thread per boundary triangle; points hashed with mode 0
__global__ void __launch_bounds__(128) k_find_pt(int nbt, const int* __restrict__ bt, const int* __restrict__ bp,
                                                 const double* __restrict__ x, double dh, double dh2, SceneGeo g,
                                                 GridView gv, CandView cv, RowSink sink) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nbt) return;
    if (g.big_tri && g.big_tri[i]) return;
    const int t0 = bt[3 * i], t1 = bt[3 * i + 1], t2 = bt[3 * i + 2];
    const int sc = g.scene(t0);
    const double inv_dx = g.idx(sc);
    const v3 A = ld3(x, t0), B = ld3(x, t1), C = ld3(x, t2);
    const v3 tmn = vmin(vmin(A, B), C), tmx = vmax(vmax(A, B), C);
    const C3 lo = cell_of(tmn, inv_dx), hi = cell_of(tmx, inv_dx);
    const v3 d = mk(dh, dh, dh);
    const float4 qlo = f32_lo(tmn - d), qhi = f32_hi(tmx + d);   // pt_aabb's triangle box
    for (long long cx = lo.x; cx <= hi.x; ++cx)
        for (long long cy = lo.y; cy <= hi.y; ++cy)
            for (long long cz = lo.z; cz <= hi.z; ++cz) {
                const int c = gv.find(gkey(g, sc, cx, cy, cz));
                if (c < 0) continue;
                for (int k = gv.us[c]; k < gv.us[c + 1]; ++k) {
                    const int j = gv.ids[k];
                    const int4 pc = __ldg(cv.cell + j);
                    const C3 first = cmax(lo, C3{pc.x, pc.y, pc.z});
                    if (first.x != cx || first.y != cy || first.z != cz) continue;
                    if (!f32_overlap(__ldg(cv.box + 2 * j), __ldg(cv.box + 2 * j + 1), qlo, qhi)) continue;
                    const int p = bp[j];
                    attempt_pt(x, dh, dh2, p, t0, t1, t2, sink);
                }
            }
}

// one thread per boundary edge (query, box +- dh); stored edges hashed with mode 1
__global__ void __launch_bounds__(128) k_find_ee(int nbe, const int* __restrict__ be, const double* __restrict__ x,
                                                 const double* __restrict__ x0, double dh, double dh2, SceneGeo g,
                                                 GridView gv, CandView cv, RowSink sink) {
    // QG lanes per query edge share the candidates of each cell
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) / QG, lane = threadIdx.x % QG;
    if (i >= nbe) return;
    if (g.big_edge && g.big_edge[i]) return;
    const int a0 = be[2 * i], a1 = be[2 * i + 1];
    const int sc = g.scene(a0);
    const double inv_dx = g.idx(sc);
    const v3 A0 = ld3(x, a0), A1 = ld3(x, a1);
    const v3 d = mk(dh, dh, dh);
    const C3 lo = cell_of(vmin(A0, A1) - d, inv_dx), hi = cell_of(vmax(A0, A1) + d, inv_dx);
    const float4 qlo = f32_lo(vmin(A0, A1)), qhi = f32_hi(vmax(A0, A1));   // ee_aabb's query edge box
    for (long long cx = lo.x; cx <= hi.x; ++cx)
        for (long long cy = lo.y; cy <= hi.y; ++cy)
            for (long long cz = lo.z; cz <= hi.z; ++cz) {
                const int c = gv.find(gkey(g, sc, cx, cy, cz));
                if (c < 0) continue;
                for (int k = gv.us[c] + lane; k < gv.us[c + 1]; k += QG) {
                    const int j = gv.ids[k];
                    if (!(i < j)) continue;
                    const int4 sc4 = __ldg(cv.cell + j);
                    const C3 first = cmax(lo, C3{sc4.x, sc4.y, sc4.z});
                    if (first.x != cx || first.y != cy || first.z != cz) continue;
                    if (!f32_overlap(__ldg(cv.box + 2 * j), __ldg(cv.box + 2 * j + 1), qlo, qhi)) continue;
                    const int b0 = be[2 * j], b1 = be[2 * j + 1];
                    attempt_ee(x, x0, dh, dh2, a0, a1, b0, b1, sink);
                }
            }
}

// ---------------------------------------------------------------- CCD step filter
// Pairs that pass the additive bound go to the exact interval test through a compacted list
// instead of running it in the candidate loop, where one lane's exact test would hold its whole
// warp (the candidate loops are divergent: lanes run different cells and candidates).  The
// minimum over pairs does not depend on where a pair's toc is computed.
struct CcdWork {
    int a, b, slot, pad;   // point-triangle: vertex, triangle; edge-edge: edge, edge; filter slot
    double d2, lb;         // current squared distance, additive lower bound
};
struct CcdList {
    CcdWork* w;            // [2 cap]: point-triangle pairs, then edge-edge pairs
    int* count;            // [2] pushes (may exceed cap: the lanes past it test inline)
    int cap;
};

// the exact tests out of line, for the candidate loops' overflow path (keeps their registers low)
__device__ __noinline__ double pt_exact_call(v3 P, v3 A, v3 B, v3 C, v3 dP, v3 dA, v3 dB, v3 dC, double eta, double d2, double lb) {
    return pt_ccd_exact(P, A, B, C, dP, dA, dB, dC, eta, d2, lb);
}
__device__ __noinline__ double ee_exact_call(v3 A0, v3 A1, v3 B0, v3 B1, v3 dA0, v3 dA1, v3 dB0, v3 dB1, double eta, double d2,
                                             double lb) {
    return ee_ccd_exact(A0, A1, B0, B1, dA0, dA1, dB0, dB1, eta, d2, lb);
}

// appends e for every calling lane (one atomic per coalesced group); false when the list is full
__device__ __forceinline__ bool ccd_push(CcdWork* w, int* count, int cap, const CcdWork& e) {
    cg::coalesced_group g = cg::coalesced_threads();
    int base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(count, (int)g.size());
    base = g.shfl(base, 0);
    const int k = base + (int)g.thread_rank();
    if (k >= cap) return false;
    w[k] = e;
    return true;
}

__device__ __forceinline__ void atomic_min_pos(unsigned long long* slot, double v) {
    if (v >= 0.0) atomicMin(slot, (unsigned long long)__double_as_longlong(v));
}

// compute_filter_3D_PT (NEWTON_IPC.py:377-406): triangles query their moving bbox
__global__ void __launch_bounds__(128) k_ccd_pt(int nbt, const int* __restrict__ bt, const int* __restrict__ bp,
                                                const double* __restrict__ x, const double* __restrict__ p, double dh, SceneGeo g,
                                                double eta, GridView gv, CandView cv, CcdList L, unsigned long long* __restrict__ alpha) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nbt) return;
    if (g.big_tri && g.big_tri[i]) return;
    const int t0 = bt[3 * i], t1 = bt[3 * i + 1], t2 = bt[3 * i + 2];
    const int sc = g.scene(t0);
    const double inv_dx = g.idx(sc);
    const v3 A = ld3(x, t0), B = ld3(x, t1), C = ld3(x, t2);
    const v3 dA = ld3(p, t0), dB = ld3(p, t1), dC = ld3(p, t2);
    const v3 mn = vmin(vmin(vmin(A, A + dA), vmin(B, B + dB)), vmin(C, C + dC));
    const v3 mx = vmax(vmax(vmax(A, A + dA), vmax(B, B + dB)), vmax(C, C + dC));
    const C3 lo = cell_of(mn, inv_dx), hi = cell_of(mx, inv_dx);
    const v3 d = mk(dh, dh, dh);
    const float4 qlo = f32_lo(mn - d), qhi = f32_hi(mx + d);   // pt_aabb_moving's triangle box
    for (long long cx = lo.x; cx <= hi.x; ++cx)
        for (long long cy = lo.y; cy <= hi.y; ++cy)
            for (long long cz = lo.z; cz <= hi.z; ++cz) {
                const int c = gv.find(gkey(g, sc, cx, cy, cz));
                if (c < 0) continue;
                for (int k = gv.us[c]; k < gv.us[c + 1]; ++k) {
                    const int j = gv.ids[k];
                    const int4 pc = __ldg(cv.cell + j);
                    const C3 first = cmax(lo, C3{pc.x, pc.y, pc.z});
                    if (first.x != cx || first.y != cy || first.z != cz) continue;
                    if (!f32_overlap(__ldg(cv.box + 2 * j), __ldg(cv.box + 2 * j + 1), qlo, qhi)) continue;
                    const int pp = bp[j];
                    if (pp == t0 || pp == t1 || pp == t2) continue;
                    const v3 P = ld3(x, pp), dP = ld3(p, pp);
                    if (!pt_aabb_moving(P, A, B, C, dP, dA, dB, dC, dh)) continue;
                    const double d2 = pt_dist2(P, A, B, C);
                    double lb;
                    if (!pt_needs_exact(dP, dA, dB, dC, eta, d2, &lb)) continue;
                    const int slot = g.vscene ? sc : 0;
                    if (!ccd_push(L.w, L.count, L.cap, CcdWork{pp, i, slot, 0, d2, lb}))
                        atomic_min_pos(alpha + slot, pt_exact_call(P, A, B, C, dP, dA, dB, dC, eta, d2, lb));
                }
            }
}

// compute_filter_3D_EE (NEWTON_IPC.py:409-440): edges query moving bbox +- dh
__global__ void __launch_bounds__(128) k_ccd_ee(int nbe, const int* __restrict__ be, const double* __restrict__ x,
                                                const double* __restrict__ p, double dh, SceneGeo g, double eta,
                                                GridView gv, CandView cv, CcdList L, unsigned long long* __restrict__ alpha) {
    // QG lanes per query edge share the candidates of each cell
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) / QG, lane = threadIdx.x % QG;
    if (i >= nbe) return;
    if (g.big_edge && g.big_edge[i]) return;
    const int a0 = be[2 * i], a1 = be[2 * i + 1];
    const int sc = g.scene(a0);
    const double inv_dx = g.idx(sc);
    const v3 A0 = ld3(x, a0), A1 = ld3(x, a1), dA0 = ld3(p, a0), dA1 = ld3(p, a1);
    const v3 d = mk(dh, dh, dh);
    const v3 mn = vmin(vmin(A0, A0 + dA0), vmin(A1, A1 + dA1)), mx = vmax(vmax(A0, A0 + dA0), vmax(A1, A1 + dA1));
    const C3 lo = cell_of(mn - d, inv_dx), hi = cell_of(mx + d, inv_dx);
    const float4 qlo = f32_lo(mn), qhi = f32_hi(mx);   // ee_aabb_moving's query edge box
    for (long long cx = lo.x; cx <= hi.x; ++cx)
        for (long long cy = lo.y; cy <= hi.y; ++cy)
            for (long long cz = lo.z; cz <= hi.z; ++cz) {
                const int c = gv.find(gkey(g, sc, cx, cy, cz));
                if (c < 0) continue;
                for (int k = gv.us[c] + lane; k < gv.us[c + 1]; k += QG) {
                    const int j = gv.ids[k];
                    if (!(i < j)) continue;
                    const int4 sc4 = __ldg(cv.cell + j);
                    const C3 first = cmax(lo, C3{sc4.x, sc4.y, sc4.z});
                    if (first.x != cx || first.y != cy || first.z != cz) continue;
                    if (!f32_overlap(__ldg(cv.box + 2 * j), __ldg(cv.box + 2 * j + 1), qlo, qhi)) continue;
                    const int b0 = be[2 * j], b1 = be[2 * j + 1];
                    if (a0 == b0 || a0 == b1 || a1 == b0 || a1 == b1) continue;
                    const v3 B0 = ld3(x, b0), B1 = ld3(x, b1), dB0 = ld3(p, b0), dB1 = ld3(p, b1);
                    if (!ee_aabb_moving(A0, A1, B0, B1, dA0, dA1, dB0, dB1, dh)) continue;
                    const double d2 = ee_dist2(A0, A1, B0, B1);
                    double lb;
                    if (!ee_needs_exact(dA0, dA1, dB0, dB1, eta, d2, &lb)) continue;
                    const int slot = g.vscene ? sc : 0;
                    if (!ccd_push(L.w + L.cap, L.count + 1, L.cap, CcdWork{i, j, slot, 0, d2, lb}))
                        atomic_min_pos(alpha + slot, ee_exact_call(A0, A1, B0, B1, dA0, dA1, dB0, dB1, eta, d2, lb));
                }
            }
}

// the exact tests of the listed pairs, one thread per pair
__global__ void __launch_bounds__(128) k_ccd_pt_exact(const int* __restrict__ bt, const double* __restrict__ x,
                                                      const double* __restrict__ p, double eta, CcdList L,
                                                      unsigned long long* __restrict__ alpha) {
    const int n = min(L.count[0], L.cap);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const CcdWork e = L.w[k];
        const int t0 = bt[3 * e.b], t1 = bt[3 * e.b + 1], t2 = bt[3 * e.b + 2];
        const v3 P = ld3(x, e.a), dP = ld3(p, e.a);
        const v3 A = ld3(x, t0), B = ld3(x, t1), C = ld3(x, t2), dA = ld3(p, t0), dB = ld3(p, t1), dC = ld3(p, t2);
        atomic_min_pos(alpha + e.slot, pt_ccd_exact(P, A, B, C, dP, dA, dB, dC, eta, e.d2, e.lb));
    }
}
__global__ void __launch_bounds__(128) k_ccd_ee_exact(const int* __restrict__ be, const double* __restrict__ x,
                                                      const double* __restrict__ p, double eta, CcdList L,
                                                      unsigned long long* __restrict__ alpha) {
    const int n = min(L.count[1], L.cap);
    const CcdWork* w = L.w + L.cap;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const CcdWork e = w[k];
        const int a0 = be[2 * e.a], a1 = be[2 * e.a + 1], b0 = be[2 * e.b], b1 = be[2 * e.b + 1];
        const v3 A0 = ld3(x, a0), A1 = ld3(x, a1), B0 = ld3(x, b0), B1 = ld3(x, b1);
        const v3 dA0 = ld3(p, a0), dA1 = ld3(p, a1), dB0 = ld3(p, b0), dB1 = ld3(p, b1);
        atomic_min_pos(alpha + e.slot, ee_ccd_exact(A0, A1, B0, B1, dA0, dA1, dB0, dB1, eta, e.d2, e.lb));
    }
}

// compute_filter_3D_inversion_free (NEWTON_IPC.py:443-453)
__global__ void __launch_bounds__(128) k_ccd_inversion(int nT, const int4* __restrict__ tets, const double* __restrict__ x,
                                                       const double* __restrict__ p, double eta, SceneGeo g,
                                                       unsigned long long* __restrict__ alpha) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nT) return;
    const int4 t = tets[e];
    const v3 X[4] = {ld3(x, t.x), ld3(x, t.y), ld3(x, t.z), ld3(x, t.w)};
    const v3 P[4] = {ld3(p, t.x), ld3(p, t.y), ld3(p, t.z), ld3(p, t.w)};
    if (inversion_cannot_flip(X, P, eta)) return;
    atomic_min_pos(alpha + (g.vscene ? g.scene(t.x) : 0), inversion_free_step(X, P, eta));
}

// check_collision_3d (NEWTON_IPC.py:855-880): triangles query bbox cells, edges hashed +- dh
__global__ void __launch_bounds__(128) k_collision(int nbt, const int* __restrict__ bt, const int* __restrict__ be,
                                                   const double* __restrict__ x, double dh, SceneGeo g,
                                                   GridView gv, CandView cv, int* __restrict__ hit) {
    // QG lanes per query triangle share the candidates of each cell
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) / QG, lane = threadIdx.x % QG;
    if (i >= nbt) return;
    if (g.big_tri && g.big_tri[i]) return;
    const int t0 = bt[3 * i], t1 = bt[3 * i + 1], t2 = bt[3 * i + 2];
    const int sc = g.scene(t0);
    const double inv_dx = g.idx(sc);
    const v3 A = ld3(x, t0), B = ld3(x, t1), C = ld3(x, t2);
    const v3 tmn = vmin(vmin(A, B), C), tmx = vmax(vmax(A, B), C);
    const C3 lo = cell_of(tmn, inv_dx), hi = cell_of(tmx, inv_dx);
    const float4 qlo = f32_lo(tmn), qhi = f32_hi(tmx);   // the triangle's box; edges carry +- dh
    hit += g.vscene ? sc : 0;
    for (long long cx = lo.x; cx <= hi.x; ++cx)
        for (long long cy = lo.y; cy <= hi.y; ++cy)
            for (long long cz = lo.z; cz <= hi.z; ++cz) {
                if (*(volatile int*)hit) return;
                const int c = gv.find(gkey(g, sc, cx, cy, cz));
                if (c < 0) continue;
                for (int k = gv.us[c] + lane; k < gv.us[c + 1]; k += QG) {
                    const int j = gv.ids[k];
                    const int4 sc4 = __ldg(cv.cell + j);
                    const C3 first = cmax(lo, C3{sc4.x, sc4.y, sc4.z});
                    if (first.x != cx || first.y != cy || first.z != cz) continue;
                    if (!f32_overlap(__ldg(cv.box + 2 * j), __ldg(cv.box + 2 * j + 1), qlo, qhi)) continue;
                    const int a0 = be[2 * j], a1 = be[2 * j + 1];
                    if (a0 == t0 || a0 == t1 || a0 == t2 || a1 == t0 || a1 == t1 || a1 == t2) continue;
                    const v3 P = ld3(x, a0), Q = ld3(x, a1);
                    if (seg_tri(P, Q, A, B, C)) atomicOr(hit, 1);
                }
            }
}

// ---------------------------------------------------------------- big primitives
// A triangle or edge whose query box covers more than BIG_CELLS cells (a ground plane meshed
// with a few large triangles next to finely meshed bodies) would enumerate, or be stored in,
// thousands of cells.  Such primitives leave the grid: each is tested against every primitive
// of its own scene with the same narrow phase, so the results are the grid's.
constexpr long long BIG_CELLS = 256;

__device__ __forceinline__ long long box_cells(v3 lo, v3 hi, double inv_dx) {
    const C3 a = cell_of(lo, inv_dx), b = cell_of(hi, inv_dx);
    return (b.x - a.x + 1) * (b.y - a.y + 1) * (b.z - a.z + 1);
}

// flags and compacted lists; triangle boxes as queried (static or moving bbox), edge boxes as
// queried (static or moving bbox +- dh).  lists: [0, nbt) triangles, [nbt, nbt + nbe) edges;
// counts[0..1] (zeroed by the caller)
__global__ void k_big_flags(int nbt, int nbe, const int* __restrict__ bt, const int* __restrict__ be, const double* __restrict__ x,
                            const double* __restrict__ p, double dh, SceneGeo g, unsigned char* __restrict__ tri_big,
                            unsigned char* __restrict__ edge_big, int* __restrict__ list, int* __restrict__ counts) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nbt) {
        const int t0 = bt[3 * k], t1 = bt[3 * k + 1], t2 = bt[3 * k + 2];
        v3 lo = vmin(vmin(ld3(x, t0), ld3(x, t1)), ld3(x, t2)), hi = vmax(vmax(ld3(x, t0), ld3(x, t1)), ld3(x, t2));
        if (p) {
            const v3 A = ld3(x, t0) + ld3(p, t0), B = ld3(x, t1) + ld3(p, t1), C = ld3(x, t2) + ld3(p, t2);
            lo = vmin(lo, vmin(vmin(A, B), C));
            hi = vmax(hi, vmax(vmax(A, B), C));
        }
        const bool big = box_cells(lo, hi, g.idx(g.scene(t0))) > BIG_CELLS;
        tri_big[k] = big;
        if (big) list[atomicAdd(&counts[0], 1)] = k;
    } else if (k < nbt + nbe) {
        const int e = k - nbt, a0 = be[2 * e], a1 = be[2 * e + 1];
        v3 lo = vmin(ld3(x, a0), ld3(x, a1)), hi = vmax(ld3(x, a0), ld3(x, a1));
        if (p) {
            const v3 A = ld3(x, a0) + ld3(p, a0), B = ld3(x, a1) + ld3(p, a1);
            lo = vmin(lo, vmin(A, B));
            hi = vmax(hi, vmax(A, B));
        }
        const v3 d = mk(dh, dh, dh);
        const bool big = box_cells(lo - d, hi + d, g.idx(g.scene(a0))) > BIG_CELLS;
        edge_big[e] = big;
        if (big) list[nbt + atomicAdd(&counts[1], 1)] = e;
    }
}

// partners of big primitive q of scene s: lists [off[s], off[s+1]) of its kind
struct BigArgs {
    const int *bp, *be, *bt;
    const int* off;        // [3][S+1]: points, edges, triangles
    int S;
    const unsigned char *tri_big, *edge_big;
    const int* list;       // [nbt + nbe]
    const int* counts;     // [2]
    int nbt;
};

// find_constraints, big triangles against every point of their scene
__global__ void k_find_pt_big(BigArgs b, const double* __restrict__ x, double dh, double dh2, SceneGeo g, RowSink sink) {
    for (int q = blockIdx.x; q < b.counts[0]; q += gridDim.x) {
        const int i = b.list[q];
        const int t0 = b.bt[3 * i], t1 = b.bt[3 * i + 1], t2 = b.bt[3 * i + 2];
        const int sc = g.scene(t0);
        for (int k = b.off[sc] + threadIdx.x; k < b.off[sc + 1]; k += blockDim.x) attempt_pt(x, dh, dh2, b.bp[k], t0, t1, t2, sink);
    }
}

// find_constraints, big edges against every edge of their scene (a pair of two big edges once,
// from its lower index); rows formed with the lower list index first as in the grid pass
__global__ void k_find_ee_big(BigArgs b, const double* __restrict__ x, const double* __restrict__ x0, double dh, double dh2,
                              SceneGeo g, RowSink sink) {
    for (int q = blockIdx.x; q < b.counts[1]; q += gridDim.x) {
        const int i = b.list[b.nbt + q];
        const int sc = g.scene(b.be[2 * i]);
        const int* off = b.off + (b.S + 1);
        for (int j = off[sc] + threadIdx.x; j < off[sc + 1]; j += blockDim.x) {
            if (j == i || (b.edge_big[j] && j < i)) continue;
            const int lo = i < j ? i : j, hi = i < j ? j : i;
            attempt_ee(x, x0, dh, dh2, b.be[2 * lo], b.be[2 * lo + 1], b.be[2 * hi], b.be[2 * hi + 1], sink);
        }
    }
}

// CCD filter, big moving triangles against every point of their scene
__global__ void k_ccd_pt_big(BigArgs b, const double* __restrict__ x, const double* __restrict__ p, double dh, double eta, SceneGeo g,
                             unsigned long long* __restrict__ alpha) {
    for (int q = blockIdx.x; q < b.counts[0]; q += gridDim.x) {
        const int i = b.list[q];
        const int t0 = b.bt[3 * i], t1 = b.bt[3 * i + 1], t2 = b.bt[3 * i + 2];
        const int sc = g.scene(t0);
        const v3 A = ld3(x, t0), B = ld3(x, t1), C = ld3(x, t2), dA = ld3(p, t0), dB = ld3(p, t1), dC = ld3(p, t2);
        for (int k = b.off[sc] + threadIdx.x; k < b.off[sc + 1]; k += blockDim.x) {
            const int pp = b.bp[k];
            if (pp == t0 || pp == t1 || pp == t2) continue;
            const v3 P = ld3(x, pp), dP = ld3(p, pp);
            if (!pt_aabb_moving(P, A, B, C, dP, dA, dB, dC, dh)) continue;
            const double d2 = pt_dist2(P, A, B, C);
            atomic_min_pos(alpha + (g.vscene ? sc : 0), pt_ccd(P, A, B, C, dP, dA, dB, dC, eta, d2));
        }
    }
}

// CCD filter, big moving edges against every edge of their scene
__global__ void k_ccd_ee_big(BigArgs b, const double* __restrict__ x, const double* __restrict__ p, double dh, double eta, SceneGeo g,
                             unsigned long long* __restrict__ alpha) {
    for (int q = blockIdx.x; q < b.counts[1]; q += gridDim.x) {
        const int i = b.list[b.nbt + q];
        const int sc = g.scene(b.be[2 * i]);
        const int* off = b.off + (b.S + 1);
        for (int j = off[sc] + threadIdx.x; j < off[sc + 1]; j += blockDim.x) {
            if (j == i || (b.edge_big[j] && j < i)) continue;
            const int lo = i < j ? i : j, hi = i < j ? j : i;
            const int a0 = b.be[2 * lo], a1 = b.be[2 * lo + 1], b0 = b.be[2 * hi], b1 = b.be[2 * hi + 1];
            if (a0 == b0 || a0 == b1 || a1 == b0 || a1 == b1) continue;
            const v3 A0 = ld3(x, a0), A1 = ld3(x, a1), B0 = ld3(x, b0), B1 = ld3(x, b1);
            const v3 dA0 = ld3(p, a0), dA1 = ld3(p, a1), dB0 = ld3(p, b0), dB1 = ld3(p, b1);
            if (!ee_aabb_moving(A0, A1, B0, B1, dA0, dA1, dB0, dB1, dh)) continue;
            const double d2 = ee_dist2(A0, A1, B0, B1);
            atomic_min_pos(alpha + (g.vscene ? sc : 0), ee_ccd(A0, A1, B0, B1, dA0, dA1, dB0, dB1, eta, d2));
        }
    }
}

// intersection check: big triangles against every edge of their scene, big edges against every
// triangle of their scene that is not big
__global__ void k_collision_big(BigArgs b, const double* __restrict__ x, SceneGeo g, int* __restrict__ hit) {
    const int nt = b.counts[0], ne = b.counts[1];
    for (int q = blockIdx.x; q < nt + ne; q += gridDim.x) {
        const bool tri = q < nt;
        const int i = tri ? b.list[q] : b.list[b.nbt + q - nt];
        const int sc = g.scene(tri ? b.bt[3 * i] : b.be[2 * i]);
        int* h = hit + (g.vscene ? sc : 0);
        const int* off = b.off + (tri ? 1 : 2) * (b.S + 1);
        for (int k = off[sc] + threadIdx.x; k < off[sc + 1]; k += blockDim.x) {
            if (*(volatile int*)h) break;
            const int e = tri ? k : i, t = tri ? i : k;
            if (!tri && b.tri_big[t]) continue;
            const int t0 = b.bt[3 * t], t1 = b.bt[3 * t + 1], t2 = b.bt[3 * t + 2], a0 = b.be[2 * e], a1 = b.be[2 * e + 1];
            if (a0 == t0 || a0 == t1 || a0 == t2 || a1 == t0 || a1 == t1 || a1 == t2) continue;
            if (seg_tri(ld3(x, a0), ld3(x, a1), ld3(x, t0), ld3(x, t1), ld3(x, t2))) atomicOr(h, 1);
        }
    }
}

// ---------------------------------------------------------------- row canonicalisation
// width-2 / width-3 rows: one 63-bit key; width-4 rows: LSD two-pass (last index, then the
// first three) with the stable radix sort.  21 bits per vertex index (< 2^21 vertices).
__global__ void k_row_keys(int n, int width, int pass, const int4* __restrict__ rows, const int* __restrict__ perm,
                           unsigned long long* __restrict__ keys, int* __restrict__ idx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int src = perm ? perm[i] : i;
    const int4 r = rows[src];
    unsigned long long k;
    if (width == 2) k = ((unsigned long long)r.x << 21) | (unsigned long long)r.y;
    else if (width == 3 || pass == 1) k = ((unsigned long long)r.x << 42) | ((unsigned long long)r.y << 21) | (unsigned long long)r.z;
    else k = (unsigned long long)r.w;
    keys[i] = k;
    idx[i] = src;
}
__global__ void k_row_gather_flag(int n, const int4* __restrict__ rows, const int* __restrict__ perm, int4* __restrict__ out,
                                  int* __restrict__ flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int4 r = rows[perm[i]];
    out[i] = r;
    int f = 1;
    if (i > 0) {
        const int4 q = rows[perm[i - 1]];
        f = !(q.x == r.x && q.y == r.y && q.z == r.z && q.w == r.w);
    }
    flag[i] = f;
}
__global__ void k_row_compact(int n, const int4* __restrict__ in, const int* __restrict__ flag, const int* __restrict__ pos,
                              int4* __restrict__ out, int* __restrict__ count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (flag[i]) out[pos[i]] = in[i];
    if (i == n - 1) *count = pos[i] + flag[i];
}

// ---------------------------------------------------------------- host side
static inline int nblk(long long n, int b) { return (int)((n + b - 1) / b); }

template <class F>
static int cub_call(fipc_ctx* c, F&& f) {
    size_t need = 0;
    if (f(nullptr, need) != cudaSuccess) return FIPC_ERR_CUDA;
    if (c->cub_tmp.ensure(need)) return FIPC_ERR_CUDA;
    size_t have = c->cub_tmp.bytes;
    if (f(c->cub_tmp.p, have) != cudaSuccess) return FIPC_ERR_CUDA;
    return FIPC_OK;
}

static SceneGeo geo(const fipc_ctx* c) {
    SceneGeo g;
    g.vscene = c->n_scenes > 1 ? c->v_scene : nullptr;
    g.inv_dx_s = c->s_hash_inv_dx;
    g.inv_dx = c->hash_inv_dx;
    return g;
}

// flag the big triangles and edges for positions x (+ direction p when moving) and return the
// scene lookup that carries the flags; *b gets the lists for the big-primitive kernels
static int big_prepare(fipc_ctx* c, const double* x, const double* p, SceneGeo* g, BigArgs* b, cudaStream_t s) {
    *g = geo(c);
    const int n = c->nBT + c->nBE;
    if (c->big_flags.ensure((size_t)n + 16) || c->big_list.ensure(4ll * (n + 2) + 16)) return FIPC_ERR_CUDA;
    unsigned char* tri_big = c->big_flags.as<unsigned char>();
    int* list = c->big_list.as<int>();
    int* counts = list + n;
    FIPC_CUDA(cudaMemsetAsync(counts, 0, 2 * sizeof(int), s));
    if (n > 0) {
        k_big_flags<<<nblk(n, 256), 256, 0, s>>>(c->nBT, c->nBE, c->bt, c->be, x, p, c->dhat, *g, tri_big, tri_big + c->nBT, list,
                                                 counts);
        FIPC_LAUNCHED();
    }
    g->big_tri = tri_big;
    g->big_edge = tri_big + c->nBT;
    b->bp = c->bp;
    b->be = c->be;
    b->bt = c->bt;
    b->off = c->prim_off;
    b->S = c->n_scenes;
    b->tri_big = g->big_tri;
    b->edge_big = g->big_edge;
    b->list = list;
    b->counts = counts;
    b->nbt = c->nBT;
    return FIPC_OK;
}
constexpr int BIG_GRID = 304, BIG_THREADS = 128;

// build grid g over n stored primitives; scal: device int scratch (overflow flag at [0])
int build_grid(fipc_ctx* c, Grid& g, int mode, int n, const int* prim, const double* x, const double* p, const SceneGeo& sg,
               cudaStream_t s) {
    g.n_entries = 0;
    g.n_unique = 0;
    if (g.counts.ensure(sizeof(long long) * (n + 1)) || g.offsets.ensure(sizeof(long long) * (n + 1)) ||
        g.ncells.ensure(sizeof(int) * 2))
        return FIPC_ERR_CUDA;
    FIPC_CUDA(cudaMemsetAsync(g.ncells.p, 0, sizeof(int) * 2, s));
    if (n == 0) return FIPC_OK;
    int* ovf = g.ncells.as<int>() + 1;
    k_cell_count<<<nblk(n, 256), 256, 0, s>>>(mode, n, prim, x, p, c->dhat, sg, g.counts.as<long long>(), ovf);
    FIPC_LAUNCHED();
    if (g.cell4.ensure(16ll * n) || g.box4.ensure(32ll * n)) return FIPC_ERR_CUDA;
    k_cand_records<<<nblk(n, 256), 256, 0, s>>>(mode, n, prim, x, p, c->dhat, sg, g.cell4.as<int4>(), g.box4.as<float4>());
    FIPC_LAUNCHED();
    long long* cnt = g.counts.as<long long>();
    long long* off = g.offsets.as<long long>();
    int st = cub_call(c, [&](void* t, size_t& b) { return cub::DeviceScan::ExclusiveSum(t, b, cnt, off, n, s); });
    if (st) return st;
    long long last_off = 0, last_cnt = 0;
    int h_ovf = 0;
    FIPC_CUDA(cudaMemcpyAsync(&last_off, off + n - 1, sizeof(long long), cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaMemcpyAsync(&last_cnt, cnt + n - 1, sizeof(long long), cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaMemcpyAsync(&h_ovf, ovf, sizeof(int), cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaStreamSynchronize(s));
    if (h_ovf) return FIPC_ERR_CAPACITY;
    const long long total = last_off + last_cnt;
    if (total > (1ll << 30)) return FIPC_ERR_CAPACITY;
    g.n_entries = (int)total;
    if (total == 0) return FIPC_OK;
    if (g.keys.ensure(8 * total) || g.keys_alt.ensure(8 * total) || g.ids.ensure(4 * total) || g.ids_alt.ensure(4 * total) ||
        g.ukeys.ensure(8 * total) || g.ustart.ensure(4 * (total + 1)) || g.tmp.ensure(4 * (total + 1)))
        return FIPC_ERR_CUDA;
    k_cell_emit<<<nblk(n, 256), 256, 0, s>>>(mode, n, prim, x, p, c->dhat, sg, off, cnt, g.keys.as<unsigned long long>(),
                                             g.ids.as<int>());
    FIPC_LAUNCHED();
    cub::DoubleBuffer<unsigned long long> kb(g.keys.as<unsigned long long>(), g.keys_alt.as<unsigned long long>());
    cub::DoubleBuffer<int> vb(g.ids.as<int>(), g.ids_alt.as<int>());
    const int N = (int)total;
    st = cub_call(c, [&](void* t, size_t& b) { return cub::DeviceRadixSort::SortPairs(t, b, kb, vb, N, 0, 63, s); });
    if (st) return st;
    if (kb.Current() != g.keys.as<unsigned long long>()) {
        FIPC_CUDA(cudaMemcpyAsync(g.keys.p, kb.Current(), 8 * total, cudaMemcpyDeviceToDevice, s));
        FIPC_CUDA(cudaMemcpyAsync(g.ids.p, vb.Current(), 4 * total, cudaMemcpyDeviceToDevice, s));
    }
    int* runs = g.tmp.as<int>();   // run lengths
    int* nu = g.ncells.as<int>();
    st = cub_call(c, [&](void* t, size_t& b) {
        return cub::DeviceRunLengthEncode::Encode(t, b, g.keys.as<unsigned long long>(), g.ukeys.as<unsigned long long>(), runs, nu,
                                                  N, s);
    });
    if (st) return st;
    st = cub_call(c, [&](void* t, size_t& b) { return cub::DeviceScan::ExclusiveSum(t, b, runs, g.ustart.as<int>(), N + 1, s); });
    if (st) return st;
    // cell table
    unsigned long long size = 1;
    while (size < 2ull * (unsigned long long)N) size <<= 1;
    if (g.hkeys.ensure(8 * size) || g.hvals.ensure(4 * size)) return FIPC_ERR_CUDA;
    FIPC_CUDA(cudaMemsetAsync(g.hkeys.p, 0xff, 8 * size, s));
    g.hmask = size - 1;
    k_hash_insert<<<nblk(N, 256), 256, 0, s>>>(g.ukeys.as<unsigned long long>(), nu, g.hkeys.as<unsigned long long>(), g.hvals.as<int>(),
                                               g.hmask);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

static CandView cands(const Grid& g) { return CandView{g.cell4.as<int4>(), g.box4.as<float4>()}; }

static GridView view(const Grid& g) {
    GridView v;
    v.hk = g.hkeys.as<unsigned long long>();
    v.hv = g.hvals.as<int>();
    v.mask = g.hmask;
    v.us = g.ustart.as<int>();
    v.ids = g.ids.as<int>();
    return v;
}

// sort + unique each list in place (rows_tmp as staging); returns counts in c->h_counts
static int canonicalize_rows(fipc_ctx* c, cudaStream_t s) {
    int h[N_TYPES + 1];
    FIPC_CUDA(cudaMemcpyAsync(h, c->d_counts, sizeof(int) * (N_TYPES + 1), cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaStreamSynchronize(s));
    if (h[N_TYPES]) return FIPC_ERR_CAPACITY;
    static const int width[N_TYPES] = {2, 3, 4, 4, 4, 4, 4};
    for (int t = 0; t < N_TYPES; ++t) {
        const int n = h[t];
        c->h_counts[t] = n;
        if (n <= 1) continue;
        if (c->rows_tmp.ensure(16ll * n) || c->sort_keys.ensure(8ll * n) || c->sort_keys_alt.ensure(8ll * n) ||
            c->sort_vals.ensure(4ll * n) || c->sort_vals_alt.ensure(4ll * n) || c->flags.ensure(4ll * n) || c->scan.ensure(4ll * n))
            return FIPC_ERR_CUDA;
        int4* rows = c->rows[t].as<int4>();
        const int* perm = nullptr;
        const int passes = width[t] == 4 ? 2 : 1;
        for (int pass = 0; pass < passes; ++pass) {
            const int kpass = width[t] == 4 ? pass : 1;
            k_row_keys<<<nblk(n, 256), 256, 0, s>>>(n, width[t], kpass, rows, perm, c->sort_keys.as<unsigned long long>(),
                                                   c->sort_vals.as<int>());
            FIPC_LAUNCHED();
            cub::DoubleBuffer<unsigned long long> kb(c->sort_keys.as<unsigned long long>(), c->sort_keys_alt.as<unsigned long long>());
            cub::DoubleBuffer<int> vb(c->sort_vals.as<int>(), c->sort_vals_alt.as<int>());
            const int end_bit = (width[t] == 2) ? 42 : ((kpass == 1) ? 63 : 32);
            int st = cub_call(c, [&](void* tm, size_t& b) { return cub::DeviceRadixSort::SortPairs(tm, b, kb, vb, n, 0, end_bit, s); });
            if (st) return st;
            if (vb.Current() != c->sort_vals.as<int>())
                FIPC_CUDA(cudaMemcpyAsync(c->sort_vals.p, vb.Current(), 4ll * n, cudaMemcpyDeviceToDevice, s));
            // the permutation for the next pass lives in sort_vals_alt
            FIPC_CUDA(cudaMemcpyAsync(c->sort_vals_alt.p, c->sort_vals.p, 4ll * n, cudaMemcpyDeviceToDevice, s));
            perm = c->sort_vals_alt.as<int>();
        }
        k_row_gather_flag<<<nblk(n, 256), 256, 0, s>>>(n, rows, perm, c->rows_tmp.as<int4>(), c->flags.as<int>());
        FIPC_LAUNCHED();
        int* flg = c->flags.as<int>();
        int* pos = c->scan.as<int>();
        int st = cub_call(c, [&](void* tm, size_t& b) { return cub::DeviceScan::ExclusiveSum(tm, b, flg, pos, n, s); });
        if (st) return st;
        k_row_compact<<<nblk(n, 256), 256, 0, s>>>(n, c->rows_tmp.as<int4>(), flg, pos, rows, c->d_counts + t);
        FIPC_LAUNCHED();
    }
    FIPC_CUDA(cudaMemcpyAsync(h, c->d_counts, sizeof(int) * N_TYPES, cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaStreamSynchronize(s));
    for (int t = 0; t < N_TYPES; ++t) c->h_counts[t] = h[t];
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int ensure_row_capacity(fipc_ctx* c, int cap) {
    if (cap <= c->cap) return FIPC_OK;
    for (int t = 0; t < N_TYPES; ++t)
        if (c->rows[t].ensure(16ll * cap)) return FIPC_ERR_CUDA;
    c->cap = cap;
    return FIPC_OK;
}

// find_constraints (NEWTON_IPC.py:337-357) into c->rows / c->h_counts
int find_constraints(fipc_ctx* c, const double* x, cudaStream_t s) {
    for (int attempt = 0; attempt < 8; ++attempt) {
        FIPC_CUDA(cudaMemsetAsync(c->d_counts, 0, sizeof(int) * (N_TYPES + 1), s));
        RowSink sink;
        for (int t = 0; t < N_TYPES; ++t) sink.rows[t] = c->rows[t].as<int4>();
        sink.counts = c->d_counts;
        sink.cap = c->cap;
        SceneGeo sg;
        BigArgs bg;
        int st = big_prepare(c, x, nullptr, &sg, &bg, s);
        if (st) return st;
        st = build_grid(c, c->gp, 0, c->nBP, c->bp, x, nullptr, sg, s);
        if (st) return st;
        if (c->gp.n_entries > 0 && c->nBT > 0) {
            k_find_pt<<<nblk(c->nBT, 128), 128, 0, s>>>(c->nBT, c->bt, c->bp, x, c->dhat, c->dhat2, sg,
                                                         view(c->gp), cands(c->gp), sink);
            FIPC_LAUNCHED();
        }
        if (c->nBT > 0 && c->nBP > 0) {
            k_find_pt_big<<<BIG_GRID, BIG_THREADS, 0, s>>>(bg, x, c->dhat, c->dhat2, sg, sink);
            FIPC_LAUNCHED();
        }
        st = build_grid(c, c->ge, 1, c->nBE, c->be, x, nullptr, sg, s);
        if (st) return st;
        if (c->ge.n_entries > 0) {
            k_find_ee<<<nblk((long long)QG * c->nBE, 128), 128, 0, s>>>(c->nBE, c->be, x, c->x0, c->dhat, c->dhat2, sg,
                                                         view(c->ge), cands(c->ge), sink);
            FIPC_LAUNCHED();
        }
        if (c->nBE > 1) {
            k_find_ee_big<<<BIG_GRID, BIG_THREADS, 0, s>>>(bg, x, c->x0, c->dhat, c->dhat2, sg, sink);
            FIPC_LAUNCHED();
        }
        FIPC_CUDA(cudaGetLastError());
        st = canonicalize_rows(c, s);
        if (st == FIPC_ERR_CAPACITY) {
            int h[N_TYPES];
            FIPC_CUDA(cudaMemcpy(h, c->d_counts, sizeof(int) * N_TYPES, cudaMemcpyDeviceToHost));
            int need = c->cap;
            for (int t = 0; t < N_TYPES; ++t) need = h[t] > need ? h[t] : need;
            if (ensure_row_capacity(c, 2 * need)) return FIPC_ERR_CUDA;
            continue;
        }
        return st;
    }
    return FIPC_ERR_CAPACITY;
}

// compute_intersection_free_step_size (NEWTON_IPC.py:456-468): the launches, min'd into
// slots (one double per scene, preset to 1.0 by the caller)
int ccd_launch(fipc_ctx* c, const double* x, const double* p, double eta, bool inversion, unsigned long long* slot, cudaStream_t s) {
    SceneGeo sg;
    BigArgs bg;
    int st = big_prepare(c, x, p, &sg, &bg, s);
    if (st) return st;
    CcdList L;
    {
        long long cap = 65536ll + c->nBE + c->nBT;
        if (cap > (1ll << 21)) cap = 1ll << 21;
        if (c->ccd_work.ensure(256 + 2 * cap * sizeof(CcdWork))) return FIPC_ERR_CUDA;
        L.count = c->ccd_work.as<int>();
        L.w = reinterpret_cast<CcdWork*>(c->ccd_work.as<char>() + 256);
        L.cap = (int)cap;
        FIPC_CUDA(cudaMemsetAsync(L.count, 0, 2 * sizeof(int), s));
    }
    st = build_grid(c, c->gp, 2, c->nBP, c->bp, x, p, sg, s);
    if (st) return st;
    if (c->gp.n_entries > 0 && c->nBT > 0) {
        k_ccd_pt<<<nblk(c->nBT, 128), 128, 0, s>>>(c->nBT, c->bt, c->bp, x, p, c->dhat, sg, eta,
                                                    view(c->gp), cands(c->gp), L, slot);
        FIPC_LAUNCHED();
        k_ccd_pt_exact<<<4 * BIG_GRID, 128, 0, s>>>(c->bt, x, p, eta, L, slot);
        FIPC_LAUNCHED();
    }
    if (c->nBT > 0 && c->nBP > 0) {
        k_ccd_pt_big<<<BIG_GRID, BIG_THREADS, 0, s>>>(bg, x, p, c->dhat, eta, sg, slot);
        FIPC_LAUNCHED();
    }
    st = build_grid(c, c->ge, 3, c->nBE, c->be, x, p, sg, s);
    if (st) return st;
    if (c->ge.n_entries > 0) {
        k_ccd_ee<<<nblk((long long)QG * c->nBE, 128), 128, 0, s>>>(c->nBE, c->be, x, p, c->dhat, sg, eta, view(c->ge), cands(c->ge),
                                                                   L, slot);
        FIPC_LAUNCHED();
        k_ccd_ee_exact<<<4 * BIG_GRID, 128, 0, s>>>(c->be, x, p, eta, L, slot);
        FIPC_LAUNCHED();
    }
    if (c->nBE > 1) {
        k_ccd_ee_big<<<BIG_GRID, BIG_THREADS, 0, s>>>(bg, x, p, c->dhat, eta, sg, slot);
        FIPC_LAUNCHED();
    }
    if (inversion && c->nT > 0) {
        k_ccd_inversion<<<nblk(c->nT, 128), 128, 0, s>>>(c->nT, (const int4*)c->tets, x, p, eta, sg, slot);
        FIPC_LAUNCHED();
    }
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

// one scene: result in *alpha_h
int ccd_step(fipc_ctx* c, const double* x, const double* p, double eta, bool inversion, double* alpha_h, cudaStream_t s) {
    if (c->scal.ensure(64)) return FIPC_ERR_CUDA;
    unsigned long long* slot = c->scal.as<unsigned long long>();
    const double one = 1.0;
    FIPC_CUDA(cudaMemcpyAsync(slot, &one, 8, cudaMemcpyHostToDevice, s));
    int st = ccd_launch(c, x, p, eta, inversion, slot, s);
    if (st) return st;
    FIPC_CUDA(cudaMemcpyAsync(alpha_h, slot, 8, cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaStreamSynchronize(s));
    return FIPC_OK;
}

// check_collision_3d (NEWTON_IPC.py:881-886): the launches, or'd into hit (one int per scene,
// zeroed by the caller)
int collision_launch(fipc_ctx* c, const double* x, int* hit, cudaStream_t s) {
    SceneGeo sg;
    BigArgs bg;
    int st = big_prepare(c, x, nullptr, &sg, &bg, s);
    if (st) return st;
    st = build_grid(c, c->ge, 4, c->nBE, c->be, x, nullptr, sg, s);
    if (st) return st;
    if (c->ge.n_entries > 0 && c->nBT > 0) {
        k_collision<<<nblk((long long)QG * c->nBT, 128), 128, 0, s>>>(c->nBT, c->bt, c->be, x, c->dhat, sg, view(c->ge),
                                                                       cands(c->ge), hit);
        FIPC_LAUNCHED();
    }
    if (c->nBT > 0 && c->nBE > 0) {
        k_collision_big<<<BIG_GRID, BIG_THREADS, 0, s>>>(bg, x, sg, hit);
        FIPC_LAUNCHED();
    }
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int check_collision(fipc_ctx* c, const double* x, int* hit_h, cudaStream_t s) {
    if (c->scal.ensure(64)) return FIPC_ERR_CUDA;
    int* hit = (int*)(c->scal.as<char>() + 16);
    FIPC_CUDA(cudaMemsetAsync(hit, 0, sizeof(int), s));
    int st = collision_launch(c, x, hit, s);
    if (st) return st;
    FIPC_CUDA(cudaMemcpyAsync(hit_h, hit, sizeof(int), cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaStreamSynchronize(s));
    return FIPC_OK;
}

}  // namespace fipc
