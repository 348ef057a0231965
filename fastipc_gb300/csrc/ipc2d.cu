// The 2D branch of the IPC Newton loop (projects/FastIPC/NEWTON_IPC.py with dim == 2):
// fixed-corotated triangles, point-point / point-edge barriers between boundary points and
// boundary edges, point-edge CCD and the point-in-triangle intersection check.
//
// Layout: positions [V][2] FP64 (the reference's x field for dim 2), triangles [T][3] int32.
// The reference tests every boundary point against every boundary edge (find_constraints_2D_PE,
// compute_filter_2D_PE) and every boundary point against every triangle (check_collision_2D).
// Here those all-pairs loops are tiled: a CTA stages a tile of edges (or triangles) with their
// vertex positions and FP32 boxes in shared memory and every thread tests its point against
// the whole tile, the conservative FP32 box test first.  The system is assembled by sorting
// (block key, contribution id) pairs and summing each run in id order, so every result is
// deterministic.  The direction comes from block-Jacobi PCG on 2x2 blocks with fixed-order
// reductions: one cooperative launch for systems that fit one CTA per SM, otherwise three
// kernels per iteration replayed from a captured CUDA graph.
#include <cuda_runtime.h>

#include <string.h>

#include <cooperative_groups.h>
#include <cub/cub.cuh>
#include <vector>

#include "barrier.cuh"
#include "ctx.cuh"
#include "fc2d.cuh"

namespace fipc {

namespace cg = cooperative_groups;

namespace {

constexpr int T2 = 256;       // threads per CTA of the 2D kernels
constexpr int TILE = 256;     // edges / triangles per shared-memory tile
constexpr int P2_RED = 304;   // fixed reduction grid (2 x 152 SMs)

inline int nb2(long long n, int b) { return (int)((n + b - 1) / b); }

// positions are read as one 16-byte double2 per vertex and rows as int4: their base addresses
// must be 16-byte aligned (every fresh device allocation is; a view at an odd offset is not)
inline bool al16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

__device__ __forceinline__ double2 ld2(const double* x, int i) { return *reinterpret_cast<const double2*>(x + 2 * (size_t)i); }

// fixed-tree block sum (blockDim.x == T2)
__device__ __forceinline__ double bsum(double v, double* sh) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = T2 / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

// atomic min / max of non-negative doubles through their bit patterns (exact, order-free)
__device__ __forceinline__ void amin_pos(double* a, double v) {
    atomicMin(reinterpret_cast<unsigned long long*>(a), (unsigned long long)__double_as_longlong(v));
}
__device__ __forceinline__ void amax_pos(double* a, double v) {
    atomicMax(reinterpret_cast<unsigned long long*>(a), (unsigned long long)__double_as_longlong(v));
}

}  // namespace

struct Ctx2 {
    int nV = 0, nT = 0, nBP = 0, nBE = 0;
    double dhat2 = 0, dhat = 0, dt = 0, kappa = 0, mean_edge = 0;
    int *tris = nullptr, *bp = nullptr, *be = nullptr;
    double *IB = nullptr, *vol = nullptr, *lam = nullptr, *mu = nullptr, *mass = nullptr;
    // per-iteration data
    DBuf elem_g, elem_H, rows[2], rows_tmp, keys, keys_alt, cnt_d, cub_tmp, scal;
    int cap[2] = {0, 0}, h_counts[2] = {0, 0};
    DBuf cg[2], cH[2];                      // barrier gradients / Hessian blocks per list
    DBuf a_keys, a_keys_alt, a_vals, a_vals_alt, a_ukeys, a_ucount, a_ustart;
    DBuf val, col, row_ptr, dpos, rhs;      // assembled 2x2-block CSR and right-hand side
    int nnzb = 0;
    DBuf pvec, ppart, pflag;                // PCG
    DBuf epart, eout;
    // PCG_CHUNK iterations captured as a CUDA graph on a private stream, keyed by the kernels'
    // arguments, and replayed on the caller's stream
    void* cap_stream = nullptr;
    void* graph_exec = nullptr;
    std::vector<unsigned char> graph_sig;
};

namespace {

// ---------------------------------------------------------------- elements
__global__ void __launch_bounds__(T2) k2_elements(int nT, const int* __restrict__ tris, const double* __restrict__ x,
                                                  const double* __restrict__ IB, const double* __restrict__ vol,
                                                  const double* __restrict__ lam, const double* __restrict__ mu, double dt2,
                                                  double* __restrict__ E, double* __restrict__ g, double* __restrict__ H) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nT) return;
    double X[6], ib[4], ge[6], He[36];
    for (int a = 0; a < 3; ++a) {
        const double2 p = ld2(x, tris[3 * (size_t)e + a]);
        X[2 * a] = p.x;
        X[2 * a + 1] = p.y;
    }
    for (int k = 0; k < 4; ++k) ib[k] = IB[4 * (size_t)e + k];
    const double psi = fc2_element(X, ib, lam[e], mu[e], dt2 * vol[e], ge, He);
    if (E) E[e] = psi;
    if (g)
        for (int k = 0; k < 6; ++k) g[6 * (size_t)e + k] = ge[k];
    if (H)
        for (int k = 0; k < 36; ++k) H[36 * (size_t)e + k] = He[k];
}

// ---------------------------------------------------------------- barrier rows (z = 0)
// type 0: PP rows (a, b); 1: PE rows (p, e0, e1).  g [n][2 nv], H [n][nv*nv][4]
__global__ void __launch_bounds__(128) k2_barrier(int type, int n, const int4* __restrict__ rows, const double* __restrict__ x,
                                                  double dh2, double kappa, double* __restrict__ E, double* __restrict__ g,
                                                  double* __restrict__ H) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int4 q = rows[r];
    const int nv = type == 0 ? 2 : 3;
    const int id[3] = {q.x, q.y, q.z};
    double X[6];
    for (int k = 0; k < nv; ++k) {
        const double2 p = ld2(x, id[k]);
        X[2 * k] = p.x;
        X[2 * k + 1] = p.y;
    }
    double e, gg[6], hh[36];
    barrier_row_2d(type, X, dh2, kappa, g != nullptr, &e, gg, hh);
    if (E) E[r] = e;
    if (!g) return;
    for (int k = 0; k < 2 * nv; ++k) g[2 * nv * (size_t)r + k] = gg[k];
    for (int k = 0; k < 4 * nv * nv; ++k) H[4 * nv * nv * (size_t)r + k] = hh[k];
}

// ---------------------------------------------------------------- constraint finding
// find_constraints_2D_PE (NEWTON_IPC.py:159-179): every boundary point against every boundary
// edge; rows go to PP (sorted pair) or PE by PE_type.  Overflow sets cnt[2] and drops the row.
// Grid: x over blocks of points, y over tiles of edges, so that every SM takes part.  GB300
// runs FP32 at many times its FP64 rate: each edge's box, grown by d-hat, is kept in FP32 with
// outward rounding, and a point outside it (tested in FP32, conservatively) skips the exact FP64
// test of the reference.
__global__ void __launch_bounds__(T2) k2_find(int nBP, const int* __restrict__ bp, int nBE, const int* __restrict__ be,
                                              const double* __restrict__ x, double dhat, double dh2, int cap_pp,
                                              int cap_pe, int4* __restrict__ pp, int4* __restrict__ pe, int* __restrict__ cnt) {
    __shared__ int se[TILE][2];
    __shared__ double sx[TILE][4];
    __shared__ float4 sb[TILE];      // (lo.x, lo.y, hi.x, hi.y) of the edge box grown by d-hat
    const int t0 = blockIdx.y * TILE;
    const int nt = min(TILE, nBE - t0);
    for (int k = threadIdx.x; k < nt; k += blockDim.x) {
        const int a = be[2 * (size_t)(t0 + k)], b = be[2 * (size_t)(t0 + k) + 1];
        se[k][0] = a;
        se[k][1] = b;
        const double2 xa = ld2(x, a), xb = ld2(x, b);
        sx[k][0] = xa.x;
        sx[k][1] = xa.y;
        sx[k][2] = xb.x;
        sx[k][3] = xb.y;
        sb[k] = make_float4(__double2float_rd(fmin(xa.x, xb.x) - dhat), __double2float_rd(fmin(xa.y, xb.y) - dhat),
                            __double2float_ru(fmax(xa.x, xb.x) + dhat), __double2float_ru(fmax(xa.y, xb.y) + dhat));
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nBP) return;
    const int p = bp[i];
    const double2 v = ld2(x, p);
    const double xp[2] = {v.x, v.y};
    const float px = (float)v.x, py = (float)v.y;
    for (int k = 0; k < nt; ++k) {
        const float4 bx = sb[k];
        if (px < bx.x || py < bx.y || px > bx.z || py > bx.w) continue;
        const int e0 = se[k][0], e1 = se[k][1];
        if (p == e0 || p == e1) continue;
        const double* x0 = &sx[k][0];
        const double* x1 = &sx[k][2];
        if (!pe2_broad(xp, x0, x1, dhat)) continue;
        const int c = pe2_type(xp, x0, x1);
        if (c < 2) {
            const int o = c == 0 ? e0 : e1;
            if (pp2_dist2(xp, c == 0 ? x0 : x1) < dh2) {
                const int slot = atomicAdd(&cnt[0], 1);
                if (slot < cap_pp) pp[slot] = make_int4(min(p, o), max(p, o), 0, 0);
                else atomicOr(&cnt[2], 1);
            }
        } else if (pe2_dist2(xp, x0, x1) < dh2) {
            const int slot = atomicAdd(&cnt[1], 1);
            if (slot < cap_pe) pe[slot] = make_int4(p, e0, e1, 0);
            else atomicOr(&cnt[2], 1);
        }
    }
}

// rows <-> 64-bit keys in lexicographic order (PP: 32 + 32 bits; PE: 21 bits per id)
__global__ void k2_row_keys(int type, int n, const int4* __restrict__ rows, unsigned long long* __restrict__ keys) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int4 q = rows[r];
    keys[r] = type == 0 ? ((unsigned long long)q.x << 32) | (unsigned)q.y
                        : ((unsigned long long)q.x << 42) | ((unsigned long long)q.y << 21) | (unsigned long long)q.z;
}
__global__ void k2_key_rows(int type, int n, const unsigned long long* __restrict__ keys, int4* __restrict__ rows) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const unsigned long long k = keys[r];
    rows[r] = type == 0 ? make_int4((int)(k >> 32), (int)(k & 0xffffffffull), 0, 0)
                        : make_int4((int)(k >> 42), (int)((k >> 21) & 0x1fffff), (int)(k & 0x1fffff), 0);
}

// ---------------------------------------------------------------- assembly
// contribution ids: [0, 9T) element blocks e*9 + a*3+b; then PP rows r*4 + v*2+w; then PE rows
// r*9 + v*3+w; then one inertia entry per vertex.  Key = row << 32 | col (vertex ids).
struct Src2 {
    int nT, nPP, nPE, nV;
    long long pp0, pe0, m0, n;
};
__global__ void k2_assembly_keys(Src2 s, const int* __restrict__ tris, const int4* __restrict__ pp, const int4* __restrict__ pe,
                                 unsigned long long* __restrict__ keys, int* __restrict__ vals) {
    const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (c >= s.n) return;
    int r, cl;
    if (c < s.pp0) {
        const long long e = c / 9;
        const int b = (int)(c % 9);
        r = tris[3 * e + b / 3];
        cl = tris[3 * e + b % 3];
    } else if (c < s.pe0) {
        const long long k = c - s.pp0;
        const int4 q = pp[k / 4];
        const int b = (int)(k % 4);
        r = (b / 2) ? q.y : q.x;
        cl = (b % 2) ? q.y : q.x;
    } else if (c < s.m0) {
        const long long k = c - s.pe0;
        const int4 q = pe[k / 9];
        const int b = (int)(k % 9);
        const int id[3] = {q.x, q.y, q.z};
        r = id[b / 3];
        cl = id[b % 3];
    } else {
        r = cl = (int)(c - s.m0);
    }
    keys[c] = ((unsigned long long)r << 32) | (unsigned)cl;
    vals[c] = (int)c;
}

// one thread per (row, col) run: the block sum in id order; a diagonal run also carries the
// gradients of its sources into rhs = -grad - m (x - xTilde) (NEWTON_IPC.py:545-567)
__global__ void k2_assembly_reduce(Src2 s, int nu, const unsigned long long* __restrict__ ukeys, const int* __restrict__ ustart,
                                   const int* __restrict__ ids, const double* __restrict__ eH, const double* __restrict__ eg,
                                   const double* __restrict__ ppH, const double* __restrict__ ppg, const double* __restrict__ peH,
                                   const double* __restrict__ peg, const double* __restrict__ mass, const double* __restrict__ x,
                                   const double* __restrict__ xt, double* __restrict__ val, int* __restrict__ col,
                                   int* __restrict__ dpos, double* __restrict__ rhs) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nu) return;
    const unsigned long long key = ukeys[u];
    const int r = (int)(key >> 32), cl = (int)(key & 0xffffffffull);
    double h[4] = {0, 0, 0, 0}, gs[2] = {0, 0};
    const bool diag = r == cl;
    for (int k = ustart[u]; k < ustart[u + 1]; ++k) {
        const long long c = ids[k];
        const double* Hb;
        const double* gb = nullptr;
        if (c < s.pp0) {
            const long long e = c / 9;
            const int b = (int)(c % 9);
            Hb = eH + 4 * c;
            if (diag) gb = eg + 6 * e + 2 * (b / 3);
        } else if (c < s.pe0) {
            const long long q = c - s.pp0;
            Hb = ppH + 4 * q;
            if (diag) gb = ppg + 4 * (q / 4) + 2 * ((q % 4) / 2);
        } else if (c < s.m0) {
            const long long q = c - s.pe0;
            Hb = peH + 4 * q;
            if (diag) gb = peg + 6 * (q / 9) + 2 * ((q % 9) / 3);
        } else {
            const double m = mass[r];
            h[0] += m;
            h[3] += m;
            gs[0] += m * (x[2 * (size_t)r] - xt[2 * (size_t)r]);
            gs[1] += m * (x[2 * (size_t)r + 1] - xt[2 * (size_t)r + 1]);
            continue;
        }
        for (int i = 0; i < 4; ++i) h[i] += Hb[i];
        if (gb) {
            gs[0] += gb[0];
            gs[1] += gb[1];
        }
    }
    for (int i = 0; i < 4; ++i) val[4 * (size_t)u + i] = h[i];
    col[u] = cl;
    if (diag) {
        dpos[r] = u;
        rhs[2 * (size_t)r] = -gs[0];
        rhs[2 * (size_t)r + 1] = -gs[1];
    }
}

// row_ptr[r] = first run whose row is >= r
__global__ void k2_row_ptr(int nV, int nu, const unsigned long long* __restrict__ ukeys, int* __restrict__ rp) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r > nV) return;
    const unsigned long long k = (unsigned long long)r << 32;
    int lo = 0, hi = nu;
    while (lo < hi) {
        const int m = (lo + hi) >> 1;
        if (ukeys[m] < k) lo = m + 1;
        else hi = m;
    }
    rp[r] = lo;
}

// ---------------------------------------------------------------- PCG on 2x2 blocks
struct PCG2 {
    int nV;
    const int* rp;
    const int* col;
    const double* val;
    const int* dpos;
    const unsigned char* fixed;
    double *x, *r, *z, *p, *q, *minv, *part;
    double* sc;        // [0] rz, [1] alpha, [2] beta, [3] |b|^2, [4] |r|^2, [5] rtol^2
    int* flag;         // [0] 1 converged / 2 stopped at maxit, [1] iterations, [2..3] tickets
    int maxit;
};

// last CTA to finish sums the per-CTA partials of n_val values in CTA order
__device__ bool last_cta(int* ticket) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(ticket, 1) == (int)gridDim.x - 1;
    __syncthreads();
    return last;
}
__device__ double sum_parts(const double* part, int n, double* sh) {
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc += part[i];
    return bsum(acc, sh);
}

__global__ void __launch_bounds__(T2) k2_pcg_start(PCG2 a, const double* __restrict__ rhs, double rtol) {
    __shared__ double sh[T2];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double rz = 0.0, bb = 0.0;
    if (i < a.nV) {
        const bool fx = a.fixed[i];
        const double b0 = fx ? 0.0 : rhs[2 * (size_t)i], b1 = fx ? 0.0 : rhs[2 * (size_t)i + 1];
        double m[4] = {1, 0, 0, 1};
        if (!fx) {
            const double* D = a.val + 4 * (size_t)a.dpos[i];
            const double det = D[0] * D[3] - D[1] * D[2];
            m[0] = D[3] / det;
            m[1] = -D[1] / det;
            m[2] = -D[2] / det;
            m[3] = D[0] / det;
        }
        for (int k = 0; k < 4; ++k) a.minv[4 * (size_t)i + k] = m[k];
        const double z0 = m[0] * b0 + m[1] * b1, z1 = m[2] * b0 + m[3] * b1;
        a.x[2 * (size_t)i] = 0.0;
        a.x[2 * (size_t)i + 1] = 0.0;
        a.r[2 * (size_t)i] = b0;
        a.r[2 * (size_t)i + 1] = b1;
        a.z[2 * (size_t)i] = z0;
        a.z[2 * (size_t)i + 1] = z1;
        a.p[2 * (size_t)i] = z0;
        a.p[2 * (size_t)i + 1] = z1;
        rz = b0 * z0 + b1 * z1;
        bb = b0 * b0 + b1 * b1;
    }
    const double s0 = bsum(rz, sh), s1 = bsum(bb, sh);
    if (threadIdx.x == 0) {
        a.part[blockIdx.x] = s0;
        a.part[gridDim.x + blockIdx.x] = s1;
    }
    if (!last_cta(&a.flag[2])) return;
    const double t0 = sum_parts(a.part, gridDim.x, sh), t1 = sum_parts(a.part + gridDim.x, gridDim.x, sh);
    if (threadIdx.x == 0) {
        a.sc[0] = t0;
        a.sc[3] = t1;
        a.sc[4] = t1;
        a.sc[5] = rtol * rtol;
        a.flag[0] = t1 == 0.0 ? 1 : (a.maxit <= 0 ? 2 : 0);
        a.flag[1] = 0;
        a.flag[2] = 0;
    }
}

// q = A p (Dirichlet rows and columns replaced by the identity, NEWTON_IPC.py:758-774), p.q
__global__ void __launch_bounds__(T2) k2_pcg_spmv(PCG2 a) {
    __shared__ double sh[T2];
    if (a.flag[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double pq = 0.0;
    if (i < a.nV) {
        double q0, q1;
        const double p0 = a.p[2 * (size_t)i], p1 = a.p[2 * (size_t)i + 1];
        if (a.fixed[i]) {
            q0 = p0;
            q1 = p1;
        } else {
            q0 = q1 = 0.0;
            for (int k = a.rp[i]; k < a.rp[i + 1]; ++k) {
                const int j = a.col[k];
                if (a.fixed[j]) continue;
                const double* B = a.val + 4 * (size_t)k;
                const double u0 = a.p[2 * (size_t)j], u1 = a.p[2 * (size_t)j + 1];
                q0 += B[0] * u0 + B[1] * u1;
                q1 += B[2] * u0 + B[3] * u1;
            }
        }
        a.q[2 * (size_t)i] = q0;
        a.q[2 * (size_t)i + 1] = q1;
        pq = p0 * q0 + p1 * q1;
    }
    const double s0 = bsum(pq, sh);
    if (threadIdx.x == 0) a.part[blockIdx.x] = s0;
    if (!last_cta(&a.flag[2])) return;
    const double t = sum_parts(a.part, gridDim.x, sh);
    if (threadIdx.x == 0) {
        a.sc[1] = a.sc[0] / t;
        a.flag[2] = 0;
    }
}

// x += alpha p, r -= alpha q, z = M^-1 r; r.z and |r|^2 give beta and the convergence test
__global__ void __launch_bounds__(T2) k2_pcg_update(PCG2 a) {
    __shared__ double sh[T2];
    if (a.flag[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double al = a.sc[1];
    double rz = 0.0, rr = 0.0;
    if (i < a.nV) {
        const size_t o = 2 * (size_t)i;
        a.x[o] += al * a.p[o];
        a.x[o + 1] += al * a.p[o + 1];
        const double r0 = a.r[o] - al * a.q[o], r1 = a.r[o + 1] - al * a.q[o + 1];
        a.r[o] = r0;
        a.r[o + 1] = r1;
        const double* m = a.minv + 4 * (size_t)i;
        const double z0 = m[0] * r0 + m[1] * r1, z1 = m[2] * r0 + m[3] * r1;
        a.z[o] = z0;
        a.z[o + 1] = z1;
        rz = r0 * z0 + r1 * z1;
        rr = r0 * r0 + r1 * r1;
    }
    const double s0 = bsum(rz, sh), s1 = bsum(rr, sh);
    if (threadIdx.x == 0) {
        a.part[blockIdx.x] = s0;
        a.part[gridDim.x + blockIdx.x] = s1;
    }
    if (!last_cta(&a.flag[3])) return;
    const double t0 = sum_parts(a.part, gridDim.x, sh), t1 = sum_parts(a.part + gridDim.x, gridDim.x, sh);
    if (threadIdx.x == 0) {
        a.sc[2] = t0 / a.sc[0];
        a.sc[0] = t0;
        a.sc[4] = t1;
        a.flag[1] += 1;
        if (t1 <= a.sc[5] * a.sc[3]) a.flag[0] = 1;
        else if (a.flag[1] >= a.maxit) a.flag[0] = 2;
        a.flag[3] = 0;
    }
}

__global__ void __launch_bounds__(T2) k2_pcg_dir(PCG2 a) {
    if (a.flag[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nV) return;
    const double be = a.sc[2];
    const size_t o = 2 * (size_t)i;
    a.p[o] = a.z[o] + be * a.p[o];
    a.p[o + 1] = a.z[o + 1] + be * a.p[o + 1];
}

// The whole PCG loop in one cooperative launch, for systems whose rows fit one CTA per SM:
// small scenes are bound by per-kernel launch and tail latency, not by bandwidth.  Three grid
// barriers per iteration; every CTA sums the per-CTA partials in the same fixed order, so all
// CTAs hold the same scalars and take the same branch, and results are deterministic.  The
// partials of p.q and of (r.z, |r|^2) live in separate arrays, so a fast CTA's next write never
// meets a slow CTA's read.  part: 3 * gridDim.x doubles.
__global__ void __launch_bounds__(T2) k2_pcg_coop(PCG2 a, const double* __restrict__ rhs, double rtol) {
    cg::grid_group grid = cg::this_grid();
    __shared__ double sh[T2];
    const int G = gridDim.x;
    const int stride = G * blockDim.x;
    double* part_pq = a.part;
    double* part_rz = a.part + G;
    double* part_rr = a.part + 2 * G;
    double rz = 0.0, bb = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nV; i += stride) {
        const bool fx = a.fixed[i];
        const double b0 = fx ? 0.0 : rhs[2 * (size_t)i], b1 = fx ? 0.0 : rhs[2 * (size_t)i + 1];
        double m[4] = {1, 0, 0, 1};
        if (!fx) {
            const double* D = a.val + 4 * (size_t)a.dpos[i];
            const double det = D[0] * D[3] - D[1] * D[2];
            m[0] = D[3] / det;
            m[1] = -D[1] / det;
            m[2] = -D[2] / det;
            m[3] = D[0] / det;
        }
        for (int k = 0; k < 4; ++k) a.minv[4 * (size_t)i + k] = m[k];
        const double z0 = m[0] * b0 + m[1] * b1, z1 = m[2] * b0 + m[3] * b1;
        const size_t o = 2 * (size_t)i;
        a.x[o] = 0.0;
        a.x[o + 1] = 0.0;
        a.r[o] = b0;
        a.r[o + 1] = b1;
        a.z[o] = z0;
        a.z[o + 1] = z1;
        a.p[o] = z0;
        a.p[o + 1] = z1;
        rz += b0 * z0 + b1 * z1;
        bb += b0 * b0 + b1 * b1;
    }
    {
        const double s0 = bsum(rz, sh), s1 = bsum(bb, sh);
        if (threadIdx.x == 0) {
            part_rz[blockIdx.x] = s0;
            part_rr[blockIdx.x] = s1;
        }
    }
    grid.sync();
    rz = sum_parts(part_rz, G, sh);
    bb = sum_parts(part_rr, G, sh);
    const double tol2 = rtol * rtol * bb;
    if (bb == 0.0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            a.flag[0] = 1;
            a.flag[1] = 0;
        }
        return;
    }
    for (int it = 1; it <= a.maxit; ++it) {
        // q = A p with the Dirichlet rows and columns replaced by the identity
        double pq = 0.0;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nV; i += stride) {
            const size_t o = 2 * (size_t)i;
            const double p0 = a.p[o], p1 = a.p[o + 1];
            double q0 = p0, q1 = p1;
            if (!a.fixed[i]) {
                q0 = q1 = 0.0;
                for (int k = a.rp[i]; k < a.rp[i + 1]; ++k) {
                    const int j = a.col[k];
                    if (a.fixed[j]) continue;
                    const double* B = a.val + 4 * (size_t)k;
                    const double u0 = a.p[2 * (size_t)j], u1 = a.p[2 * (size_t)j + 1];
                    q0 += B[0] * u0 + B[1] * u1;
                    q1 += B[2] * u0 + B[3] * u1;
                }
            }
            a.q[o] = q0;
            a.q[o + 1] = q1;
            pq += p0 * q0 + p1 * q1;
        }
        {
            const double s0 = bsum(pq, sh);
            if (threadIdx.x == 0) part_pq[blockIdx.x] = s0;
        }
        grid.sync();
        const double alpha = rz / sum_parts(part_pq, G, sh);
        double rz_new = 0.0, rr = 0.0;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nV; i += stride) {
            const size_t o = 2 * (size_t)i;
            a.x[o] += alpha * a.p[o];
            a.x[o + 1] += alpha * a.p[o + 1];
            const double r0 = a.r[o] - alpha * a.q[o], r1 = a.r[o + 1] - alpha * a.q[o + 1];
            a.r[o] = r0;
            a.r[o + 1] = r1;
            const double* m = a.minv + 4 * (size_t)i;
            const double z0 = m[0] * r0 + m[1] * r1, z1 = m[2] * r0 + m[3] * r1;
            a.z[o] = z0;
            a.z[o + 1] = z1;
            rz_new += r0 * z0 + r1 * z1;
            rr += r0 * r0 + r1 * r1;
        }
        {
            const double s0 = bsum(rz_new, sh), s1 = bsum(rr, sh);
            if (threadIdx.x == 0) {
                part_rz[blockIdx.x] = s0;
                part_rr[blockIdx.x] = s1;
            }
        }
        grid.sync();
        rz_new = sum_parts(part_rz, G, sh);
        rr = sum_parts(part_rr, G, sh);
        if (rr <= tol2) {
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                a.flag[0] = 1;
                a.flag[1] = it;
            }
            return;
        }
        const double beta = rz_new / rz;
        rz = rz_new;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nV; i += stride) {
            const size_t o = 2 * (size_t)i;
            a.p[o] = a.z[o] + beta * a.p[o];
            a.p[o + 1] = a.z[o + 1] + beta * a.p[o + 1];
        }
        grid.sync();
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.flag[0] = 2;
        a.flag[1] = a.maxit;
    }
}

// ---------------------------------------------------------------- energy, residual, CCD, collision
// compute_energy (NEWTON_IPC.py:514-542, dim 2): inertia, elasticity and the two barrier lists
// over one index space, per-CTA partials on a fixed grid
__global__ void __launch_bounds__(T2) k2_energy(int nV, int nT, int nPP, int nPE, const double* __restrict__ x,
                                                const double* __restrict__ xt, const double* __restrict__ mass,
                                                const int* __restrict__ tris, const double* __restrict__ IB,
                                                const double* __restrict__ vol, const double* __restrict__ lam,
                                                const double* __restrict__ mu, double dt2, const int4* __restrict__ pp,
                                                const int4* __restrict__ pe, double dh2, double kappa, double* __restrict__ part) {
    __shared__ double sh[T2];
    double acc = 0.0;
    const long long n = (long long)nV + nT + nPP + nPE;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        if (k < nV) {
            const double dx = x[2 * k] - xt[2 * k], dy = x[2 * k + 1] - xt[2 * k + 1];
            acc += 0.5 * mass[k] * (dx * dx + dy * dy);
        } else if (k < (long long)nV + nT) {
            const long long e = k - nV;
            double X[6];
            for (int a = 0; a < 3; ++a) {
                const double2 p = ld2(x, tris[3 * e + a]);
                X[2 * a] = p.x;
                X[2 * a + 1] = p.y;
            }
            const double* ib = IB + 4 * e;
            const double Ds[4] = {X[2] - X[0], X[4] - X[0], X[3] - X[1], X[5] - X[1]};
            const double F[4] = {Ds[0] * ib[0] + Ds[1] * ib[2], Ds[0] * ib[1] + Ds[1] * ib[3], Ds[2] * ib[0] + Ds[3] * ib[2],
                                 Ds[2] * ib[1] + Ds[3] * ib[3]};
            acc += fc2_psi_F(F, lam[e], mu[e]) * dt2 * vol[e];
        } else {
            const bool isPP = k < (long long)nV + nT + nPP;
            const int4 q = isPP ? pp[k - nV - nT] : pe[k - nV - nT - nPP];
            const double2 a = ld2(x, q.x), b = ld2(x, q.y);
            const double pa[2] = {a.x, a.y}, pb[2] = {b.x, b.y};
            double d;
            if (isPP) {
                d = pp2_dist2(pa, pb);
            } else {
                const double2 c = ld2(x, q.z);
                const double pc[2] = {c.x, c.y};
                d = pe2_dist2(pa, pb, pc);
            }
            acc += barrier_E(d, dh2, kappa);
        }
    }
    const double s = bsum(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}
__global__ void __launch_bounds__(T2) k2_sum(int n, const double* __restrict__ part, double* __restrict__ out) {
    __shared__ double sh[T2];
    const double s = sum_parts(part, n, sh);
    if (threadIdx.x == 0) *out = s;
}

__global__ void __launch_bounds__(T2) k2_absmax(int n, const double* __restrict__ p, double* __restrict__ out) {
    __shared__ double sh[T2];
    double m = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) m = fmax(m, fabs(p[i]));
    sh[threadIdx.x] = m;
    __syncthreads();
    for (int s = T2 / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) amax_pos(out, sh[0]);
}

// compute_filter_2D_PE (NEWTON_IPC.py:361-374): min over boundary point / edge pairs.  Grid as
// k2_find; the moving boxes of the moving broad phase (ipc.py:374-381) are pre-tested in FP32
// with outward rounding.
__global__ void __launch_bounds__(T2) k2_ccd(int nBP, const int* __restrict__ bp, int nBE, const int* __restrict__ be,
                                             const double* __restrict__ x, const double* __restrict__ d, double dhat, double eta,
                                             double* __restrict__ alpha) {
    __shared__ int se[TILE][2];
    __shared__ double sx[TILE][8];
    __shared__ float4 sb[TILE];
    __shared__ double red[T2];
    const int t0 = blockIdx.y * TILE;
    const int nt = min(TILE, nBE - t0);
    for (int k = threadIdx.x; k < nt; k += blockDim.x) {
        const int a = be[2 * (size_t)(t0 + k)], b = be[2 * (size_t)(t0 + k) + 1];
        se[k][0] = a;
        se[k][1] = b;
        const double2 xa = ld2(x, a), xb = ld2(x, b), da = ld2(d, a), db = ld2(d, b);
        sx[k][0] = xa.x;
        sx[k][1] = xa.y;
        sx[k][2] = xb.x;
        sx[k][3] = xb.y;
        sx[k][4] = da.x;
        sx[k][5] = da.y;
        sx[k][6] = db.x;
        sx[k][7] = db.y;
        const double ax = xa.x + da.x, ay = xa.y + da.y, bx = xb.x + db.x, by = xb.y + db.y;
        sb[k] = make_float4(__double2float_rd(fmin(fmin(xa.x, xb.x), fmin(ax, bx)) - dhat),
                            __double2float_rd(fmin(fmin(xa.y, xb.y), fmin(ay, by)) - dhat),
                            __double2float_ru(fmax(fmax(xa.x, xb.x), fmax(ax, bx)) + dhat),
                            __double2float_ru(fmax(fmax(xa.y, xb.y), fmax(ay, by)) + dhat));
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double best = 1.0;
    if (i < nBP) {
        const int p = bp[i];
        const double2 v = ld2(x, p), w = ld2(d, p);
        const double xp[2] = {v.x, v.y}, dp[2] = {w.x, w.y};
        // the point's swept box in FP32, rounded outward
        const float plx = __double2float_rd(fmin(v.x, v.x + w.x)), ply = __double2float_rd(fmin(v.y, v.y + w.y));
        const float phx = __double2float_ru(fmax(v.x, v.x + w.x)), phy = __double2float_ru(fmax(v.y, v.y + w.y));
        for (int k = 0; k < nt; ++k) {
            const float4 bx = sb[k];
            if (phx < bx.x || phy < bx.y || plx > bx.z || ply > bx.w) continue;
            if (p == se[k][0] || p == se[k][1]) continue;
            const double* s = sx[k];
            if (pe2_moving_broad(xp, s, s + 2, dp, s + 4, s + 6, dhat)) best = fmin(best, pe2_ccd(xp, s, s + 2, dp, s + 4, s + 6, eta));
        }
    }
    red[threadIdx.x] = best;
    __syncthreads();
    for (int s = T2 / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] = fmin(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0 && red[0] < 1.0) amin_pos(alpha, red[0]);
}

// check_collision_2D (NEWTON_IPC.py:843-854): a boundary point inside a triangle it is not a
// vertex of.  Grid as k2_find; the triangle's box (FP32, rounded outward) is tested first.
__global__ void __launch_bounds__(T2) k2_collision(int nBP, const int* __restrict__ bp, int nT, const int* __restrict__ tris,
                                                   const double* __restrict__ x, int* __restrict__ hit) {
    __shared__ int st[TILE][3];
    __shared__ double sx[TILE][6];
    __shared__ float4 sb[TILE];
    const int t0 = blockIdx.y * TILE;
    const int nt = min(TILE, nT - t0);
    for (int k = threadIdx.x; k < nt; k += blockDim.x) {
        double lx = 1e300, ly = 1e300, hx = -1e300, hy = -1e300;
        for (int a = 0; a < 3; ++a) {
            const int v = tris[3 * (size_t)(t0 + k) + a];
            st[k][a] = v;
            const double2 xv = ld2(x, v);
            sx[k][2 * a] = xv.x;
            sx[k][2 * a + 1] = xv.y;
            lx = fmin(lx, xv.x);
            ly = fmin(ly, xv.y);
            hx = fmax(hx, xv.x);
            hy = fmax(hy, xv.y);
        }
        sb[k] = make_float4(__double2float_rd(lx), __double2float_rd(ly), __double2float_ru(hx), __double2float_ru(hy));
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nBP) return;
    const int p = bp[i];
    const double2 v = ld2(x, p);
    const double xp[2] = {v.x, v.y};
    const float px = (float)v.x, py = (float)v.y;
    for (int k = 0; k < nt; ++k) {
        const float4 bx = sb[k];
        if (px < bx.x || py < bx.y || px > bx.z || py > bx.w) continue;
        if (p == st[k][0] || p == st[k][1] || p == st[k][2]) continue;
        if (point_in_tri2(xp, sx[k], sx[k] + 2, sx[k] + 4)) {
            atomicOr(hit, 1);
            return;
        }
    }
}

// ---------------------------------------------------------------- vector updates (dim 2)
__global__ void k2_xn_xtilde(int n2, const double* __restrict__ x, const double* __restrict__ v, double dt, double gravity,
                             double* __restrict__ xn, double* __restrict__ xt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n2) return;
    const double xi = x[i];
    xn[i] = xi;
    double t = xi + dt * v[i];
    if (i % 2 == 1) t += dt * dt * gravity;
    xt[i] = t;
}
__global__ void k2_move_nodes(int n2, const unsigned char* __restrict__ fixed, const double* __restrict__ target,
                              double* __restrict__ x, double* __restrict__ xt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n2 || !fixed[i / 2]) return;
    x[i] = target[i];
    xt[i] = target[i];
}
__global__ void k2_apply_sol(int n2, const double* __restrict__ xp, const double* __restrict__ sol, double alpha,
                             double* __restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n2) x[i] = xp[i] + sol[i] * alpha;
}
__global__ void k2_compute_v(int n2, const double* __restrict__ x, const double* __restrict__ xn, double dt, double* __restrict__ v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n2) v[i] = (x[i] - xn[i]) / dt;
}

__global__ void k2_ccd_pairs(int n, const double* __restrict__ xq, const double* __restrict__ pq, double eta,
                             double* __restrict__ toc) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const double* X = xq + 6 * (size_t)c;
    const double* P = pq + 6 * (size_t)c;
    toc[c] = pe2_ccd(X, X + 2, X + 4, P, P + 2, P + 4, eta);
}

constexpr int PCG_CHUNK = 32;   // iterations between host checks of the convergence flag

void pcg_chunk(const PCG2& a, int nb, cudaStream_t s) {
    for (int k = 0; k < PCG_CHUNK; ++k) {
        k2_pcg_spmv<<<nb, T2, 0, s>>>(a);
        k2_pcg_update<<<nb, T2, 0, s>>>(a);
        k2_pcg_dir<<<nb, T2, 0, s>>>(a);
    }
}

void drop_graph2(Ctx2* c) {
    if (c->graph_exec) cudaGraphExecDestroy((cudaGraphExec_t)c->graph_exec);
    c->graph_exec = nullptr;
    c->graph_sig.clear();
}

// the chunk graph for these arguments; false when capture is unavailable (the caller then
// launches the kernels directly)
bool pcg_graph(Ctx2* c, const PCG2& a, int nb) {
    std::vector<unsigned char> sig(sizeof(PCG2) + sizeof(int));
    memcpy(sig.data(), &a, sizeof(PCG2));
    memcpy(sig.data() + sizeof(PCG2), &nb, sizeof(int));
    if (c->graph_exec && sig == c->graph_sig) return true;
    drop_graph2(c);
    if (!c->cap_stream) {
        cudaStream_t cs;
        if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) return false;
        c->cap_stream = cs;
    }
    cudaStream_t cs = (cudaStream_t)c->cap_stream;
    if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return false;
    pcg_chunk(a, nb, cs);
    cudaGraph_t g = nullptr;
    if (cudaStreamEndCapture(cs, &g) != cudaSuccess || !g) {
        cudaGetLastError();
        return false;
    }
    cudaGraphExec_t ex = nullptr;
    const bool ok = cudaGraphInstantiate(&ex, g, 0ull) == cudaSuccess;
    cudaGraphDestroy(g);
    if (!ok) {
        cudaGetLastError();
        return false;
    }
    c->graph_exec = ex;
    c->graph_sig = sig;
    return true;
}

template <class F>
int cub2(Ctx2* c, F&& f) {
    size_t need = 0;
    if (f(nullptr, need) != cudaSuccess) return FIPC_ERR_CUDA;
    if (c->cub_tmp.ensure(need)) return FIPC_ERR_CUDA;
    size_t have = c->cub_tmp.bytes;
    if (f(c->cub_tmp.p, have) != cudaSuccess) return FIPC_ERR_CUDA;
    return FIPC_OK;
}

template <class T>
int upload2(T** dst, const T* src, size_t n) {
    *dst = nullptr;
    if (n == 0) return FIPC_OK;
    if (cudaMalloc((void**)dst, sizeof(T) * n) != cudaSuccess) return FIPC_ERR_CUDA;
    if (cudaMemcpy(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice) != cudaSuccess) return FIPC_ERR_CUDA;
    return FIPC_OK;
}

void release_ctx2(Ctx2* c) {
    cudaFree(c->tris);
    cudaFree(c->bp);
    cudaFree(c->be);
    cudaFree(c->IB);
    cudaFree(c->vol);
    cudaFree(c->lam);
    cudaFree(c->mu);
    cudaFree(c->mass);
    DBuf* bufs[] = {&c->elem_g, &c->elem_H, &c->rows[0], &c->rows[1], &c->rows_tmp, &c->keys, &c->keys_alt, &c->cnt_d,
                    &c->cub_tmp, &c->scal, &c->cg[0], &c->cg[1], &c->cH[0], &c->cH[1], &c->a_keys, &c->a_keys_alt,
                    &c->a_vals, &c->a_vals_alt, &c->a_ukeys, &c->a_ucount, &c->a_ustart, &c->val, &c->col, &c->row_ptr,
                    &c->dpos, &c->rhs, &c->pvec, &c->ppart, &c->pflag, &c->epart, &c->eout};
    for (DBuf* b : bufs) b->release();
    drop_graph2(c);
    if (c->cap_stream) cudaStreamDestroy((cudaStream_t)c->cap_stream);
    c->cap_stream = nullptr;
}

}  // namespace
}  // namespace fipc

using namespace fipc;

struct fipc2d_ctx_impl {
    Ctx2 c;
};

extern "C" {

int fipc2d_ctx_create(fipc2d_ctx_impl** out, int n_verts, int n_tris, const int* tris_h, const double* x_rest_h,
                      const double* lam_h, const double* mu_h, double rho, int n_bp, const int* bp_h, int n_be,
                      const int* be_h, double dhat2, double dt) {
    if (!out || n_verts <= 0 || n_verts >= (1 << 21) || n_tris < 0 || n_bp < 0 || n_be < 0 || !x_rest_h ||
        (n_tris && (!tris_h || !lam_h || !mu_h)) || (n_bp && !bp_h) || (n_be && !be_h) || dhat2 <= 0 || dt <= 0)
        return FIPC_ERR_ARGUMENT;
    *out = nullptr;
    for (long long k = 0; k < 3ll * n_tris; ++k)
        if (tris_h[k] < 0 || tris_h[k] >= n_verts) return FIPC_ERR_ARGUMENT;
    for (int k = 0; k < n_bp; ++k)
        if (bp_h[k] < 0 || bp_h[k] >= n_verts) return FIPC_ERR_ARGUMENT;
    for (long long k = 0; k < 2ll * n_be; ++k)
        if (be_h[k] < 0 || be_h[k] >= n_verts) return FIPC_ERR_ARGUMENT;
    // compute_restT_and_m (NEWTON_IPC.py:485-494): restT = [x1-x0, x2-x0], vol0 = det / 2,
    // mass = vol0 rho / 3 to each vertex
    std::vector<double> IB(4ull * n_tris), vol(n_tris), mass(n_verts, 0.0);
    for (int e = 0; e < n_tris; ++e) {
        const int* t = tris_h + 3ll * e;
        const double* a = x_rest_h + 2ll * t[0];
        const double* b = x_rest_h + 2ll * t[1];
        const double* c = x_rest_h + 2ll * t[2];
        const double T00 = b[0] - a[0], T01 = c[0] - a[0], T10 = b[1] - a[1], T11 = c[1] - a[1];
        const double det = T00 * T11 - T01 * T10;
        if (!(det > 0)) return FIPC_ERR_ARGUMENT;   // inverted or degenerate rest triangle
        IB[4ll * e] = T11 / det;
        IB[4ll * e + 1] = -T01 / det;
        IB[4ll * e + 2] = -T10 / det;
        IB[4ll * e + 3] = T00 / det;
        vol[e] = det / 2;
        const double m = vol[e] * rho / 3;
        for (int k = 0; k < 3; ++k) mass[t[k]] += m;
    }
    fipc2d_ctx_impl* h = new fipc2d_ctx_impl();
    Ctx2* c = &h->c;
    c->nV = n_verts;
    c->nT = n_tris;
    c->nBP = n_bp;
    c->nBE = n_be;
    c->dhat2 = dhat2;
    c->dhat = sqrt(dhat2);
    c->dt = dt;
    // compute_adaptive_kappa x 10 (NEWTON_IPC.py:116-124, 943)
    double total = 0.0;
    for (int i = 0; i < n_verts; ++i) total += mass[i];
    c->kappa = 1.0e13 * total / n_verts / (4.0e-16 * barrier_H(1.0e-16, dhat2, 1.0)) * 10.0;
    // compute_mean_of_boundary_edges (NEWTON_IPC.py:127-134)
    double len = 0.0;
    for (int k = 0; k < n_be; ++k) {
        const double* a = x_rest_h + 2ll * be_h[2 * k];
        const double* b = x_rest_h + 2ll * be_h[2 * k + 1];
        len += sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]));
    }
    c->mean_edge = n_be ? len / n_be : 0.0;
    int st = upload2(&c->tris, tris_h, 3ull * n_tris);
    st |= upload2(&c->bp, bp_h, (size_t)n_bp);
    st |= upload2(&c->be, be_h, 2ull * n_be);
    st |= upload2(&c->IB, IB.data(), IB.size());
    st |= upload2(&c->vol, vol.data(), vol.size());
    st |= upload2(&c->lam, lam_h, (size_t)n_tris);
    st |= upload2(&c->mu, mu_h, (size_t)n_tris);
    st |= upload2(&c->mass, mass.data(), mass.size());
    if (st) {
        release_ctx2(c);
        delete h;
        return FIPC_ERR_CUDA;
    }
    *out = h;
    return FIPC_OK;
}

int fipc2d_ctx_destroy(fipc2d_ctx_impl* h) {
    if (!h) return FIPC_ERR_ARGUMENT;
    release_ctx2(&h->c);
    delete h;
    return FIPC_OK;
}

int fipc2d_ctx_params(fipc2d_ctx_impl* h, double* kappa_h, double* mean_edge_h) {
    if (!h) return FIPC_ERR_ARGUMENT;
    if (kappa_h) *kappa_h = h->c.kappa;
    if (mean_edge_h) *mean_edge_h = h->c.mean_edge;
    return FIPC_OK;
}

int fipc2d_ctx_set_kappa(fipc2d_ctx_impl* h, double kappa) {
    if (!h || !(kappa > 0)) return FIPC_ERR_ARGUMENT;
    h->c.kappa = kappa;
    return FIPC_OK;
}

int fipc2d_ctx_mass(fipc2d_ctx_impl* h, double* mass_h) {
    if (!h || !mass_h) return FIPC_ERR_ARGUMENT;
    FIPC_CUDA(cudaMemcpy(mass_h, h->c.mass, sizeof(double) * h->c.nV, cudaMemcpyDeviceToHost));
    return FIPC_OK;
}

int fipc2d_compute_xn_and_xtilde(int n_verts, const double* x, const double* v, double dt, double gravity, double* xn,
                                 double* xtilde, void* stream) {
    if (n_verts < 0 || !x || !v || !xn || !xtilde) return FIPC_ERR_ARGUMENT;
    if (!n_verts) return FIPC_OK;
    k2_xn_xtilde<<<nb2(2ll * n_verts, 256), 256, 0, (cudaStream_t)stream>>>(2 * n_verts, x, v, dt, gravity, xn, xtilde);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc2d_move_nodes(int n_verts, const unsigned char* fixed, const double* target, double* x, double* xtilde, void* stream) {
    if (n_verts < 0 || !fixed || !target || !x || !xtilde) return FIPC_ERR_ARGUMENT;
    if (!n_verts) return FIPC_OK;
    k2_move_nodes<<<nb2(2ll * n_verts, 256), 256, 0, (cudaStream_t)stream>>>(2 * n_verts, fixed, target, x, xtilde);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc2d_apply_sol(int n_verts, const double* xprev, const double* sol, double alpha, double* x, void* stream) {
    if (n_verts < 0 || !xprev || !sol || !x) return FIPC_ERR_ARGUMENT;
    if (!n_verts) return FIPC_OK;
    k2_apply_sol<<<nb2(2ll * n_verts, 256), 256, 0, (cudaStream_t)stream>>>(2 * n_verts, xprev, sol, alpha, x);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc2d_compute_v(int n_verts, const double* x, const double* xn, double dt, double* v, void* stream) {
    if (n_verts < 0 || !x || !xn || !v || dt == 0.0) return FIPC_ERR_ARGUMENT;
    if (!n_verts) return FIPC_OK;
    k2_compute_v<<<nb2(2ll * n_verts, 256), 256, 0, (cudaStream_t)stream>>>(2 * n_verts, x, xn, dt, v);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc2d_elements(int n_tris, const int* tris, const double* x, const double* ib, const double* vol, const double* lam,
                    const double* mu, double dt, double* E, double* g, double* H, void* stream) {
    if (n_tris < 0 || !tris || !x || !ib || !vol || !lam || !mu || !al16(x)) return FIPC_ERR_ARGUMENT;
    if (!n_tris) return FIPC_OK;
    k2_elements<<<nb2(n_tris, T2), T2, 0, (cudaStream_t)stream>>>(n_tris, tris, x, ib, vol, lam, mu, dt * dt, E, g, H);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc2d_barrier_rows(int type, int n_rows, const int* rows, const double* x, double dhat2, double kappa, double* E, double* g,
                        double* H, void* stream) {
    if ((type != 0 && type != 1) || n_rows < 0 || !rows || !x || ((g == nullptr) != (H == nullptr)) || !al16(x) || !al16(rows))
        return FIPC_ERR_ARGUMENT;
    if (!n_rows) return FIPC_OK;
    k2_barrier<<<nb2(n_rows, 128), 128, 0, (cudaStream_t)stream>>>(type, n_rows, (const int4*)rows, x, dhat2, kappa, E, g, H);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc2d_ccd_pairs(int n, const double* xq, const double* pq, double eta, double* toc, void* stream) {
    if (n < 0 || !xq || !pq || !toc) return FIPC_ERR_ARGUMENT;
    if (!n) return FIPC_OK;
    k2_ccd_pairs<<<nb2(n, 128), 128, 0, (cudaStream_t)stream>>>(n, xq, pq, eta, toc);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc2d_find_constraints(fipc2d_ctx_impl* h, const double* x, int* counts_h, void* stream) {
    if (!h || !x || !al16(x)) return FIPC_ERR_ARGUMENT;
    Ctx2* c = &h->c;
    cudaStream_t s = (cudaStream_t)stream;
    if (c->cnt_d.ensure(16) || c->scal.ensure(64)) return FIPC_ERR_CUDA;
    int* cnt = c->cnt_d.as<int>();
    for (int t = 0; t < 2; ++t)
        if (c->cap[t] == 0) {
            c->cap[t] = 1024;
            if (c->rows[t].ensure(16ull * c->cap[t])) return FIPC_ERR_CUDA;
        }
    int hc[3] = {0, 0, 0};
    for (int attempt = 0; attempt < 8; ++attempt) {
        FIPC_CUDA(cudaMemsetAsync(cnt, 0, 16, s));
        if (c->nBP && c->nBE) {
            k2_find<<<dim3(nb2(c->nBP, T2), nb2(c->nBE, TILE)), T2, 0, s>>>(c->nBP, c->bp, c->nBE, c->be, x, c->dhat, c->dhat2, c->cap[0], c->cap[1],
                                                  c->rows[0].as<int4>(), c->rows[1].as<int4>(), cnt);
            FIPC_LAUNCHED();
        }
        FIPC_CUDA(cudaMemcpyAsync(hc, cnt, 12, cudaMemcpyDeviceToHost, s));
        FIPC_CUDA(cudaStreamSynchronize(s));
        if (!hc[2]) break;
        for (int t = 0; t < 2; ++t)
            if (hc[t] > c->cap[t]) {
                c->cap[t] = hc[t] + hc[t] / 2 + 1024;
                if (c->rows[t].ensure(16ull * c->cap[t])) return FIPC_ERR_CUDA;
            }
    }
    if (hc[2]) return FIPC_ERR_CAPACITY;
    // np.unique(rows, axis=0) (NEWTON_IPC.py:348-356): sort the packed keys, drop repeats
    for (int t = 0; t < 2; ++t) {
        const int n = hc[t];
        c->h_counts[t] = 0;
        if (!n) continue;
        if (c->keys.ensure(8ull * n) || c->keys_alt.ensure(8ull * n)) return FIPC_ERR_CUDA;
        unsigned long long* k0 = c->keys.as<unsigned long long>();
        unsigned long long* k1 = c->keys_alt.as<unsigned long long>();
        k2_row_keys<<<nb2(n, 256), 256, 0, s>>>(t, n, c->rows[t].as<int4>(), k0);
        FIPC_LAUNCHED();
        cub::DoubleBuffer<unsigned long long> kb(k0, k1);
        int st = cub2(c, [&](void* tm, size_t& b) { return cub::DeviceRadixSort::SortKeys(tm, b, kb, n, 0, 64, s); });
        if (st) return st;
        unsigned long long* sorted = kb.Current();
        unsigned long long* uniq = sorted == k0 ? k1 : k0;
        int* nu_d = (int*)(c->scal.as<char>() + 16);
        st = cub2(c, [&](void* tm, size_t& b) { return cub::DeviceSelect::Unique(tm, b, sorted, uniq, nu_d, n, s); });
        if (st) return st;
        int nu = 0;
        FIPC_CUDA(cudaMemcpyAsync(&nu, nu_d, 4, cudaMemcpyDeviceToHost, s));
        FIPC_CUDA(cudaStreamSynchronize(s));
        k2_key_rows<<<nb2(nu, 256), 256, 0, s>>>(t, nu, uniq, c->rows[t].as<int4>());
        FIPC_LAUNCHED();
        c->h_counts[t] = nu;
    }
    FIPC_CUDA(cudaGetLastError());
    if (counts_h) {
        counts_h[0] = c->h_counts[0];
        counts_h[1] = c->h_counts[1];
    }
    return FIPC_OK;
}

int fipc2d_get_constraints(fipc2d_ctx_impl* h, int type, int* rows, void* stream) {
    if (!h || (type != 0 && type != 1) || !rows) return FIPC_ERR_ARGUMENT;
    if (!h->c.h_counts[type]) return FIPC_OK;
    FIPC_CUDA(cudaMemcpyAsync(rows, h->c.rows[type].p, 16ull * h->c.h_counts[type], cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
    return FIPC_OK;
}

int fipc2d_compute_hessian_and_gradient(fipc2d_ctx_impl* h, const double* x, const double* xtilde, void* stream) {
    if (!h || !x || !xtilde || !al16(x)) return FIPC_ERR_ARGUMENT;
    Ctx2* c = &h->c;
    cudaStream_t s = (cudaStream_t)stream;
    const int nPP = c->h_counts[0], nPE = c->h_counts[1];
    if (c->elem_g.ensure(48ull * c->nT + 8) || c->elem_H.ensure(288ull * c->nT + 8) || c->cg[0].ensure(32ull * nPP + 8) ||
        c->cH[0].ensure(128ull * nPP + 8) || c->cg[1].ensure(48ull * nPE + 8) || c->cH[1].ensure(288ull * nPE + 8))
        return FIPC_ERR_CUDA;
    const double dt2 = c->dt * c->dt;
    if (c->nT) {
        k2_elements<<<nb2(c->nT, T2), T2, 0, s>>>(c->nT, c->tris, x, c->IB, c->vol, c->lam, c->mu, dt2, nullptr,
                                                  c->elem_g.as<double>(), c->elem_H.as<double>());
        FIPC_LAUNCHED();
    }
    for (int t = 0; t < 2; ++t)
        if (c->h_counts[t]) {
            k2_barrier<<<nb2(c->h_counts[t], 128), 128, 0, s>>>(t, c->h_counts[t], c->rows[t].as<int4>(), x, c->dhat2, c->kappa,
                                                                nullptr, c->cg[t].as<double>(), c->cH[t].as<double>());
            FIPC_LAUNCHED();
        }
    Src2 src;
    src.nT = c->nT;
    src.nPP = nPP;
    src.nPE = nPE;
    src.nV = c->nV;
    src.pp0 = 9ll * c->nT;
    src.pe0 = src.pp0 + 4ll * nPP;
    src.m0 = src.pe0 + 9ll * nPE;
    src.n = src.m0 + c->nV;
    if (src.n >= (1ll << 31)) return FIPC_ERR_CAPACITY;
    const int N = (int)src.n;
    if (c->a_keys.ensure(8ull * N) || c->a_keys_alt.ensure(8ull * N) || c->a_vals.ensure(4ull * N) || c->a_vals_alt.ensure(4ull * N) ||
        c->a_ukeys.ensure(8ull * N) || c->a_ucount.ensure(4ull * (N + 1)) || c->a_ustart.ensure(4ull * (N + 1)) ||
        c->val.ensure(32ull * N) || c->col.ensure(4ull * N) || c->row_ptr.ensure(4ull * (c->nV + 1)) ||
        c->dpos.ensure(4ull * c->nV) || c->rhs.ensure(16ull * c->nV) || c->scal.ensure(64))
        return FIPC_ERR_CUDA;
    k2_assembly_keys<<<nb2(N, 256), 256, 0, s>>>(src, c->tris, c->rows[0].as<int4>(), c->rows[1].as<int4>(),
                                                c->a_keys.as<unsigned long long>(), c->a_vals.as<int>());
    FIPC_LAUNCHED();
    cub::DoubleBuffer<unsigned long long> kb(c->a_keys.as<unsigned long long>(), c->a_keys_alt.as<unsigned long long>());
    cub::DoubleBuffer<int> vb(c->a_vals.as<int>(), c->a_vals_alt.as<int>());
    int st = cub2(c, [&](void* tm, size_t& b) { return cub::DeviceRadixSort::SortPairs(tm, b, kb, vb, N, 0, 53, s); });
    if (st) return st;
    int* nu_d = (int*)(c->scal.as<char>() + 32);
    unsigned long long* sk = kb.Current();
    st = cub2(c, [&](void* tm, size_t& b) {
        return cub::DeviceRunLengthEncode::Encode(tm, b, sk, c->a_ukeys.as<unsigned long long>(), c->a_ucount.as<int>(), nu_d, N, s);
    });
    if (st) return st;
    int nu = 0;
    FIPC_CUDA(cudaMemcpyAsync(&nu, nu_d, 4, cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaStreamSynchronize(s));
    st = cub2(c, [&](void* tm, size_t& b) {
        return cub::DeviceScan::ExclusiveSum(tm, b, c->a_ucount.as<int>(), c->a_ustart.as<int>(), nu + 1, s);
    });
    if (st) return st;
    k2_assembly_reduce<<<nb2(nu, 128), 128, 0, s>>>(src, nu, c->a_ukeys.as<unsigned long long>(), c->a_ustart.as<int>(), vb.Current(),
                                                    c->elem_H.as<double>(), c->elem_g.as<double>(), c->cH[0].as<double>(),
                                                    c->cg[0].as<double>(), c->cH[1].as<double>(), c->cg[1].as<double>(), c->mass, x,
                                                    xtilde, c->val.as<double>(), c->col.as<int>(), c->dpos.as<int>(),
                                                    c->rhs.as<double>());
    FIPC_LAUNCHED();
    k2_row_ptr<<<nb2(c->nV + 1, 256), 256, 0, s>>>(c->nV, nu, c->a_ukeys.as<unsigned long long>(), c->row_ptr.as<int>());
    FIPC_LAUNCHED();
    c->nnzb = nu;
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc2d_system_nnzb(fipc2d_ctx_impl* h, int* nnzb_h) {
    if (!h || !nnzb_h) return FIPC_ERR_ARGUMENT;
    *nnzb_h = h->c.nnzb;
    return FIPC_OK;
}

int fipc2d_export_system(fipc2d_ctx_impl* h, int* row_ptr, int* col_idx, double* val, double* rhs, void* stream) {
    if (!h) return FIPC_ERR_ARGUMENT;
    Ctx2* c = &h->c;
    cudaStream_t s = (cudaStream_t)stream;
    if (row_ptr) FIPC_CUDA(cudaMemcpyAsync(row_ptr, c->row_ptr.p, 4ull * (c->nV + 1), cudaMemcpyDeviceToDevice, s));
    if (col_idx && c->nnzb) FIPC_CUDA(cudaMemcpyAsync(col_idx, c->col.p, 4ull * c->nnzb, cudaMemcpyDeviceToDevice, s));
    if (val && c->nnzb) FIPC_CUDA(cudaMemcpyAsync(val, c->val.p, 32ull * c->nnzb, cudaMemcpyDeviceToDevice, s));
    if (rhs) FIPC_CUDA(cudaMemcpyAsync(rhs, c->rhs.p, 16ull * c->nV, cudaMemcpyDeviceToDevice, s));
    return FIPC_OK;
}

int fipc2d_solve_system(fipc2d_ctx_impl* h, const unsigned char* fixed, double rtol, int maxit, double* sol, int* iters_h,
                        void* stream) {
    if (!h || !fixed || !sol || maxit < 0 || !(rtol >= 0)) return FIPC_ERR_ARGUMENT;
    Ctx2* c = &h->c;
    if (!c->nnzb) return FIPC_ERR_ARGUMENT;   // no system assembled
    cudaStream_t s = (cudaStream_t)stream;
    const int nb = nb2(c->nV, T2);
    const size_t n2 = 2ull * c->nV;
    if (c->pvec.ensure(8 * (4 * n2 + 4ull * c->nV)) || c->ppart.ensure(24ull * nb + 64) || c->pflag.ensure(64 + 16)) return FIPC_ERR_CUDA;
    PCG2 a;
    a.nV = c->nV;
    a.rp = c->row_ptr.as<int>();
    a.col = c->col.as<int>();
    a.val = c->val.as<double>();
    a.dpos = c->dpos.as<int>();
    a.fixed = fixed;
    double* v = c->pvec.as<double>();
    a.x = sol;
    a.r = v;
    a.z = v + n2;
    a.p = v + 2 * n2;
    a.q = v + 3 * n2;
    a.minv = v + 4 * n2;
    a.part = c->ppart.as<double>();
    a.sc = c->pflag.as<double>();
    a.flag = (int*)(c->pflag.as<char>() + 64);
    a.maxit = maxit;
    FIPC_CUDA(cudaMemsetAsync(a.flag, 0, 16, s));
    int hf[2] = {0, 0};
    // one cooperative launch when the rows fit one CTA per SM
    int dev = 0, nsm = 0, per = 0;
    FIPC_CUDA(cudaGetDevice(&dev));
    FIPC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    FIPC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k2_pcg_coop, T2, 0));
    if (maxit > 0 && per >= 1 && nb <= nsm) {
        const double* rhs = c->rhs.as<double>();
        void* args[] = {&a, &rhs, &rtol};
        if (cudaLaunchCooperativeKernel((const void*)k2_pcg_coop, dim3(nb), dim3(T2), args, 0, s) == cudaSuccess) {
            FIPC_LAUNCHED();
            FIPC_CUDA(cudaMemcpyAsync(hf, a.flag, 8, cudaMemcpyDeviceToHost, s));
            FIPC_CUDA(cudaStreamSynchronize(s));
            FIPC_CUDA(cudaGetLastError());
            if (iters_h) *iters_h = hf[1];
            return hf[0] == 1 ? FIPC_OK : FIPC_ERR_ITERATION;
        }
        cudaGetLastError();   // not launchable here: the multi-kernel path below
    }
    k2_pcg_start<<<nb, T2, 0, s>>>(a, c->rhs.as<double>(), rtol);
    FIPC_LAUNCHED();
    // whole chunks: the iteration that converges or reaches maxit turns the rest of its chunk
    // into early exits
    const bool graph = maxit > 0 && pcg_graph(c, a, nb);
    for (int k0 = 0; k0 < maxit; k0 += PCG_CHUNK) {
        if (graph) FIPC_CUDA(cudaGraphLaunch((cudaGraphExec_t)c->graph_exec, s));
        else pcg_chunk(a, nb, s);
        g_launches.fetch_add(3 * PCG_CHUNK, std::memory_order_relaxed);
        FIPC_CUDA(cudaMemcpyAsync(hf, a.flag, 8, cudaMemcpyDeviceToHost, s));
        FIPC_CUDA(cudaStreamSynchronize(s));
        if (hf[0]) break;
    }
    if (maxit == 0) {
        FIPC_CUDA(cudaMemcpyAsync(hf, a.flag, 8, cudaMemcpyDeviceToHost, s));
        FIPC_CUDA(cudaStreamSynchronize(s));
    }
    FIPC_CUDA(cudaGetLastError());
    if (iters_h) *iters_h = hf[1];
    return hf[0] == 1 ? FIPC_OK : FIPC_ERR_ITERATION;
}

int fipc2d_output_residual(fipc2d_ctx_impl* h, const double* sol, double* res_h, void* stream) {
    if (!h || !sol || !res_h) return FIPC_ERR_ARGUMENT;
    Ctx2* c = &h->c;
    cudaStream_t s = (cudaStream_t)stream;
    if (c->eout.ensure(16)) return FIPC_ERR_CUDA;
    double* o = c->eout.as<double>();
    FIPC_CUDA(cudaMemsetAsync(o, 0, 8, s));
    k2_absmax<<<P2_RED, T2, 0, s>>>(2 * c->nV, sol, o);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaMemcpyAsync(res_h, o, 8, cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaStreamSynchronize(s));
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc2d_compute_energy(fipc2d_ctx_impl* h, const double* x, const double* xtilde, double* e_h, void* stream) {
    if (!h || !x || !xtilde || !e_h || !al16(x)) return FIPC_ERR_ARGUMENT;
    Ctx2* c = &h->c;
    cudaStream_t s = (cudaStream_t)stream;
    if (c->epart.ensure(8ull * P2_RED) || c->eout.ensure(16)) return FIPC_ERR_CUDA;
    k2_energy<<<P2_RED, T2, 0, s>>>(c->nV, c->nT, c->h_counts[0], c->h_counts[1], x, xtilde, c->mass, c->tris, c->IB, c->vol, c->lam,
                                    c->mu, c->dt * c->dt, c->rows[0].as<int4>(), c->rows[1].as<int4>(), c->dhat2, c->kappa,
                                    c->epart.as<double>());
    FIPC_LAUNCHED();
    k2_sum<<<1, T2, 0, s>>>(P2_RED, c->epart.as<double>(), c->eout.as<double>());
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaMemcpyAsync(e_h, c->eout.p, 8, cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaStreamSynchronize(s));
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc2d_compute_intersection_free_step_size(fipc2d_ctx_impl* h, const double* x, const double* sol, double eta, double* alpha_h,
                                               void* stream) {
    if (!h || !x || !sol || !alpha_h || !al16(x) || !al16(sol)) return FIPC_ERR_ARGUMENT;
    Ctx2* c = &h->c;
    cudaStream_t s = (cudaStream_t)stream;
    if (c->eout.ensure(16)) return FIPC_ERR_CUDA;
    double* o = c->eout.as<double>();
    const double one = 1.0;
    FIPC_CUDA(cudaMemcpyAsync(o, &one, 8, cudaMemcpyHostToDevice, s));
    if (c->nBP && c->nBE) {
        k2_ccd<<<dim3(nb2(c->nBP, T2), nb2(c->nBE, TILE)), T2, 0, s>>>(c->nBP, c->bp, c->nBE, c->be, x, sol, c->dhat, eta, o);
        FIPC_LAUNCHED();
    }
    FIPC_CUDA(cudaMemcpyAsync(alpha_h, o, 8, cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaStreamSynchronize(s));
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc2d_check_collision(fipc2d_ctx_impl* h, const double* x, int* hit_h, void* stream) {
    if (!h || !x || !hit_h || !al16(x)) return FIPC_ERR_ARGUMENT;
    Ctx2* c = &h->c;
    cudaStream_t s = (cudaStream_t)stream;
    if (c->cnt_d.ensure(16)) return FIPC_ERR_CUDA;
    int* hit = c->cnt_d.as<int>() + 3;
    FIPC_CUDA(cudaMemsetAsync(hit, 0, 4, s));
    if (c->nBP && c->nT) {
        k2_collision<<<dim3(nb2(c->nBP, T2), nb2(c->nT, TILE)), T2, 0, s>>>(c->nBP, c->bp, c->nT, c->tris, x, hit);
        FIPC_LAUNCHED();
    }
    FIPC_CUDA(cudaMemcpyAsync(hit_h, hit, 4, cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaStreamSynchronize(s));
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

}  // extern "C"
