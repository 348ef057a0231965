// Two-level preconditioner for the PCG direction solve: block-Jacobi plus a coarse correction
// on the six rigid-body modes (three translations, three rotations) of each aggregate of
// consecutive vertices,
//     M^-1 r = D^-1 r + P Ac^-1 P^T r,   Ac = P^T A P,   P_i = [I, -[d_i]x]  (3 x 6),
// with d_i the offset of vertex i from its aggregate's centroid and Dirichlet rows of P zero.
// Both terms are symmetric positive (semi)definite, so CG keeps converging to the solution of
// the reference's system (NEWTON_IPC.py:750-777); only the iteration count changes.  Long or
// stacked bodies have low-frequency modes that block-Jacobi resolves only one mesh layer per
// iteration; the coarse space removes them.
//
// Aggregates are runs of cs_agg_rows vertices, a multiple of the PCG block, so each PCG block
// restricts its residuals into its own aggregate with one fixed-order block sum, and the
// aggregate's last block (atomic ticket) totals them.  Ac is built from the elastic + inertia
// blocks (one CTA per coupled aggregate pair, fixed-order sums), inverted densely in place by a
// symmetric block sweep in one cooperative launch, and applied per PCG iteration as one dense
// matrix-vector kernel followed by the prolongation.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "ctx.cuh"
#include "pcg.cuh"

namespace cg = cooperative_groups;

namespace fipc {

static inline int nblk_c(long long n, int b) { return (int)((n + b - 1) / b); }

// one CTA per aggregate: centroid of its vertices (fixed order), then d_i = x_i - centroid
constexpr int CS_THREADS = 128;
__global__ void __launch_bounds__(CS_THREADS) k_cs_offsets(int nV, int agg_rows, const double* __restrict__ x, double* __restrict__ d) {
    __shared__ double sh[3][CS_THREADS];
    const int a = blockIdx.x, i0 = a * agg_rows, i1 = min(nV, i0 + agg_rows);
    double c[3] = {0.0, 0.0, 0.0};
    for (int i = i0 + threadIdx.x; i < i1; i += CS_THREADS)
        for (int k = 0; k < 3; ++k) c[k] += x[3 * (size_t)i + k];
    for (int k = 0; k < 3; ++k) sh[k][threadIdx.x] = c[k];
    __syncthreads();
    for (int s = CS_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int k = 0; k < 3; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + s];
        __syncthreads();
    }
    const double inv = 1.0 / (double)(i1 - i0);
    const double cx = sh[0][0] * inv, cy = sh[1][0] * inv, cz = sh[2][0] * inv;
    for (int i = i0 + threadIdx.x; i < i1; i += CS_THREADS) {
        d[3 * (size_t)i] = x[3 * (size_t)i] - cx;
        d[3 * (size_t)i + 1] = x[3 * (size_t)i + 1] - cy;
        d[3 * (size_t)i + 2] = x[3 * (size_t)i + 2] - cz;
    }
}

// C += P_i^T B P_j for the 3x3 block B (row-major, entries at B[32 * e])
__device__ __forceinline__ void add_coarse_block(double (&C)[36], const double* __restrict__ B, const double (&di)[3],
                                                 const double (&dj)[3]) {
    double b[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) b[e] = __ldg(B + 32 * e);
    // S(d) v = d x v;  BS = B S(dj), SB = S(di) B, SBS = S(di) B S(dj)
    const double Sj[9] = {0.0, -dj[2], dj[1], dj[2], 0.0, -dj[0], -dj[1], dj[0], 0.0};
    const double Si[9] = {0.0, -di[2], di[1], di[2], 0.0, -di[0], -di[1], di[0], 0.0};
    double BS[9], SB[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            BS[3 * r + c] = b[3 * r] * Sj[c] + b[3 * r + 1] * Sj[3 + c] + b[3 * r + 2] * Sj[6 + c];
            SB[3 * r + c] = Si[3 * r] * b[c] + Si[3 * r + 1] * b[3 + c] + Si[3 * r + 2] * b[6 + c];
        }
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double sbs = Si[3 * r] * BS[c] + Si[3 * r + 1] * BS[3 + c] + Si[3 * r + 2] * BS[6 + c];
            C[6 * r + c] += b[3 * r + c];
            C[6 * r + 3 + c] -= BS[3 * r + c];
            C[6 * (3 + r) + c] += SB[3 * r + c];
            C[6 * (3 + r) + 3 + c] -= sbs;
        }
}

// one CTA per coupled aggregate pair (I, J): the 6x6 block Ac[I][J] = sum over free i in I and
// free j in J of P_i^T A_ij P_j (elastic + inertia blocks), fixed-order sums, into dense Ac
constexpr int CS_BUILD_THREADS = 512;
__global__ void __launch_bounds__(CS_BUILD_THREADS) k_cs_build(int nV, int agg_rows, int n, const int* __restrict__ pairs,
                                                         const int* __restrict__ soff, const int* __restrict__ scol,
                                                         const int* __restrict__ rlen, const double* __restrict__ sval,
                                                         const unsigned char* __restrict__ fixed, const double* __restrict__ d,
                                                         double* __restrict__ Ac) {
    __shared__ double sh[36][CS_BUILD_THREADS / 32];
    const int I = pairs[2 * blockIdx.x], J = pairs[2 * blockIdx.x + 1];
    const int i0 = I * agg_rows, i1 = min(nV, i0 + agg_rows), j0 = J * agg_rows, j1 = min(nV, j0 + agg_rows);
    double C[36];
#pragma unroll
    for (int e = 0; e < 36; ++e) C[e] = 0.0;
    for (int i = i0 + threadIdx.x; i < i1; i += CS_BUILD_THREADS) {
        if (fixed[i]) continue;
        const double di[3] = {d[3 * (size_t)i], d[3 * (size_t)i + 1], d[3 * (size_t)i + 2]};
        const int sl = i >> 5, lane = i & 31, base = soff[sl], len = rlen[i];
        for (int k = 0; k < len; ++k) {
            const size_t slot = (size_t)(base + k);
            const int j = __ldg(scol + slot * 32 + lane);
            if (j < j0 || j >= j1 || fixed[j]) continue;
            const double dj[3] = {d[3 * (size_t)j], d[3 * (size_t)j + 1], d[3 * (size_t)j + 2]};
            add_coarse_block(C, sval + slot * 288 + lane, di, dj);
        }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int e = 0; e < 36; ++e) {
        double v = C[e];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sh[e][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x < 36) {
        double t = 0.0;
        for (int w = 0; w < CS_BUILD_THREADS / 32; ++w) t += sh[threadIdx.x][w];
        const int r = threadIdx.x / 6, c = threadIdx.x % 6;
        Ac[(size_t)(6 * I + r) * n + 6 * J + c] = t;
    }
}

// zero diagonals (modes without free vertices: their rows and columns are zero) become 1; the
// others get a 1e-12 relative shift that keeps nearly degenerate rotation modes invertible
__global__ void k_cs_regularize(int n, double* __restrict__ Ac) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double* dk = Ac + (size_t)k * n + k;
    *dk = *dk > 0.0 ? *dk * (1.0 + 1e-12) : 1.0;
}

// In-place inverse of the SPD matrix A (n x n row-major, n a multiple of GJ_B) by the symmetric
// block sweep (the Gauss-Jordan sweep operator): sweeping block K of a symmetric matrix maps
//     A_KK -> -A_KK^-1,  A_IK -> A_IK T,  A_KJ -> T A_KJ,  A_IJ -> A_IJ - A_IK T A_KJ   (T = A_KK^-1),
// which keeps the matrix symmetric, and sweeping every block leaves -A^-1.  No pivoting is
// needed: the A_KK met are Schur complements of an SPD matrix.  Only the tiles on and below the
// diagonal are kept, which halves the FP64 work of a full Gauss-Jordan inverse; the upper
// triangle is filled at the end.  One cooperative launch:
//   prologue   CTA 0: T = A_00^-1 (Gauss-Jordan on one tile in shared memory)
//   per K      A: every CTA: panel P_I = A_IK (tile (K, I) transposed for I < K) and W_I = P_I T
//              B: CTA 0 writes A_KK = -T, then updates tile (K+1, K+1) and inverts it into T
//                 (the next block's T, ready by the next barrier); the other CTAs take the other
//                 lower tiles: A_IJ -= W_I P_J^T, A_IK = W_I, A_KJ = W_J^T
//   epilogue   upper triangle = -(lower triangle)^T, then the lower triangle negated
// buf: T (B^2) + P (n B) + W (n B) doubles.  Every sum runs in a fixed order.
constexpr int GJ_B = 32, GJ_THREADS = 256;

// in-place Gauss-Jordan inverse of the SPD tile s (shared memory, row stride GJ_B + 1)
__device__ void gj_tile_inverse(double (*s)[GJ_B + 1], double* prow, double* pcol) {
    const int t = threadIdx.x;
    for (int k = 0; k < GJ_B; ++k) {
        if (t < GJ_B) {
            const double inv = 1.0 / s[k][k];
            prow[t] = t == k ? inv : s[k][t] * inv;
            pcol[t] = s[t][k];
        }
        __syncthreads();
        for (int e = t; e < GJ_B * GJ_B; e += GJ_THREADS) {
            const int i = e / GJ_B, j = e % GJ_B;
            double v;
            if (i == k) v = prow[j];
            else if (j == k) v = -pcol[i] * prow[k];
            else v = fma(-pcol[i], prow[j], s[i][j]);
            s[i][j] = v;
        }
        __syncthreads();
    }
}

// lower tile number t -> (I, J), I >= J
__device__ __forceinline__ void lower_tile(int t, int& I, int& J) {
    int i = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
    while ((i + 1) * (i + 2) / 2 <= t) ++i;
    while (i * (i + 1) / 2 > t) --i;
    I = i;
    J = t - i * (i + 1) / 2;
}

__global__ void __launch_bounds__(GJ_THREADS) k_cs_gauss_jordan(int n, double* __restrict__ A, double* __restrict__ buf) {
    cg::grid_group grid = cg::this_grid();
    __shared__ double sa[GJ_B][GJ_B + 1];
    __shared__ double sb[GJ_B][GJ_B + 1];
    __shared__ double prow[GJ_B], pcol[GJ_B];
    const int nb = n / GJ_B, t = threadIdx.x;
    const long long gtid = (long long)blockIdx.x * GJ_THREADS + t, gthr = (long long)gridDim.x * GJ_THREADS;
    double* T = buf;
    double* P = buf + GJ_B * GJ_B;
    double* W = P + (size_t)n * GJ_B;
    const int c = t & 31, rb = t >> 5;   // tile column and first row (rows rb, rb + 8, rb + 16, rb + 24)
    const bool solo = gridDim.x == 1;
    const int worker = solo ? 0 : (int)blockIdx.x - 1, workers = solo ? 1 : (int)gridDim.x - 1;
    const int n_lower = nb * (nb + 1) / 2;
    if (blockIdx.x == 0) {
        for (int e = t; e < GJ_B * GJ_B; e += GJ_THREADS) sa[e / GJ_B][e % GJ_B] = A[(size_t)(e / GJ_B) * n + e % GJ_B];
        __syncthreads();
        gj_tile_inverse(sa, prow, pcol);
        for (int e = t; e < GJ_B * GJ_B; e += GJ_THREADS) T[e] = sa[e / GJ_B][e % GJ_B];
    }
    grid.sync();
    for (int K = 0; K < nb; ++K) {
        const int k0 = K * GJ_B;
        // A: P_I and W_I = P_I T for every row outside block K
        for (int e = t; e < GJ_B * GJ_B; e += GJ_THREADS) sa[e / GJ_B][e % GJ_B] = T[e];
        __syncthreads();
        for (long long e = gtid; e < (long long)n * GJ_B; e += gthr) {
            const int i = (int)(e / GJ_B), m = (int)(e % GJ_B), I = i / GJ_B;
            if (I == K) continue;
            const double* src = I > K ? A + (size_t)i * n + k0 : A + (size_t)k0 * n + i;
            const size_t st = I > K ? 1 : (size_t)n;
            double w = 0.0;
#pragma unroll 8
            for (int q = 0; q < GJ_B; ++q) w = fma(src[q * st], sa[q][m], w);
            P[e] = src[m * st];
            W[e] = w;
        }
        grid.sync();
        // B
        if (blockIdx.x == 0) {
            for (int e = t; e < GJ_B * GJ_B; e += GJ_THREADS) A[(size_t)(k0 + e / GJ_B) * n + k0 + e % GJ_B] = -T[e];
            if (K + 1 < nb) {
                const int i0 = k0 + GJ_B;
                __syncthreads();
                for (int e = t; e < GJ_B * GJ_B; e += GJ_THREADS) {
                    sa[e / GJ_B][e % GJ_B] = W[(size_t)i0 * GJ_B + e];
                    sb[e / GJ_B][e % GJ_B] = P[(size_t)i0 * GJ_B + e];
                }
                __syncthreads();
                double acc[4] = {0.0, 0.0, 0.0, 0.0};
                for (int q = 0; q < GJ_B; ++q) {
                    const double pj = sb[c][q];
#pragma unroll
                    for (int u = 0; u < 4; ++u) acc[u] = fma(sa[rb + 8 * u][q], pj, acc[u]);
                }
                double v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) v[u] = A[(size_t)(i0 + rb + 8 * u) * n + i0 + c] - acc[u];
                __syncthreads();
#pragma unroll
                for (int u = 0; u < 4; ++u) sa[rb + 8 * u][c] = v[u];
                __syncthreads();
                gj_tile_inverse(sa, prow, pcol);
                for (int e = t; e < GJ_B * GJ_B; e += GJ_THREADS) T[e] = sa[e / GJ_B][e % GJ_B];
            }
        }
        if (blockIdx.x != 0 || solo) {
            for (int tile = worker; tile < n_lower; tile += workers) {
                int I, J;
                lower_tile(tile, I, J);
                if ((I == K && J == K) || (I == K + 1 && J == K + 1)) continue;
                const int i0 = I * GJ_B, j0 = J * GJ_B;
                if (J == K) {            // A_IK = W_I (I > K)
                    for (int e = t; e < GJ_B * GJ_B; e += GJ_THREADS)
                        A[(size_t)(i0 + e / GJ_B) * n + k0 + e % GJ_B] = W[(size_t)i0 * GJ_B + e];
                    continue;
                }
                if (I == K) {            // A_KJ = W_J^T (J < K)
                    for (int e = t; e < GJ_B * GJ_B; e += GJ_THREADS) {
                        const int r = e / GJ_B, cc = e % GJ_B;
                        A[(size_t)(k0 + r) * n + j0 + cc] = W[(size_t)(j0 + cc) * GJ_B + r];
                    }
                    continue;
                }
                __syncthreads();
                for (int e = t; e < GJ_B * GJ_B; e += GJ_THREADS) {
                    sa[e / GJ_B][e % GJ_B] = W[(size_t)i0 * GJ_B + e];
                    sb[e / GJ_B][e % GJ_B] = P[(size_t)j0 * GJ_B + e];
                }
                __syncthreads();
                double acc[4] = {0.0, 0.0, 0.0, 0.0};
                for (int q = 0; q < GJ_B; ++q) {
                    const double pj = sb[c][q];
#pragma unroll
                    for (int u = 0; u < 4; ++u) acc[u] = fma(sa[rb + 8 * u][q], pj, acc[u]);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    double* out = A + (size_t)(i0 + rb + 8 * u) * n + j0 + c;
                    *out = *out - acc[u];
                }
            }
        }
        grid.sync();
    }
    // epilogue: the lower triangle holds -A^-1
    for (long long e = gtid; e < (long long)n * n; e += gthr) {
        const int i = (int)(e / n), j = (int)(e % n);
        if (i < j) A[e] = -A[(size_t)j * n + i];
    }
    grid.sync();
    for (long long e = gtid; e < (long long)n * n; e += gthr) {
        const int i = (int)(e / n), j = (int)(e % n);
        if (i >= j) A[e] = -A[e];
    }
}

// cooperative launch of the inverse over a grid that fits the GPU (n a multiple of GJ_B)
static int launch_gauss_jordan(int n, double* A, double* buf, cudaStream_t s) {
    int dev = 0, nsm = 0, per = 0;
    FIPC_CUDA(cudaGetDevice(&dev));
    FIPC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    FIPC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_cs_gauss_jordan, GJ_THREADS, 0));
    if (per < 1) return FIPC_ERR_CUDA;
    int grid = nsm * (per < 2 ? per : 2);
    const int nb = n / GJ_B, tiles = nb * (nb + 1) / 2 + 1;   // the lower tiles, plus CTA 0's own work
    if (grid > tiles) grid = tiles;
    void* args[] = {&n, &A, &buf};
    FIPC_CUDA(cudaLaunchCooperativeKernel((const void*)k_cs_gauss_jordan, dim3(grid), dim3(GJ_THREADS), args, 0, s));
    FIPC_LAUNCHED();
    return FIPC_OK;
}

// y = Ac^-1 g: g (the aggregate restrictions, complete once the last PCG kernel ran) is staged in
// shared memory, then one warp per row, fixed-order lane sums and shuffle tree
constexpr int CS_MV_THREADS = 256;
__global__ void __launch_bounds__(CS_MV_THREADS) k_cs_coarse(PCGArgs a) {
    extern __shared__ double g[];
    if (*(volatile int*)&a.flag[0]) return;
    for (int q = threadIdx.x; q < a.cs_n; q += CS_MV_THREADS) g[q] = a.cs_g[q];
    __syncthreads();
    const int lane = threadIdx.x & 31, warps = CS_MV_THREADS / 32;
    for (int row = blockIdx.x * warps + (threadIdx.x >> 5); row < a.cs_n; row += gridDim.x * warps) {
        const double* Ar = a.cs_ainv + (size_t)row * a.cs_ld;
        double t = 0.0;
        for (int j = lane; j < a.cs_n; j += 32) t += __ldg(Ar + j) * g[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0) a.cs_y[row] = t;
    }
}

// u_i += P_i y_I = y_t + y_w x d_i on free vertices
__global__ void __launch_bounds__(PCG_THREADS) k_cs_prolong(PCGArgs a) {
    if (*(volatile int*)&a.flag[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nV || a.fixed[i]) return;
    const double* y = a.cs_y + 6 * (size_t)(blockIdx.x / a.cs_blocks);
    const double dx = __ldg(a.cs_d + 3 * (size_t)i), dy = __ldg(a.cs_d + 3 * (size_t)i + 1), dz = __ldg(a.cs_d + 3 * (size_t)i + 2);
    const double y0 = y[0], y1 = y[1], y2 = y[2], y3 = y[3], y4 = y[4], y5 = y[5];
    a.u[4 * (size_t)i] += y0 + (y4 * dz - y5 * dy);
    a.u[4 * (size_t)i + 1] += y1 + (y5 * dx - y3 * dz);
    a.u[4 * (size_t)i + 2] += y2 + (y3 * dy - y4 * dx);
}

// ---------------------------------------------------------------- host side
// aggregate pairs coupled by the static pattern (host, at context creation or on a change of
// the aggregate size)
void pcg_graph_reset(fipc_ctx* c);

int cs_setup(fipc_ctx* c, int agg_rows, const int* row_ptr_h, const int* col_idx_h) {
    pcg_graph_reset(c);
    if (c->cs_pairs) cudaFree(c->cs_pairs);
    c->cs_pairs = nullptr;
    c->cs_agg_rows = 0;
    c->cs_n_agg = 0;
    c->cs_n_pairs = 0;
    if (agg_rows <= 0) return FIPC_OK;
    if (agg_rows % PCG_THREADS) return FIPC_ERR_ARGUMENT;
    const int na = (c->nV + agg_rows - 1) / agg_rows;
    if (na > 1024) return FIPC_ERR_ARGUMENT;   // dense coarse matrix of at most 6144^2
    std::vector<unsigned long long> keys;
    for (int i = 0; i < c->nV; ++i)
        for (int k = row_ptr_h[i]; k < row_ptr_h[i + 1]; ++k)
            keys.push_back(((unsigned long long)(i / agg_rows) << 32) | (unsigned)(col_idx_h[k] / agg_rows));
    std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    std::vector<int> pairs(2 * keys.size());
    for (size_t q = 0; q < keys.size(); ++q) {
        pairs[2 * q] = (int)(keys[q] >> 32);
        pairs[2 * q + 1] = (int)(keys[q] & 0xffffffffu);
    }
    if (cudaMalloc((void**)&c->cs_pairs, sizeof(int) * pairs.size()) != cudaSuccess) return FIPC_ERR_CUDA;
    if (cudaMemcpy(c->cs_pairs, pairs.data(), sizeof(int) * pairs.size(), cudaMemcpyHostToDevice) != cudaSuccess) return FIPC_ERR_CUDA;
    c->cs_agg_rows = agg_rows;
    c->cs_n_agg = na;
    c->cs_n_pairs = (int)keys.size();
    // offsets from the rest shape until the next assembly sets them at its positions (any
    // centre spans the same rigid-body modes, so the coarse space is valid either way)
    if (c->cs_d.ensure(24ll * c->nV)) return FIPC_ERR_CUDA;
    k_cs_offsets<<<c->cs_n_agg, CS_THREADS>>>(c->nV, c->cs_agg_rows, c->x0, c->cs_d.as<double>());
    FIPC_LAUNCHED();
    if (cudaDeviceSynchronize() != cudaSuccess) return FIPC_ERR_CUDA;
    return FIPC_OK;
}

int mg_offsets(fipc_ctx* c, const double* x, cudaStream_t s);

// the symmetric block-sweep inverse for other preconditioner levels (n a multiple of GJ_B)
int cs_gauss_jordan(int n, double* A, double* buf, cudaStream_t s) { return launch_gauss_jordan(n, A, buf, s); }

// offsets from the aggregate centroids at the Newton iterate x (called by the assembly), and the
// multigrid hierarchy's when it is in use
int cs_offsets(fipc_ctx* c, const double* x, cudaStream_t s) {
    if (c->mg) {
        const int st = mg_offsets(c, x, s);
        if (st) return st;
    }
    if (!c->cs_agg_rows) return FIPC_OK;
    if (c->cs_d.ensure(24ll * c->nV)) return FIPC_ERR_CUDA;
    k_cs_offsets<<<c->cs_n_agg, CS_THREADS, 0, s>>>(c->nV, c->cs_agg_rows, x, c->cs_d.as<double>());
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

// Ac^-1 for the assembled system and the Dirichlet mask; fills the coarse fields of a
int cs_prepare(fipc_ctx* c, const unsigned char* fixed, PCGArgs& a, cudaStream_t s) {
    a.cs_blocks = 0;
    if (!c->cs_agg_rows) return FIPC_OK;
    const int n = 6 * c->cs_n_agg, nb = nblk_c(c->nV, PCG_THREADS);
    const int ld = ((n + GJ_B - 1) / GJ_B) * GJ_B;   // padded with identity rows to whole GJ blocks
    if (c->cs_Ac.ensure(8ll * ld * ld) || c->cs_buf.ensure(8ll * (GJ_B * GJ_B + 2ll * ld * GJ_B)) || c->cs_part.ensure(48ll * nb) ||
        c->cs_gbuf.ensure(16ll * n) || c->cs_tick.ensure(4ll * c->cs_n_agg))
        return FIPC_ERR_CUDA;
    FIPC_CUDA(cudaMemsetAsync(c->cs_tick.p, 0, 4ll * c->cs_n_agg, s));   // aggregate tickets
    double* Ac = c->cs_Ac.as<double>();
    FIPC_CUDA(cudaMemsetAsync(Ac, 0, 8ll * ld * ld, s));
    k_cs_build<<<c->cs_n_pairs, CS_BUILD_THREADS, 0, s>>>(c->nV, c->cs_agg_rows, ld, c->cs_pairs, c->sell_off, c->sell_col, c->row_len,
                                                          c->sell_val, fixed, c->cs_d.as<double>(), Ac);
    FIPC_LAUNCHED();
    k_cs_regularize<<<nblk_c(ld, 128), 128, 0, s>>>(ld, Ac);
    FIPC_LAUNCHED();
    int st = launch_gauss_jordan(ld, Ac, c->cs_buf.as<double>(), s);
    if (st) return st;
    a.cs_blocks = c->cs_agg_rows / PCG_THREADS;
    a.cs_d = c->cs_d.as<double>();
    a.cs_part = c->cs_part.as<double>();
    a.cs_g = c->cs_gbuf.as<double>();
    a.cs_y = a.cs_g + n;
    a.cs_ticket = c->cs_tick.as<int>();
    a.cs_ainv = Ac;
    a.cs_n = n;
    a.cs_ld = ld;
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

// the coarse correction u += P Ac^-1 P^T r for the aggregate restrictions the last PCG kernel wrote
void cs_apply(const fipc_ctx* c, const PCGArgs& a, cudaStream_t s) {
    k_cs_coarse<<<nblk_c(a.cs_n, CS_MV_THREADS / 32), CS_MV_THREADS, 8 * (size_t)a.cs_n, s>>>(a);
    FIPC_LAUNCHED();
    k_cs_prolong<<<nblk_c(c->nV, PCG_THREADS), PCG_THREADS, 0, s>>>(a);
    FIPC_LAUNCHED();
}

void cs_free(fipc_ctx* c) {
    if (c->cs_pairs) cudaFree(c->cs_pairs);
    c->cs_pairs = nullptr;
    DBuf* bufs[] = {&c->cs_d, &c->cs_Ac, &c->cs_tick, &c->cs_buf, &c->cs_part, &c->cs_gbuf};
    for (DBuf* b : bufs) b->release();
}

}  // namespace fipc

using namespace fipc;

// in-place inverse of a dense SPD matrix (n a multiple of 32, row-major); work: 1024 + 64 n doubles
extern "C" int fipc_dense_spd_inverse(int n, double* A, double* work, void* stream) {
    if (n <= 0 || n % GJ_B || !A || !work) return FIPC_ERR_ARGUMENT;
    const int st = launch_gauss_jordan(n, A, work, (cudaStream_t)stream);
    if (st) return st;
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}
