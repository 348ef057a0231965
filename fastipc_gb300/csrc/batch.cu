// Batched scenes: S independent IPC scenes in one context, each with its own Newton loop.
//
// The scenes' meshes are concatenated (scene s owns vertices [voff[s], voff[s+1]) and tets
// [toff[s], toff[s+1]); every boundary primitive lies in one scene).  Everything that is
// per element (Neo-Hookean tets, barrier rows, assembly, SpMV rows) runs over the union as
// for one scene; what the reference reduces over a scene is reduced per scene here:
//   * spatial hash: cell keys carry the scene id and each scene uses its own cell size, so the
//     constraint lists are the union of the per-scene lists (NEWTON_IPC.py:337-357);
//   * kappa per scene (NEWTON_IPC.py:116-124) in the barrier rows;
//   * energy, residual, CCD step and intersection flag per scene (one value per scene);
//   * PCG with per-scene scalars: rows are cut into tiles that never cross a scene; each tile
//     writes its dot-product partials and the last tile of a scene to finish (atomic ticket per
//     scene) sums that scene's partials in tile order and derives its alpha / beta, so every
//     scene converges on its own and the sums are reproducible.  The kernels are persistent
//     (a fixed grid strides over the tile table), a chunk of iterations is replayed as one
//     captured CUDA graph, and the tile size and grid are picked by timing on the live system.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "barrier.cuh"
#include "ctx.cuh"
#include "geometry.cuh"
#include "nh.cuh"
#include "pcg.cuh"

namespace fipc {

// the seven constraint lists of a context
struct RowLists {
    const int4* rows[N_TYPES];
    int n[N_TYPES];
};

static inline int nblk(long long n, int b) { return (int)((n + b - 1) / b); }

// ---------------------------------------------------------------- per-scene reductions
template <int NT>
__device__ __forceinline__ double block_sum_t(double v, double* sh) {
    sh[threadIdx.x] = v;
    __syncthreads();
#pragma unroll
    for (int s = NT / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

// first row of each list whose leading vertex is >= voff[s] (lists are sorted), s = 0..S
__global__ void k_scene_row_offsets(int S, const int* __restrict__ voff, RowLists rl, int* __restrict__ roff) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s > S) return;
    const int v = voff[s];
    for (int t = 0; t < N_TYPES; ++t) {
        const int4* r = rl.rows[t];
        int lo = 0, hi = rl.n[t];
        while (lo < hi) {
            const int m = (lo + hi) >> 1;
            if (r[m].x < v) lo = m + 1;
            else hi = m;
        }
        roff[t * (S + 1) + s] = lo;
    }
}

// incremental potential per scene (NEWTON_IPC.py:515-542): one block per scene
constexpr int SE_THREADS = 256;
__global__ void __launch_bounds__(SE_THREADS) k_scene_energy(int S, const int* __restrict__ voff, const int* __restrict__ toff,
                                                             const int* __restrict__ roff, RowLists rl, const double* __restrict__ x,
                                                             const double* __restrict__ xt, const double* __restrict__ m,
                                                             const int4* __restrict__ tets, const double* __restrict__ dminv,
                                                             const double* __restrict__ vol, const double* __restrict__ lam,
                                                             const double* __restrict__ mu, double dt2, const double* __restrict__ x0,
                                                             double dh2, const double* __restrict__ kap_s, double* __restrict__ out) {
    __shared__ double sh[SE_THREADS];
    const int s = blockIdx.x;
    double acc = 0.0;
    for (int i = voff[s] + threadIdx.x; i < voff[s + 1]; i += SE_THREADS) acc += 0.5 * m[i] * sq(ld3(x, i) - ld3(xt, i));
    double total = block_sum_t<SE_THREADS>(acc, sh);
    acc = 0.0;
    for (int e = toff[s] + threadIdx.x; e < toff[s + 1]; e += SE_THREADS) {
        const int4 t = tets[e];
        const v3 X[4] = {ld3(x, t.x), ld3(x, t.y), ld3(x, t.z), ld3(x, t.w)};
        double IB[9], F[9];
        for (int i = 0; i < 9; ++i) IB[i] = dminv[9 * (size_t)e + i];
        deformation_gradient(X, IB, F);
        acc += nh_psi_F(F, lam[e], mu[e]) * dt2 * vol[e];
    }
    total += block_sum_t<SE_THREADS>(acc, sh);
    const double kappa = kap_s[s];
    for (int type = 0; type < N_TYPES; ++type) {
        const int r0 = roff[type * (S + 1) + s], r1 = roff[type * (S + 1) + s + 1];
        if (r0 >= r1) continue;
        const int nv = type_nverts(type);
        acc = 0.0;
        for (int r = r0 + threadIdx.x; r < r1; r += SE_THREADS) {
            const int4 q = rl.rows[type][r];
            const int id[4] = {q.x, q.y, nv > 2 ? q.z : q.x, nv > 3 ? q.w : q.x};
            v3 X[4], X0[4];
            for (int k = 0; k < 4; ++k) {
                X[k] = ld3(x, id[k]);
                X0[k] = type >= T_EEM ? ld3(x0, id[k]) : mk(0, 0, 0);
            }
            double e;
            barrier_row(type, X, X0, dh2, kappa, 0, &e, nullptr, nullptr);
            acc += e;
        }
        total += block_sum_t<SE_THREADS>(acc, sh);
    }
    if (threadIdx.x == 0) out[s] = total;
}

// max |p| per scene (NEWTON_IPC.py:805-812)
__global__ void __launch_bounds__(SE_THREADS) k_scene_absmax(const int* __restrict__ voff, const double* __restrict__ p,
                                                             double* __restrict__ out) {
    __shared__ double sh[SE_THREADS];
    const int s = blockIdx.x;
    double mx = 0.0;
    for (long long i = 3ll * voff[s] + threadIdx.x; i < 3ll * voff[s + 1]; i += SE_THREADS) mx = fmax(mx, fabs(p[i]));
    sh[threadIdx.x] = mx;
    __syncthreads();
    for (int k = SE_THREADS / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + k]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[s] = sh[0];
}

// x = xPrev + alpha[scene] p (NEWTON_IPC.py:792-796)
__global__ void k_apply_sol_scenes(int n3, const int* __restrict__ vscene, const double* __restrict__ xprev, const double* __restrict__ sol,
                                   const double* __restrict__ alpha, double* __restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n3) x[i] = xprev[i] + sol[i] * alpha[vscene[i / 3]];
}

__global__ void k_fill_f64(int n, double* __restrict__ a, double v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}

}  // namespace fipc

// ---------------------------------------------------------------- batched PCG
namespace fipc {

struct BPCG {
    PCGArgs m{};                  // operands and vectors; m.part / m.sc / m.flag unused
    int S, n_tiles, maxit, dry;   // dry: SpMV only (timing), no partials and no scalars
    const int* tile_scene;        // [n_tiles]
    const int* tile_row0;         // [n_tiles]
    const int* voff;              // [S + 1]
    const int* scene_tile0;       // [S + 1]
    double* part;                 // [3][n_tiles]
    double* sc;                   // [S][SC_COUNT]
    int* sflag;                   // [S][4]: done, iterations, ticket, failed
    int* ndone;                   // scenes finished
    double rtol;
};

// scene of tile t, read once by thread 0 (block-uniform), or -1 when the scene is finished
template <int TR>
__device__ __forceinline__ int tile_scene_live(const BPCG& a, int t) {
    __shared__ int sh;
    if (threadIdx.x == 0) {
        const int s = a.tile_scene[t];
        sh = *(volatile int*)&a.sflag[4 * s] ? -1 : s;
    }
    __syncthreads();
    const int s = sh;
    __syncthreads();
    return s;
}

// tile sums of NV values into part[c * n_tiles + t]; true in every thread of the scene's last tile
template <int TR, int NV>
__device__ __forceinline__ bool tile_partials(const BPCG& a, int t, int s, const double (&v)[NV]) {
    // the values go through shared memory and warp c sums component c in a fixed order (fewer
    // FP64 adds than a shuffle tree in every warp)
    __shared__ double sv[NV][TR];
    __shared__ double tot[NV];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < NV; ++c) sv[c][threadIdx.x] = v[c];
    __syncthreads();
    for (int c = wid; c < NV; c += TR / 32) {
        double x = sv[c][lane];
#pragma unroll
        for (int k = 1; k < TR / 32; ++k) x += sv[c][lane + 32 * k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) tot[c] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int c = 0; c < NV; ++c) a.part[(size_t)c * a.n_tiles + t] = tot[c];
        __threadfence();
        const int ticket = atomicAdd(&a.sflag[4 * s + 2], 1);
        last = ticket == a.scene_tile0[s + 1] - a.scene_tile0[s] - 1;
    }
    __syncthreads();
    const bool r = last;
    __syncthreads();
    return r;
}

// in the scene's last tile: out[c] = sum of the scene's tile partials in tile order
template <int TR, int NV>
__device__ __forceinline__ void scene_sums(const BPCG& a, int s, double (&out)[NV]) {
    __shared__ double sh[NV][TR / 32];
    __threadfence();
    const int t0 = a.scene_tile0[s], t1 = a.scene_tile0[s + 1];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        double q = 0.0;
        for (int t = t0 + threadIdx.x; t < t1; t += TR) q += *(volatile double*)&a.part[(size_t)c * a.n_tiles + t];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) q += __shfl_down_sync(0xffffffffu, q, o);
        if (lane == 0) sh[c][wid] = q;
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        double q = 0.0;
        for (int k = 0; k < TR / 32; ++k) q += sh[c][k];
        out[c] = q;
    }
    __syncthreads();
}

// ndone is zeroed by the caller before this launch
__global__ void k_bpcg_init(int S, const unsigned char* __restrict__ active, int* __restrict__ sflag, int* __restrict__ ndone) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const int off = active && !active[s];
    sflag[4 * s] = off;
    sflag[4 * s + 1] = 0;
    sflag[4 * s + 2] = 0;
    sflag[4 * s + 3] = 0;
    if (off) atomicAdd(ndone, 1);
}

// residual of the initial guess, preconditioner, u = M^-1 r; per-scene |r|^2, |b|^2 and tolerance
template <int TR>
__global__ void __launch_bounds__(TR) k_bpcg_start(BPCG a, const double* __restrict__ rhs) {
    for (int t = blockIdx.x; t < a.n_tiles; t += gridDim.x) {
        const int s = tile_scene_live<TR>(a, t);
        const int i = a.tile_row0[t] + threadIdx.x;
        if (s < 0) {   // inactive scene: zero direction
            const int sr = a.tile_scene[t];
            if (i < a.voff[sr + 1]) a.m.x[3 * i] = a.m.x[3 * i + 1] = a.m.x[3 * i + 2] = 0.0;
            continue;
        }
        double rr = 0.0, bb = 0.0;
        if (i < a.voff[s + 1]) {
            double Mi[9];
            const bool fx = a.m.fixed[i] != 0;
            jacobi_block_inverse(a.m, i, fx, Mi);
            for (int k = 0; k < 9; ++k) a.m.minv[9 * (size_t)i + k] = Mi[k];
            double y0, y1, y2;
            row_apply<3>(a.m, i, a.m.x, y0, y1, y2);
            const double r0 = fx ? 0.0 : rhs[3 * i] - y0, r1 = fx ? 0.0 : rhs[3 * i + 1] - y1, r2 = fx ? 0.0 : rhs[3 * i + 2] - y2;
            a.m.r[3 * i] = r0;
            a.m.r[3 * i + 1] = r1;
            a.m.r[3 * i + 2] = r2;
            if (!fx) bb = rhs[3 * i] * rhs[3 * i] + rhs[3 * i + 1] * rhs[3 * i + 1] + rhs[3 * i + 2] * rhs[3 * i + 2];
            for (int d = 0; d < 3; ++d) {
                a.m.u[4 * i + d] = Mi[3 * d] * r0 + Mi[3 * d + 1] * r1 + Mi[3 * d + 2] * r2;
                a.m.p[3 * i + d] = 0.0;
                a.m.s[3 * i + d] = 0.0;
            }
            a.m.u[4 * i + 3] = 0.0;
            rr = r0 * r0 + r1 * r1 + r2 * r2;
        }
        const double v[2] = {rr, bb};
        if (tile_partials<TR, 2>(a, t, s, v)) {
            double tt[2];
            scene_sums<TR, 2>(a, s, tt);
            if (threadIdx.x == 0) {
                double* sc = a.sc + SC_COUNT * s;
                sc[SC_RR0] = tt[0];
                sc[SC_TOL2] = a.rtol * a.rtol * tt[1];
                sc[SC_GAMMA] = 1.0;
                sc[SC_ALPHA] = 1.0;
                a.sflag[4 * s + 2] = 0;
                if (tt[0] == 0.0 || tt[0] <= a.rtol * a.rtol * tt[1]) {
                    a.sflag[4 * s] = 1;
                    atomicAdd(a.ndone, 1);
                }
            }
        }
    }
}

// w = A u with the per-scene dot products; each scene's last tile derives its alpha and beta
template <int TR>
__global__ void __launch_bounds__(TR) k_bpcg_spmv(BPCG a) {
    for (int t = blockIdx.x; t < a.n_tiles; t += gridDim.x) {
        const int s = a.dry ? a.tile_scene[t] : tile_scene_live<TR>(a, t);
        if (s < 0) continue;
        const int i = a.tile_row0[t] + threadIdx.x;
        double g = 0.0, dl = 0.0, rr = 0.0;
        if (i < a.voff[s + 1]) {
            double y0 = 0.0, y1 = 0.0, y2 = 0.0;
            if (!a.m.fixed[i]) row_apply<4>(a.m, i, a.m.u, y0, y1, y2);
            a.m.w[3 * i] = y0;
            a.m.w[3 * i + 1] = y1;
            a.m.w[3 * i + 2] = y2;
            const double u0 = a.m.u[4 * i], u1 = a.m.u[4 * i + 1], u2 = a.m.u[4 * i + 2];
            const double r0 = a.m.r[3 * i], r1 = a.m.r[3 * i + 1], r2 = a.m.r[3 * i + 2];
            g = r0 * u0 + r1 * u1 + r2 * u2;
            dl = y0 * u0 + y1 * u1 + y2 * u2;
            rr = r0 * r0 + r1 * r1 + r2 * r2;
        }
        if (a.dry) continue;
        const double v[3] = {g, dl, rr};
        if (tile_partials<TR, 3>(a, t, s, v)) {
            double tt[3];
            scene_sums<TR, 3>(a, s, tt);
            if (threadIdx.x == 0) {
                double* sc = a.sc + SC_COUNT * s;
                int* f = a.sflag + 4 * s;
                const double G = tt[0], Dl = tt[1], R = tt[2];
                const int k = f[1];
                f[2] = 0;
                if (R <= sc[SC_TOL2] || k >= a.maxit) {
                    f[3] = R <= sc[SC_TOL2] ? 0 : 1;
                    f[0] = 1;
                    atomicAdd(a.ndone, 1);
                } else {
                    const double beta = k == 0 ? 0.0 : G / sc[SC_GAMMA];
                    const double alpha = k == 0 ? G / Dl : G / (Dl - beta * G / sc[SC_ALPHA]);
                    sc[SC_GAMMA] = G;
                    sc[SC_DELTA] = Dl;
                    sc[SC_RR] = R;
                    sc[SC_BETA] = beta;
                    sc[SC_ALPHA] = alpha;
                    f[1] = k + 1;
                }
            }
        }
    }
}

// p = u + beta p, s = w + beta s, x += alpha p, r -= alpha s, u = M^-1 r with the scene's scalars
template <int TR>
__global__ void __launch_bounds__(TR) k_bpcg_update(BPCG a) {
    for (int t = blockIdx.x; t < a.n_tiles; t += gridDim.x) {
        const int s = tile_scene_live<TR>(a, t);
        if (s < 0) continue;
        const int i = a.tile_row0[t] + threadIdx.x;
        if (i >= a.voff[s + 1]) continue;
        const double alpha = a.sc[SC_COUNT * s + SC_ALPHA], beta = a.sc[SC_COUNT * s + SC_BETA];
        // every load before the first store (the arrays are not declared distinct)
        double u[3], p[3], w[3], sv[3], x[3], r[3], M[9];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int q = 3 * i + d;
            u[d] = a.m.u[4 * i + d];
            p[d] = a.m.p[q];
            w[d] = a.m.w[q];
            sv[d] = a.m.s[q];
            x[d] = a.m.x[q];
            r[d] = a.m.r[q];
        }
#pragma unroll
        for (int k = 0; k < 9; ++k) M[k] = __ldg(a.m.minv + 9 * (size_t)i + k);
        double r3[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int q = 3 * i + d;
            const double pn = u[d] + beta * p[d], sn = w[d] + beta * sv[d];
            r3[d] = r[d] - alpha * sn;
            a.m.p[q] = pn;
            a.m.s[q] = sn;
            a.m.x[q] = x[d] + alpha * pn;
            a.m.r[q] = r3[d];
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) a.m.u[4 * i + d] = M[3 * d] * r3[0] + M[3 * d + 1] * r3[1] + M[3 * d + 2] * r3[2];
    }
}

__global__ void k_bpcg_iters(int S, const int* __restrict__ sflag, int* __restrict__ iters) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < S) iters[s] = sflag[4 * s + 1];
}

}  // namespace fipc

// ---------------------------------------------------------------- host side
namespace fipc {

int find_constraints(fipc_ctx* c, const double* x, cudaStream_t s);
int ccd_launch(fipc_ctx* c, const double* x, const double* p, double eta, bool inversion, unsigned long long* slot, cudaStream_t s);
int collision_launch(fipc_ctx* c, const double* x, int* hit, cudaStream_t s);

constexpr int BPCG_CHUNK = 32;   // iterations per captured graph

static RowLists row_lists(const fipc_ctx* c) {
    RowLists rl;
    for (int t = 0; t < N_TYPES; ++t) {
        rl.rows[t] = c->rows[t].as<int4>();
        rl.n[t] = c->h_counts[t];
    }
    return rl;
}

// tiles of at most tr rows, never crossing a scene
static int build_tiles(fipc_ctx* c, int tr, cudaStream_t s) {
    std::vector<int> ts, tr0, st0(c->n_scenes + 1, 0);
    for (int q = 0; q < c->n_scenes; ++q) {
        for (int r = c->h_voff[q]; r < c->h_voff[q + 1]; r += tr) {
            ts.push_back(q);
            tr0.push_back(r);
        }
        st0[q + 1] = (int)ts.size();
    }
    const int nt = (int)ts.size();
    if (c->tile_scene.ensure(4ll * nt + 4) || c->tile_row0.ensure(4ll * nt + 4) || c->scene_tile0.ensure(4ll * (c->n_scenes + 1)) ||
        c->bpcg_part.ensure(8ll * 3 * nt + 64))
        return FIPC_ERR_CUDA;
    FIPC_CUDA(cudaMemcpyAsync(c->tile_scene.p, ts.data(), 4ll * nt, cudaMemcpyHostToDevice, s));
    FIPC_CUDA(cudaMemcpyAsync(c->tile_row0.p, tr0.data(), 4ll * nt, cudaMemcpyHostToDevice, s));
    FIPC_CUDA(cudaMemcpyAsync(c->scene_tile0.p, st0.data(), 4ll * (c->n_scenes + 1), cudaMemcpyHostToDevice, s));
    FIPC_CUDA(cudaStreamSynchronize(s));   // host vectors go out of scope
    c->n_tiles = nt;
    c->tile_rows = tr;
    return FIPC_OK;
}

template <int TR>
static void launch_start(const BPCG& a, int grid, const double* rhs, cudaStream_t s) {
    k_bpcg_start<TR><<<grid, TR, 0, s>>>(a, rhs);
}
template <int TR>
static void launch_iter(const BPCG& a, int grid, cudaStream_t s) {
    k_bpcg_spmv<TR><<<grid, TR, 0, s>>>(a);
    k_bpcg_update<TR><<<grid, TR, 0, s>>>(a);
}
template <int TR>
static void launch_spmv(const BPCG& a, int grid, cudaStream_t s) {
    k_bpcg_spmv<TR><<<grid, TR, 0, s>>>(a);
}
static void dispatch_start(int tr, const BPCG& a, int grid, const double* rhs, cudaStream_t s) {
    if (tr == 64) launch_start<64>(a, grid, rhs, s);
    else if (tr == 256) launch_start<256>(a, grid, rhs, s);
    else launch_start<128>(a, grid, rhs, s);
}
static void dispatch_iter(int tr, const BPCG& a, int grid, cudaStream_t s) {
    if (tr == 64) launch_iter<64>(a, grid, s);
    else if (tr == 256) launch_iter<256>(a, grid, s);
    else launch_iter<128>(a, grid, s);
}
static void dispatch_spmv(int tr, const BPCG& a, int grid, cudaStream_t s) {
    if (tr == 64) launch_spmv<64>(a, grid, s);
    else if (tr == 256) launch_spmv<256>(a, grid, s);
    else launch_spmv<128>(a, grid, s);
}

static void fill_tables(const fipc_ctx* c, BPCG& a) {
    a.n_tiles = c->n_tiles;
    a.tile_scene = c->tile_scene.as<int>();
    a.tile_row0 = c->tile_row0.as<int>();
    a.scene_tile0 = c->scene_tile0.as<int>();
    a.part = c->bpcg_part.as<double>();
}

// persistent grid of the batched PCG, chosen by timing the SpMV on the live system: every
// candidate runs its SpMV without reductions, best of three launches.  The tile (rows per tile =
// threads per block) stays at 128 rows: it sets the order of the per-scene sums, so choosing it by
// timing would make the directions depend on the timing; the grid does not change any sum.
static int autotune(fipc_ctx* c, BPCG a, cudaStream_t s) {
    int dev = 0, nsm = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaEvent_t e0, e1;
    FIPC_CUDA(cudaEventCreate(&e0));
    FIPC_CUDA(cudaEventCreate(&e1));
    const int trs[1] = {128};
    const int mult[5] = {2, 4, 8, 16, 0};   // 0: one block per tile
    float best = 1e30f;
    int best_tr = 128, best_grid = 0;
    a.dry = 1;
    for (int tr : trs) {
        int st = build_tiles(c, tr, s);
        if (st) return st;
        fill_tables(c, a);
        for (int m : mult) {
            int grid = m ? m * nsm : c->n_tiles;
            if (grid > c->n_tiles) grid = c->n_tiles;
            if (grid < 1) grid = 1;
            dispatch_spmv(tr, a, grid, s);   // warm-up
            FIPC_LAUNCHED();
            float tmin = 1e30f;
            for (int rep = 0; rep < 3; ++rep) {
                FIPC_CUDA(cudaEventRecord(e0, s));
                dispatch_spmv(tr, a, grid, s);
                FIPC_LAUNCHED();
                FIPC_CUDA(cudaEventRecord(e1, s));
                FIPC_CUDA(cudaEventSynchronize(e1));
                float ms = 0.f;
                FIPC_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                tmin = ms < tmin ? ms : tmin;
            }
            if (tmin < best) {
                best = tmin;
                best_tr = tr;
                best_grid = m ? m * nsm : 0;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    FIPC_CUDA(cudaGetLastError());
    int st = build_tiles(c, best_tr, s);
    if (st) return st;
    c->pcg_grid = best_grid ? (best_grid < c->n_tiles ? best_grid : c->n_tiles) : c->n_tiles;
    c->tune_ms = best;
    return FIPC_OK;
}

static void drop_graph(fipc_ctx* c) {
    if (c->graph_exec) cudaGraphExecDestroy((cudaGraphExec_t)c->graph_exec);
    c->graph_exec = nullptr;
    c->graph_sig.clear();
}

// a graph of BPCG_CHUNK iterations for these kernel arguments (captured on a private stream,
// replayed on the caller's); false when capture is unavailable
static bool chunk_graph(fipc_ctx* c, const BPCG& a) {
    const unsigned char* sig = reinterpret_cast<const unsigned char*>(&a);
    if (c->graph_exec && c->graph_sig.size() == sizeof(BPCG) && std::equal(sig, sig + sizeof(BPCG), c->graph_sig.begin()))
        return true;
    drop_graph(c);
    if (!c->cap_stream) {
        cudaStream_t cs;
        if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) return false;
        c->cap_stream = cs;
    }
    cudaStream_t cs = (cudaStream_t)c->cap_stream;
    if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return false;
    for (int k = 0; k < BPCG_CHUNK; ++k) dispatch_iter(c->tile_rows, a, c->pcg_grid, cs);
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
    c->graph_sig.assign(sig, sig + sizeof(BPCG));
    return true;
}

int batch_pcg(fipc_ctx* c, const unsigned char* fixed, const unsigned char* active, double rtol, int maxit, double* sol, int* iters,
              int* failed_h, cudaStream_t s) {
    const int S = c->n_scenes;
    const long long n3 = 3ll * c->nV;
    if (c->pcg_vec.ensure(8 * (n3 * 4 + 13ll * c->nV) + 64) || c->bpcg_sc.ensure(8ll * SC_COUNT * S + 64) ||
        c->bpcg_flag.ensure(4ll * (4 * S + 4)))
        return FIPC_ERR_CUDA;
    if (c->c_nnzb == 0 && (c->c_rowptr.ensure(4ll * (c->nV + 1)) || cudaMemsetAsync(c->c_rowptr.p, 0, 4ll * (c->nV + 1), s)))
        return FIPC_ERR_CUDA;
    if (c->c_val.ensure(72) || c->c_col.ensure(4)) return FIPC_ERR_CUDA;
    BPCG a;
    memset(&a, 0, sizeof(a));
    a.m.nV = c->nV;
    a.m.soff = c->sell_off;
    a.m.scol = c->sell_col;
    a.m.rlen = c->row_len;
    a.m.sval = c->sell_val;
    a.m.crp = c->c_rowptr.as<int>();
    a.m.cci = c->c_col.as<int>();
    a.m.cva = c->c_val.as<double>();
    a.m.fixed = fixed;
    a.m.diag_spos = c->diag_spos;
    double* v = c->pcg_vec.as<double>();
    a.m.x = sol;
    a.m.u = v;
    a.m.r = v + 4ll * c->nV;
    a.m.w = a.m.r + n3;
    a.m.p = a.m.w + n3;
    a.m.s = a.m.p + n3;
    a.m.minv = a.m.s + n3;
    a.S = S;
    a.maxit = maxit;
    a.voff = c->voff_d;
    a.sc = c->bpcg_sc.as<double>();
    a.sflag = c->bpcg_flag.as<int>();
    a.ndone = a.sflag + 4 * S;
    a.rtol = rtol;
    if (c->tile_rows == 0) {
        int st = autotune(c, a, s);
        if (st) return st;
    }
    fill_tables(c, a);
    a.dry = 0;
    FIPC_CUDA(cudaMemsetAsync(a.ndone, 0, sizeof(int), s));
    k_bpcg_init<<<nblk(S, 128), 128, 0, s>>>(S, active, a.sflag, a.ndone);
    FIPC_LAUNCHED();
    dispatch_start(c->tile_rows, a, c->pcg_grid, c->rhs, s);
    FIPC_LAUNCHED();
    const bool graph = chunk_graph(c, a);
    int ndone = 0;
    for (long long it = 0; it <= (long long)maxit + BPCG_CHUNK; it += BPCG_CHUNK) {
        if (graph) {
            FIPC_CUDA(cudaGraphLaunch((cudaGraphExec_t)c->graph_exec, s));
        } else {
            for (int k = 0; k < BPCG_CHUNK; ++k) dispatch_iter(c->tile_rows, a, c->pcg_grid, s);
        }
        g_launches.fetch_add(2 * BPCG_CHUNK, std::memory_order_relaxed);
        FIPC_CUDA(cudaMemcpyAsync(&ndone, a.ndone, sizeof(int), cudaMemcpyDeviceToHost, s));
        FIPC_CUDA(cudaStreamSynchronize(s));
        if (ndone >= S) break;
    }
    if (iters) {
        k_bpcg_iters<<<nblk(S, 128), 128, 0, s>>>(S, a.sflag, iters);
        FIPC_LAUNCHED();
    }
    std::vector<int> f(4 * S);
    FIPC_CUDA(cudaMemcpyAsync(f.data(), a.sflag, 16ll * S, cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaStreamSynchronize(s));
    int failed = 0;
    for (int q = 0; q < S; ++q) failed += (f[4 * q] == 0 || f[4 * q + 3]) ? 1 : 0;
    if (failed_h) *failed_h = failed;
    FIPC_CUDA(cudaGetLastError());
    return failed ? FIPC_ERR_ITERATION : FIPC_OK;
}

void free_batch(fipc_ctx* c) {
    drop_graph(c);
    if (c->cap_stream) cudaStreamDestroy((cudaStream_t)c->cap_stream);
    c->cap_stream = nullptr;
    void* ptrs[] = {c->v_scene, c->voff_d, c->toff_d, c->s_kappa, c->s_inv_dx, c->s_hash_inv_dx};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    DBuf* bufs[] = {&c->tile_scene, &c->tile_row0, &c->scene_tile0, &c->bpcg_vec, &c->bpcg_sc, &c->bpcg_part, &c->bpcg_flag, &c->s_red,
                    &c->s_rowoff};
    for (DBuf* b : bufs) b->release();
}

}  // namespace fipc

// ---------------------------------------------------------------- C ABI
using namespace fipc;

extern "C" int fipc_ctx_create(fipc_ctx** out, int n_verts, int n_tets, const int* tets, const double* x_rest, const double* lam,
                               const double* mu, double rho, int n_bp, const int* bp, int n_be, const int* be, int n_bt, const int* bt,
                               double dhat2, double dt);
extern "C" int fipc_ctx_destroy(fipc_ctx* c);
namespace fipc {
int cs_setup(fipc_ctx* c, int agg_rows, const int* row_ptr_h, const int* col_idx_h);
void mg_free(fipc_ctx* c);
double median_edge_inv(const double* x, const int* be, int e0, int e1, double fallback);
}

namespace {
template <class T>
int upload_vec(T** dst, const std::vector<T>& v) {
    *dst = nullptr;
    if (v.empty()) return FIPC_OK;
    if (cudaMalloc((void**)dst, sizeof(T) * v.size()) != cudaSuccess) return FIPC_ERR_CUDA;
    if (cudaMemcpy(*dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice) != cudaSuccess) return FIPC_ERR_CUDA;
    return FIPC_OK;
}
}  // namespace

extern "C" {

int fipc_batch_create(fipc_ctx** out, int n_scenes, const int* vert_off, const int* tet_off, const int* be_off, int n_verts, int n_tets,
                      const int* tets, const double* x_rest, const double* lam, const double* mu, double rho, int n_bp, const int* bp,
                      int n_be, const int* be, int n_bt, const int* bt, double dhat2, double dt) {
    if (!out || n_scenes < 1 || n_scenes > 1024 || !vert_off || !tet_off || !be_off) return FIPC_ERR_ARGUMENT;
    *out = nullptr;
    const int S = n_scenes;
    if (vert_off[0] != 0 || tet_off[0] != 0 || be_off[0] != 0 || vert_off[S] != n_verts || tet_off[S] != n_tets || be_off[S] != n_be)
        return FIPC_ERR_ARGUMENT;
    std::vector<int> vs(n_verts > 0 ? n_verts : 0);
    for (int q = 0; q < S; ++q) {
        if (vert_off[q + 1] <= vert_off[q] || tet_off[q + 1] < tet_off[q] || be_off[q + 1] < be_off[q]) return FIPC_ERR_ARGUMENT;
        for (int i = vert_off[q]; i < vert_off[q + 1]; ++i) vs[i] = q;
    }
    // every element and boundary primitive inside one scene (its own offsets for tets / edges)
    for (int q = 0; q < S; ++q) {
        for (long long k = 4ll * tet_off[q]; k < 4ll * tet_off[q + 1]; ++k)
            if (tets[k] < 0 || tets[k] >= n_verts || vs[tets[k]] != q) return FIPC_ERR_ARGUMENT;
        for (long long k = 2ll * be_off[q]; k < 2ll * be_off[q + 1]; ++k)
            if (be[k] < 0 || be[k] >= n_verts || vs[be[k]] != q) return FIPC_ERR_ARGUMENT;
    }
    for (int k = 0; k < n_bt; ++k) {
        const int a = bt[3 * k], b = bt[3 * k + 1], d = bt[3 * k + 2];
        if (a < 0 || a >= n_verts || b < 0 || b >= n_verts || d < 0 || d >= n_verts || vs[a] != vs[b] || vs[a] != vs[d])
            return FIPC_ERR_ARGUMENT;
    }
    for (int k = 0; k < n_bp; ++k)
        if (bp[k] < 0 || bp[k] >= n_verts) return FIPC_ERR_ARGUMENT;
    // each scene's boundary points, edges and triangles are one run of their list, in scene order
    std::vector<int> poff(3 * (S + 1), 0);
    {
        const int nl[3] = {n_bp, n_be, n_bt};
        for (int l = 0; l < 3; ++l) {
            int* o = poff.data() + l * (S + 1);
            int q = 0;
            for (int k = 0; k < nl[l]; ++k) {
                const int sk = vs[l == 0 ? bp[k] : (l == 1 ? be[2 * k] : bt[3 * k])];
                if (sk < q) return FIPC_ERR_ARGUMENT;
                while (q < sk) o[++q] = k;
            }
            while (q < S) o[++q] = nl[l];
        }
    }
    fipc_ctx* c = nullptr;
    int st = fipc_ctx_create(&c, n_verts, n_tets, tets, x_rest, lam, mu, rho, n_bp, bp, n_be, be, n_bt, bt, dhat2, dt);
    if (st) return st;
    cs_setup(c, 0, nullptr, nullptr);   // the batched PCG preconditions with block-Jacobi
    mg_free(c);
    // per-scene kappa (NEWTON_IPC.py:116-124, x10 at :943) and hash cell (:127-134)
    std::vector<double> mass(n_verts), kap(S), idx(S), hidx(S);
    if (cudaMemcpy(mass.data(), c->mass, 8ll * n_verts, cudaMemcpyDeviceToHost) != cudaSuccess) {
        fipc_ctx_destroy(c);
        return FIPC_ERR_CUDA;
    }
    const double Hb = barrier_H(1.0e-16, dhat2, 1.0);
    for (int q = 0; q < S; ++q) {
        double total = 0.0;
        for (int i = vert_off[q]; i < vert_off[q + 1]; ++i) total += mass[i];
        kap[q] = 1.0e13 * total / (vert_off[q + 1] - vert_off[q]) / (4.0e-16 * Hb) * 10.0;
        double len = 0.0;
        for (int k = be_off[q]; k < be_off[q + 1]; ++k) {
            const int a = be[2 * k], b = be[2 * k + 1];
            const double dx = x_rest[3 * a] - x_rest[3 * b], dy = x_rest[3 * a + 1] - x_rest[3 * b + 1],
                         dz = x_rest[3 * a + 2] - x_rest[3 * b + 2];
            len += std::sqrt(dx * dx + dy * dy + dz * dz);
        }
        const int ne = be_off[q + 1] - be_off[q];
        idx[q] = ne ? 1.0 / (len / (double)ne) : 1.0;
        hidx[q] = median_edge_inv(x_rest, be, be_off[q], be_off[q + 1], idx[q]);
    }
    c->n_scenes = S;
    c->h_voff.assign(vert_off, vert_off + S + 1);
    c->h_toff.assign(tet_off, tet_off + S + 1);
    c->h_kappa = kap;
    c->h_inv_dx = idx;
    if (c->prim_off) cudaFree(c->prim_off);
    st = upload_vec(&c->v_scene, vs) | upload_vec(&c->voff_d, c->h_voff) | upload_vec(&c->toff_d, c->h_toff) |
         upload_vec(&c->s_kappa, kap) | upload_vec(&c->s_inv_dx, idx) | upload_vec(&c->s_hash_inv_dx, hidx) |
         upload_vec(&c->prim_off, poff);
    if (st) {
        fipc_ctx_destroy(c);
        return FIPC_ERR_CUDA;
    }
    *out = c;
    return FIPC_OK;
}

int fipc_batch_params(fipc_ctx* c, int* n_scenes, double* kappa, double* inv_dx) {
    if (!c) return FIPC_ERR_ARGUMENT;
    if (n_scenes) *n_scenes = c->n_scenes;
    for (int q = 0; q < (int)c->h_kappa.size(); ++q) {
        if (kappa) kappa[q] = c->h_kappa[q];
        if (inv_dx) inv_dx[q] = c->h_inv_dx[q];
    }
    return FIPC_OK;
}

int fipc_batch_compute_energy(fipc_ctx* c, const double* x, const double* xt, double* energy, void* stream) {
    if (!c || c->n_scenes < 2 || !x || !xt || !energy) return FIPC_ERR_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    const int S = c->n_scenes;
    if (c->s_rowoff.ensure(4ll * N_TYPES * (S + 1))) return FIPC_ERR_CUDA;
    const RowLists rl = row_lists(c);
    k_scene_row_offsets<<<nblk(S + 1, 128), 128, 0, s>>>(S, c->voff_d, rl, c->s_rowoff.as<int>());
    FIPC_LAUNCHED();
    k_scene_energy<<<S, SE_THREADS, 0, s>>>(S, c->voff_d, c->toff_d, c->s_rowoff.as<int>(), rl, x, xt, c->mass, (const int4*)c->tets,
                                            c->dminv, c->vol, c->lam, c->mu, c->dt * c->dt, c->x0, c->dhat2, c->s_kappa, energy);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc_batch_output_residual(fipc_ctx* c, const double* sol, double* residual, void* stream) {
    if (!c || c->n_scenes < 2 || !sol || !residual) return FIPC_ERR_ARGUMENT;
    k_scene_absmax<<<c->n_scenes, SE_THREADS, 0, (cudaStream_t)stream>>>(c->voff_d, sol, residual);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc_batch_step_size(fipc_ctx* c, const double* x, const double* sol, double eta, int inversion, double* alpha, void* stream) {
    if (!c || c->n_scenes < 2 || !x || !sol || !alpha) return FIPC_ERR_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    k_fill_f64<<<nblk(c->n_scenes, 128), 128, 0, s>>>(c->n_scenes, alpha, 1.0);
    FIPC_LAUNCHED();
    return ccd_launch(c, x, sol, eta, inversion != 0, reinterpret_cast<unsigned long long*>(alpha), s);
}

int fipc_batch_check_collision(fipc_ctx* c, const double* x, int* hit, void* stream) {
    if (!c || c->n_scenes < 2 || !x || !hit) return FIPC_ERR_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    FIPC_CUDA(cudaMemsetAsync(hit, 0, sizeof(int) * c->n_scenes, s));
    return collision_launch(c, x, hit, s);
}

int fipc_batch_apply_sol(fipc_ctx* c, const double* xprev, const double* sol, const double* alpha, double* x, void* stream) {
    if (!c || c->n_scenes < 2 || !xprev || !sol || !alpha || !x) return FIPC_ERR_ARGUMENT;
    k_apply_sol_scenes<<<nblk(3ll * c->nV, 256), 256, 0, (cudaStream_t)stream>>>(3 * c->nV, c->v_scene, xprev, sol, alpha, x);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc_batch_solve_system(fipc_ctx* c, const unsigned char* fixed, const unsigned char* active, double rtol, int maxit, int use_guess,
                            double* sol, int* iters, int* n_failed, void* stream) {
    if (!c || c->n_scenes < 2 || !fixed || !sol || maxit <= 0 || !(rtol >= 0)) return FIPC_ERR_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    if (!use_guess) FIPC_CUDA(cudaMemsetAsync(sol, 0, sizeof(double) * 3ull * c->nV, s));
    return batch_pcg(c, fixed, active, rtol, maxit, sol, iters, n_failed, s);
}

int fipc_batch_pcg_shape(fipc_ctx* c, int* tile_rows, int* grid, int* n_tiles, float* spmv_ms) {
    if (!c) return FIPC_ERR_ARGUMENT;
    if (tile_rows) *tile_rows = c->tile_rows;
    if (grid) *grid = c->pcg_grid;
    if (n_tiles) *n_tiles = c->n_tiles;
    if (spmv_ms) *spmv_ms = c->tune_ms;
    return FIPC_OK;
}

}  // extern "C"
