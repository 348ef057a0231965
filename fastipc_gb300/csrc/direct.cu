// Direct solve of the Newton system: the role of the reference's CHOLMOD factorisation
// (projects/FastIPC/NEWTON_IPC.py:764-776), for the iterations where PCG reaches its iteration
// limit, or for callers that want the reference's exact solve.
//
// A multifrontal Cholesky factorisation written for this GPU (no library factorisation):
//  * analysis on the host (mf_plan.h): nested-dissection ordering of the free vertices from the
//    elastic and contact block patterns, the assembly tree, one dense frontal matrix per tree
//    node, extend-add maps and the task tables of the numeric phase;
//  * the edited system's 3x3 blocks (Dirichlet rows and columns removed: their solution is 0,
//    as NEWTON_IPC.py:758-772 makes it) scattered into the fronts, elastic then contact;
//  * per tree height, children's update matrices pulled into their parents (each entry sums its
//    children in a fixed order), then every front of the height factored panel by panel: the
//    64 x 64 diagonal tile by one CTA, the rows below it in 64-row chunks, and the trailing
//    update in 64 x 64 tiles (4 x 4 register blocks, operands staged in shared memory) across
//    all fronts of the height at once;
//  * forward and backward substitution through the tree (one CTA per front).
// Every sum runs in a fixed order, so the solve is deterministic.  FP64 throughout: the
// trailing update, which holds nearly all the flops, is bound by the FP64 pipe.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <vector>

#include "ctx.cuh"
#include "mf_plan.h"

namespace fipc {

int sell_to_bsr(fipc_ctx* c, double* out, cudaStream_t s);

namespace {

constexpr int MF_THREADS = 256;
constexpr int MF_LDS = MF_TILE + 1;   // padded shared-memory column stride of a tile

inline int nbd(long long n, int b) { return (int)((n + b - 1) / b); }

// device copy of the plan (pointers into one arena) and the numeric buffers
struct MfDev {
    double* F;                       // fronts
    double* W;                       // per-front solve vectors
    double* Y;                       // per-front pivot results of the forward sweep
    const int *nvf, *npiv, *piv0, *child0, *children, *cmap, *fidx, *order, *level_nodes, *task_front, *ext_front;
    const long long *foff, *woff, *cmap0, *fidx0, *task_chunk0, *task_tile0, *ext_col0;
    int* flag;                       // [0]: a non-positive or non-finite pivot
};

// ---------------------------------------------------------------- assembly into the fronts
// block k of a block matrix to its front position (column-major, leading dimension ld[k])
__global__ void k_mf_scatter(long long nb, const double* __restrict__ val, const long long* __restrict__ dst, const int* __restrict__ ld,
                             double* __restrict__ F, int add) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nb) return;
    const long long d = dst[k];
    if (d < 0) return;
    const long long L = ld[k];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            const double v = val[9 * k + 3 * a + b];
            double* p = F + d + a + b * L;
            *p = add ? *p + v : v;
        }
}

// extend-add, pull form: one CTA per (front, column j); each lower entry (i >= j) adds the
// matching entries of its children's update matrices, children in tree order
__global__ void __launch_bounds__(MF_THREADS) k_mf_extend(MfDev d, const int* __restrict__ fronts, const long long* __restrict__ col0,
                                                          int nf) {
    const long long q = blockIdx.x;
    const int e = mf_find(col0, nf + 1, q);
    const int f = fronts[e];
    const int j = (int)(q - col0[e]);
    const int N = 3 * d.nvf[f];
    double* F = d.F + d.foff[f];
    const int J = j / 3, jb = j % 3;
    for (int i = j + threadIdx.x; i < N; i += MF_THREADS) {
        const int I = i / 3, ib = i % 3;
        double v = 0.0;
        for (int t = d.child0[f]; t < d.child0[f + 1]; ++t) {
            const int c = d.children[t];
            const int* m = d.cmap + d.cmap0[c];
            const int ci = m[I], cj = m[J];
            if (ci < 0 || cj < 0) continue;
            const long long Nc = 3ll * d.nvf[c];
            v += d.F[d.foff[c] + (3 * ci + ib) + (3ll * cj + jb) * Nc];
        }
        F[i + (long long)j * N] += v;
    }
}

// ---------------------------------------------------------------- panel factorisation
struct PanelArgs {
    int k;                           // panel index: columns [k MF_TILE, k MF_TILE + kb)
    int n_fronts;
    long long t0;                    // offset into task_front
    const long long* chunk0;         // prefix of row chunks (n_fronts + 1)
    const long long* tile0;          // prefix of trailing tiles (n_fronts + 1)
};

__device__ __forceinline__ void panel_geometry(const MfDev& d, const PanelArgs& p, int e, int* f, int* N, int* c0, int* kb) {
    *f = d.task_front[p.t0 + e];
    *N = 3 * d.nvf[*f];
    *c0 = p.k * MF_TILE;
    *kb = min(MF_TILE, 3 * d.npiv[*f] - *c0);
}

// Cholesky of the diagonal tile, one CTA per front, right-looking in shared memory
__global__ void __launch_bounds__(MF_THREADS) k_mf_potrf(MfDev d, PanelArgs p) {
    __shared__ double T[MF_TILE * MF_LDS];
    int f, N, c0, kb;
    panel_geometry(d, p, blockIdx.x, &f, &N, &c0, &kb);
    double* F = d.F + d.foff[f] + c0 + (long long)c0 * N;
    for (int idx = threadIdx.x; idx < kb * kb; idx += MF_THREADS) {
        const int i = idx % kb, j = idx / kb;
        if (i >= j) T[i + j * MF_LDS] = F[i + (long long)j * N];
    }
    __syncthreads();
    for (int j = 0; j < kb; ++j) {
        if (threadIdx.x == 0) {
            double dj = T[j + j * MF_LDS];
            if (!(dj > 0.0) || !isfinite(dj)) {
                atomicOr(d.flag, 1);
                dj = 1.0;
            }
            T[j + j * MF_LDS] = sqrt(dj);
        }
        __syncthreads();
        const double piv = T[j + j * MF_LDS];
        for (int i = j + 1 + threadIdx.x; i < kb; i += MF_THREADS) T[i + j * MF_LDS] /= piv;
        __syncthreads();
        const int r = kb - j - 1;
        for (int idx = threadIdx.x; idx < r * r; idx += MF_THREADS) {
            const int i = j + 1 + idx % r, l = j + 1 + idx / r;
            if (i >= l) T[i + l * MF_LDS] -= T[i + j * MF_LDS] * T[l + j * MF_LDS];
        }
        __syncthreads();
    }
    for (int idx = threadIdx.x; idx < kb * kb; idx += MF_THREADS) {
        const int i = idx % kb, j = idx / kb;
        if (i >= j) F[i + (long long)j * N] = T[i + j * MF_LDS];
    }
}

// rows below the diagonal tile, 64 per CTA: X L^T = B, right-looking over the panel's columns
__global__ void __launch_bounds__(MF_THREADS) k_mf_trsm(MfDev d, PanelArgs p) {
    extern __shared__ double sm[];
    double* L = sm;
    double* B = sm + MF_TILE * MF_LDS;
    const int e = mf_find(p.chunk0, p.n_fronts + 1, blockIdx.x);
    int f, N, c0, kb;
    panel_geometry(d, p, e, &f, &N, &c0, &kb);
    const int r0 = c0 + kb + (int)(blockIdx.x - p.chunk0[e]) * MF_TILE;
    const int nr = min(MF_TILE, N - r0);
    const double* Fd = d.F + d.foff[f] + c0 + (long long)c0 * N;
    double* Fb = d.F + d.foff[f] + r0 + (long long)c0 * N;
    for (int idx = threadIdx.x; idx < kb * kb; idx += MF_THREADS) {
        const int i = idx % kb, j = idx / kb;
        if (i >= j) L[i + j * MF_LDS] = Fd[i + (long long)j * N];
    }
    for (int idx = threadIdx.x; idx < nr * kb; idx += MF_THREADS) {
        const int r = idx % nr, j = idx / nr;
        B[r + j * MF_LDS] = Fb[r + (long long)j * N];
    }
    __syncthreads();
    for (int j = 0; j < kb; ++j) {
        const double piv = L[j + j * MF_LDS];
        for (int r = threadIdx.x; r < nr; r += MF_THREADS) B[r + j * MF_LDS] /= piv;
        __syncthreads();
        const int w = kb - j - 1;
        for (int idx = threadIdx.x; idx < nr * w; idx += MF_THREADS) {
            const int r = idx % nr, l = j + 1 + idx / nr;
            B[r + l * MF_LDS] -= B[r + j * MF_LDS] * L[l + j * MF_LDS];
        }
        __syncthreads();
    }
    for (int idx = threadIdx.x; idx < nr * kb; idx += MF_THREADS) {
        const int r = idx % nr, j = idx / nr;
        Fb[r + (long long)j * N] = B[r + j * MF_LDS];
    }
}

// trailing update of one 64 x 64 lower tile: C -= A_i A_j^T over the panel's kb columns.
// Thread (tr, tc) owns rows tr + 16 a and columns tc + 16 b (a, b < 4): a warp's loads and
// stores of C cover 16 consecutive rows of two columns.
__global__ void __launch_bounds__(MF_THREADS) k_mf_update(MfDev d, PanelArgs p) {
    extern __shared__ double sm[];
    double* As = sm;                      // [l][row], 64 x 64
    double* Bs = sm + MF_TILE * MF_TILE;
    const int e = mf_find(p.tile0, p.n_fronts + 1, blockIdx.x);
    int f, N, c0, kb;
    panel_geometry(d, p, e, &f, &N, &c0, &kb);
    int ti, tj;
    mf_tile(blockIdx.x - p.tile0[e], &ti, &tj);
    const int s0 = c0 + kb;
    const int i0 = s0 + ti * MF_TILE, j0 = s0 + tj * MF_TILE;
    const int ni = min(MF_TILE, N - i0), nj = min(MF_TILE, N - j0);
    const double* F = d.F + d.foff[f];
    for (int idx = threadIdx.x; idx < MF_TILE * kb; idx += MF_THREADS) {
        const int r = idx % MF_TILE, l = idx / MF_TILE;
        As[l * MF_TILE + r] = r < ni ? F[(i0 + r) + (long long)(c0 + l) * N] : 0.0;
        Bs[l * MF_TILE + r] = r < nj ? F[(j0 + r) + (long long)(c0 + l) * N] : 0.0;
    }
    __syncthreads();
    const int tr = threadIdx.x & 15, tc = threadIdx.x >> 4;
    double acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
    for (int l = 0; l < kb; ++l) {
        double av[4], bv[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            av[a] = As[l * MF_TILE + tr + 16 * a];
            bv[a] = Bs[l * MF_TILE + tc + 16 * a];
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a][b] = fma(av[a], bv[b], acc[a][b]);
    }
    double* C = d.F + d.foff[f];
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const int j = tc + 16 * b;
        if (j >= nj) continue;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int i = tr + 16 * a;
            if (i < ni) C[(i0 + i) + (long long)(j0 + j) * N] -= acc[a][b];
        }
    }
}

// ---------------------------------------------------------------- substitution
// forward: w = gathered right-hand side + children's updates; pivots solved column by column
// (pivot results to Y), the rest of w updated; one CTA per front of the height
__global__ void __launch_bounds__(MF_THREADS) k_mf_forward(MfDev d, int h0, const double* __restrict__ rhs) {
    const int f = d.level_nodes[h0 + blockIdx.x];
    const int N = 3 * d.nvf[f], P = 3 * d.npiv[f];
    double* w = d.W + d.woff[f];
    double* y = d.Y + d.woff[f];
    const double* F = d.F + d.foff[f];
    for (int i = threadIdx.x; i < N; i += MF_THREADS) {
        const int I = i / 3, ib = i % 3;
        double v = I < d.npiv[f] ? rhs[3ll * d.order[d.piv0[f] + I] + ib] : 0.0;
        for (int t = d.child0[f]; t < d.child0[f + 1]; ++t) {
            const int c = d.children[t];
            const int m = d.cmap[d.cmap0[c] + I];
            if (m >= 0) v += d.W[d.woff[c] + 3 * m + ib];
        }
        w[i] = v;
    }
    __syncthreads();
    for (int j = 0; j < P; ++j) {
        const double wj = w[j] / F[j + (long long)j * N];
        if (threadIdx.x == 0) y[j] = wj;
        for (int i = j + 1 + threadIdx.x; i < N; i += MF_THREADS) w[i] -= F[i + (long long)j * N] * wj;
        __syncthreads();
    }
    for (int j = threadIdx.x; j < P; j += MF_THREADS) w[j] = y[j];
}

// backward, one CTA per front of the height (parents first): the structure's values from the
// solution, w_j -= L_ij x_i over them (a warp per column), then the pivots' triangle by one
// warp, written to the solution
__global__ void __launch_bounds__(MF_THREADS) k_mf_backward(MfDev d, int h0, double* __restrict__ sol) {
    const int f = d.level_nodes[h0 + blockIdx.x];
    const int N = 3 * d.nvf[f], P = 3 * d.npiv[f];
    double* w = d.W + d.woff[f];
    const double* F = d.F + d.foff[f];
    const int* fl = d.fidx + d.fidx0[f];
    for (int i = P + threadIdx.x; i < N; i += MF_THREADS) w[i] = sol[3ll * d.order[fl[i / 3]] + i % 3];
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int j = wid; j < P; j += MF_THREADS / 32) {
        double s = 0.0;
        for (int i = P + lane; i < N; i += 32) s += F[i + (long long)j * N] * w[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) w[j] -= s;
    }
    __syncthreads();
    if (wid == 0) {
        for (int j = P - 1; j >= 0; --j) {
            double s = 0.0;
            for (int i = j + 1 + lane; i < P; i += 32) s += F[i + (long long)j * N] * w[i];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
            if (lane == 0) w[j] = (w[j] - s) / F[j + (long long)j * N];
            __syncwarp();
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < P; j += MF_THREADS) sol[3ll * d.order[d.piv0[f] + j / 3] + j % 3] = w[j];
}

struct DevMem {
    void* p = nullptr;
    ~DevMem() {
        if (p) cudaFree(p);
    }
    bool alloc(size_t n) { return cudaMalloc(&p, n ? n : 16) == cudaSuccess; }
    template <class T>
    T* as() const { return (T*)p; }
};

// packs host vectors into one device arena (16-byte aligned pieces)
struct Arena {
    std::vector<char> host;
    std::vector<std::pair<size_t, const void**>> fix;
    template <class T>
    void add(const std::vector<T>& v, const T** out) {
        size_t off = (host.size() + 15) & ~size_t(15);
        host.resize(off + sizeof(T) * v.size());
        if (!v.empty()) memcpy(host.data() + off, v.data(), sizeof(T) * v.size());
        fix.push_back({off, (const void**)out});
    }
    bool upload(DevMem& m, cudaStream_t s) {
        if (!m.alloc(host.size())) return false;
        if (cudaMemcpyAsync(m.p, host.data(), host.size(), cudaMemcpyHostToDevice, s) != cudaSuccess) return false;
        for (auto& f : fix) *f.second = (const void*)((char*)m.p + f.first);
        return true;
    }
};

bool g_attr_set = false;

}  // namespace
}  // namespace fipc

using namespace fipc;

extern "C" {

int fipc_solve_system_direct(fipc_ctx* c, const unsigned char* fixed, double* sol, int* nnz_h, void* stream) {
    if (!c || !fixed || !sol) return FIPC_ERR_ARGUMENT;
    const int* crp_d = c->c_rowptr.as<int>();
    if (!crp_d) return FIPC_ERR_ARGUMENT;   // no system assembled
    cudaStream_t s = (cudaStream_t)stream;
    const int nV = c->nV;
    const int e_nnzb = c->nnzb, c_nnzb = c->c_nnzb;
    // patterns, Dirichlet mask and rest positions to the host for the analysis
    std::vector<int> rp(nV + 1), ci(e_nnzb), crp(nV + 1), cci(c_nnzb);
    std::vector<unsigned char> fx(nV);
    std::vector<double> x0(3ll * nV);
    FIPC_CUDA(cudaMemcpyAsync(rp.data(), c->row_ptr, 4ll * (nV + 1), cudaMemcpyDeviceToHost, s));
    if (e_nnzb) FIPC_CUDA(cudaMemcpyAsync(ci.data(), c->col_idx, 4ll * e_nnzb, cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaMemcpyAsync(crp.data(), crp_d, 4ll * (nV + 1), cudaMemcpyDeviceToHost, s));
    if (c_nnzb) FIPC_CUDA(cudaMemcpyAsync(cci.data(), c->c_col.p, 4ll * c_nnzb, cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaMemcpyAsync(fx.data(), fixed, nV, cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaMemcpyAsync(x0.data(), c->x0, 24ll * nV, cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaStreamSynchronize(s));
    MfPlan P;
    const auto t_an = std::chrono::steady_clock::now();
    if (mf_analyse(nV, rp.data(), ci.data(), c_nnzb ? crp.data() : nullptr, c_nnzb ? cci.data() : nullptr, fx.data(), x0.data(), P))
        return FIPC_ERR_ARGUMENT;
    c->mf_analyse_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_an).count();
    c->mf_fronts = P.n_nodes;
    c->mf_front_doubles = P.f_total;
    c->mf_flops = P.flops;
    FIPC_CUDA(cudaMemsetAsync(sol, 0, 24ll * nV, s));
    if (nnz_h) {
        long long stored = 0;
        for (int f = 0; f < P.n_nodes; ++f) stored += 9ll * P.nvf[f] * (P.nvf[f] + 1) / 2 + 3ll * P.nvf[f];
        *nnz_h = (int)std::min<long long>(stored, INT_MAX);
    }
    if (P.n_nodes == 0) return FIPC_OK;
    // the fronts must fit
    size_t free_b = 0, total_b = 0;
    FIPC_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const double need = 8.0 * ((double)P.f_total + 2.0 * (double)P.w_total) + 72.0 * e_nnzb;
    if (need > 0.85 * (double)free_b) return FIPC_ERR_CAPACITY;
    // extend-add tasks per height: fronts with children, prefix of their columns
    std::vector<int> ext_front;
    std::vector<long long> ext_col0;
    std::vector<long long> ext_at(P.height_max + 2, 0);   // per height: start in ext_front
    std::vector<long long> ext_pre_at(P.height_max + 2, 0);
    for (int h = 0; h <= P.height_max; ++h) {
        ext_at[h] = (long long)ext_front.size();
        ext_pre_at[h] = (long long)ext_col0.size();
        long long acc = 0;
        ext_col0.push_back(0);
        for (int q = P.lvl0[h]; q < P.lvl0[h + 1]; ++q) {
            const int f = P.level_nodes[q];
            if (P.child0[f + 1] == P.child0[f]) continue;
            ext_front.push_back(f);
            acc += 3ll * P.nvf[f];
            ext_col0.push_back(acc);
        }
    }
    ext_at[P.height_max + 1] = (long long)ext_front.size();
    MfDev d{};
    Arena ar;
    ar.add(P.nvf, &d.nvf);
    ar.add(P.npiv, &d.npiv);
    ar.add(P.piv0, &d.piv0);
    ar.add(P.child0, &d.child0);
    ar.add(P.children, &d.children);
    ar.add(P.cmap, &d.cmap);
    ar.add(P.fidx, &d.fidx);
    ar.add(P.order, &d.order);
    ar.add(P.level_nodes, &d.level_nodes);
    ar.add(P.task_front, &d.task_front);
    ar.add(ext_front, &d.ext_front);
    ar.add(P.foff, &d.foff);
    ar.add(P.woff, &d.woff);
    ar.add(P.cmap0, &d.cmap0);
    ar.add(P.fidx0, &d.fidx0);
    ar.add(P.task_chunk0, &d.task_chunk0);
    ar.add(P.task_tile0, &d.task_tile0);
    ar.add(ext_col0, &d.ext_col0);
    const long long *e_dst = nullptr, *c_dst = nullptr;
    const int *e_ld = nullptr, *c_ld = nullptr;
    ar.add(P.e_dst, &e_dst);
    ar.add(P.e_ld, &e_ld);
    ar.add(P.c_dst, &c_dst);
    ar.add(P.c_ld, &c_ld);
    DevMem plan, fronts, vecs, ev, flag;
    if (!ar.upload(plan, s)) return FIPC_ERR_CUDA;
    if (!fronts.alloc(8ull * P.f_total) || !vecs.alloc(16ull * P.w_total) || !ev.alloc(72ull * e_nnzb) || !flag.alloc(16))
        return FIPC_ERR_CUDA;
    d.F = fronts.as<double>();
    d.W = vecs.as<double>();
    d.Y = d.W + P.w_total;
    d.flag = flag.as<int>();
    FIPC_CUDA(cudaMemsetAsync(d.F, 0, 8ull * P.f_total, s));
    FIPC_CUDA(cudaMemsetAsync(d.flag, 0, 16, s));
    if (!g_attr_set) {
        FIPC_CUDA(cudaFuncSetAttribute(k_mf_update, cudaFuncAttributeMaxDynamicSharedMemorySize, 16 * MF_TILE * MF_TILE));
        FIPC_CUDA(cudaFuncSetAttribute(k_mf_trsm, cudaFuncAttributeMaxDynamicSharedMemorySize, 16 * MF_TILE * MF_LDS));
        g_attr_set = true;
    }
    int st = sell_to_bsr(c, ev.as<double>(), s);
    if (st) return st;
    if (e_nnzb) {
        k_mf_scatter<<<nbd(e_nnzb, 256), 256, 0, s>>>(e_nnzb, ev.as<double>(), e_dst, e_ld, d.F, 0);
        FIPC_LAUNCHED();
    }
    if (c_nnzb) {
        k_mf_scatter<<<nbd(c_nnzb, 256), 256, 0, s>>>(c_nnzb, c->c_val.as<double>(), c_dst, c_ld, d.F, 1);
        FIPC_LAUNCHED();
    }
    size_t pn = 0;
    for (int h = 0; h <= P.height_max; ++h) {
        const int nf = (int)(ext_at[h + 1] - ext_at[h]);
        const long long cols = nf > 0 ? ext_col0[ext_pre_at[h] + nf] : 0;
        if (cols > 0) {
            k_mf_extend<<<(unsigned)cols, MF_THREADS, 0, s>>>(d, d.ext_front + ext_at[h], d.ext_col0 + ext_pre_at[h], nf);
            FIPC_LAUNCHED();
        }
        for (; pn < P.panels.size() && P.panels[pn].height == h; ++pn) {
            const MfPlan::Panel& pl = P.panels[pn];
            PanelArgs pa{pl.k, pl.n_fronts, pl.t0, d.task_chunk0 + P.task_off[pn], d.task_tile0 + P.task_off[pn]};
            k_mf_potrf<<<pl.n_fronts, MF_THREADS, 0, s>>>(d, pa);
            FIPC_LAUNCHED();
            if (pl.n_chunks) {
                k_mf_trsm<<<(unsigned)pl.n_chunks, MF_THREADS, 16 * MF_TILE * MF_LDS, s>>>(d, pa);
                FIPC_LAUNCHED();
            }
            if (pl.n_tiles) {
                k_mf_update<<<(unsigned)pl.n_tiles, MF_THREADS, 16 * MF_TILE * MF_TILE, s>>>(d, pa);
                FIPC_LAUNCHED();
            }
        }
    }
    // right-hand side with zeros at fixed vertices is implied: only free vertices are gathered
    for (int h = 0; h <= P.height_max; ++h) {
        k_mf_forward<<<P.lvl0[h + 1] - P.lvl0[h], MF_THREADS, 0, s>>>(d, P.lvl0[h], c->rhs);
        FIPC_LAUNCHED();
    }
    for (int h = P.height_max; h >= 0; --h) {
        k_mf_backward<<<P.lvl0[h + 1] - P.lvl0[h], MF_THREADS, 0, s>>>(d, P.lvl0[h], sol);
        FIPC_LAUNCHED();
    }
    FIPC_CUDA(cudaGetLastError());
    int bad = 0;
    FIPC_CUDA(cudaMemcpyAsync(&bad, d.flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaStreamSynchronize(s));
    return bad ? FIPC_ERR_NONFINITE : FIPC_OK;
}

int fipc_direct_stats(const fipc_ctx* c, int* fronts_h, long long* front_doubles_h, double* flops_h, double* analyse_ms_h) {
    if (!c) return FIPC_ERR_ARGUMENT;
    if (fronts_h) *fronts_h = c->mf_fronts;
    if (front_doubles_h) *front_doubles_h = c->mf_front_doubles;
    if (flops_h) *flops_h = c->mf_flops;
    if (analyse_ms_h) *analyse_ms_h = c->mf_analyse_ms;
    return FIPC_OK;
}

}  // extern "C"
