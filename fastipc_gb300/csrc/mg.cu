// Multigrid preconditioner of the PCG direction solve: geometric aggregation with rigid-body
// modes (hierarchy from mg_plan.h), one symmetric V(1,1)-cycle per PCG iteration.
//
//     level 0 (vertices, 3x3 blocks):  z = w0 D^-1 r;  t = r - A z;  restrict;  ...;  prolong;
//                                      u = z + w0 D^-1 (r - A z)            (u: the PCG's B r)
//     levels 1 .. L-2 (6x6 blocks):    the same on the Galerkin matrices A_l = P^T A_{l-1} P
//     level L-1 (coarsest):            dense inverse (symmetric block sweep)
//
// D^-1 is the block-Jacobi inverse (level 0: the PCG's own, identity at Dirichlet vertices) and
// w_l = 4 / (3 * 1.05 * rho_l) with rho_l an 8-step power-iteration estimate of the spectral
// radius of D_l^-1 A_l from a fixed start vector (it underestimates rho by up to about 15%, which
// keeps w_l rho_l < 1.6 < 2), so the smoother converges and the cycle is symmetric positive
// definite:
// CG converges to the solution of the same system as with block-Jacobi, in far fewer
// iterations.  Dirichlet vertices have zero rows in every prolongator and a zero output.
//
// Per Newton iteration (mg_prepare / mg_start): contact patterns of every level (host, from the
// system's contact pattern), aggregate centroids and member offsets at the current positions,
// the Galerkin products (one warp per coarse block, fixed-order sums over its contribution
// list), 6x6 block inverses, the dense coarsest inverse and the smoother weights.  Every sum
// runs in a fixed order, so the preconditioner is deterministic.
#include <cuda_runtime.h>

#include <vector>

#include "ctx.cuh"
#include "mg_plan.h"
#include "pcg.cuh"

namespace fipc {

int cs_gauss_jordan(int n, double* A, double* buf, cudaStream_t s);
constexpr int MG_GJ_B = 32;                 // block of the dense inverse (its row padding)
constexpr int MG_POWER_ITERS = 8;          // power iterations per level and solve
constexpr int MG_THREADS = 128;
constexpr int MG_MIN_VERTICES = 1000;      // smaller scenes keep the two-level preconditioner

static inline int nblk_m(long long n, int b) { return (int)((n + b - 1) / b); }

void mg_vcycle(const fipc_ctx* c, const PCGArgs& a, cudaStream_t s);
int mg_launches_per_cycle(int levels);
int mg_offsets(fipc_ctx* c, const double* x, cudaStream_t s);

// device buffers of one level
struct MgLevelBufs {
    DBuf mem_ptr, mem, agg_of, rot;                  // levels >= 1 (rot: level 1)
    DBuf s_rp, s_ci, s_cp, s_src, s_row, s_col;      // static pattern and contributions
    DBuf c_rp, c_ci, c_cp, c_src, c_row, c_col;      // contact pattern and contributions
    DBuf s_val, c_val, minv, cent, d, g, z, z2, t;   // values, inverses, geometry, vectors
    DBuf pv0, pv1, part, nrm;                        // power iteration
    void release() {
        DBuf* all[] = {&mem_ptr, &mem, &agg_of, &rot, &s_rp, &s_ci, &s_cp, &s_src, &s_row, &s_col, &c_rp, &c_ci, &c_cp, &c_src, &c_row,
                       &c_col, &s_val, &c_val, &minv, &cent, &d, &g, &z, &z2, &t, &pv0, &pv1, &part, &nrm};
        for (DBuf* b : all) b->release();
    }
};

struct MgState {
    MgPlan plan;
    std::vector<MgLevelBufs> B;
    DBuf dense, gj_buf, omega, t0, z0, terms, v32, z0f;
    int n_dense = 0, ld_dense = 0;
    bool fp32 = false;                               // FP32 smoothing products on level 0
    bool contact_empty = true;                       // the per-level contact patterns are empty
    MgArgs args{};                                   // kernel arguments of the V-cycle
    ~MgState() {
        for (MgLevelBufs& b : B) b.release();
        DBuf* all[] = {&dense, &gj_buf, &omega, &t0, &z0, &terms, &v32, &z0f};
        for (DBuf* b : all) b->release();
    }
};

template <class T>
static int upload_vec(DBuf& b, const std::vector<T>& v, cudaStream_t s) {
    if (b.ensure(sizeof(T) * (v.size() ? v.size() : 1))) return FIPC_ERR_CUDA;
    if (!v.empty()) FIPC_CUDA(cudaMemcpyAsync(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s));
    return FIPC_OK;
}

// ---------------------------------------------------------------- set-up kernels
// centroid of each aggregate of level l from its members' positions (vertices: x; nodes: the
// finer level's centroids), then each member's offset from it
__global__ void k_mg_centroid(int n, const int* __restrict__ mem_ptr, const int* __restrict__ mem, const double* __restrict__ pos,
                              const unsigned char* __restrict__ rot, double* __restrict__ cent, double* __restrict__ d) {
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= n) return;
    double c0 = 0.0, c1 = 0.0, c2 = 0.0;
    const int k0 = mem_ptr[I], k1 = mem_ptr[I + 1];
    for (int k = k0; k < k1; ++k) {
        const int i = mem[k];
        c0 += pos[3 * (size_t)i];
        c1 += pos[3 * (size_t)i + 1];
        c2 += pos[3 * (size_t)i + 2];
    }
    const double inv = 1.0 / (double)(k1 - k0);
    c0 *= inv;
    c1 *= inv;
    c2 *= inv;
    cent[3 * (size_t)I] = c0;
    cent[3 * (size_t)I + 1] = c1;
    cent[3 * (size_t)I + 2] = c2;
    const bool r = !rot || rot[I];   // translation-only nodes: zero offsets, so zero rotation columns
    for (int k = k0; k < k1; ++k) {
        const int i = mem[k];
        d[3 * (size_t)i] = r ? pos[3 * (size_t)i] - c0 : 0.0;
        d[3 * (size_t)i + 1] = r ? pos[3 * (size_t)i + 1] - c1 : 0.0;
        d[3 * (size_t)i + 2] = r ? pos[3 * (size_t)i + 2] - c2 : 0.0;
    }
}

// C (6x6) += P_i^T B P_j for a finer block B (BxB, row-major, entry e at B[e * es]); P of a
// vertex (B = 3) is [I, -[d]x], of a node (B = 6) [[I, -[d]x], [0, I]]
template <int NB>
__device__ __forceinline__ void gal_add(double (&C)[36], const double* __restrict__ Bp, int es, const double* di, const double* dj) {
    double b[NB * NB];
#pragma unroll
    for (int e = 0; e < NB * NB; ++e) b[e] = __ldg(Bp + (size_t)e * es);
    const double Sj[9] = {0.0, -dj[2], dj[1], dj[2], 0.0, -dj[0], -dj[1], dj[0], 0.0};
    const double Si[9] = {0.0, -di[2], di[1], di[2], 0.0, -di[0], -di[1], di[0], 0.0};
    // X = B P_j (NB x 6): X[:, 0:3] = B[:, 0:3];  X[:, 3:6] = -B[:, 0:3] Sj + B[:, 3:6]
    double X[NB * 6];
#pragma unroll
    for (int r = 0; r < NB; ++r) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            X[6 * r + c] = b[NB * r + c];
            double v = -(b[NB * r] * Sj[c] + b[NB * r + 1] * Sj[3 + c] + b[NB * r + 2] * Sj[6 + c]);
            if (NB == 6) v += b[NB * r + 3 + c];
            X[6 * r + 3 + c] = v;
        }
    }
    // C += P_i^T X: rows 0..2 += X[0:3, :];  rows 3..5 += Si X[0:3, :] (+ X[3:6, :] for nodes)
#pragma unroll
    for (int c = 0; c < 6; ++c) {
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            C[6 * r + c] += X[6 * r + c];
            double v = Si[3 * r] * X[c] + Si[3 * r + 1] * X[6 + c] + Si[3 * r + 2] * X[12 + c];
            if (NB == 6) v += X[6 * (3 + r) + c];
            C[6 * (3 + r) + c] += v;
        }
    }
}

// Galerkin block values of level l, one warp per block: the contributions (lane-strided, then a
// shuffle tree) of the finer level's blocks.  Level 1 reads the system's blocks: the elastic
// ones from the sliced-ELL values (sell position of each BSR block in bsr2sell), the contact
// ones from the contact block values; Dirichlet vertices contribute nothing.
template <int NB, bool SELL>
__global__ void __launch_bounds__(MG_THREADS) k_mg_galerkin(int nnz, const int* __restrict__ cp, const int* __restrict__ src,
                                                          const int* __restrict__ srow, const int* __restrict__ scol,
                                                          const double* __restrict__ fval, const int* __restrict__ bsr2sell,
                                                          const unsigned char* __restrict__ fixed, const double* __restrict__ d,
                                                          double* __restrict__ out) {
    const int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (b >= nnz) return;
    double C[36];
#pragma unroll
    for (int e = 0; e < 36; ++e) C[e] = 0.0;
    for (int q = cp[b] + lane; q < cp[b + 1]; q += 32) {
        const int i = srow[q], j = scol[q];
        if (fixed && (fixed[i] || fixed[j])) continue;
        const double di[3] = {d[3 * (size_t)i], d[3 * (size_t)i + 1], d[3 * (size_t)i + 2]};
        const double dj[3] = {d[3 * (size_t)j], d[3 * (size_t)j + 1], d[3 * (size_t)j + 2]};
        if (SELL) {
            const int ps = bsr2sell[src[q]];
            gal_add<NB>(C, fval + (size_t)(ps >> 5) * 288 + (ps & 31), 32, di, dj);
        } else {
            gal_add<NB>(C, fval + (size_t)NB * NB * src[q], 1, di, dj);
        }
    }
#pragma unroll
    for (int e = 0; e < 36; ++e) {
        double v = C[e];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) out[36 * (size_t)b + e] = v;
    }
}

// Level 1 from the system's 3x3 blocks, in two passes (fewer registers per thread than one warp
// per coarse block, so far more contributions are in flight): every contribution's 6x6 product
// P_i^T A_ij P_j into terms [contribution][36] (zeros for Dirichlet vertices), then every coarse
// block sums its contiguous run of terms in list order, one lane per entry.
template <bool SELL>
__global__ void __launch_bounds__(MG_THREADS) k_mg_gal_terms(int nq, const int* __restrict__ src, const int* __restrict__ srow,
                                                             const int* __restrict__ scol, const double* __restrict__ fval,
                                                             const int* __restrict__ bsr2sell, const unsigned char* __restrict__ fixed,
                                                             const double* __restrict__ d, double* __restrict__ terms) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    double C[36];
#pragma unroll
    for (int e = 0; e < 36; ++e) C[e] = 0.0;
    const int i = srow[q], j = scol[q];
    if (!fixed[i] && !fixed[j]) {
        const double di[3] = {d[3 * (size_t)i], d[3 * (size_t)i + 1], d[3 * (size_t)i + 2]};
        const double dj[3] = {d[3 * (size_t)j], d[3 * (size_t)j + 1], d[3 * (size_t)j + 2]};
        if (SELL) {
            const int ps = bsr2sell[src[q]];
            gal_add<3>(C, fval + (size_t)(ps >> 5) * 288 + (ps & 31), 32, di, dj);
        } else {
            gal_add<3>(C, fval + 9 * (size_t)src[q], 1, di, dj);
        }
    }
#pragma unroll
    for (int e = 0; e < 36; ++e) terms[36 * (size_t)q + e] = C[e];
}

__global__ void __launch_bounds__(MG_THREADS) k_mg_gal_sum(int nnz, const int* __restrict__ cp, const double* __restrict__ terms,
                                                           double* __restrict__ out) {
    const int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (b >= nnz) return;
    for (int e = lane; e < 36; e += 32) {
        double t = 0.0;
        for (int q = cp[b]; q < cp[b + 1]; ++q) t += terms[36 * (size_t)q + e];
        out[36 * (size_t)b + e] = t;
    }
}

// block-Jacobi inverse of every node of a level: the diagonal blocks of both patterns, shifted
// by 1e-10 of their largest diagonal entry (identity for a node whose modes are all inert)
__global__ void k_mg_inverse(int n, const int* __restrict__ srp, const int* __restrict__ sci, const double* __restrict__ sval,
                             const int* __restrict__ crp, const int* __restrict__ cci, const double* __restrict__ cval,
                             double* __restrict__ minv) {
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= n) return;
    double A[36];
#pragma unroll
    for (int e = 0; e < 36; ++e) A[e] = 0.0;
    for (int k = srp[I]; k < srp[I + 1]; ++k)
        if (sci[k] == I)
            for (int e = 0; e < 36; ++e) A[e] += sval[36 * (size_t)k + e];
    if (crp)
        for (int k = crp[I]; k < crp[I + 1]; ++k)
            if (cci[k] == I)
                for (int e = 0; e < 36; ++e) A[e] += cval[36 * (size_t)k + e];
    double mx = 0.0;
    for (int p = 0; p < 6; ++p) mx = fmax(mx, A[7 * p]);
    if (!(mx > 0.0)) {
        for (int e = 0; e < 36; ++e) A[e] = (e % 7 == 0) ? 1.0 : 0.0;
    } else {
        for (int p = 0; p < 6; ++p) A[7 * p] += 1e-10 * mx;
        // Gauss-Jordan without pivoting (symmetric positive definite)
        for (int k = 0; k < 6; ++k) {
            const double ip = 1.0 / A[7 * k];
            for (int j = 0; j < 6; ++j) A[6 * k + j] *= ip;
            A[7 * k] = ip;
            for (int i = 0; i < 6; ++i) {
                if (i == k) continue;
                const double f = A[6 * i + k];
                for (int j = 0; j < 6; ++j) A[6 * i + j] -= f * A[6 * k + j];
                A[6 * i + k] = -f * ip;
            }
        }
    }
    for (int e = 0; e < 36; ++e) minv[36 * (size_t)I + e] = A[e];
}

// the coarsest level's blocks into the dense matrix (row stride ld); add: the second pattern
__global__ void k_mg_dense_fill(int n, const int* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ val, int ld,
                                double* __restrict__ D, int add) {
    const int I = blockIdx.x;
    if (I >= n) return;
    for (int k = rp[I]; k < rp[I + 1]; ++k) {
        const int J = ci[k];
        for (int e = threadIdx.x; e < 36; e += blockDim.x) {
            double* p = D + (size_t)(6 * I + e / 6) * ld + 6 * J + e % 6;
            *p = add ? *p + val[36 * (size_t)k + e] : val[36 * (size_t)k + e];
        }
    }
}

__global__ void k_mg_regularize(int ld, double* __restrict__ D) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ld) return;
    double* dk = D + (size_t)k * ld + k;
    *dk = *dk > 0.0 ? *dk * (1.0 + 1e-12) : 1.0;
}

// ---------------------------------------------------------------- power iteration
// deterministic start vector (free DOFs only) and its squared-norm partials
__global__ void __launch_bounds__(MG_THREADS) k_mg_pinit(int n_nodes, int bs, int st, const unsigned char* __restrict__ fixed,
                                                         double* __restrict__ v, double* __restrict__ part) {
    __shared__ double sh[MG_THREADS];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double s = 0.0;
    if (i < n_nodes) {
        for (int k = 0; k < bs; ++k) {
            const unsigned long long h = ((unsigned long long)(i * bs + k) * 2654435761ull) % 1000ull;
            const double val = (fixed && fixed[i]) ? 0.0 : (double)h / 1000.0 - 0.5;
            v[(size_t)st * i + k] = val;
            s += val * val;
        }
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = MG_THREADS / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// nrm[0] = sqrt(sum of part[0 .. nb)), fixed order (one block)
__global__ void k_mg_norm(int nb, const double* __restrict__ part, double* __restrict__ nrm) {
    __shared__ double sh[256];
    double s = 0.0;
    for (int k = threadIdx.x; k < nb; k += 256) s += part[k];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) nrm[0] = sqrt(sh[0]);
}

// level 0: vout = D^-1 A (vin / |vin|) on free vertices (stride 4)
__global__ void __launch_bounds__(MG_THREADS) k_mg_power0(PCGArgs a, const double* __restrict__ vin, const double* __restrict__ nrm,
                                                          double* __restrict__ vout, double* __restrict__ part) {
    __shared__ double sh[MG_THREADS];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double s = 0.0;
    if (i < a.nV) {
        double y[3] = {0.0, 0.0, 0.0};
        if (!a.fixed[i]) {
            row_apply<4>(a, i, vin, y[0], y[1], y[2]);
            const double sc = 1.0 / nrm[0];
            for (int k = 0; k < 3; ++k) y[k] *= sc;
        }
        for (int k = 0; k < 3; ++k) {
            const double o = a.minv[9 * (size_t)i + 3 * k] * y[0] + a.minv[9 * (size_t)i + 3 * k + 1] * y[1] + a.minv[9 * (size_t)i + 3 * k + 2] * y[2];
            vout[4 * (size_t)i + k] = o;
            s += o * o;
        }
        vout[4 * (size_t)i + 3] = 0.0;
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = MG_THREADS / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// y_p = (A v)_{I,p} at level >= 1 (both patterns), one warp per node: lane = 6 kk + p (kk < 5;
// lanes 30, 31 idle) takes output p of the row's blocks kk, kk + 5, ...; the five partial sums of
// each output are added in a fixed order.  Every lane returns y for its p = lane % 6.
__device__ __forceinline__ double mg_row_warp(const MgLev& L, int I, const double* __restrict__ v, int lane) {
    const int kk = lane / 6, p = lane % 6;
    double y = 0.0;
    if (lane < 30) {
        for (int pass = 0; pass < 2; ++pass) {
            const int* rp = pass ? L.c_rp : L.s_rp;
            if (!rp) continue;
            const int* ci = pass ? L.c_ci : L.s_ci;
            const double* val = pass ? L.c_val : L.s_val;
            for (int k = rp[I] + kk; k < rp[I + 1]; k += 5) {
                const double* B = val + 36 * (size_t)k + 6 * p;
                const double* x = v + 6 * (size_t)ci[k];
#pragma unroll
                for (int q = 0; q < 6; ++q) y = fma(__ldg(B + q), x[q], y);
            }
        }
    }
    const unsigned full = 0xffffffffu;
    const double y1 = __shfl_sync(full, y, p + 6), y2 = __shfl_sync(full, y, p + 12), y3 = __shfl_sync(full, y, p + 18),
                 y4 = __shfl_sync(full, y, p + 24);
    const double y0 = __shfl_sync(full, y, p);
    return ((y0 + y1) + (y2 + y3)) + y4;
}

// z_p = w sum_q M_pq s_q for the lane's p, with s_q held by lane q (q < 6)
__device__ __forceinline__ double mg_minv_warp(const double* __restrict__ M, double s, double w, int lane) {
    const int p = lane % 6;
    double z = 0.0;
#pragma unroll
    for (int q = 0; q < 6; ++q) z = fma(__ldg(M + 6 * p + q), __shfl_sync(0xffffffffu, s, q), z);
    return w * z;
}

// level l >= 1: vout = D_l^-1 A_l (vin / |vin|), one warp per node
__global__ void __launch_bounds__(MG_THREADS) k_mg_powerl(MgLev L, const double* __restrict__ vin, const double* __restrict__ nrm,
                                                          double* __restrict__ vout, double* __restrict__ part) {
    __shared__ double sh[MG_THREADS / 32];
    const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    double s = 0.0;
    if (I < L.n) {
        const double y = mg_row_warp(L, I, vin, lane) * (1.0 / nrm[0]);
        const double z = mg_minv_warp(L.minv + 36 * (size_t)I, y, 1.0, lane);
        if (lane < 6) {
            vout[6 * (size_t)I + lane] = z;
            s = z * z;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < MG_THREADS / 32; ++w) t += sh[w];
        part[blockIdx.x] = t;
    }
}

// w_l = 4 / (3 * 1.05 * rho_l)
__global__ void k_mg_omega(const double* __restrict__ rho, double* __restrict__ omega) {
    if (threadIdx.x == 0) omega[0] = rho[0] > 0.0 ? 4.0 / (3.0 * 1.05 * rho[0]) : 1.0;
}

// ---------------------------------------------------------------- V-cycle kernels
// z0 = w0 u  (u = D^-1 r from the PCG's start kernel)
__global__ void k_mg_scale0(PCGArgs a, double* __restrict__ z0, const double* __restrict__ omega) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nV) return;
    const double w = omega[0];
    for (int k = 0; k < 3; ++k) {
        const double v = w * a.u[4 * (size_t)i + k];
        z0[4 * (size_t)i + k] = v;
        if (a.mg_z0f) a.mg_z0f[4 * (size_t)i + k] = (float)v;
    }
    z0[4 * (size_t)i + 3] = 0.0;
    if (a.mg_z0f) a.mg_z0f[4 * (size_t)i + 3] = 0.f;
}

// FP32 copies of the level-0 values (elastic sliced ELL, contact blocks) for the smoothing products
__global__ void k_mg_to_f32(long long n, const double* __restrict__ in, float* __restrict__ out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

// t0 = r - A z0 (free vertices; Dirichlet vertices 0)
__global__ void __launch_bounds__(PCG_THREADS) k_mg_res0(PCGArgs a, const double* __restrict__ z0, double* __restrict__ t0) {
    if (*(volatile int*)&a.flag[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nV) return;
    double y0 = 0.0, y1 = 0.0, y2 = 0.0;
    const bool fx = a.fixed[i];
    if (!fx) row_apply<4>(a, i, z0, y0, y1, y2);
    t0[3 * (size_t)i] = fx ? 0.0 : a.r[3 * (size_t)i] - y0;
    t0[3 * (size_t)i + 1] = fx ? 0.0 : a.r[3 * (size_t)i + 1] - y1;
    t0[3 * (size_t)i + 2] = fx ? 0.0 : a.r[3 * (size_t)i + 2] - y2;
}

// t0 = r - A z0 with FP32 products (values and z0 as FP32, FP32 sums); the residual in FP64
__global__ void __launch_bounds__(PCG_THREADS) k_mg_res0_f32(PCGArgs a, const float* __restrict__ v32, const float* __restrict__ c32,
                                                             const float4* __restrict__ z0f, double* __restrict__ t0) {
    if (*(volatile int*)&a.flag[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nV) return;
    float y0 = 0.f, y1 = 0.f, y2 = 0.f;
    const bool fx = a.fixed[i];
    if (!fx) row_apply_f32(a, v32, c32, i, z0f, y0, y1, y2);
    t0[3 * (size_t)i] = fx ? 0.0 : a.r[3 * (size_t)i] - (double)y0;
    t0[3 * (size_t)i + 1] = fx ? 0.0 : a.r[3 * (size_t)i + 1] - (double)y1;
    t0[3 * (size_t)i + 2] = fx ? 0.0 : a.r[3 * (size_t)i + 2] - (double)y2;
}

// restriction of the finer residual t (vertices: stride 3, Dirichlet vertices skipped; nodes:
// stride 6) into level L, one warp per node: lanes take members lane, lane + 32, ... and the six
// sums are added by a fixed shuffle tree; below the coarsest also z = w D^-1 g
__global__ void __launch_bounds__(MG_THREADS) k_mg_restrict(PCGArgs a, MgLev L, const double* __restrict__ t, int from_vertices,
                                                            const double* __restrict__ omega, int coarsest) {
    if (*(volatile int*)&a.flag[0]) return;
    const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (I >= L.n) return;
    double g[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    const int st = from_vertices ? 3 : 6;
    for (int k = L.mem_ptr[I] + lane; k < L.mem_ptr[I + 1]; k += 32) {
        const int i = L.mem[k];
        if (from_vertices && a.fixed[i]) continue;
        const double t0 = t[(size_t)st * i], t1 = t[(size_t)st * i + 1], t2 = t[(size_t)st * i + 2];
        const double d0 = L.d[3 * (size_t)i], d1 = L.d[3 * (size_t)i + 1], d2 = L.d[3 * (size_t)i + 2];
        g[0] += t0;
        g[1] += t1;
        g[2] += t2;
        g[3] += d1 * t2 - d2 * t1;
        g[4] += d2 * t0 - d0 * t2;
        g[5] += d0 * t1 - d1 * t0;
        if (!from_vertices) {
            g[3] += t[6 * (size_t)i + 3];
            g[4] += t[6 * (size_t)i + 4];
            g[5] += t[6 * (size_t)i + 5];
        }
    }
#pragma unroll
    for (int q = 0; q < 6; ++q) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) g[q] += __shfl_down_sync(0xffffffffu, g[q], o);
        g[q] = __shfl_sync(0xffffffffu, g[q], 0);
    }
    const int p = lane % 6;
    double gp = g[0];
#pragma unroll
    for (int q = 1; q < 6; ++q)
        if (p == q) gp = g[q];
    if (lane < 6) L.g[6 * (size_t)I + lane] = gp;
    if (!coarsest) {
        const double z = mg_minv_warp(L.minv + 36 * (size_t)I, gp, omega[0], lane);
        if (lane < 6) L.z[6 * (size_t)I + lane] = z;
    }
}

// level >= 1, one warp per node: post = 0: t = g - A z;  post = 1: z2 = z + w D^-1 (g - A z)
__global__ void __launch_bounds__(MG_THREADS) k_mg_smooth(PCGArgs a, MgLev L, const double* __restrict__ omega, int post) {
    if (*(volatile int*)&a.flag[0]) return;
    const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (I >= L.n) return;
    const int p = lane % 6;
    const double r = L.g[6 * (size_t)I + p] - mg_row_warp(L, I, L.z, lane);
    if (!post) {
        if (lane < 6) L.t[6 * (size_t)I + lane] = r;
        return;
    }
    const double z = mg_minv_warp(L.minv + 36 * (size_t)I, r, omega[0], lane);
    if (lane < 6) L.z2[6 * (size_t)I + lane] = L.z[6 * (size_t)I + lane] + z;
}

// coarsest: z = D^-1 g (dense, row stride ld), one warp per row, fixed-order lane sums and
// shuffle tree
__global__ void __launch_bounds__(MG_THREADS) k_mg_coarsest(PCGArgs a, MgLev L, const double* __restrict__ D, int n, int ld) {
    if (*(volatile int*)&a.flag[0]) return;
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (row >= n) return;
    const double* Dr = D + (size_t)row * ld;
    double t = 0.0;
    for (int j = lane; j < n; j += 32) t += __ldg(Dr + j) * L.g[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (lane == 0) L.z[row] = t;
}

// prolongation from level L into its finer level: zf += P Y (Y: the coarsest's z, else z2);
// into vertices (zf stride 4, Dirichlet vertices skipped) or into nodes (stride 6)
__global__ void __launch_bounds__(MG_THREADS) k_mg_prolong(PCGArgs a, MgLev L, const double* __restrict__ Y0, double* __restrict__ zf,
                                                           int nf, int to_vertices) {
    if (*(volatile int*)&a.flag[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf) return;
    if (to_vertices && a.fixed[i]) return;
    const double* Y = Y0 + 6 * (size_t)L.agg_of[i];
    const double d0 = L.d[3 * (size_t)i], d1 = L.d[3 * (size_t)i + 1], d2 = L.d[3 * (size_t)i + 2];
    const double u0 = Y[0] + (Y[4] * d2 - Y[5] * d1), u1 = Y[1] + (Y[5] * d0 - Y[3] * d2), u2 = Y[2] + (Y[3] * d1 - Y[4] * d0);
    if (to_vertices) {
        const double z0 = zf[4 * (size_t)i] + u0, z1 = zf[4 * (size_t)i + 1] + u1, z2 = zf[4 * (size_t)i + 2] + u2;
        zf[4 * (size_t)i] = z0;
        zf[4 * (size_t)i + 1] = z1;
        zf[4 * (size_t)i + 2] = z2;
        if (a.mg_z0f) {
            a.mg_z0f[4 * (size_t)i] = (float)z0;
            a.mg_z0f[4 * (size_t)i + 1] = (float)z1;
            a.mg_z0f[4 * (size_t)i + 2] = (float)z2;
        }
    } else {
        double* z = zf + 6 * (size_t)i;
        z[0] += u0;
        z[1] += u1;
        z[2] += u2;
        z[3] += Y[3];
        z[4] += Y[4];
        z[5] += Y[5];
    }
}

// level 0 post-smoothing into the PCG's u: u = z0 + w0 D^-1 (r - A z0); Dirichlet vertices 0
__global__ void __launch_bounds__(PCG_THREADS) k_mg_post0(PCGArgs a, const double* __restrict__ z0, const double* __restrict__ omega) {
    if (*(volatile int*)&a.flag[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nV) return;
    if (a.fixed[i]) {
        a.u[4 * (size_t)i] = a.u[4 * (size_t)i + 1] = a.u[4 * (size_t)i + 2] = 0.0;
        return;
    }
    double y0, y1, y2;
    row_apply<4>(a, i, z0, y0, y1, y2);
    const double s0 = a.r[3 * (size_t)i] - y0, s1 = a.r[3 * (size_t)i + 1] - y1, s2 = a.r[3 * (size_t)i + 2] - y2;
    const double* M = a.minv + 9 * (size_t)i;
    const double w = omega[0];
    a.u[4 * (size_t)i] = z0[4 * (size_t)i] + w * (M[0] * s0 + M[1] * s1 + M[2] * s2);
    a.u[4 * (size_t)i + 1] = z0[4 * (size_t)i + 1] + w * (M[3] * s0 + M[4] * s1 + M[5] * s2);
    a.u[4 * (size_t)i + 2] = z0[4 * (size_t)i + 2] + w * (M[6] * s0 + M[7] * s1 + M[8] * s2);
}

// the same with FP32 products
__global__ void __launch_bounds__(PCG_THREADS) k_mg_post0_f32(PCGArgs a, const float* __restrict__ v32, const float* __restrict__ c32,
                                                              const float4* __restrict__ z0f, const double* __restrict__ z0,
                                                              const double* __restrict__ omega) {
    if (*(volatile int*)&a.flag[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nV) return;
    if (a.fixed[i]) {
        a.u[4 * (size_t)i] = a.u[4 * (size_t)i + 1] = a.u[4 * (size_t)i + 2] = 0.0;
        return;
    }
    float y0, y1, y2;
    row_apply_f32(a, v32, c32, i, z0f, y0, y1, y2);
    const double s0 = a.r[3 * (size_t)i] - (double)y0, s1 = a.r[3 * (size_t)i + 1] - (double)y1, s2 = a.r[3 * (size_t)i + 2] - (double)y2;
    const double* M = a.minv + 9 * (size_t)i;
    const double w = omega[0];
    a.u[4 * (size_t)i] = z0[4 * (size_t)i] + w * (M[0] * s0 + M[1] * s1 + M[2] * s2);
    a.u[4 * (size_t)i + 1] = z0[4 * (size_t)i + 1] + w * (M[3] * s0 + M[4] * s1 + M[5] * s2);
    a.u[4 * (size_t)i + 2] = z0[4 * (size_t)i + 2] + w * (M[6] * s0 + M[7] * s1 + M[8] * s2);
}

// ---------------------------------------------------------------- host side
static MgState* state(fipc_ctx* c) { return reinterpret_cast<MgState*>(c->mg); }

// the hierarchy of the context's static pattern (h: aggregation cell; <= 0: the hash cell)
void pcg_graph_reset(fipc_ctx* c);

int mg_setup(fipc_ctx* c, double h) {
    pcg_graph_reset(c);
    if (c->mg) {
        delete state(c);
        c->mg = nullptr;
    }
    c->mg_levels = 0;
    if (c->n_scenes > 1 || c->nV < MG_MIN_VERTICES) return FIPC_OK;
    const int nV = c->nV;
    std::vector<int> rp(nV + 1), ci(c->nnzb);
    std::vector<double> x0(3ll * nV);
    if (cudaMemcpy(rp.data(), c->row_ptr, 4ll * (nV + 1), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(ci.data(), c->col_idx, 4ll * c->nnzb, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(x0.data(), c->x0, 24ll * nV, cudaMemcpyDeviceToHost) != cudaSuccess)
        return FIPC_ERR_CUDA;
    if (!(h > 0.0)) h = c->hash_inv_dx > 0.0 ? 1.0 / c->hash_inv_dx : 1.0 / c->inv_dx;
    MgState* M = new MgState();
    mg_build(nV, x0.data(), rp.data(), ci.data(), h, M->plan);
    if (M->plan.levels < 2) {
        delete M;
        return FIPC_OK;
    }
    const int NL = M->plan.levels;
    M->B.resize(NL);
    cudaStream_t s = 0;
    int st = FIPC_OK;
    for (int l = 1; l < NL && st == FIPC_OK; ++l) {
        const MgLevelPlan& p = M->plan.L[l];
        MgLevelBufs& b = M->B[l];
        st |= upload_vec(b.mem_ptr, p.mem_ptr, s);
        st |= upload_vec(b.mem, p.mem, s);
        st |= upload_vec(b.agg_of, p.agg_of, s);
        if (l == 1) st |= upload_vec(b.rot, p.rot, s);
        st |= upload_vec(b.s_rp, p.S.rp, s);
        st |= upload_vec(b.s_ci, p.S.ci, s);
        st |= upload_vec(b.s_cp, p.S.con_ptr, s);
        st |= upload_vec(b.s_src, p.S.src, s);
        st |= upload_vec(b.s_row, p.S.src_row, s);
        st |= upload_vec(b.s_col, p.S.src_col, s);
        const size_t nf = l == 1 ? (size_t)nV : (size_t)M->plan.L[l - 1].n;
        if (b.s_val.ensure(288ull * (p.S.nnz() + 1)) || b.minv.ensure(288ull * p.n) || b.cent.ensure(24ull * p.n) || b.d.ensure(24ull * nf) ||
            b.g.ensure(48ull * p.n) || b.z.ensure(48ull * p.n) || b.z2.ensure(48ull * p.n) || b.t.ensure(48ull * p.n) ||
            b.pv0.ensure(48ull * p.n) || b.pv1.ensure(48ull * p.n) || b.part.ensure(8ull * (nblk_m(32ll * p.n, MG_THREADS) + 1)) ||
            b.nrm.ensure(8ull * (MG_POWER_ITERS + 2)))
            st = FIPC_ERR_CUDA;
    }
    MgLevelBufs& b0 = M->B[0];
    const int nb0 = nblk_m(nV, MG_THREADS);
    if (st == FIPC_OK && (M->t0.ensure(24ull * nV) || M->z0.ensure(32ull * nV) || b0.pv0.ensure(32ull * nV) || b0.pv1.ensure(32ull * nV) ||
                          b0.part.ensure(8ull * (nb0 + 1)) || b0.nrm.ensure(8ull * (MG_POWER_ITERS + 2)) || M->omega.ensure(8ull * NL)))
        st = FIPC_ERR_CUDA;
    const int nc = M->plan.L[NL - 1].n;
    M->n_dense = 6 * nc;
    M->ld_dense = ((M->n_dense + MG_GJ_B - 1) / MG_GJ_B) * MG_GJ_B;
    if (st == FIPC_OK && (M->dense.ensure(8ull * M->ld_dense * M->ld_dense) ||
                          M->gj_buf.ensure(8ull * (MG_GJ_B * MG_GJ_B + 2ull * M->ld_dense * MG_GJ_B))))
        st = FIPC_ERR_CUDA;
    if (st == FIPC_OK && cudaDeviceSynchronize() != cudaSuccess) st = FIPC_ERR_CUDA;
    if (st != FIPC_OK) {
        delete M;
        return st;
    }
    c->mg = M;
    c->mg_levels = NL;
    // offsets from the rest shape until the next assembly sets them at its positions (any
    // centre spans the same rigid-body modes)
    st = mg_offsets(c, c->x0, 0);
    if (st == FIPC_OK && cudaDeviceSynchronize() != cudaSuccess) st = FIPC_ERR_CUDA;
    return st;
}

void mg_free(fipc_ctx* c) {
    if (c->mg) pcg_graph_reset(c);
    if (c->mg) delete state(c);
    c->mg = nullptr;
    c->mg_levels = 0;
}

// centroids and offsets of every level at the positions x (called by the assembly)
int mg_offsets(fipc_ctx* c, const double* x, cudaStream_t s) {
    MgState* M = state(c);
    if (!M) return FIPC_OK;
    for (int l = 1; l < M->plan.levels; ++l) {
        const int n = M->plan.L[l].n;
        const double* pos = l == 1 ? x : M->B[l - 1].cent.as<double>();
        k_mg_centroid<<<nblk_m(n, MG_THREADS), MG_THREADS, 0, s>>>(n, M->B[l].mem_ptr.as<int>(), M->B[l].mem.as<int>(), pos,
                                                                    l == 1 ? M->B[l].rot.as<unsigned char>() : nullptr,
                                                                    M->B[l].cent.as<double>(), M->B[l].d.as<double>());
        FIPC_LAUNCHED();
    }
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

// per-level contact patterns of the current system (host), the Galerkin products, block
// inverses and the dense coarsest inverse; fills a's multigrid fields
int mg_prepare(fipc_ctx* c, const unsigned char* fixed, PCGArgs& a, cudaStream_t s) {
    MgState* M = state(c);
    a.mg = nullptr;
    a.mg_z0 = nullptr;
    a.mg_omega = nullptr;
    a.mg_z0f = nullptr;
    if (!M) return FIPC_OK;
    const int NL = M->plan.levels, nV = c->nV;
    // contact patterns of every level
    if (c->c_nnzb > 0) {
        std::vector<int> crp(nV + 1), cci(c->c_nnzb);
        FIPC_CUDA(cudaMemcpyAsync(crp.data(), c->c_rowptr.p, 4ll * (nV + 1), cudaMemcpyDeviceToHost, s));
        FIPC_CUDA(cudaMemcpyAsync(cci.data(), c->c_col.p, 4ll * c->c_nnzb, cudaMemcpyDeviceToHost, s));
        FIPC_CUDA(cudaStreamSynchronize(s));
        mg_contact(M->plan, nV, crp.data(), cci.data());
        M->contact_empty = false;
        for (int l = 1; l < NL; ++l) {
            const MgPattern& C = M->plan.L[l].C;
            MgLevelBufs& b = M->B[l];
            if (C.nnz() == 0) continue;
            if (upload_vec(b.c_rp, C.rp, s) || upload_vec(b.c_ci, C.ci, s) || upload_vec(b.c_cp, C.con_ptr, s) ||
                upload_vec(b.c_src, C.src, s) || upload_vec(b.c_row, C.src_row, s) || upload_vec(b.c_col, C.src_col, s) ||
                b.c_val.ensure(288ull * C.nnz()))
                return FIPC_ERR_CUDA;
        }
    } else if (!M->contact_empty) {
        mg_contact(M->plan, nV, nullptr, nullptr);
        M->contact_empty = true;
    }
    // Galerkin products, level by level
    for (int l = 1; l < NL; ++l) {
        const MgLevelPlan& p = M->plan.L[l];
        MgLevelBufs& b = M->B[l];
        const double* d = b.d.as<double>();
        const int ns = p.S.nnz(), ncn = p.C.nnz();
        if (l == 1) {
            const int nqs = (int)p.S.src.size(), nqc = (int)p.C.src.size();
            if (M->terms.ensure(288ull * (nqs > nqc ? nqs : nqc) + 8)) return FIPC_ERR_CUDA;
            double* terms = M->terms.as<double>();
            if (ns) {
                k_mg_gal_terms<true><<<nblk_m(nqs, MG_THREADS), MG_THREADS, 0, s>>>(
                    nqs, b.s_src.as<int>(), b.s_row.as<int>(), b.s_col.as<int>(), c->sell_val, c->bsr2sell, fixed, d, terms);
                k_mg_gal_sum<<<nblk_m(32ll * ns, MG_THREADS), MG_THREADS, 0, s>>>(ns, b.s_cp.as<int>(), terms, b.s_val.as<double>());
                g_launches.fetch_add(1, std::memory_order_relaxed);
            }
            if (ncn) {
                k_mg_gal_terms<false><<<nblk_m(nqc, MG_THREADS), MG_THREADS, 0, s>>>(
                    nqc, b.c_src.as<int>(), b.c_row.as<int>(), b.c_col.as<int>(), c->c_val.as<double>(), nullptr, fixed, d, terms);
                k_mg_gal_sum<<<nblk_m(32ll * ncn, MG_THREADS), MG_THREADS, 0, s>>>(ncn, b.c_cp.as<int>(), terms, b.c_val.as<double>());
                g_launches.fetch_add(1, std::memory_order_relaxed);
            }
        } else {
            const MgLevelBufs& f = M->B[l - 1];
            if (ns)
                k_mg_galerkin<6, false><<<nblk_m(32ll * ns, MG_THREADS), MG_THREADS, 0, s>>>(
                    ns, b.s_cp.as<int>(), b.s_src.as<int>(), b.s_row.as<int>(), b.s_col.as<int>(), f.s_val.as<double>(), nullptr,
                    nullptr, d, b.s_val.as<double>());
            if (ncn)
                k_mg_galerkin<6, false><<<nblk_m(32ll * ncn, MG_THREADS), MG_THREADS, 0, s>>>(
                    ncn, b.c_cp.as<int>(), b.c_src.as<int>(), b.c_row.as<int>(), b.c_col.as<int>(), f.c_val.as<double>(), nullptr,
                    nullptr, d, b.c_val.as<double>());
        }
        g_launches.fetch_add((ns ? 1 : 0) + (ncn ? 1 : 0), std::memory_order_relaxed);
        if (l < NL - 1) {
            k_mg_inverse<<<nblk_m(p.n, MG_THREADS), MG_THREADS, 0, s>>>(p.n, b.s_rp.as<int>(), b.s_ci.as<int>(), b.s_val.as<double>(),
                                                                        ncn ? b.c_rp.as<int>() : nullptr, b.c_ci.as<int>(),
                                                                        b.c_val.as<double>(), b.minv.as<double>());
            FIPC_LAUNCHED();
        }
    }
    // the coarsest level, dense and inverted (padding rows: identity)
    {
        const MgLevelPlan& p = M->plan.L[NL - 1];
        MgLevelBufs& b = M->B[NL - 1];
        const int ld = M->ld_dense;
        double* D = M->dense.as<double>();
        FIPC_CUDA(cudaMemsetAsync(D, 0, 8ull * ld * ld, s));
        k_mg_dense_fill<<<p.n, 64, 0, s>>>(p.n, b.s_rp.as<int>(), b.s_ci.as<int>(), b.s_val.as<double>(), ld, D, 0);
        FIPC_LAUNCHED();
        if (p.C.nnz()) {
            k_mg_dense_fill<<<p.n, 64, 0, s>>>(p.n, b.c_rp.as<int>(), b.c_ci.as<int>(), b.c_val.as<double>(), ld, D, 1);
            FIPC_LAUNCHED();
        }
        k_mg_regularize<<<nblk_m(ld, 128), 128, 0, s>>>(ld, D);
        FIPC_LAUNCHED();
        int st = cs_gauss_jordan(ld, D, M->gj_buf.as<double>(), s);
        if (st) return st;
    }
    // kernel arguments
    MgArgs& m = M->args;
    m = MgArgs{};
    m.levels = NL;
    m.z0 = M->z0.as<double>();
    m.t0 = M->t0.as<double>();
    m.omega = M->omega.as<double>();
    m.dense = M->dense.as<double>();
    m.n_dense = M->n_dense;
    m.ld_dense = M->ld_dense;
    for (int l = 1; l < NL; ++l) {
        const MgLevelPlan& p = M->plan.L[l];
        MgLevelBufs& b = M->B[l];
        MgLev& L = m.L[l];
        L.n = p.n;
        L.mem_ptr = b.mem_ptr.as<int>();
        L.mem = b.mem.as<int>();
        L.agg_of = b.agg_of.as<int>();
        L.d = b.d.as<double>();
        L.s_rp = b.s_rp.as<int>();
        L.s_ci = b.s_ci.as<int>();
        L.s_val = b.s_val.as<double>();
        const bool hc = p.C.nnz() > 0;
        L.c_rp = hc ? b.c_rp.as<int>() : nullptr;
        L.c_ci = hc ? b.c_ci.as<int>() : nullptr;
        L.c_val = hc ? b.c_val.as<double>() : nullptr;
        L.minv = b.minv.as<double>();
        L.g = b.g.as<double>();
        L.z = b.z.as<double>();
        L.z2 = b.z2.as<double>();
        L.t = b.t.as<double>();
    }
    M->fp32 = c->mg_fp32 != 0;
    if (M->fp32) {
        const long long ne = 288ll * c->n_slots, nc = 9ll * c->c_nnzb;
        if (M->v32.ensure(4ull * (ne + nc) + 64) || M->z0f.ensure(16ull * nV + 64)) return FIPC_ERR_CUDA;
        float* v32 = M->v32.as<float>();
        k_mg_to_f32<<<1216, 256, 0, s>>>(ne, c->sell_val, v32);
        FIPC_LAUNCHED();
        if (nc) {
            k_mg_to_f32<<<nblk_m(nc, 256), 256, 0, s>>>(nc, c->c_val.as<double>(), v32 + ne);
            FIPC_LAUNCHED();
        }
        m.v32 = v32;
        m.c32 = v32 + ne;
        m.z0f = M->z0f.as<float>();
    }
    a.mg = &M->args;
    a.mg_z0 = m.z0;
    a.mg_omega = m.omega;
    a.mg_z0f = m.z0f;
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

// smoother weights (power iteration: level 0 needs the block-Jacobi inverse of the PCG's start
// kernel), then z0 = w0 D^-1 r0 and the first V-cycle
int mg_start(fipc_ctx* c, const PCGArgs& a, cudaStream_t s) {
    MgState* M = state(c);
    const MgArgs& m = M->args;
    const int NL = M->plan.levels, nV = c->nV;
    for (int l = 0; l < NL - 1; ++l) {
        MgLevelBufs& b = M->B[l];
        const int n = l == 0 ? nV : M->plan.L[l].n;
        const int nb = nblk_m(n, MG_THREADS), nbw = nblk_m(32ll * n, MG_THREADS);
        double* v0 = b.pv0.as<double>();
        double* v1 = b.pv1.as<double>();
        double* nrm = b.nrm.as<double>();
        // a fixed start vector every solve, so that a solve depends on its system alone
        const int iters = MG_POWER_ITERS;
        k_mg_pinit<<<nb, MG_THREADS, 0, s>>>(n, l == 0 ? 3 : 6, l == 0 ? 4 : 6, l == 0 ? a.fixed : nullptr, v0, b.part.as<double>());
        k_mg_norm<<<1, 256, 0, s>>>(nb, b.part.as<double>(), nrm);
        g_launches.fetch_add(2, std::memory_order_relaxed);
        for (int k = 0; k < iters; ++k) {
            if (l == 0)
                k_mg_power0<<<nb, MG_THREADS, 0, s>>>(a, v0, nrm + k, v1, b.part.as<double>());
            else
                k_mg_powerl<<<nbw, MG_THREADS, 0, s>>>(m.L[l], v0, nrm + k, v1, b.part.as<double>());
            k_mg_norm<<<1, 256, 0, s>>>(l == 0 ? nb : nbw, b.part.as<double>(), nrm + k + 1);
            std::swap(v0, v1);
        }
        k_mg_omega<<<1, 32, 0, s>>>(nrm + iters, M->omega.as<double>() + l);
        g_launches.fetch_add(1 + 2 * iters, std::memory_order_relaxed);
    }
    k_mg_scale0<<<nblk_m(nV, MG_THREADS), MG_THREADS, 0, s>>>(a, m.z0, m.omega);
    FIPC_LAUNCHED();
    mg_vcycle(c, a, s);
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

// one V-cycle on the residual a.r, from z0 = w0 D^-1 r (written by the PCG's update kernel) to u
void mg_vcycle(const fipc_ctx* c, const PCGArgs& a, cudaStream_t s) {
    const MgState* M = reinterpret_cast<const MgState*>(c->mg);
    const MgArgs& m = M->args;
    const int NL = m.levels, nV = c->nV;
    const int nb0 = nblk_m(nV, PCG_THREADS);
    if (m.z0f) k_mg_res0_f32<<<nb0, PCG_THREADS, 0, s>>>(a, m.v32, m.c32, reinterpret_cast<const float4*>(m.z0f), m.t0);
    else k_mg_res0<<<nb0, PCG_THREADS, 0, s>>>(a, m.z0, m.t0);
    for (int l = 1; l < NL; ++l) {
        const MgLev& L = m.L[l];
        k_mg_restrict<<<nblk_m(32ll * L.n, MG_THREADS), MG_THREADS, 0, s>>>(a, L, l == 1 ? m.t0 : m.L[l - 1].t, l == 1, m.omega + l,
                                                                            l == NL - 1);
        if (l < NL - 1) k_mg_smooth<<<nblk_m(32ll * L.n, MG_THREADS), MG_THREADS, 0, s>>>(a, L, m.omega + l, 0);
    }
    k_mg_coarsest<<<nblk_m(32ll * m.n_dense, MG_THREADS), MG_THREADS, 0, s>>>(a, m.L[NL - 1], m.dense, m.n_dense, m.ld_dense);
    for (int l = NL - 1; l >= 1; --l) {
        const MgLev& L = m.L[l];
        const int nf = l == 1 ? nV : m.L[l - 1].n;
        k_mg_prolong<<<nblk_m(nf, MG_THREADS), MG_THREADS, 0, s>>>(a, L, l == NL - 1 ? L.z : L.z2, l == 1 ? m.z0 : m.L[l - 1].z, nf,
                                                                    l == 1);
        if (l - 1 >= 1) k_mg_smooth<<<nblk_m(32ll * nf, MG_THREADS), MG_THREADS, 0, s>>>(a, m.L[l - 1], m.omega + (l - 1), 1);
    }
    if (m.z0f) k_mg_post0_f32<<<nb0, PCG_THREADS, 0, s>>>(a, m.v32, m.c32, reinterpret_cast<const float4*>(m.z0f), m.z0, m.omega);
    else k_mg_post0<<<nb0, PCG_THREADS, 0, s>>>(a, m.z0, m.omega);
    g_launches.fetch_add(mg_launches_per_cycle(NL), std::memory_order_relaxed);
}

// kernels of one V-cycle: residual, restrictions and smoothing down, coarsest, prolongations
// and smoothing up, level-0 post-smoothing
int mg_launches_per_cycle(int levels) { return 4 * levels - 3; }

}  // namespace fipc

extern "C" int fipc_ctx_set_multigrid_fp32(fipc_ctx* c, int on) {
    using namespace fipc;
    if (!c) return FIPC_ERR_ARGUMENT;
    c->mg_fp32 = on ? 1 : 0;
    pcg_graph_reset(c);
    return FIPC_OK;
}

extern "C" int fipc_ctx_multigrid(fipc_ctx* c, int* levels, int* nodes_h) {
    using namespace fipc;
    if (!c) return FIPC_ERR_ARGUMENT;
    if (levels) *levels = c->mg_levels;
    const MgState* M = reinterpret_cast<const MgState*>(c->mg);
    if (nodes_h)
        for (int l = 0; l < MG_MAX_LEVELS; ++l) nodes_h[l] = (M && l < M->plan.levels) ? M->plan.L[l].n : 0;
    return FIPC_OK;
}
