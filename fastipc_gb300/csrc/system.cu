// Newton system: assembly into 3x3 block-sparse rows and the PCG direction solve.  Replaces the triplet assembly of NEWTON_IPC.py:545-747 and the CHOLMOD solve of
// NEWTON_IPC.py:750-777.
//
// Assembly has no order-dependent atomics.  The elastic+inertia pattern is static: each
// upper block (i <= j) owns a precomputed, fixed-order list of (tet, local block, transposed)
// contributions; one thread sums its list and writes block (i,j) and its transpose (j,i).
// Contact blocks change every iteration: (row vertex, column vertex) keys of all 3x3 blocks
// of all constraint rows are radix-sorted (stable, so equal keys keep generation order) and
// each run is summed by one thread into a second block-sparse matrix.  The same runs on the
// diagonal carry the constraint gradients into the right-hand side.
//
// PCG: block-Jacobi preconditioner (inverse 3x3 diagonal blocks) plus, by default, the
// rigid-body coarse correction of coarse.cu; Dirichlet vertices removed by zero rows/columns
// (the reference's DBC_set_zeros + identity, NEWTON_IPC.py:756-772).  Per iteration an SpMV and
// an update kernel on a fixed grid (plus the two coarse kernels); dot products are per-block
// partials summed in a fixed order by the last block, so results are bitwise reproducible.
#include <algorithm>

#include <cub/cub.cuh>

#include <vector>
#include <cuda_runtime.h>

#include "ctx.cuh"
#include "pcg.cuh"
#include "profile.cuh"

namespace fipc {

// ---------------------------------------------------------------- elastic + inertia
__device__ __forceinline__ double* sell_block(double* val, int enc) {
    return val + (size_t)(enc >> 5) * 288 + (enc & 31);
}

// one thread per upper block: fixed-order sum of its contributions, written to (i,j) and
// transposed to (j,i) in the sliced-ELL value array (entry stride 32).  A contribution is
// (position of its 3x3 block in the tiled element-Hessian array / 9) << 1 | transposed.
__global__ void k_assemble_elastic(int n_upper, const int* __restrict__ cptr, const int* __restrict__ contrib,
                                   const int* __restrict__ spos, const int* __restrict__ tspos, const int* __restrict__ urow,
                                   const double* __restrict__ elem_H, const double* __restrict__ mass, double* __restrict__ val) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= n_upper) return;
    double s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = cptr[u]; k < cptr[u + 1]; ++k) {
        const int c = contrib[k];
        const double* H = elem_H + 9 * (size_t)(c >> 1);
        if (c & 1) {
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) s[i * 3 + j] += H[j * 3 + i];
        } else {
#pragma unroll
            for (int i = 0; i < 9; ++i) s[i] += H[i];
        }
    }
    const int p = spos[u], q = tspos[u];
    if (p == q) {
        const double m = mass[urow[u]];
        s[0] += m;
        s[4] += m;
        s[8] += m;
    }
    double* dp = sell_block(val, p);
#pragma unroll
    for (int i = 0; i < 9; ++i) dp[32 * i] = s[i];
    if (p != q) {
        double* dq = sell_block(val, q);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) dq[32 * (i * 3 + j)] = s[j * 3 + i];
    }
}

// sliced-ELL -> block-CSR order (export for tests)
__global__ void k_sell_to_bsr(int nnzb, const int* __restrict__ bsr2sell, const double* __restrict__ sval, double* __restrict__ bval) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nnzb) return;
    const double* src = sval + (size_t)(bsr2sell[k] >> 5) * 288 + (bsr2sell[k] & 31);
#pragma unroll
    for (int i = 0; i < 9; ++i) bval[9 * (size_t)k + i] = src[32 * i];
}

// rhs = -(m (x - xt) + sum of element gradients)   (NEWTON_IPC.py:558-567, 679-690)
__global__ void k_assemble_rhs(int nV, const int* __restrict__ vt_ptr, const int* __restrict__ vt_list,
                               const double* __restrict__ elem_g, const double* __restrict__ mass, const double* __restrict__ x,
                               const double* __restrict__ xt, double* __restrict__ rhs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nV) return;
    const double m = mass[i];
    double r0 = -m * (x[3 * i] - xt[3 * i]), r1 = -m * (x[3 * i + 1] - xt[3 * i + 1]), r2 = -m * (x[3 * i + 2] - xt[3 * i + 2]);
    for (int k = vt_ptr[i]; k < vt_ptr[i + 1]; ++k) {
        const int c = vt_list[k];   // tet * 4 + local vertex
        const double* g = elem_g + 12 * (size_t)(c >> 2) + 3 * (c & 3);
        r0 -= g[0];
        r1 -= g[1];
        r2 -= g[2];
    }
    rhs[3 * i] = r0;
    rhs[3 * i + 1] = r1;
    rhs[3 * i + 2] = r2;
}

// ---------------------------------------------------------------- contact blocks
// one thread per constraint row (global index over the concatenated lists)
__global__ void k_contact_keys(int n_rows, const int4* __restrict__ rows, TypeTable tt, unsigned long long* __restrict__ keys,
                               int* __restrict__ vals) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rows) return;
    int t = 0;
    while (t < N_TYPES - 1 && r >= tt.row0[t + 1]) ++t;
    const int nv = type_nverts(t);
    const int4 q = rows[r];
    const int id[4] = {q.x, q.y, q.z, q.w};
    long long o = tt.ent0[t] + (long long)(r - tt.row0[t]) * nv * nv;
    for (int v = 0; v < nv; ++v)
        for (int w = 0; w < nv; ++w) {
            keys[o] = ((unsigned long long)id[v] << 32) | (unsigned long long)id[w];
            vals[o] = r * 16 + v * 4 + w;
            ++o;
        }
}

// one thread per unique block: sum its run; diagonal runs also fold the gradients into rhs
__global__ void k_contact_reduce(int nu, const unsigned long long* __restrict__ ukeys, const int* __restrict__ ustart,
                                 const int* __restrict__ vals, const double* __restrict__ cH, const double* __restrict__ cg,
                                 double* __restrict__ cval, int* __restrict__ ccol, double* __restrict__ rhs) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nu) return;
    const unsigned long long key = ukeys[b];
    const int row = (int)(key >> 32), col = (int)(key & 0xffffffffu);
    double s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double gs[3] = {0, 0, 0};
    for (int k = ustart[b]; k < ustart[b + 1]; ++k) {
        const int e = vals[k];
        const int r = e >> 4, vw = e & 15;
        const double* H = cH + 144 * (size_t)r + 9 * vw;
#pragma unroll
        for (int i = 0; i < 9; ++i) s[i] += H[i];
        if (row == col) {
            const int v = vw >> 2;
            gs[0] += cg[12 * (size_t)r + 3 * v];
            gs[1] += cg[12 * (size_t)r + 3 * v + 1];
            gs[2] += cg[12 * (size_t)r + 3 * v + 2];
        }
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) cval[9 * (size_t)b + i] = s[i];
    ccol[b] = col;
    if (row == col) {
        rhs[3 * row] -= gs[0];
        rhs[3 * row + 1] -= gs[1];
        rhs[3 * row + 2] -= gs[2];
    }
}

__global__ void k_contact_rowptr(int nV, int nu, const unsigned long long* __restrict__ ukeys, int* __restrict__ rowptr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > nV) return;
    const unsigned long long key = (unsigned long long)i << 32;
    int lo = 0, hi = nu;
    while (lo < hi) {
        const int m = (lo + hi) >> 1;
        if (ukeys[m] < key) lo = m + 1;
        else hi = m;
    }
    rowptr[i] = lo;
}

// ---------------------------------------------------------------- PCG
// Chronopoulos-Gear form of preconditioned CG: per iteration one SpMV w = A u (u = M^-1 r,
// already formed) fused with the three dot products (r,u), (w,u), (r,r), and one vector update
//   p = u + beta p, s = w + beta s, x += alpha p, r -= alpha s, u = M^-1 r.
// Dot products: per-block partials; the last block to finish (atomic ticket) sums them in block
// order and derives alpha/beta, so the scalars are bitwise reproducible and need no launch.
// block sums of up to 3 values into part[c * nblk + block]; returns true in every thread of
// the last block to finish, which then reduces the partials with final_sums
template <int NV>
__device__ __forceinline__ bool block_partials(const PCGArgs& a, const double (&v)[NV]) {
    __shared__ double tot[NV];
    __shared__ bool last;
    block_sums<NV>(v, tot);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int c = 0; c < NV; ++c) a.part[c * gridDim.x + blockIdx.x] = tot[c];
        __threadfence();
        const int ticket = atomicAdd(&a.flag[2], 1);
        last = ticket == (int)gridDim.x - 1;
    }
    __syncthreads();
    return last;
}

// in the last block: out[c] = sum over blocks of part[c * nblk + b], every thread striding the
// blocks in a fixed order and a fixed shuffle/shared tree (bitwise reproducible)
template <int NV>
__device__ __forceinline__ void final_sums(const PCGArgs& a, double (&out)[NV]) {
    __shared__ double sh[NV][PCG_THREADS / 32];
    __threadfence();
    const int nb = gridDim.x, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        double t = 0.0;
        for (int b = threadIdx.x; b < nb; b += PCG_THREADS) t += *(volatile double*)&a.part[c * nb + b];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0) sh[c][wid] = t;
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        double t = 0.0;
        for (int k = 0; k < PCG_THREADS / 32; ++k) t += sh[c][k];
        out[c] = t;
    }
}

// residual of the initial guess, block-Jacobi inverse, u = M^-1 r; partials of (r,r)
__global__ void __launch_bounds__(PCG_THREADS) k_pcg_start(PCGArgs a, const double* __restrict__ rhs, double rtol, int maxit) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double rr = 0.0, bb = 0.0, r3[3] = {0.0, 0.0, 0.0};
    if (i < a.nV) {
        double Mi[9];
        const bool fx = a.fixed[i] != 0;
        jacobi_block_inverse(a, i, fx, Mi);
        for (int k = 0; k < 9; ++k) a.minv[9 * (size_t)i + k] = Mi[k];
        double y0, y1, y2;
        row_apply<3>(a, i, a.x, y0, y1, y2);
        const double r0 = fx ? 0.0 : rhs[3 * i] - y0, r1 = fx ? 0.0 : rhs[3 * i + 1] - y1, r2 = fx ? 0.0 : rhs[3 * i + 2] - y2;
        a.r[3 * i] = r0;
        a.r[3 * i + 1] = r1;
        a.r[3 * i + 2] = r2;
        if (!fx) bb = rhs[3 * i] * rhs[3 * i] + rhs[3 * i + 1] * rhs[3 * i + 1] + rhs[3 * i + 2] * rhs[3 * i + 2];
        for (int d = 0; d < 3; ++d) {
            a.u[4 * i + d] = Mi[3 * d] * r0 + Mi[3 * d + 1] * r1 + Mi[3 * d + 2] * r2;
            a.p[3 * i + d] = 0.0;
            a.s[3 * i + d] = 0.0;
        }
        a.u[4 * i + 3] = 0.0;
        rr = r0 * r0 + r1 * r1 + r2 * r2;
        r3[0] = r0;
        r3[1] = r1;
        r3[2] = r2;
    }
    if (a.cs_blocks) {
        double d3[3] = {0.0, 0.0, 0.0};
        if (i < a.nV)
            for (int k = 0; k < 3; ++k) d3[k] = a.cs_d[3 * (size_t)i + k];
        block_restrict(a, i < a.nV, i, r3, d3);
    }
    // the tolerance is relative to |b| on the free DOFs (= |r0| when starting from zero)
    const double v[2] = {rr, bb};
    if (block_partials<2>(a, v)) {
        double tt[2];
        final_sums<2>(a, tt);
        if (threadIdx.x != 0) return;
        const double t = tt[0];
        a.sc[SC_RR0] = t;
        a.sc[SC_TOL2] = rtol * rtol * tt[1];
        a.sc[SC_GAMMA] = 1.0;
        a.sc[SC_ALPHA] = 1.0;
        a.flag[0] = (t == 0.0 || t <= rtol * rtol * tt[1]) ? 1 : 0;
        a.flag[1] = 0;
        a.flag[2] = 0;
        a.flag[3] = 0;
        a.flag[4] = maxit;
    }
}

// iteration k (= flag[3], kept on the device so that a captured chunk of iterations replays
// unchanged), part 1: w = A u and the dot products; the last block derives alpha, beta
__global__ void __launch_bounds__(PCG_THREADS) k_pcg_spmv(PCGArgs a) {
    if (*(volatile int*)&a.flag[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double g = 0.0, dl = 0.0, rr = 0.0;
    if (i < a.nV) {
        double y0 = 0.0, y1 = 0.0, y2 = 0.0;
        if (!a.fixed[i]) row_apply<4>(a, i, a.u, y0, y1, y2);
        a.w[3 * i] = y0;
        a.w[3 * i + 1] = y1;
        a.w[3 * i + 2] = y2;
        const double u0 = a.u[4 * i], u1 = a.u[4 * i + 1], u2 = a.u[4 * i + 2];
        const double r0 = a.r[3 * i], r1 = a.r[3 * i + 1], r2 = a.r[3 * i + 2];
        g = r0 * u0 + r1 * u1 + r2 * u2;
        dl = y0 * u0 + y1 * u1 + y2 * u2;
        rr = r0 * r0 + r1 * r1 + r2 * r2;
    }
    const double v[3] = {g, dl, rr};
    if (block_partials<3>(a, v)) {
        double tt[3];
        final_sums<3>(a, tt);
        if (threadIdx.x != 0) return;
        const double G = tt[0], Dl = tt[1], R = tt[2];
        const int k = a.flag[3];
        a.flag[2] = 0;
        if (R <= a.sc[SC_TOL2]) {
            a.flag[0] = 1;
            a.flag[1] = k;
            return;
        }
        a.flag[3] = k + 1;
        const double beta = k == 0 ? 0.0 : G / a.sc[SC_GAMMA];
        const double alpha = k == 0 ? G / Dl : G / (Dl - beta * G / a.sc[SC_ALPHA]);
        a.sc[SC_GAMMA] = G;
        a.sc[SC_DELTA] = Dl;
        a.sc[SC_RR] = R;
        a.sc[SC_BETA] = beta;
        a.sc[SC_ALPHA] = alpha;
    }
}

// iteration k, part 2: recurrences and the preconditioner
__global__ void __launch_bounds__(PCG_THREADS) k_pcg_update(PCGArgs a) {
    if (*(volatile int*)&a.flag[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double rn[3] = {0.0, 0.0, 0.0}, d3[3] = {0.0, 0.0, 0.0};
    if (i < a.nV) {
        const double alpha = a.sc[SC_ALPHA], beta = a.sc[SC_BETA];
        // every load before the first store: the vectors are separate arrays, but nothing tells
        // the compiler so, and a store between two loads would serialise them
        double u[3], p[3], w[3], s[3], x[3], r[3], M[9];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int q = 3 * i + d;
            u[d] = a.u[4 * i + d];
            p[d] = a.p[q];
            w[d] = a.w[q];
            s[d] = a.s[q];
            x[d] = a.x[q];
            r[d] = a.r[q];
        }
#pragma unroll
        for (int k = 0; k < 9; ++k) M[k] = __ldg(a.minv + 9 * (size_t)i + k);
        if (a.cs_blocks)
#pragma unroll
            for (int d = 0; d < 3; ++d) d3[d] = __ldg(a.cs_d + 3 * (size_t)i + d);
        double pn[3], sn[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            pn[d] = u[d] + beta * p[d];
            sn[d] = w[d] + beta * s[d];
            rn[d] = r[d] - alpha * sn[d];
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int q = 3 * i + d;
            a.p[q] = pn[d];
            a.s[q] = sn[d];
            a.x[q] = x[d] + alpha * pn[d];
            a.r[q] = rn[d];
            const double z = M[3 * d] * rn[0] + M[3 * d + 1] * rn[1] + M[3 * d + 2] * rn[2];
            if (a.mg_z0) {
                const double z0 = a.mg_omega[0] * z;
                a.mg_z0[4 * i + d] = z0;
                if (a.mg_z0f) a.mg_z0f[4 * i + d] = (float)z0;
            } else {
                a.u[4 * i + d] = z;
            }
        }
    }
    if (a.cs_blocks) block_restrict(a, i < a.nV, i, rn, d3);
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

int launch_elasticity(int nT, const int* tets, const double* x, const double* dminv, const double* vol, const double* lam,
                      const double* mu, double dt, double* E, double* g, double* Hu, cudaStream_t s, bool tiled);
int launch_barrier_rows(int type, int n, const int* rows, const double* x, const double* x0, double dh2, double kappa,
                        const double* kap_s, const int* vscene, double* E, double* g, double* Hb, int* status, cudaStream_t s);

int cs_offsets(fipc_ctx* c, const double* x, cudaStream_t s);
int cs_prepare(fipc_ctx* c, const unsigned char* fixed, PCGArgs& a, cudaStream_t s);
void cs_apply(const fipc_ctx* c, const PCGArgs& a, cudaStream_t s);
int mg_prepare(fipc_ctx* c, const unsigned char* fixed, PCGArgs& a, cudaStream_t s);
int mg_start(fipc_ctx* c, const PCGArgs& a, cudaStream_t s);
void mg_vcycle(const fipc_ctx* c, const PCGArgs& a, cudaStream_t s);
int mg_launches_per_cycle(int levels);

int contact_prepare(fipc_ctx* c, TypeTable* tt, int* nrows_out, long long* nent_out, cudaStream_t s);

// the elastic + inertia matrix (sliced ELL) from the element blocks in elem_H (tiled layout)
// and the lumped mass on the diagonal blocks
int assemble_elastic(fipc_ctx* c, cudaStream_t s) {
    k_assemble_elastic<<<nblk(c->n_upper, 128), 128, 0, s>>>(c->n_upper, c->up_cptr, c->up_contrib, c->up_spos, c->up_tspos,
                                                             c->up_row, c->elem_H, c->mass, c->sell_val);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}
int contact_reduce(fipc_ctx* c, const TypeTable& tt, int nrows, long long nent, cudaStream_t s);

// compute_hessian_and_gradient (NEWTON_IPC.py:736-747) for the current constraint lists
int assemble_system(fipc_ctx* c, const double* x, const double* xt, cudaStream_t s) {
    int st = cs_offsets(c, x, s);
    if (st) return st;
    st = launch_elasticity(c->nT, c->tets, x, c->dminv, c->vol, c->lam, c->mu, c->dt, nullptr, c->elem_g, c->elem_H, s, true);
    if (st) return st;
    st = assemble_elastic(c, s);
    if (st) return st;
    k_assemble_rhs<<<nblk(c->nV, 128), 128, 0, s>>>(c->nV, c->vt_ptr, c->vt_list, c->elem_g, c->mass, x, xt, c->rhs);
    FIPC_LAUNCHED();
    TypeTable tt;
    int nrows = 0;
    long long nent = 0;
    st = contact_prepare(c, &tt, &nrows, &nent, s);
    if (st || nrows == 0) return st;
    // the rows' barrier gradients / projected Hessians
    for (int t = 0; t < N_TYPES; ++t) {
        if (!c->h_counts[t]) continue;
        const int off = tt.row0[t];
        st = launch_barrier_rows(t, c->h_counts[t], c->rows[t].as<int>(), x, c->x0, c->dhat2, c->kappa,
                                 c->n_scenes > 1 ? c->s_kappa : nullptr, c->v_scene, nullptr,
                                 c->c_g.as<double>() + 12ll * off, c->c_H.as<double>() + 144ll * off, nullptr, s);
        if (st) return st;
    }
    return contact_reduce(c, tt, nrows, nent, s);
}

// The contact rows of the current lists, concatenated in list order into rows_tmp: the type
// table, the row and block-entry counts, and buffers for the per-row gradients c_g [rows][12]
// and 3x3 blocks c_H [rows][16][9] that the caller fills.  With no rows the contact matrix is
// left empty.
int contact_prepare(fipc_ctx* c, TypeTable* tt, int* nrows_out, long long* nent_out, cudaStream_t s) {
    int nrows = 0;
    long long nent = 0;
    for (int t = 0; t < N_TYPES; ++t) {
        nrows += c->h_counts[t];
        nent += (long long)c->h_counts[t] * type_nverts(t) * type_nverts(t);
    }
    *nrows_out = nrows;
    *nent_out = nent;
    c->c_rows = nrows;
    c->c_nnzb = 0;
    if (c->c_rowptr.ensure(4ll * (c->nV + 1))) return FIPC_ERR_CUDA;
    if (nrows == 0) {
        FIPC_CUDA(cudaMemsetAsync(c->c_rowptr.p, 0, 4ll * (c->nV + 1), s));
        FIPC_CUDA(cudaGetLastError());
        return FIPC_OK;
    }
    if (c->c_g.ensure(96ll * nrows) || c->c_H.ensure(1152ll * nrows) || c->c_keys.ensure(8 * nent) || c->c_keys_alt.ensure(8 * nent) ||
        c->c_vals.ensure(4 * nent) || c->c_vals_alt.ensure(4 * nent) || c->c_ukeys.ensure(8 * nent) || c->c_ucount.ensure(4 * (nent + 1)) ||
        c->c_ustart.ensure(4 * (nent + 1)) || c->c_val.ensure(72 * nent) || c->c_col.ensure(4 * nent) || c->rows_tmp.ensure(16ll * nrows))
        return FIPC_ERR_CUDA;
    int4* all = c->rows_tmp.as<int4>();
    int off = 0;
    long long eoff = 0;
    for (int t = 0; t < N_TYPES; ++t) {
        tt->row0[t] = off;
        tt->ent0[t] = eoff;
        if (c->h_counts[t]) FIPC_CUDA(cudaMemcpyAsync(all + off, c->rows[t].p, 16ll * c->h_counts[t], cudaMemcpyDeviceToDevice, s));
        off += c->h_counts[t];
        eoff += (long long)c->h_counts[t] * type_nverts(t) * type_nverts(t);
    }
    tt->row0[N_TYPES] = off;
    tt->ent0[N_TYPES] = eoff;
    return FIPC_OK;
}

// The contact matrix (block CSR, fixed-order sums of every (row, column) block of the rows) and
// the rows' gradients folded into rhs, from c_g / c_H filled for the rows contact_prepare set up
int contact_reduce(fipc_ctx* c, const TypeTable& tt, int nrows, long long nent, cudaStream_t s) {
    const int4* all = c->rows_tmp.as<int4>();
    k_contact_keys<<<nblk(nrows, 128), 128, 0, s>>>(nrows, all, tt, c->c_keys.as<unsigned long long>(), c->c_vals.as<int>());
    FIPC_LAUNCHED();
    const int N = (int)nent;
    cub::DoubleBuffer<unsigned long long> kb(c->c_keys.as<unsigned long long>(), c->c_keys_alt.as<unsigned long long>());
    cub::DoubleBuffer<int> vb(c->c_vals.as<int>(), c->c_vals_alt.as<int>());
    int st = cub_call(c, [&](void* tm, size_t& b) { return cub::DeviceRadixSort::SortPairs(tm, b, kb, vb, N, 0, 53, s); });
    if (st) return st;
    unsigned long long* sk = kb.Current();
    int* sv = vb.Current();
    if (c->scal.ensure(64)) return FIPC_ERR_CUDA;
    int* nu_d = (int*)(c->scal.as<char>() + 32);
    st = cub_call(c, [&](void* tm, size_t& b) {
        return cub::DeviceRunLengthEncode::Encode(tm, b, sk, c->c_ukeys.as<unsigned long long>(), c->c_ucount.as<int>(), nu_d, N, s);
    });
    if (st) return st;
    int nu = 0;
    FIPC_CUDA(cudaMemcpyAsync(&nu, nu_d, sizeof(int), cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaStreamSynchronize(s));
    int* cnt = c->c_ucount.as<int>();
    int* ustart = c->c_ustart.as<int>();
    st = cub_call(c, [&](void* tm, size_t& b) { return cub::DeviceScan::ExclusiveSum(tm, b, cnt, ustart, nu + 1, s); });
    if (st) return st;
    k_contact_reduce<<<nblk(nu, 128), 128, 0, s>>>(nu, c->c_ukeys.as<unsigned long long>(), ustart, sv, c->c_H.as<double>(),
                                                   c->c_g.as<double>(), c->c_val.as<double>(), c->c_col.as<int>(), c->rhs);
    FIPC_LAUNCHED();
    k_contact_rowptr<<<nblk(c->nV + 1, 256), 256, 0, s>>>(c->nV, nu, c->c_ukeys.as<unsigned long long>(), c->c_rowptr.as<int>());
    FIPC_LAUNCHED();
    c->c_nnzb = nu;
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int sell_to_bsr(fipc_ctx* c, double* out, cudaStream_t s) {
    k_sell_to_bsr<<<nblk(c->nnzb, 256), 256, 0, s>>>(c->nnzb, c->bsr2sell, c->sell_val, out);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

// The single-scene PCG replays from one captured graph per solve: a while-loop (conditional)
// node whose body holds PCG3_BODY iterations (SpMV, update, preconditioner) and a one-thread
// kernel that keeps the loop going while the solve has not converged and another body fits the
// iteration budget.  Convergence is decided on the device; the host launches the graph once and
// reads the flags once.  Iterations after convergence inside the last body return at their
// first instruction (at most PCG3_BODY - 1 of them).  Iterations left over below the budget,
// and solves whose per-launch timing is requested, run as plain launches in chunks of
// PCG3_CHUNK iterations.
constexpr int PCG3_BODY = 4, PCG3_CHUNK = 32;

// flag[0]: converged, flag[3]: iterations begun, flag[4]: iteration budget
__global__ void k_pcg_continue(const int* __restrict__ flag, cudaGraphConditionalHandle h) {
    if (threadIdx.x != 0) return;
    const volatile int* f = flag;
    const bool go = f[0] == 0 && f[3] + PCG3_BODY <= f[4];
    cudaGraphSetConditional(h, go ? 1u : 0u);
}

// drops the captured PCG graph (its kernels hold the preconditioner's buffers)
void pcg_graph_reset(fipc_ctx* c) {
    if (c->pcg3_exec) cudaGraphExecDestroy((cudaGraphExec_t)c->pcg3_exec);
    c->pcg3_exec = nullptr;
    c->pcg3_sig.clear();
}

// the while-loop graph for these kernel arguments, captured on the context's private stream and
// replayed on the caller's; reused while the arguments (buffers, sizes) stay the same; false when
// conditional graphs are unavailable
static bool pcg3_graph(fipc_ctx* c, const PCGArgs& a) {
    std::vector<unsigned char> sig(reinterpret_cast<const unsigned char*>(&a), reinterpret_cast<const unsigned char*>(&a) + sizeof(PCGArgs));
    if (a.mg) sig.insert(sig.end(), reinterpret_cast<const unsigned char*>(a.mg), reinterpret_cast<const unsigned char*>(a.mg) + sizeof(MgArgs));
    if (c->pcg3_exec && c->pcg3_sig == sig) return true;
    pcg_graph_reset(c);
    if (!c->cap_stream) {
        cudaStream_t cs;
        if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) return false;
        c->cap_stream = cs;
    }
    cudaStream_t cs = (cudaStream_t)c->cap_stream;
    const int nb = nblk(c->nV, PCG_THREADS);
    cudaGraph_t g = nullptr;
    if (cudaGraphCreate(&g, 0) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    bool ok = false;
    do {
        cudaGraphConditionalHandle h;
        if (cudaGraphConditionalHandleCreate(&h, g, 1u, cudaGraphCondAssignDefault) != cudaSuccess) break;
        cudaGraphNodeParams np{};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        if (cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np) != cudaSuccess) break;
        cudaGraph_t body = np.conditional.phGraph_out[0];
        const long long counted = g_launches.load();   // captured launches run (and count) at replay
        if (cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) != cudaSuccess) break;
        for (int k = 0; k < PCG3_BODY; ++k) {
            k_pcg_spmv<<<nb, PCG_THREADS, 0, cs>>>(a);
            k_pcg_update<<<nb, PCG_THREADS, 0, cs>>>(a);
            if (a.mg) mg_vcycle(c, a, cs);
            else if (a.cs_blocks) cs_apply(c, a, cs);
        }
        k_pcg_continue<<<1, 32, 0, cs>>>(a.flag, h);
        g_launches.store(counted);
        cudaGraph_t captured = nullptr;
        if (cudaStreamEndCapture(cs, &captured) != cudaSuccess || captured != body) break;
        cudaGraphExec_t ex = nullptr;
        if (cudaGraphInstantiate(&ex, g, 0ull) != cudaSuccess) break;
        c->pcg3_exec = ex;
        c->pcg3_sig = sig;
        ok = true;
    } while (false);
    cudaGraphDestroy(g);
    if (!ok) cudaGetLastError();
    return ok;
}

// solve_system (NEWTON_IPC.py:750-777) by block-Jacobi PCG; sol: device [3 nV] holding the
// initial guess on entry (zero for the reference's semantics) and the solution on return
int pcg_solve(fipc_ctx* c, const unsigned char* fixed, const int* /*diag_pos*/, double rtol, int maxit, double* sol, int* iters,
              cudaStream_t s) {
    const long long n3 = 3ll * c->nV;
    const int nb = nblk(c->nV, PCG_THREADS);
    if (c->pcg_vec.ensure(8 * (n3 * 4 + 13ll * c->nV) + 64) || c->pcg_part.ensure(8ll * (3 * nb + SC_COUNT) + 64) || c->scal.ensure(80))
        return FIPC_ERR_CUDA;
    if (c->c_nnzb == 0 && (c->c_rowptr.ensure(4ll * (c->nV + 1)) || cudaMemsetAsync(c->c_rowptr.p, 0, 4ll * (c->nV + 1), s)))
        return FIPC_ERR_CUDA;
    if (c->c_val.ensure(72) || c->c_col.ensure(4)) return FIPC_ERR_CUDA;
    PCGArgs a{};
    a.nV = c->nV;
    a.soff = c->sell_off;
    a.scol = c->sell_col;
    a.rlen = c->row_len;
    a.sval = c->sell_val;
    a.crp = c->c_rowptr.as<int>();
    a.cci = c->c_col.as<int>();
    a.cva = c->c_val.as<double>();
    a.fixed = fixed;
    a.diag_spos = c->diag_spos;
    double* v = c->pcg_vec.as<double>();
    a.x = sol;
    a.u = v;                       // 4 nV, first so that it is 32-byte aligned
    a.r = v + 4ll * c->nV;
    a.w = a.r + n3;
    a.p = a.w + n3;
    a.s = a.p + n3;
    a.minv = a.s + n3;
    a.part = c->pcg_part.as<double>();
    a.sc = a.part + 3 * nb;
    a.flag = (int*)(c->scal.as<char>() + 48);
    FIPC_CUDA(cudaMemsetAsync(a.flag, 0, 5 * sizeof(int), s));
    int st = c->mg ? mg_prepare(c, fixed, a, s) : cs_prepare(c, fixed, a, s);
    if (st) return st;
    if (a.mg) a.cs_blocks = 0;
    // traffic model per launch: matrix blocks and column ids once (padding slots included),
    // row data, the gathered vector once, w written, r read
    const double slots = 32.0 * (double)c->n_slots, nv = (double)c->nV, cn = (double)c->c_nnzb;
    const double spmv_bytes = slots * (72.0 + 4.0) + cn * 76.0 + nv * (4.0 + 4.0 + 1.0 + 32.0 + 24.0 + 24.0);
    const double spmv_flops = (double)(c->nnzb + c->c_nnzb) * 18.0 + nv * 18.0;
    const double upd_bytes = nv * (32.0 * 2 + 24.0 * 2 * 4 + 24.0 + 72.0);
    const double upd_flops = nv * 36.0;
    k_pcg_start<<<nb, PCG_THREADS, 0, s>>>(a, c->rhs, rtol, maxit);
    FIPC_LAUNCHED();
    if (a.mg) {
        st = mg_start(c, a, s);
        if (st) return st;
    } else if (a.cs_blocks) {
        cs_apply(c, a, s);
    }
    int h_flag[4] = {0, 0, 0, 0};
    // per-launch timing of the SpMV or the update needs plain launches; otherwise the iterations
    // replay from the captured while-loop graph, and only a remainder below the budget runs plainly
    const int pk = profile_kernel();
    const bool timed = pk == PK_PCG_SPMV || pk == PK_PCG_UPDATE;
    const int per_iter = a.mg ? 2 + mg_launches_per_cycle(c->mg_levels) : (a.cs_blocks ? 4 : 2);
    int k0 = 0;
    if (!timed && maxit >= PCG3_BODY && pcg3_graph(c, a)) {
        FIPC_CUDA(cudaGraphLaunch((cudaGraphExec_t)c->pcg3_exec, s));
        FIPC_CUDA(cudaMemcpyAsync(h_flag, a.flag, sizeof(int) * 4, cudaMemcpyDeviceToHost, s));
        FIPC_CUDA(cudaStreamSynchronize(s));
        // bodies run: up to and including the one that saw convergence, else whole budget-sized ones
        const long long bodies = h_flag[0] ? h_flag[3] / PCG3_BODY + 1 : h_flag[3] / PCG3_BODY;
        g_launches.fetch_add(bodies * (PCG3_BODY * per_iter + 1), std::memory_order_relaxed);
        k0 = h_flag[3];
    }
    while (!h_flag[0] && k0 < maxit) {
        const int k1 = (k0 + PCG3_CHUNK < maxit) ? k0 + PCG3_CHUNK : maxit;
        for (int k = k0; k < k1; ++k) {
            {
                ProfScope ps(PK_PCG_SPMV, s, spmv_bytes, spmv_flops);
                k_pcg_spmv<<<nb, PCG_THREADS, 0, s>>>(a);
            }
            FIPC_LAUNCHED();
            {
                ProfScope ps(PK_PCG_UPDATE, s, upd_bytes, upd_flops);
                k_pcg_update<<<nb, PCG_THREADS, 0, s>>>(a);
            }
            FIPC_LAUNCHED();
            if (a.mg) mg_vcycle(c, a, s);
            else if (a.cs_blocks) cs_apply(c, a, s);
        }
        k0 = k1;
        FIPC_CUDA(cudaMemcpyAsync(h_flag, a.flag, sizeof(int) * 4, cudaMemcpyDeviceToHost, s));
        FIPC_CUDA(cudaStreamSynchronize(s));
    }
    FIPC_CUDA(cudaGetLastError());
    if (iters) *iters = h_flag[0] ? h_flag[1] : maxit;
    return h_flag[0] ? FIPC_OK : FIPC_ERR_ITERATION;
}

}  // namespace fipc
