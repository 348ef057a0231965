// Newton system: assembly into 3x3 block-sparse rows and the block-Jacobi PCG direction
// solve.  Replaces the triplet assembly of NEWTON_IPC.py:545-747 and the CHOLMOD solve of
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
// PCG: block-Jacobi preconditioner (inverse 3x3 diagonal blocks), Dirichlet vertices removed
// by zero rows/columns (the reference's DBC_set_zeros + identity, NEWTON_IPC.py:756-772).
// Two kernels per iteration on a fixed grid; dot products are per-block partials summed in a
// fixed order by every consumer block, so results are bitwise reproducible.
#include <cub/cub.cuh>
#include <cuda_runtime.h>

#include "ctx.cuh"
#include "profile.cuh"

namespace fipc {

// ---------------------------------------------------------------- elastic + inertia
__global__ void k_assemble_elastic(int n_upper, const int* __restrict__ cptr, const int* __restrict__ contrib,
                                   const int* __restrict__ pos, const int* __restrict__ tpos, const int* __restrict__ urow,
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
    const int p = pos[u], q = tpos[u];
    if (p == q) {
        const double m = mass[urow[u]];
        s[0] += m;
        s[4] += m;
        s[8] += m;
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) val[9 * (size_t)p + i] = s[i];
    if (p != q) {
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) val[9 * (size_t)q + i * 3 + j] = s[j * 3 + i];
    }
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
// row ranges of the concatenated lists: rows [row0[t], row0[t+1]) are of type t and their
// nv(t)^2 blocks start at ent0[t] + (r - row0[t]) nv(t)^2
struct TypeTable {
    int row0[N_TYPES + 1];
    long long ent0[N_TYPES + 1];
};

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
struct PCGArgs {
    int nV;
    const int *rp, *ci;          // elastic BSR
    const double* va;
    const int *crp, *cci;        // contact BSR
    const double* cva;
    const unsigned char* fixed;
    double *x, *r, *z, *p0, *p1, *ap, *minv;
    double *part;                // [5][RED_BLOCKS]: rz(2), rr(2), pAp
    double* sc;                  // [0] rz_prev, [1] rr0, [2] rtol^2
    int* flag;                   // [0] done, [1] iterations
};

__device__ __forceinline__ double sum_parts(const double* __restrict__ p, double* sh) {
    double a = 0.0;
    for (int i = threadIdx.x; i < RED_BLOCKS; i += blockDim.x) a += p[i];
    sh[threadIdx.x] = a;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

__device__ __forceinline__ void inv3x3(const double* A, double* R) {
    const double c00 = A[4] * A[8] - A[5] * A[7], c01 = A[5] * A[6] - A[3] * A[8], c02 = A[3] * A[7] - A[4] * A[6];
    const double det = A[0] * c00 + A[1] * c01 + A[2] * c02, id = 1.0 / det;
    R[0] = c00 * id;
    R[1] = (A[2] * A[7] - A[1] * A[8]) * id;
    R[2] = (A[1] * A[5] - A[2] * A[4]) * id;
    R[3] = c01 * id;
    R[4] = (A[0] * A[8] - A[2] * A[6]) * id;
    R[5] = (A[2] * A[3] - A[0] * A[5]) * id;
    R[6] = c02 * id;
    R[7] = (A[1] * A[6] - A[0] * A[7]) * id;
    R[8] = (A[0] * A[4] - A[1] * A[3]) * id;
}

// setup: M^-1 from diagonal blocks, x = 0, r = masked rhs, z = M^-1 r, partials of r.z, r.r
__global__ void __launch_bounds__(RED_THREADS) k_pcg_init(PCGArgs a, const double* __restrict__ rhs, const int* __restrict__ diag_pos) {
    __shared__ double sh[RED_THREADS];
    double rz = 0.0, rr = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nV; i += gridDim.x * blockDim.x) {
        double D[9], Mi[9];
        const bool fx = a.fixed[i] != 0;
        if (fx) {
            for (int k = 0; k < 9; ++k) Mi[k] = (k % 4 == 0) ? 1.0 : 0.0;
        } else {
            const double* E = a.va + 9 * (size_t)diag_pos[i];
            for (int k = 0; k < 9; ++k) D[k] = E[k];
            for (int k = a.crp[i]; k < a.crp[i + 1]; ++k)
                if (a.cci[k] == i)
                    for (int q = 0; q < 9; ++q) D[q] += a.cva[9 * (size_t)k + q];
            inv3x3(D, Mi);
        }
        for (int k = 0; k < 9; ++k) a.minv[9 * (size_t)i + k] = Mi[k];
        double r3[3];
        for (int d = 0; d < 3; ++d) {
            r3[d] = fx ? 0.0 : rhs[3 * i + d];
            a.r[3 * i + d] = r3[d];
            a.x[3 * i + d] = 0.0;
            a.p1[3 * i + d] = 0.0;
        }
        for (int d = 0; d < 3; ++d) {
            const double zd = Mi[3 * d] * r3[0] + Mi[3 * d + 1] * r3[1] + Mi[3 * d + 2] * r3[2];
            a.z[3 * i + d] = zd;
            rz += r3[d] * zd;
            rr += r3[d] * r3[d];
        }
    }
    sh[threadIdx.x] = rz;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) a.part[0 * RED_BLOCKS + blockIdx.x] = sh[0];
    __syncthreads();
    sh[threadIdx.x] = rr;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) a.part[2 * RED_BLOCKS + blockIdx.x] = sh[0];
}

__global__ void k_pcg_init_scalars(PCGArgs a, double rtol) {
    __shared__ double sh[RED_THREADS];
    const double rr0 = sum_parts(a.part + 2 * RED_BLOCKS, sh);
    if (threadIdx.x == 0) {
        a.sc[0] = 1.0;
        a.sc[1] = rr0;
        a.sc[2] = rtol * rtol * rr0;
        a.flag[0] = rr0 == 0.0 ? 1 : 0;
        a.flag[1] = 0;
    }
}

// K1 of iteration k: beta, p_k = z + beta p_{k-1}, Ap = A p_k (masked), partials of p.Ap
__global__ void __launch_bounds__(RED_THREADS) k_pcg_spmv(PCGArgs a, int k) {
    __shared__ double sh[RED_THREADS];
    if (*(volatile int*)&a.flag[0]) return;
    const int par = k & 1;
    const double rz = sum_parts(a.part + par * RED_BLOCKS, sh);
    const double rr = sum_parts(a.part + (2 + par) * RED_BLOCKS, sh);
    if (rr <= a.sc[2]) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            a.flag[0] = 1;
            a.flag[1] = k;
        }
        return;
    }
    const double beta = k == 0 ? 0.0 : rz / a.sc[0];
    const double* pp = (k & 1) ? a.p0 : a.p1;   // p_{k-1}
    double* pn = (k & 1) ? a.p1 : a.p0;         // p_k
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nV; i += gridDim.x * blockDim.x) {
        double y0 = 0.0, y1 = 0.0, y2 = 0.0;
        const double q0 = a.z[3 * i] + beta * pp[3 * i], q1 = a.z[3 * i + 1] + beta * pp[3 * i + 1],
                     q2 = a.z[3 * i + 2] + beta * pp[3 * i + 2];
        pn[3 * i] = q0;
        pn[3 * i + 1] = q1;
        pn[3 * i + 2] = q2;
        if (!a.fixed[i]) {
            for (int e = a.rp[i]; e < a.rp[i + 1]; ++e) {
                const int j = a.ci[e];
                const double* B = a.va + 9 * (size_t)e;
                const double p0 = a.z[3 * j] + beta * pp[3 * j], p1 = a.z[3 * j + 1] + beta * pp[3 * j + 1],
                             p2 = a.z[3 * j + 2] + beta * pp[3 * j + 2];
                y0 += B[0] * p0 + B[1] * p1 + B[2] * p2;
                y1 += B[3] * p0 + B[4] * p1 + B[5] * p2;
                y2 += B[6] * p0 + B[7] * p1 + B[8] * p2;
            }
            for (int e = a.crp[i]; e < a.crp[i + 1]; ++e) {
                const int j = a.cci[e];
                const double* B = a.cva + 9 * (size_t)e;
                const double p0 = a.z[3 * j] + beta * pp[3 * j], p1 = a.z[3 * j + 1] + beta * pp[3 * j + 1],
                             p2 = a.z[3 * j + 2] + beta * pp[3 * j + 2];
                y0 += B[0] * p0 + B[1] * p1 + B[2] * p2;
                y1 += B[3] * p0 + B[4] * p1 + B[5] * p2;
                y2 += B[6] * p0 + B[7] * p1 + B[8] * p2;
            }
        }
        a.ap[3 * i] = y0;
        a.ap[3 * i + 1] = y1;
        a.ap[3 * i + 2] = y2;
        acc += q0 * y0 + q1 * y1 + q2 * y2;
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) a.part[4 * RED_BLOCKS + blockIdx.x] = sh[0];
}

// K2 of iteration k: alpha, x += alpha p, r -= alpha Ap, z = M^-1 r, partials of r.z, r.r
__global__ void __launch_bounds__(RED_THREADS) k_pcg_update(PCGArgs a, int k) {
    __shared__ double sh[RED_THREADS];
    if (*(volatile int*)&a.flag[0]) return;
    const int par = k & 1;
    const double rz = sum_parts(a.part + par * RED_BLOCKS, sh);
    const double pAp = sum_parts(a.part + 4 * RED_BLOCKS, sh);
    const double alpha = rz / pAp;
    const double* pk = (k & 1) ? a.p1 : a.p0;
    double rzn = 0.0, rrn = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nV; i += gridDim.x * blockDim.x) {
        double r3[3];
        for (int d = 0; d < 3; ++d) {
            a.x[3 * i + d] += alpha * pk[3 * i + d];
            r3[d] = a.r[3 * i + d] - alpha * a.ap[3 * i + d];
            a.r[3 * i + d] = r3[d];
        }
        const double* Mi = a.minv + 9 * (size_t)i;
        for (int d = 0; d < 3; ++d) {
            const double zd = Mi[3 * d] * r3[0] + Mi[3 * d + 1] * r3[1] + Mi[3 * d + 2] * r3[2];
            a.z[3 * i + d] = zd;
            rzn += r3[d] * zd;
            rrn += r3[d] * r3[d];
        }
    }
    const int npar = (k + 1) & 1;
    sh[threadIdx.x] = rzn;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) a.part[npar * RED_BLOCKS + blockIdx.x] = sh[0];
    __syncthreads();
    sh[threadIdx.x] = rrn;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.part[(2 + npar) * RED_BLOCKS + blockIdx.x] = sh[0];
        if (blockIdx.x == 0) a.sc[0] = rz;
    }
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
                      const double* mu, double dt, double* E, double* g, double* Hu, cudaStream_t s);
int launch_barrier_rows(int type, int n, const int* rows, const double* x, const double* x0, double dh2, double kappa, double* E,
                        double* g, double* Hb, int* status, cudaStream_t s);

// compute_hessian_and_gradient (NEWTON_IPC.py:736-747) for the current constraint lists
int assemble_system(fipc_ctx* c, const double* x, const double* xt, cudaStream_t s) {
    int st = launch_elasticity(c->nT, c->tets, x, c->dminv, c->vol, c->lam, c->mu, c->dt, nullptr, c->elem_g, c->elem_H, s);
    if (st) return st;
    k_assemble_elastic<<<nblk(c->n_upper, 128), 128, 0, s>>>(c->n_upper, c->up_cptr, c->up_contrib, c->up_pos, c->up_tpos, c->up_row,
                                                             c->elem_H, c->mass, c->bsr_val);
    FIPC_LAUNCHED();
    k_assemble_rhs<<<nblk(c->nV, 128), 128, 0, s>>>(c->nV, c->vt_ptr, c->vt_list, c->elem_g, c->mass, x, xt, c->rhs);
    FIPC_LAUNCHED();
    // contact rows, concatenated in list order
    int nrows = 0;
    long long nent = 0;
    for (int t = 0; t < N_TYPES; ++t) {
        nrows += c->h_counts[t];
        nent += (long long)c->h_counts[t] * type_nverts(t) * type_nverts(t);
    }
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
    // concatenated rows (list order) and their barrier gradients / projected Hessians
    int4* all = c->rows_tmp.as<int4>();
    TypeTable tt;
    int off = 0;
    long long eoff = 0;
    for (int t = 0; t < N_TYPES; ++t) {
        tt.row0[t] = off;
        tt.ent0[t] = eoff;
        if (c->h_counts[t]) {
            FIPC_CUDA(cudaMemcpyAsync(all + off, c->rows[t].p, 16ll * c->h_counts[t], cudaMemcpyDeviceToDevice, s));
            st = launch_barrier_rows(t, c->h_counts[t], c->rows[t].as<int>(), x, c->x0, c->dhat2, c->kappa, nullptr,
                                     c->c_g.as<double>() + 12ll * off, c->c_H.as<double>() + 144ll * off, nullptr, s);
            if (st) return st;
        }
        off += c->h_counts[t];
        eoff += (long long)c->h_counts[t] * type_nverts(t) * type_nverts(t);
    }
    tt.row0[N_TYPES] = off;
    tt.ent0[N_TYPES] = eoff;
    k_contact_keys<<<nblk(nrows, 128), 128, 0, s>>>(nrows, all, tt, c->c_keys.as<unsigned long long>(), c->c_vals.as<int>());
    FIPC_LAUNCHED();
    const int N = (int)nent;
    cub::DoubleBuffer<unsigned long long> kb(c->c_keys.as<unsigned long long>(), c->c_keys_alt.as<unsigned long long>());
    cub::DoubleBuffer<int> vb(c->c_vals.as<int>(), c->c_vals_alt.as<int>());
    st = cub_call(c, [&](void* tm, size_t& b) { return cub::DeviceRadixSort::SortPairs(tm, b, kb, vb, N, 0, 53, s); });
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

// solve_system (NEWTON_IPC.py:750-777) by block-Jacobi PCG; sol: device [3 nV]
int pcg_solve(fipc_ctx* c, const unsigned char* fixed, const int* diag_pos, double rtol, int maxit, double* sol, int* iters,
              cudaStream_t s) {
    const long long n3 = 3ll * c->nV;
    if (c->pcg_vec.ensure(8 * (n3 * 6 + 9ll * c->nV)) || c->pcg_part.ensure(8ll * 5 * RED_BLOCKS + 64) || c->scal.ensure(64))
        return FIPC_ERR_CUDA;
    if (c->c_nnzb == 0 && (c->c_rowptr.ensure(4ll * (c->nV + 1)) || cudaMemsetAsync(c->c_rowptr.p, 0, 4ll * (c->nV + 1), s)))
        return FIPC_ERR_CUDA;
    if (c->c_val.ensure(72) || c->c_col.ensure(4)) return FIPC_ERR_CUDA;
    PCGArgs a;
    a.nV = c->nV;
    a.rp = c->row_ptr;
    a.ci = c->col_idx;
    a.va = c->bsr_val;
    a.crp = c->c_rowptr.as<int>();
    a.cci = c->c_col.as<int>();
    a.cva = c->c_val.as<double>();
    a.fixed = fixed;
    double* v = c->pcg_vec.as<double>();
    a.x = sol;
    a.r = v;
    a.z = v + n3;
    a.p0 = v + 2 * n3;
    a.p1 = v + 3 * n3;
    a.ap = v + 4 * n3;
    a.minv = v + 5 * n3;
    a.part = c->pcg_part.as<double>();
    a.sc = c->pcg_part.as<double>() + 5 * RED_BLOCKS;
    a.flag = (int*)(c->scal.as<char>() + 48);
    k_pcg_init<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, c->rhs, diag_pos);
    FIPC_LAUNCHED();
    k_pcg_init_scalars<<<1, RED_THREADS, 0, s>>>(a, rtol);
    FIPC_LAUNCHED();
    int h_flag[2] = {0, 0};
    const int chunk = 32;
    // algorithmic traffic per launch: every matrix block and column index once, the vertex
    // vectors once each (z and p_{k-1} read, p_k and Ap written), row pointers and flags
    const double nnz = (double)c->nnzb + (double)c->c_nnzb, nv = (double)c->nV;
    const double spmv_bytes = nnz * 76.0 + nv * (4.0 + 4.0 + 1.0 + 4 * 24.0);
    const double spmv_flops = nnz * 24.0 + nv * 12.0;
    const double upd_bytes = nv * (2 * 24.0 + 2 * 24.0 + 24.0 + 24.0 + 24.0 + 72.0);
    const double upd_flops = nv * 42.0;
    for (int k0 = 0; k0 < maxit; k0 += chunk) {
        for (int k = k0; k < k0 + chunk && k < maxit; ++k) {
            {
                ProfScope ps(PK_PCG_SPMV, s, spmv_bytes, spmv_flops);
                k_pcg_spmv<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, k);
            }
            FIPC_LAUNCHED();
            {
                ProfScope ps(PK_PCG_UPDATE, s, upd_bytes, upd_flops);
                k_pcg_update<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, k);
            }
            FIPC_LAUNCHED();
        }
        FIPC_CUDA(cudaMemcpyAsync(h_flag, a.flag, sizeof(int) * 2, cudaMemcpyDeviceToHost, s));
        FIPC_CUDA(cudaStreamSynchronize(s));
        if (h_flag[0]) break;
    }
    FIPC_CUDA(cudaGetLastError());
    if (iters) *iters = h_flag[0] ? h_flag[1] : maxit;
    return h_flag[0] ? FIPC_OK : FIPC_ERR_ITERATION;
}

}  // namespace fipc
