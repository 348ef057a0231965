// Shared by the single-scene and batched PCG: the system operands and the per-row product
// w_i = sum_j A_ij v_j over the elastic sliced-ELL rows and the contact block-CSR rows.
#pragma once

#include "ctx.cuh"

namespace fipc {

struct PCGArgs {
    int nV;
    const int *soff, *scol, *rlen;   // elastic matrix, sliced-ELL
    const double* sval;
    const int *crp, *cci;            // contact matrix, block-CSR
    const double* cva;
    const unsigned char* fixed;
    const int* diag_spos;
    double *x, *r, *u, *w, *p, *s, *minv;   // u: stride 4 (padded); the others stride 3
    double* part;                    // [3][nblk]
    double* sc;                      // scalars, see SC_*
    int* flag;                       // [0] done, [1] iterations, [2] ticket
    // coarse space (cs_blocks = PCG blocks per aggregate; 0: block-Jacobi only)
    int cs_blocks;
    const double* cs_d;              // [V][3] vertex offset from its aggregate's centroid
    double* cs_part;                 // [nblk][6] per-block restriction (force, torque) of r
    double* cs_g;                    // [6 n_agg] restriction per aggregate
    double* cs_y;                    // [6 n_agg] coarse correction Ac^-1 g
    int* cs_ticket;                  // [n_agg] blocks of the aggregate done (reset by its last block)
    const double* cs_ainv;           // inverse coarse matrix, row stride cs_ld
    int cs_n, cs_ld;                 // 6 n_agg; padded row stride
    // multigrid preconditioner (mg non-null, host pointer): the update kernel writes the
    // pre-smoothed z0 = w0 D^-1 r (stride 4) instead of u, and the V-cycle produces u
    const struct MgArgs* mg;
    double* mg_z0;
    const double* mg_omega;          // [levels] smoother weights (device)
    float* mg_z0f;                   // FP32 copy of z0 (stride 4) for FP32 smoothing products, or null
};

// one level >= 1 of the multigrid hierarchy (6 DOFs per node), as the V-cycle kernels see it
struct MgLev {
    int n;                           // nodes
    const int *mem_ptr, *mem;        // members (finer-level ids) of each node
    const int* agg_of;               // node of each finer-level node
    const double* d;                 // [3 n_finer] offsets of the finer nodes from their node's centroid
    const int *s_rp, *s_ci;          // static pattern, 6x6 blocks
    const double* s_val;
    const int *c_rp, *c_ci;          // contact pattern (c_rp null: none)
    const double* c_val;
    const double* minv;              // [36 n] block-Jacobi inverses
    double *g, *z, *z2, *t;          // [6 n]: restricted residual, iterate, post-smoothed, residual
};
constexpr int MG_LEVELS_CAP = 8;
struct MgArgs {
    int levels;
    MgLev L[MG_LEVELS_CAP];          // L[1 .. levels - 1]
    double* z0;                      // [4 nV] level-0 iterate
    double* t0;                      // [3 nV] level-0 residual
    const double* omega;             // [levels]
    const double* dense;             // coarsest inverse, row stride ld_dense
    int n_dense, ld_dense;
    // FP32 smoothing products on level 0 (null: FP64): the elastic values in the sliced-ELL
    // layout and the contact values as FP32 copies, and z0 as FP32 (stride 4)
    const float *v32, *c32;
    float* z0f;
};
enum { SC_GAMMA = 0, SC_DELTA, SC_RR, SC_ALPHA, SC_BETA, SC_RR0, SC_TOL2, SC_COUNT };
constexpr int PCG_THREADS = 128;

// w_i = sum_j A_ij v_j over the elastic (sliced-ELL) and contact (block-CSR) rows of vertex i;
// v is stored with stride ST doubles per vertex (ST = 4: 32-byte aligned, two vector loads)
template <int ST>
__device__ __forceinline__ void load_v(const double* __restrict__ v, int j, double& a, double& b, double& c) {
    if (ST == 4) {
        const double2 ab = __ldg(reinterpret_cast<const double2*>(v + 4 * (size_t)j));
        a = ab.x;
        b = ab.y;
        c = __ldg(v + 4 * (size_t)j + 2);
    } else {
        a = __ldg(v + 3 * (size_t)j);
        b = __ldg(v + 3 * (size_t)j + 1);
        c = __ldg(v + 3 * (size_t)j + 2);
    }
}

template <int ST>
__device__ __forceinline__ void row_apply(const PCGArgs& a, int i, const double* __restrict__ v, double& y0, double& y1, double& y2) {
    y0 = y1 = y2 = 0.0;
    const int sl = i >> 5, lane = i & 31;
    const int base = a.soff[sl], len = a.rlen[i];
    int k = 0;
    // two blocks per trip: their index, value and vector loads are independent
    for (; k + 1 < len; k += 2) {
        const size_t s0 = (size_t)(base + k), s1 = s0 + 1;
        const int j0 = __ldg(a.scol + s0 * 32 + lane), j1 = __ldg(a.scol + s1 * 32 + lane);
        const double* B = a.sval + s0 * 288 + lane;
        const double* C = a.sval + s1 * 288 + lane;
        double b[9], c[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            b[q] = __ldg(B + 32 * q);
            c[q] = __ldg(C + 32 * q);
        }
        double p0, p1, p2, q0, q1, q2;
        load_v<ST>(v, j0, p0, p1, p2);
        load_v<ST>(v, j1, q0, q1, q2);
        // pure FMA chains: three DFMA per block row
        y0 = fma(b[0], p0, fma(b[1], p1, fma(b[2], p2, y0)));
        y1 = fma(b[3], p0, fma(b[4], p1, fma(b[5], p2, y1)));
        y2 = fma(b[6], p0, fma(b[7], p1, fma(b[8], p2, y2)));
        y0 = fma(c[0], q0, fma(c[1], q1, fma(c[2], q2, y0)));
        y1 = fma(c[3], q0, fma(c[4], q1, fma(c[5], q2, y1)));
        y2 = fma(c[6], q0, fma(c[7], q1, fma(c[8], q2, y2)));
    }
    if (k < len) {
        const size_t s0 = (size_t)(base + k);
        const int j0 = __ldg(a.scol + s0 * 32 + lane);
        const double* B = a.sval + s0 * 288 + lane;
        double p0, p1, p2;
        load_v<ST>(v, j0, p0, p1, p2);
        y0 = fma(__ldg(B + 0), p0, fma(__ldg(B + 32), p1, fma(__ldg(B + 64), p2, y0)));
        y1 = fma(__ldg(B + 96), p0, fma(__ldg(B + 128), p1, fma(__ldg(B + 160), p2, y1)));
        y2 = fma(__ldg(B + 192), p0, fma(__ldg(B + 224), p1, fma(__ldg(B + 256), p2, y2)));
    }
    for (int e = a.crp[i]; e < a.crp[i + 1]; ++e) {
        const int j = a.cci[e];
        const double* B = a.cva + 9 * (size_t)e;
        double v0, v1, v2;
        load_v<ST>(v, j, v0, v1, v2);
        y0 = fma(B[0], v0, fma(B[1], v1, fma(B[2], v2, y0)));
        y1 = fma(B[3], v0, fma(B[4], v1, fma(B[5], v2, y1)));
        y2 = fma(B[6], v0, fma(B[7], v1, fma(B[8], v2, y2)));
    }
}

// y = A v with FP32 copies of the values (v32: the sliced-ELL layout of sval; c32: the contact
// blocks) and an FP32 vector (stride 4), accumulated in FP32: the multigrid's smoothing products
__device__ __forceinline__ void row_apply_f32(const PCGArgs& a, const float* __restrict__ v32, const float* __restrict__ c32, int i,
                                              const float4* __restrict__ v, float& y0, float& y1, float& y2) {
    y0 = y1 = y2 = 0.f;
    const int sl = i >> 5, lane = i & 31;
    const int base = a.soff[sl], len = a.rlen[i];
    int k = 0;
    for (; k + 1 < len; k += 2) {
        const size_t s0 = (size_t)(base + k), s1 = s0 + 1;
        const int j0 = __ldg(a.scol + s0 * 32 + lane), j1 = __ldg(a.scol + s1 * 32 + lane);
        const float* B = v32 + s0 * 288 + lane;
        const float* C = v32 + s1 * 288 + lane;
        float b[9], c[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            b[q] = __ldg(B + 32 * q);
            c[q] = __ldg(C + 32 * q);
        }
        const float4 p = __ldg(v + j0), q = __ldg(v + j1);
        y0 = fmaf(b[0], p.x, fmaf(b[1], p.y, fmaf(b[2], p.z, y0)));
        y1 = fmaf(b[3], p.x, fmaf(b[4], p.y, fmaf(b[5], p.z, y1)));
        y2 = fmaf(b[6], p.x, fmaf(b[7], p.y, fmaf(b[8], p.z, y2)));
        y0 = fmaf(c[0], q.x, fmaf(c[1], q.y, fmaf(c[2], q.z, y0)));
        y1 = fmaf(c[3], q.x, fmaf(c[4], q.y, fmaf(c[5], q.z, y1)));
        y2 = fmaf(c[6], q.x, fmaf(c[7], q.y, fmaf(c[8], q.z, y2)));
    }
    if (k < len) {
        const size_t s0 = (size_t)(base + k);
        const int j0 = __ldg(a.scol + s0 * 32 + lane);
        const float* B = v32 + s0 * 288 + lane;
        const float4 p = __ldg(v + j0);
        y0 = fmaf(__ldg(B + 0), p.x, fmaf(__ldg(B + 32), p.y, fmaf(__ldg(B + 64), p.z, y0)));
        y1 = fmaf(__ldg(B + 96), p.x, fmaf(__ldg(B + 128), p.y, fmaf(__ldg(B + 160), p.z, y1)));
        y2 = fmaf(__ldg(B + 192), p.x, fmaf(__ldg(B + 224), p.y, fmaf(__ldg(B + 256), p.z, y2)));
    }
    for (int e = a.crp[i]; e < a.crp[i + 1]; ++e) {
        const float* B = c32 + 9 * (size_t)e;
        const float4 p = __ldg(v + a.cci[e]);
        y0 = fmaf(B[0], p.x, fmaf(B[1], p.y, fmaf(B[2], p.z, y0)));
        y1 = fmaf(B[3], p.x, fmaf(B[4], p.y, fmaf(B[5], p.z, y1)));
        y2 = fmaf(B[6], p.x, fmaf(B[7], p.y, fmaf(B[8], p.z, y2)));
    }
}

// block sums of NV per-thread values into the shared array out[NV] (valid in every thread on
// return).  The values go through shared memory and warp c sums component c (four rows per lane,
// then a shuffle tree), so the block spends about 8 FP64 adds per component per lane of one warp
// instead of a full shuffle tree in every warp; the order is fixed.
template <int NV>
__device__ __forceinline__ void block_sums(const double (&v)[NV], double* out) {
    __shared__ double sv[NV][PCG_THREADS];
#pragma unroll
    for (int c = 0; c < NV; ++c) sv[c][threadIdx.x] = v[c];
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int c = wid; c < NV; c += PCG_THREADS / 32) {
        double x = sv[c][lane];
#pragma unroll
        for (int k = 1; k < PCG_THREADS / 32; ++k) x += sv[c][lane + 32 * k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) out[c] = x;
    }
    __syncthreads();
}

// restriction of one block's residuals onto the rigid-body modes of its aggregate: the block's
// sum over rows of (r_i, d_i x r_i) into cs_part[block] (fixed shuffle / shared order); the
// aggregate's last block to finish (atomic ticket) sums its blocks' partials in block order
// into cs_g, so the aggregate totals need no extra launch and are reproducible
__device__ __forceinline__ void block_restrict(const PCGArgs& a, bool valid, int i, const double (&r)[3], const double (&d)[3]) {
    __shared__ double tot[6];
    __shared__ bool last;
    double v[6] = {0, 0, 0, 0, 0, 0};
    if (valid) {
        v[0] = r[0];
        v[1] = r[1];
        v[2] = r[2];
        v[3] = d[1] * r[2] - d[2] * r[1];
        v[4] = d[2] * r[0] - d[0] * r[2];
        v[5] = d[0] * r[1] - d[1] * r[0];
    }
    block_sums<6>(v, tot);
    const int I = blockIdx.x / a.cs_blocks;
    if (threadIdx.x < 6) {
        a.cs_part[6 * (size_t)blockIdx.x + threadIdx.x] = tot[threadIdx.x];
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nblocks = min((int)gridDim.x - I * a.cs_blocks, a.cs_blocks);
        last = atomicAdd(&a.cs_ticket[I], 1) == nblocks - 1;
    }
    __syncthreads();
    if (last && threadIdx.x < 6) {
        __threadfence();
        const int b0 = I * a.cs_blocks, b1 = min((int)gridDim.x, b0 + a.cs_blocks);
        double t = 0.0;
        for (int b = b0; b < b1; ++b) t += *(volatile double*)&a.cs_part[6 * (size_t)b + threadIdx.x];
        a.cs_g[6 * I + threadIdx.x] = t;
        if (threadIdx.x == 0) a.cs_ticket[I] = 0;
    }
}

// block-Jacobi preconditioner: the inverse of vertex i's 3x3 diagonal block (elastic + contact);
// identity at Dirichlet vertices
__device__ __forceinline__ void jacobi_block_inverse(const PCGArgs& a, int i, bool fx, double (&Mi)[9]) {
    if (fx) {
        for (int k = 0; k < 9; ++k) Mi[k] = (k % 4 == 0) ? 1.0 : 0.0;
    } else {
        double D[9];
        const double* E = a.sval + (size_t)(a.diag_spos[i] >> 5) * 288 + (a.diag_spos[i] & 31);
        for (int k = 0; k < 9; ++k) D[k] = E[32 * k];
        for (int k = a.crp[i]; k < a.crp[i + 1]; ++k)
            if (a.cci[k] == i)
                for (int q = 0; q < 9; ++q) D[q] += a.cva[9 * (size_t)k + q];
        const double c00 = D[4] * D[8] - D[5] * D[7], c01 = D[5] * D[6] - D[3] * D[8], c02 = D[3] * D[7] - D[4] * D[6];
        const double id = 1.0 / (D[0] * c00 + D[1] * c01 + D[2] * c02);
        Mi[0] = c00 * id;
        Mi[1] = (D[2] * D[7] - D[1] * D[8]) * id;
        Mi[2] = (D[1] * D[5] - D[2] * D[4]) * id;
        Mi[3] = c01 * id;
        Mi[4] = (D[0] * D[8] - D[2] * D[6]) * id;
        Mi[5] = (D[2] * D[3] - D[0] * D[5]) * id;
        Mi[6] = c02 * id;
        Mi[7] = (D[1] * D[6] - D[0] * D[7]) * id;
        Mi[8] = (D[0] * D[4] - D[1] * D[3]) * id;
    }
}

}  // namespace fipc
