// Per-element and per-constraint kernels: Neo-Hookean tets, IPC barrier rows, energies,
// the vector updates of the Newton loop, and the stateless C-ABI entries around them.
#include <cuda_runtime.h>

#include "barrier.cuh"
#include "ccd.cuh"
#include "ctx.cuh"
#include "geometry.cuh"
#include "nh.cuh"
#include "profile.cuh"

namespace fipc {

std::atomic<long long> g_launches{0};

// ---------------------------------------------------------------- Neo-Hookean element
// One thread per tet: gradient g[T,12] and the 10 upper Hessian blocks of dt^2 vol0 psi(F)
// (NEWTON_IPC.py:568-691); energy E[T] when requested.  Hessian layouts:
//  * TILED = false: Hu[T][90] (the stateless entry point's documented layout);
//  * TILED = true (the context's assembly input): tiles of 32 consecutive tets, block b of tet
//    e at Hu[((e / 32) * 10 + b) * 288 + (e % 32) * 9 + i], so each warp's block b is one
//    contiguous 2,304-byte run, staged through shared memory and stored as full sectors (a
//    per-thread 720-byte record written straight from registers reaches DRAM about twice).
//    The buffer holds whole tiles.
template <bool TILED>
__global__ void __launch_bounds__(128) k_elasticity(int nT, const int4* __restrict__ tets, const double* __restrict__ x,
                                                    const double* __restrict__ dminv, const double* __restrict__ vol,
                                                    const double* __restrict__ lam, const double* __restrict__ mu, double dt2,
                                                    double* __restrict__ E, double* __restrict__ g, double* __restrict__ Hu) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (!TILED && e >= nT) return;
    double ge[12], He[90];
    if (e < nT) {
        const int4 t = tets[e];
        v3 X[4] = {ld3(x, t.x), ld3(x, t.y), ld3(x, t.z), ld3(x, t.w)};
        double IB[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) IB[i] = dminv[9 * (size_t)e + i];
        const double psi = nh_element(X, IB, lam[e], mu[e], dt2 * vol[e], ge, He);
        if (E) E[e] = psi;
#pragma unroll
        for (int i = 0; i < 12; ++i) g[12 * (size_t)e + i] = ge[i];
    } else {
#pragma unroll
        for (int i = 0; i < 90; ++i) He[i] = 0.0;
    }
    if (!TILED) {
#pragma unroll
        for (int i = 0; i < 90; ++i) Hu[90 * (size_t)e + i] = He[i];
        return;
    }
    if ((e & ~31) >= nT) return;                   // a whole warp past the last tile
    __shared__ double stage[4][32 * 9];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double* tile = Hu + (size_t)(e >> 5) * 2880;   // the warp's 32 tets share e >> 5
#pragma unroll
    for (int b = 0; b < 10; ++b) {
#pragma unroll
        for (int i = 0; i < 9; ++i) stage[w][lane * 9 + i] = He[b * 9 + i];
        __syncwarp();
#pragma unroll
        for (int k = 0; k < 9; ++k) tile[b * 288 + k * 32 + lane] = stage[w][k * 32 + lane];
        __syncwarp();
    }
}

// ---------------------------------------------------------------- barrier rows
// One thread per constraint row: E[n], g[n,12] (3 nv used) and Hb[n,16,9] 3x3 vertex blocks
// (v*4+w, nv x nv used) of the projected barrier Hessian (common/math/ipc.py *_g_and_H).
__global__ void __launch_bounds__(128) k_barrier_rows(int type, int n, const int4* __restrict__ rows,
                                                      const double* __restrict__ x, const double* __restrict__ x0, double dh2,
                                                      double kappa, const double* __restrict__ kap_s, const int* __restrict__ vscene,
                                                      double* __restrict__ E, double* __restrict__ g, double* __restrict__ Hb,
                                                      int* __restrict__ status) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int4 q = rows[r];
    if (kap_s) kappa = kap_s[vscene[q.x]];   // batched scenes: the row's own scene
    const int nv = type_nverts(type);
    const int id[4] = {q.x, q.y, nv > 2 ? q.z : q.x, nv > 3 ? q.w : q.x};
    v3 X[4], X0[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        X[k] = ld3(x, id[k]);
        X0[k] = type >= T_EEM ? ld3(x0, id[k]) : mk(0, 0, 0);
    }
    double e, gg[12], hb[144];
    const int st = barrier_row(type, X, X0, dh2, kappa, g != nullptr, &e, gg, hb);
    if (st && status) atomicOr(status, 1);
    if (E) E[r] = e;
    if (!g) return;
    for (int i = 0; i < 3 * nv; ++i) g[12 * (size_t)r + i] = gg[i];
    for (int v = 0; v < nv; ++v)
        for (int w = 0; w < nv; ++w)
            for (int i = 0; i < 9; ++i) Hb[144 * (size_t)r + (v * 4 + w) * 9 + i] = hb[(v * 4 + w) * 9 + i];
}

// ---------------------------------------------------------------- deterministic reductions
// Fixed grid (RED_BLOCKS x RED_THREADS), grid-stride accumulation, fixed tree: the same
// inputs always give the same bits.
__device__ __forceinline__ double block_sum(double v, double* sh) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

// inertia 0.5 m |x - xt|^2  (NEWTON_IPC.py:518-519)
__global__ void __launch_bounds__(RED_THREADS) k_energy_inertia(int nV, const double* __restrict__ x, const double* __restrict__ xt,
                                                                const double* __restrict__ m, double* __restrict__ part) {
    __shared__ double sh[RED_THREADS];
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nV; i += gridDim.x * blockDim.x) {
        const v3 d = ld3(x, i) - ld3(xt, i);
        acc += 0.5 * m[i] * sq(d);
    }
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// elasticity dt^2 vol0 psi(F) from |F|^2 and det F (NEWTON_IPC.py:521-525)
__global__ void __launch_bounds__(RED_THREADS) k_energy_elastic(int nT, const int4* __restrict__ tets, const double* __restrict__ x,
                                                                const double* __restrict__ dminv, const double* __restrict__ vol,
                                                                const double* __restrict__ lam, const double* __restrict__ mu,
                                                                double dt2, double* __restrict__ part) {
    __shared__ double sh[RED_THREADS];
    double acc = 0.0;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nT; e += gridDim.x * blockDim.x) {
        const int4 t = tets[e];
        const v3 X[4] = {ld3(x, t.x), ld3(x, t.y), ld3(x, t.z), ld3(x, t.w)};
        double IB[9], F[9];
        for (int i = 0; i < 9; ++i) IB[i] = dminv[9 * (size_t)e + i];
        deformation_gradient(X, IB, F);
        acc += nh_psi_F(F, lam[e], mu[e]) * dt2 * vol[e];
    }
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// barrier energies of one list (NEWTON_IPC.py:527-541)
__global__ void __launch_bounds__(RED_THREADS) k_energy_barrier(int type, int n, const int4* __restrict__ rows,
                                                                const double* __restrict__ x, const double* __restrict__ x0,
                                                                double dh2, double kappa, const double* __restrict__ kap_s,
                                                                const int* __restrict__ vscene, double* __restrict__ part) {
    __shared__ double sh[RED_THREADS];
    double acc = 0.0;
    const int nv = type_nverts(type);
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const int4 q = rows[r];
        const double kap = kap_s ? kap_s[vscene[q.x]] : kappa;
        const int id[4] = {q.x, q.y, nv > 2 ? q.z : q.x, nv > 3 ? q.w : q.x};
        v3 X[4], X0[4];
        for (int k = 0; k < 4; ++k) {
            X[k] = ld3(x, id[k]);
            X0[k] = type >= T_EEM ? ld3(x0, id[k]) : mk(0, 0, 0);
        }
        double e;
        barrier_row(type, X, X0, dh2, kap, 0, &e, nullptr, nullptr);
        acc += e;
    }
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// sum of n_parts partial vectors of RED_BLOCKS each, in fixed order
__global__ void k_sum_parts(int n_parts, const double* __restrict__ part, double* __restrict__ out) {
    __shared__ double sh[RED_THREADS];
    double acc = 0.0;
    for (int p = 0; p < n_parts; ++p)
        for (int i = threadIdx.x; i < RED_BLOCKS; i += blockDim.x) acc += part[p * RED_BLOCKS + i];
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) *out = s;
}

// max |p| (NEWTON_IPC.py:805-812)
__global__ void __launch_bounds__(RED_THREADS) k_absmax(int n, const double* __restrict__ p, double* __restrict__ part) {
    __shared__ double sh[RED_THREADS];
    double m = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) m = fmax(m, fabs(p[i]));
    sh[threadIdx.x] = m;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}
__global__ void k_max_parts(const double* __restrict__ part, double* __restrict__ out) {
    __shared__ double sh[RED_THREADS];
    double m = 0.0;
    for (int i = threadIdx.x; i < RED_BLOCKS; i += blockDim.x) m = fmax(m, part[i]);
    sh[threadIdx.x] = m;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

// ---------------------------------------------------------------- vector updates
// NEWTON_IPC.py:497-502
__global__ void k_xn_xtilde(int nV, const double* __restrict__ x, const double* __restrict__ v, double dt, double gravity,
                            double* __restrict__ xn, double* __restrict__ xt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * nV) return;
    const double xi = x[i];
    xn[i] = xi;
    double t = xi + dt * v[i];
    if (i % 3 == 1) t += dt * dt * gravity;
    xt[i] = t;
}
// NEWTON_IPC.py:505-511
__global__ void k_move_nodes(int nV, const unsigned char* __restrict__ fixed, const double* __restrict__ target,
                             double* __restrict__ x, double* __restrict__ xt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * nV) return;
    if (fixed[i / 3]) {
        x[i] = target[i];
        xt[i] = target[i];
    }
}
// settings['dirichlet'](t) of projects/FastIPC/reader.py:154-357 evaluated on the device for
// schedules that are rigid motions of vertex groups: group g moves its rest positions by the
// rotation about the unit axis a through c at omega rad/s (Rodrigues' formula), then
// translates them by u t.  motion[g] = (c[3], a[3], omega, u[3]).  Vertices with group < 0
// are free and keep their rest position as target, as the reference's copy of the particles
// does.  One thread per vertex.
__global__ void k_dirichlet_script(int nV, const double* __restrict__ xr, const int* __restrict__ group, int n_groups,
                                   const double* __restrict__ motion, double t, unsigned char* __restrict__ fixed,
                                   double* __restrict__ target) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nV) return;
    const int g = group[i];
    const double px = xr[3 * (size_t)i], py = xr[3 * (size_t)i + 1], pz = xr[3 * (size_t)i + 2];
    if (g < 0 || g >= n_groups) {
        fixed[i] = 0;
        target[3 * (size_t)i] = px;
        target[3 * (size_t)i + 1] = py;
        target[3 * (size_t)i + 2] = pz;
        return;
    }
    const double* m = motion + 10 * (size_t)g;
    const double rx = px - m[0], ry = py - m[1], rz = pz - m[2];
    const double ax = m[3], ay = m[4], az = m[5];
    double sn, cs;
    sincos(m[6] * t, &sn, &cs);
    // R r = r cos + (a x r) sin + a (a . r)(1 - cos)
    const double ad = (ax * rx + ay * ry + az * rz) * (1.0 - cs);
    const double qx = rx * cs + (ay * rz - az * ry) * sn + ax * ad;
    const double qy = ry * cs + (az * rx - ax * rz) * sn + ay * ad;
    const double qz = rz * cs + (ax * ry - ay * rx) * sn + az * ad;
    fixed[i] = 1;
    target[3 * (size_t)i] = m[0] + qx + m[7] * t;
    target[3 * (size_t)i + 1] = m[1] + qy + m[8] * t;
    target[3 * (size_t)i + 2] = m[2] + qz + m[9] * t;
}
// NEWTON_IPC.py:792-796
__global__ void k_apply_sol(int n, const double* __restrict__ xprev, const double* __restrict__ sol, double alpha,
                            double* __restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = xprev[i] + sol[i] * alpha;
}
// NEWTON_IPC.py:799-802
__global__ void k_compute_v(int n, const double* __restrict__ x, const double* __restrict__ xn, double dt,
                            double* __restrict__ v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = (x[i] - xn[i]) / dt;
}

// ---------------------------------------------------------------- explicit-pair CCD (tests)
__global__ void k_ccd_pairs(int kind, int n, const double* __restrict__ xq, const double* __restrict__ pq, double eta,
                            double* __restrict__ toc) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    v3 Q[4], D[4];
    for (int k = 0; k < 4; ++k) {
        Q[k] = load3(xq + 12 * (size_t)c, k);
        D[k] = load3(pq + 12 * (size_t)c, k);
    }
    if (kind == 0) toc[c] = pt_ccd(Q[0], Q[1], Q[2], Q[3], D[0], D[1], D[2], D[3], eta, pt_dist2(Q[0], Q[1], Q[2], Q[3]));
    else toc[c] = ee_ccd(Q[0], Q[1], Q[2], Q[3], D[0], D[1], D[2], D[3], eta, ee_dist2(Q[0], Q[1], Q[2], Q[3]));
}
__global__ void k_inversion_pairs(int n, const double* __restrict__ xs, const double* __restrict__ ps, double eta,
                                  double* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    v3 X[4], P[4];
    for (int k = 0; k < 4; ++k) {
        X[k] = load3(xs + 12 * (size_t)c, k);
        P[k] = load3(ps + 12 * (size_t)c, k);
    }
    out[c] = inversion_free_step(X, P, eta);
}

// ---------------------------------------------------------------- host launchers
static inline int nblk(long long n, int b) { return (int)((n + b - 1) / b); }

int launch_elasticity(int nT, const int* tets, const double* x, const double* dminv, const double* vol, const double* lam,
                      const double* mu, double dt, double* E, double* g, double* Hu, cudaStream_t s, bool tiled) {
    if (nT <= 0) return FIPC_OK;
    {
        // per tet: 4 indices, 4 positions, Dm^-1, vol/lam/mu in; gradient and 10 blocks out
        ProfScope ps(PK_ELASTICITY, s, nT * (16.0 + 96.0 + 72.0 + 24.0 + 96.0 + 720.0 + (E ? 8.0 : 0.0)), 0.0);
        if (tiled)
            k_elasticity<true><<<nblk(nT, 128), 128, 0, s>>>(nT, (const int4*)tets, x, dminv, vol, lam, mu, dt * dt, E, g, Hu);
        else
            k_elasticity<false><<<nblk(nT, 128), 128, 0, s>>>(nT, (const int4*)tets, x, dminv, vol, lam, mu, dt * dt, E, g, Hu);
    }
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int launch_barrier_rows(int type, int n, const int* rows, const double* x, const double* x0, double dh2, double kappa,
                        const double* kap_s, const int* vscene, double* E, double* g, double* Hb, int* status, cudaStream_t s) {
    if (n <= 0) return FIPC_OK;
    k_barrier_rows<<<nblk(n, 128), 128, 0, s>>>(type, n, (const int4*)rows, x, x0, dh2, kappa, kap_s, vscene, E, g, Hb, status);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

// total incremental potential into *out (device); part: scratch of (2 + N_TYPES) * RED_BLOCKS
int launch_energy(const fipc_ctx* c, const double* x, const double* xt, const int* const* rows, const int* counts, double* part,
                  double* out, cudaStream_t s) {
    k_energy_inertia<<<RED_BLOCKS, RED_THREADS, 0, s>>>(c->nV, x, xt, c->mass, part);
    FIPC_LAUNCHED();
    k_energy_elastic<<<RED_BLOCKS, RED_THREADS, 0, s>>>(c->nT, (const int4*)c->tets, x, c->dminv, c->vol, c->lam, c->mu,
                                                       c->dt * c->dt, part + RED_BLOCKS);
    FIPC_LAUNCHED();
    int np = 2;
    for (int t = 0; t < N_TYPES; ++t) {
        if (counts[t] <= 0) continue;
        k_energy_barrier<<<RED_BLOCKS, RED_THREADS, 0, s>>>(t, counts[t], (const int4*)rows[t], x, c->x0, c->dhat2, c->kappa,
                                                           c->n_scenes > 1 ? c->s_kappa : nullptr, c->v_scene,
                                                           part + (size_t)np * RED_BLOCKS);
        FIPC_LAUNCHED();
        ++np;
    }
    k_sum_parts<<<1, RED_THREADS, 0, s>>>(np, part, out);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int launch_absmax(int n, const double* p, double* part, double* out, cudaStream_t s) {
    k_absmax<<<RED_BLOCKS, RED_THREADS, 0, s>>>(n, p, part);
    FIPC_LAUNCHED();
    k_max_parts<<<1, RED_THREADS, 0, s>>>(part, out);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

}  // namespace fipc

using namespace fipc;

extern "C" {

int fipc_elasticity(int n_tets, const int* tets, const double* x, const double* dm_inv, const double* vol, const double* lam,
                    const double* mu, double dt, double* E, double* g, double* Hu, void* stream) {
    if (n_tets < 0 || !tets || !x || !dm_inv || !vol || !lam || !mu || !g || !Hu) return FIPC_ERR_ARGUMENT;
    return launch_elasticity(n_tets, tets, x, dm_inv, vol, lam, mu, dt, E, g, Hu, (cudaStream_t)stream, false);
}

int fipc_barrier_rows(int type, int n_rows, const int* rows, const double* x, const double* x0, double dhat2, double kappa,
                      double* E, double* g, double* H, void* stream) {
    if (type < 0 || type >= N_TYPES || n_rows < 0 || !rows || !x || (type >= T_EEM && !x0)) return FIPC_ERR_ARGUMENT;
    if ((g == nullptr) != (H == nullptr)) return FIPC_ERR_ARGUMENT;
    return launch_barrier_rows(type, n_rows, rows, x, x0, dhat2, kappa, nullptr, nullptr, E, g, H, nullptr, (cudaStream_t)stream);
}

int fipc_ccd_pairs(int kind, int n, const double* xq, const double* pq, double eta, double* toc, void* stream) {
    if ((kind != 0 && kind != 1) || n < 0 || !xq || !pq || !toc) return FIPC_ERR_ARGUMENT;
    if (n == 0) return FIPC_OK;
    k_ccd_pairs<<<nblk(n, 128), 128, 0, (cudaStream_t)stream>>>(kind, n, xq, pq, eta, toc);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc_inversion_free_pairs(int n, const double* xs, const double* ps, double eta, double* out, void* stream) {
    if (n < 0 || !xs || !ps || !out) return FIPC_ERR_ARGUMENT;
    if (n == 0) return FIPC_OK;
    k_inversion_pairs<<<nblk(n, 128), 128, 0, (cudaStream_t)stream>>>(n, xs, ps, eta, out);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc_compute_xn_and_xtilde(int n_verts, const double* x, const double* v, double dt, double gravity, double* xn, double* xtilde,
                               void* stream) {
    if (n_verts < 0 || !x || !v || !xn || !xtilde) return FIPC_ERR_ARGUMENT;
    if (n_verts == 0) return FIPC_OK;
    k_xn_xtilde<<<nblk(3ll * n_verts, 256), 256, 0, (cudaStream_t)stream>>>(n_verts, x, v, dt, gravity, xn, xtilde);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc_move_nodes(int n_verts, const unsigned char* fixed, const double* target, double* x, double* xtilde, void* stream) {
    if (n_verts < 0 || !fixed || !target || !x || !xtilde) return FIPC_ERR_ARGUMENT;
    if (n_verts == 0) return FIPC_OK;
    k_move_nodes<<<nblk(3ll * n_verts, 256), 256, 0, (cudaStream_t)stream>>>(n_verts, fixed, target, x, xtilde);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc_dirichlet_script(int n_verts, const double* x_rest, const int* group, int n_groups, const double* motion, double t,
                          unsigned char* fixed, double* target, void* stream) {
    if (n_verts < 0 || n_groups < 0 || !x_rest || !group || (n_groups > 0 && !motion) || !fixed || !target)
        return FIPC_ERR_ARGUMENT;
    if (n_verts == 0) return FIPC_OK;
    k_dirichlet_script<<<nblk(n_verts, 256), 256, 0, (cudaStream_t)stream>>>(n_verts, x_rest, group, n_groups, motion, t, fixed,
                                                                             target);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc_apply_sol(int n_verts, const double* xprev, const double* sol, double alpha, double* x, void* stream) {
    if (n_verts < 0 || !xprev || !sol || !x) return FIPC_ERR_ARGUMENT;
    if (n_verts == 0) return FIPC_OK;
    k_apply_sol<<<nblk(3ll * n_verts, 256), 256, 0, (cudaStream_t)stream>>>(3 * n_verts, xprev, sol, alpha, x);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc_compute_v(int n_verts, const double* x, const double* xn, double dt, double* v, void* stream) {
    if (n_verts < 0 || !x || !xn || !v || dt == 0.0) return FIPC_ERR_ARGUMENT;
    if (n_verts == 0) return FIPC_OK;
    k_compute_v<<<nblk(3ll * n_verts, 256), 256, 0, (cudaStream_t)stream>>>(3 * n_verts, x, xn, dt, v);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

long long fipc_launch_count(void) { return g_launches.load(); }

const char* fipc_status_string(int status) {
    switch (status) {
        case FIPC_OK: return "ok";
        case FIPC_ERR_CAPACITY: return "capacity exceeded";
        case FIPC_ERR_ITERATION: return "iteration limit reached";
        case FIPC_ERR_NONFINITE: return "non-finite value";
        case FIPC_ERR_CUDA: return "CUDA error";
        case FIPC_ERR_ARGUMENT: return "invalid argument";
        case FIPC_ERR_IO: return "file I/O error";
        default: return "unknown status";
    }
}

}  // extern "C"
