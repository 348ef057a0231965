// Allocation-free variant of the incremental-potential energy (compute_energy).
//
// Some callers cannot allocate device memory while they run: a host application that owns
// every byte of device memory in one arena reserved at start-up (a game or VFX engine plug-in,
// a real-time control loop) forbids cudaMalloc later, because it synchronises the device, can
// fail when the arena has taken the memory, and breaks a fixed memory budget.  Such a caller
// also cannot create a scene context (fipc_ctx_create allocates).  This entry point needs
// neither: the caller passes every input and the output; the only scratch, the per-block
// partial sums of the reduction, lives in the file-scope array below, which exists once per
// GPU that loads the library and stays allocated until the process exits.
//
// Set-up: the first call on a device (with that device current) looks up the array's device
// address with cudaGetSymbolAddress, caches it for that device, and loads this file's kernels
// (under CUDA's lazy module loading a kernel's first launch would otherwise load it, and
// loading can allocate device memory and synchronise).  So make that first call at start-up,
// before the arena takes the device memory and before any stream capture; a call with zero
// vertices, tets and rows does the set-up and writes 0.  The cached address does not survive
// cudaDeviceReset: a process that resets a device must not call this entry point afterwards.
// Every call on a device shares the one array and overwrites it, so calls whose kernels
// overlap on the GPU (different streams, different host threads) race; order them on one
// stream.
#include <cuda_runtime.h>

#include <mutex>

#include "barrier.cuh"
#include "ctx.cuh"
#include "nh.cuh"

namespace fipc {

// maximum number of per-block partial sums: one per 256 vertices, tets or constraint rows,
// i.e. about 16.7 million elements in total per call (512 KiB of device memory)
constexpr int NOALLOC_MAX_PARTIALS = 1 << 16;
constexpr int NOALLOC_THREADS = 256;
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) double g_noalloc_partials[NOALLOC_MAX_PARTIALS];

namespace {
std::mutex g_noalloc_mu;
double* g_noalloc_addr[NOALLOC_MAX_DEVICES] = {nullptr};

int noalloc_load_kernels();

// device address of g_noalloc_partials for the current device (looked up once per device,
// which also loads this file's kernels on that device)
int noalloc_scratch(double** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES) return FIPC_ERR_CUDA;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_partials) != cudaSuccess || !p) return FIPC_ERR_CUDA;
        const int st = noalloc_load_kernels();
        if (st) return st;
        g_noalloc_addr[dev] = static_cast<double*>(p);
    }
    *out = g_noalloc_addr[dev];
    return FIPC_OK;
}
}  // namespace

__device__ __forceinline__ void na_block_store(double v, double* part) {
    __shared__ double sh[NOALLOC_THREADS];
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = NOALLOC_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// one thread per vertex: 0.5 m |x - xt|^2 (NEWTON_IPC.py:518-519)
__global__ void __launch_bounds__(NOALLOC_THREADS) k_na_inertia(int nV, const double* __restrict__ x, const double* __restrict__ xt,
                                                                const double* __restrict__ m, double* __restrict__ part) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0.0;
    if (i < nV) e = 0.5 * m[i] * sq(ld3(x, i) - ld3(xt, i));
    na_block_store(e, part);
}

// one thread per tet: dt^2 vol0 psi(F) (NEWTON_IPC.py:521-525)
__global__ void __launch_bounds__(NOALLOC_THREADS) k_na_elastic(int nT, const int4* __restrict__ tets, const double* __restrict__ x,
                                                                const double* __restrict__ dminv, const double* __restrict__ vol,
                                                                const double* __restrict__ lam, const double* __restrict__ mu, double dt2,
                                                                double* __restrict__ part) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    double acc = 0.0;
    if (e < nT) {
        const int4 t = tets[e];
        const v3 X[4] = {ld3(x, t.x), ld3(x, t.y), ld3(x, t.z), ld3(x, t.w)};
        double IB[9], F[9];
        for (int i = 0; i < 9; ++i) IB[i] = dminv[9 * (size_t)e + i];
        deformation_gradient(X, IB, F);
        acc = nh_psi_F(F, lam[e], mu[e]) * dt2 * vol[e];
    }
    na_block_store(acc, part);
}

// one thread per constraint row of one list (NEWTON_IPC.py:527-541)
__global__ void __launch_bounds__(NOALLOC_THREADS) k_na_barrier(int type, int n, const int4* __restrict__ rows,
                                                                const double* __restrict__ x, const double* __restrict__ x0,
                                                                double dh2, double kappa, double* __restrict__ part) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0.0;
    if (r < n) {
        const int nv = type_nverts(type);
        const int4 q = rows[r];
        const int id[4] = {q.x, q.y, nv > 2 ? q.z : q.x, nv > 3 ? q.w : q.x};
        v3 X[4], X0[4];
        for (int k = 0; k < 4; ++k) {
            X[k] = ld3(x, id[k]);
            X0[k] = type >= T_EEM ? ld3(x0, id[k]) : mk(0, 0, 0);
        }
        barrier_row(type, X, X0, dh2, kappa, 0, &e, nullptr, nullptr);
    }
    na_block_store(e, part);
}

// sum of the first `total` partials in index order (one block, fixed tree)
__global__ void __launch_bounds__(NOALLOC_THREADS) k_na_sum(int total, const double* __restrict__ part, double* __restrict__ out) {
    __shared__ double sh[NOALLOC_THREADS];
    double a = 0.0;
    for (int i = threadIdx.x; i < total; i += NOALLOC_THREADS) a += part[i];
    sh[threadIdx.x] = a;
    __syncthreads();
    for (int s = NOALLOC_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

namespace {
// cudaFuncGetAttributes loads a kernel on the current device, so the set-up call pays every
// module load and later calls launch already-loaded kernels
int noalloc_load_kernels() {
    cudaFuncAttributes a;
    if (cudaFuncGetAttributes(&a, k_na_inertia) != cudaSuccess) return FIPC_ERR_CUDA;
    if (cudaFuncGetAttributes(&a, k_na_elastic) != cudaSuccess) return FIPC_ERR_CUDA;
    if (cudaFuncGetAttributes(&a, k_na_barrier) != cudaSuccess) return FIPC_ERR_CUDA;
    if (cudaFuncGetAttributes(&a, k_na_sum) != cudaSuccess) return FIPC_ERR_CUDA;
    return FIPC_OK;
}

// int4 row and tet loads need 16-byte alignment, double loads 8-byte
inline bool al16(const void* p) { return ((uintptr_t)p & 15u) == 0; }
inline bool al8(const void* p) { return ((uintptr_t)p & 7u) == 0; }
}  // namespace

}  // namespace fipc

using namespace fipc;

extern "C" {

int fipc_compute_energy_noalloc(int n_verts, const double* x, const double* xtilde, const double* mass, int n_tets, const int* tets,
                                const double* dm_inv, const double* vol, const double* lam, const double* mu, double dt,
                                const int* counts_h, const int* const* rows_h, const double* x0, double dhat2, double kappa,
                                double* energy, void* stream) {
    if (n_verts < 0 || n_tets < 0 || !counts_h) return FIPC_ERR_ARGUMENT;
    // partials needed: one per 256 vertices, tets and rows of each list
    long long blocks = ((long long)n_verts + NOALLOC_THREADS - 1) / NOALLOC_THREADS +
                       ((long long)n_tets + NOALLOC_THREADS - 1) / NOALLOC_THREADS;
    for (int t = 0; t < N_TYPES; ++t) {
        if (counts_h[t] < 0) return FIPC_ERR_ARGUMENT;
        blocks += ((long long)counts_h[t] + NOALLOC_THREADS - 1) / NOALLOC_THREADS;
    }
    if (blocks > NOALLOC_MAX_PARTIALS) return FIPC_ERR_CAPACITY;   // beyond the fixed scratch
    if (!energy || (n_verts && (!x || !xtilde || !mass)) || (n_tets && (!tets || !dm_inv || !vol || !lam || !mu))) return FIPC_ERR_ARGUMENT;
    bool any_rows = false;
    for (int t = 0; t < N_TYPES; ++t) {
        if (counts_h[t] <= 0) continue;
        any_rows = true;
        if (!rows_h || !rows_h[t] || (t >= T_EEM && !x0)) return FIPC_ERR_ARGUMENT;
        if (!al16(rows_h[t])) return FIPC_ERR_ARGUMENT;
    }
    // a misaligned vector load would raise a sticky CUDA error in the caller's context: refuse
    // such pointers before anything is launched
    if (!al8(energy)) return FIPC_ERR_ARGUMENT;
    if ((n_verts || any_rows) && !al8(x)) return FIPC_ERR_ARGUMENT;
    if (n_verts && (!al8(xtilde) || !al8(mass))) return FIPC_ERR_ARGUMENT;
    if (n_tets && (!al16(tets) || !al8(x) || !al8(dm_inv) || !al8(vol) || !al8(lam) || !al8(mu))) return FIPC_ERR_ARGUMENT;
    if (x0 && !al8(x0)) return FIPC_ERR_ARGUMENT;
    double* part = nullptr;
    const int st = noalloc_scratch(&part);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    int off = 0;
    auto nb = [](long long n) { return (int)((n + NOALLOC_THREADS - 1) / NOALLOC_THREADS); };
    if (n_verts > 0) {
        k_na_inertia<<<nb(n_verts), NOALLOC_THREADS, 0, s>>>(n_verts, x, xtilde, mass, part + off);
        FIPC_LAUNCHED();
        off += nb(n_verts);
    }
    if (n_tets > 0) {
        k_na_elastic<<<nb(n_tets), NOALLOC_THREADS, 0, s>>>(n_tets, (const int4*)tets, x, dm_inv, vol, lam, mu, dt * dt, part + off);
        FIPC_LAUNCHED();
        off += nb(n_tets);
    }
    for (int t = 0; t < N_TYPES; ++t) {
        if (counts_h[t] <= 0) continue;
        k_na_barrier<<<nb(counts_h[t]), NOALLOC_THREADS, 0, s>>>(t, counts_h[t], (const int4*)rows_h[t], x, x0, dhat2, kappa, part + off);
        FIPC_LAUNCHED();
        off += nb(counts_h[t]);
    }
    k_na_sum<<<1, NOALLOC_THREADS, 0, s>>>(off, part, energy);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

}  // extern "C"
