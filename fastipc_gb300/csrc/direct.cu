// Direct solve of the Newton system: the role of the reference's CHOLMOD factorisation
// (projects/FastIPC/NEWTON_IPC.py:764-776), for the iterations where PCG reaches its iteration
// limit, or for callers that want the reference's exact solve.
//
// The elastic + inertia blocks and the contact blocks are expanded into scalar (row, column,
// value) entries with the Dirichlet edit of NEWTON_IPC.py:758-772 (rows and columns of fixed
// DOFs zero, one on their diagonal), radix-sorted by position and summed per position in a
// fixed order into CSR; the right-hand side gets zeros at fixed DOFs.  The factorisation is
// cuSOLVER's sparse Cholesky (a library routine, like CHOLMOD in the reference), loaded at run
// time so that the library builds and runs without it; when it cannot be loaded the entry
// point returns status 4 and the caller keeps its PCG result.
#include <cuda_runtime.h>
#include <cusolverSp.h>   // types and prototypes only: the library is opened with dlopen
#include <dlfcn.h>

#include <cub/cub.cuh>

#include "ctx.cuh"

namespace fipc {

int sell_to_bsr(fipc_ctx* c, double* out, cudaStream_t s);

namespace {

inline int nbd(long long n, int b) { return (int)((n + b - 1) / b); }

// one thread per block row: the 9 scalar entries of each elastic and contact block, in a
// fixed layout (row i's entries start at 9 * (elastic_rowptr[i] + contact_rowptr[i]))
__global__ void k_direct_entries(int nV, const int* __restrict__ erp, const int* __restrict__ eci, const double* __restrict__ ev,
                                 const int* __restrict__ crp, const int* __restrict__ cci, const double* __restrict__ cv,
                                 const unsigned char* __restrict__ fixed, unsigned long long* __restrict__ keys,
                                 double* __restrict__ vals) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nV) return;
    long long o = 9ll * (erp[i] + crp[i]);
    const bool fi = fixed[i];
    for (int pass = 0; pass < 2; ++pass) {
        const int* rp = pass ? crp : erp;
        const int* ci = pass ? cci : eci;
        const double* v = pass ? cv : ev;
        for (int k = rp[i]; k < rp[i + 1]; ++k) {
            const int j = ci[k];
            const bool fj = fixed[j];
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    double val = v[9ll * k + 3 * a + b];
                    if (fi || fj) val = (pass == 0 && i == j && a == b) ? 1.0 : 0.0;
                    keys[o] = ((unsigned long long)(3 * i + a) << 32) | (unsigned)(3 * j + b);
                    vals[o] = val;
                    ++o;
                }
        }
    }
}

__global__ void k_direct_sum(int nu, const unsigned long long* __restrict__ ukeys, const int* __restrict__ start,
                             const double* __restrict__ vals, double* __restrict__ out, int* __restrict__ col) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nu) return;
    double s = 0.0;
    for (int k = start[u]; k < start[u + 1]; ++k) s += vals[k];
    out[u] = s;
    col[u] = (int)(ukeys[u] & 0xffffffffull);
}

__global__ void k_direct_rowptr(int n, int nu, const unsigned long long* __restrict__ ukeys, int* __restrict__ rp) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r > n) return;
    const unsigned long long k = (unsigned long long)r << 32;
    int lo = 0, hi = nu;
    while (lo < hi) {
        const int m = (lo + hi) >> 1;
        if (ukeys[m] < k) lo = m + 1;
        else hi = m;
    }
    rp[r] = lo;
}

__global__ void k_direct_rhs(int nV, const double* __restrict__ rhs, const unsigned char* __restrict__ fixed, double* __restrict__ b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 3 * nV) b[i] = fixed[i / 3] ? 0.0 : rhs[i];
}

// cuSOLVER / cuSPARSE entry points, resolved once
struct SpLib {
    bool tried = false, ok = false;
    cusolverStatus_t (*create)(cusolverSpHandle_t*) = nullptr;
    cusolverStatus_t (*destroy)(cusolverSpHandle_t) = nullptr;
    cusolverStatus_t (*set_stream)(cusolverSpHandle_t, cudaStream_t) = nullptr;
    cusolverStatus_t (*chol)(cusolverSpHandle_t, int, int, const cusparseMatDescr_t, const double*, const int*, const int*,
                             const double*, double, int, double*, int*) = nullptr;
    cusparseStatus_t (*create_descr)(cusparseMatDescr_t*) = nullptr;
    cusparseStatus_t (*destroy_descr)(cusparseMatDescr_t) = nullptr;
    cusparseStatus_t (*set_type)(cusparseMatDescr_t, cusparseMatrixType_t) = nullptr;
    cusparseStatus_t (*set_base)(cusparseMatDescr_t, cusparseIndexBase_t) = nullptr;
};

SpLib& splib() {
    static SpLib L;
    if (L.tried) return L;
    L.tried = true;
    // the loader's search path first, then the toolkit's own directory
    auto open_any = [](const char* const* names) -> void* {
        for (int k = 0; names[k]; ++k)
            if (void* h = dlopen(names[k], RTLD_NOW | RTLD_LOCAL)) return h;
        return nullptr;
    };
    static const char* const sparse_names[] = {"libcusparse.so", "libcusparse.so.12", "/usr/local/cuda/lib64/libcusparse.so",
                                               "/usr/local/cuda/lib64/libcusparse.so.12", nullptr};
    static const char* const solver_names[] = {"libcusolver.so", "libcusolver.so.12", "/usr/local/cuda/lib64/libcusolver.so",
                                               "/usr/local/cuda/lib64/libcusolver.so.12", nullptr};
    void* hp = open_any(sparse_names);
    void* hs = open_any(solver_names);
    if (!hs || !hp) return L;
    L.create = (decltype(L.create))dlsym(hs, "cusolverSpCreate");
    L.destroy = (decltype(L.destroy))dlsym(hs, "cusolverSpDestroy");
    L.set_stream = (decltype(L.set_stream))dlsym(hs, "cusolverSpSetStream");
    L.chol = (decltype(L.chol))dlsym(hs, "cusolverSpDcsrlsvchol");
    L.create_descr = (decltype(L.create_descr))dlsym(hp, "cusparseCreateMatDescr");
    L.destroy_descr = (decltype(L.destroy_descr))dlsym(hp, "cusparseDestroyMatDescr");
    L.set_type = (decltype(L.set_type))dlsym(hp, "cusparseSetMatType");
    L.set_base = (decltype(L.set_base))dlsym(hp, "cusparseSetMatIndexBase");
    L.ok = L.create && L.destroy && L.set_stream && L.chol && L.create_descr && L.destroy_descr && L.set_type && L.set_base;
    return L;
}

struct DevMem {
    void* p = nullptr;
    ~DevMem() {
        if (p) cudaFree(p);
    }
    bool alloc(size_t n) { return cudaMalloc(&p, n ? n : 8) == cudaSuccess; }
    template <class T>
    T* as() const { return (T*)p; }
};

}  // namespace
}  // namespace fipc

using namespace fipc;

extern "C" {

int fipc_solve_system_direct(fipc_ctx* c, const unsigned char* fixed, double* sol, int* nnz_h, void* stream) {
    if (!c || !fixed || !sol) return FIPC_ERR_ARGUMENT;
    SpLib& L = splib();
    if (!L.ok) return FIPC_ERR_CUDA;
    cudaStream_t s = (cudaStream_t)stream;
    const int nV = c->nV, n = 3 * nV;
    // block row pointers of both matrices on the host sizes the entry layout
    int e_nnzb = c->nnzb, c_nnzb = c->c_nnzb;
    const long long N = 9ll * (e_nnzb + c_nnzb);
    if (N >= (1ll << 31)) return FIPC_ERR_CAPACITY;
    DevMem ev, keys, keys2, vals, vals2, ukeys, cnt, start, nu_d, val, col, rp, b, tmp;
    if (!ev.alloc(72ull * e_nnzb) || !keys.alloc(8ull * N) || !keys2.alloc(8ull * N) || !vals.alloc(8ull * N) ||
        !vals2.alloc(8ull * N) || !ukeys.alloc(8ull * N) || !cnt.alloc(4ull * (N + 1)) || !start.alloc(4ull * (N + 1)) ||
        !nu_d.alloc(8) || !val.alloc(8ull * N) || !col.alloc(4ull * N) || !rp.alloc(4ull * (n + 1)) || !b.alloc(8ull * n))
        return FIPC_ERR_CUDA;
    int st = sell_to_bsr(c, ev.as<double>(), s);
    if (st) return st;
    const int* crp = c->c_rowptr.as<int>();
    if (!crp) return FIPC_ERR_ARGUMENT;   // no system assembled
    k_direct_entries<<<nbd(nV, 128), 128, 0, s>>>(nV, c->row_ptr, c->col_idx, ev.as<double>(), crp, c->c_col.as<int>(),
                                                   c->c_val.as<double>(), fixed, keys.as<unsigned long long>(), vals.as<double>());
    FIPC_LAUNCHED();
    cub::DoubleBuffer<unsigned long long> kb(keys.as<unsigned long long>(), keys2.as<unsigned long long>());
    cub::DoubleBuffer<double> vb(vals.as<double>(), vals2.as<double>());
    size_t need = 0;
    const int Ni = (int)N;
    FIPC_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, need, kb, vb, Ni, 0, 64, s));
    if (!tmp.alloc(need)) return FIPC_ERR_CUDA;
    FIPC_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, need, kb, vb, Ni, 0, 64, s));
    DevMem tmp2;
    size_t need2 = 0;
    int* nu_p = nu_d.as<int>();
    FIPC_CUDA(cub::DeviceRunLengthEncode::Encode(nullptr, need2, kb.Current(), ukeys.as<unsigned long long>(), cnt.as<int>(), nu_p, Ni, s));
    if (!tmp2.alloc(need2)) return FIPC_ERR_CUDA;
    FIPC_CUDA(cub::DeviceRunLengthEncode::Encode(tmp2.p, need2, kb.Current(), ukeys.as<unsigned long long>(), cnt.as<int>(), nu_p, Ni, s));
    int nu = 0;
    FIPC_CUDA(cudaMemcpyAsync(&nu, nu_p, 4, cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaStreamSynchronize(s));
    DevMem tmp3;
    size_t need3 = 0;
    FIPC_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, need3, cnt.as<int>(), start.as<int>(), nu + 1, s));
    if (!tmp3.alloc(need3)) return FIPC_ERR_CUDA;
    FIPC_CUDA(cub::DeviceScan::ExclusiveSum(tmp3.p, need3, cnt.as<int>(), start.as<int>(), nu + 1, s));
    k_direct_sum<<<nbd(nu, 256), 256, 0, s>>>(nu, ukeys.as<unsigned long long>(), start.as<int>(), vb.Current(), val.as<double>(),
                                              col.as<int>());
    FIPC_LAUNCHED();
    k_direct_rowptr<<<nbd(n + 1, 256), 256, 0, s>>>(n, nu, ukeys.as<unsigned long long>(), rp.as<int>());
    FIPC_LAUNCHED();
    k_direct_rhs<<<nbd(n, 256), 256, 0, s>>>(nV, c->rhs, fixed, b.as<double>());
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    cusolverSpHandle_t h = nullptr;
    cusparseMatDescr_t d = nullptr;
    if (L.create(&h) != CUSOLVER_STATUS_SUCCESS) return FIPC_ERR_CUDA;
    int sing = -1;
    cusolverStatus_t cs = L.set_stream(h, s);
    if (cs == CUSOLVER_STATUS_SUCCESS && L.create_descr(&d) == CUSPARSE_STATUS_SUCCESS) {
        L.set_type(d, CUSPARSE_MATRIX_TYPE_GENERAL);
        L.set_base(d, CUSPARSE_INDEX_BASE_ZERO);
        // reorder 3: METIS nested dissection (fill-reducing, as CHOLMOD's default ordering)
        cs = L.chol(h, n, nu, d, val.as<double>(), rp.as<int>(), col.as<int>(), b.as<double>(), 0.0, 3, sol, &sing);
    } else {
        cs = CUSOLVER_STATUS_INTERNAL_ERROR;
    }
    if (d) L.destroy_descr(d);
    L.destroy(h);
    FIPC_CUDA(cudaStreamSynchronize(s));
    if (cs != CUSOLVER_STATUS_SUCCESS) return FIPC_ERR_CUDA;
    if (nnz_h) *nnz_h = nu;
    return sing >= 0 ? FIPC_ERR_NONFINITE : FIPC_OK;   // singularity >= 0: not positive definite
}

}  // extern "C"
