// Event-pair timing of one selected kernel (see profile.cuh).
#include <mutex>
#include <vector>

#include "common.cuh"
#include "ctx.cuh"
#include "profile.cuh"

namespace fipc {

namespace {
struct Rec {
    cudaEvent_t a, b;
};
std::mutex g_mu;
int g_kernel = PK_NONE;
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_pool;
double g_bytes = 0.0, g_flops = 0.0;

cudaEvent_t get_event() {
    if (!g_pool.empty()) {
        cudaEvent_t e = g_pool.back();
        g_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}
}  // namespace

int profile_kernel() {
    std::lock_guard<std::mutex> lk(g_mu);
    return g_kernel;
}

ProfScope::ProfScope(int kernel, cudaStream_t stream, double bytes_, double flops_) : id(kernel), s(stream), bytes(bytes_), flops(flops_) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_kernel != id) return;
    a = get_event();
    b = get_event();
    cudaEventRecord(a, s);
}

ProfScope::~ProfScope() {
    if (!a) return;
    std::lock_guard<std::mutex> lk(g_mu);
    cudaEventRecord(b, s);
    g_recs.push_back({a, b});
    g_bytes += bytes;
    g_flops += flops;
}

// FP64 throughput probe: 8 independent FMA chains per thread (enough independent work to fill
// the FP64 pipe), iters rounds; every thread writes its sum so nothing is optimised away.
// Flops per launch = blocks x 256 x iters x 16.
__global__ void __launch_bounds__(256) k_fp64_fma_probe(int iters, double b, double c, double* __restrict__ out) {
    const double s0 = 1e-9 * threadIdx.x;
    double a0 = s0, a1 = s0 + 1e-3, a2 = s0 + 2e-3, a3 = s0 + 3e-3, a4 = s0 + 4e-3, a5 = s0 + 5e-3, a6 = s0 + 6e-3,
           a7 = s0 + 7e-3;
    for (int i = 0; i < iters; ++i) {
        a0 = fma(a0, b, c);
        a1 = fma(a1, b, c);
        a2 = fma(a2, b, c);
        a3 = fma(a3, b, c);
        a4 = fma(a4, b, c);
        a5 = fma(a5, b, c);
        a6 = fma(a6, b, c);
        a7 = fma(a7, b, c);
    }
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
}

}  // namespace fipc

using namespace fipc;

extern "C" {

// start timing every launch of kernel `kernel_id` (1 PCG SpMV, 2 PCG update, 3 Neo-Hookean
// element, 4 barrier rows, 5 elastic assembly); 0 stops.  Clears previous records.
int fipc_profile_enable(int kernel_id) {
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto& r : g_recs) {
        g_pool.push_back(r.a);
        g_pool.push_back(r.b);
    }
    g_recs.clear();
    g_bytes = g_flops = 0.0;
    g_kernel = kernel_id;
    return FIPC_OK;
}

// sum of the recorded launch times (ms), launch count, algorithmic bytes and flops
int fipc_profile_read(double* total_ms, long long* launches, double* bytes, double* flops) {
    std::lock_guard<std::mutex> lk(g_mu);
    double t = 0.0;
    for (auto& r : g_recs) {
        if (cudaEventSynchronize(r.b) != cudaSuccess) return FIPC_ERR_CUDA;
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess) return FIPC_ERR_CUDA;
        t += ms;
    }
    if (total_ms) *total_ms = t;
    if (launches) *launches = (long long)g_recs.size();
    if (bytes) *bytes = g_bytes;
    if (flops) *flops = g_flops;
    return FIPC_OK;
}

// one launch of the FP64 FMA probe: blocks x 256 threads, out [blocks * 256] (device)
int fipc_fp64_fma_probe(int blocks, int iters, double* out, void* stream) {
    if (blocks <= 0 || iters <= 0 || !out) return FIPC_ERR_ARGUMENT;
    k_fp64_fma_probe<<<blocks, 256, 0, (cudaStream_t)stream>>>(iters, 0.999999, 1e-6, out);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

}  // extern "C"
