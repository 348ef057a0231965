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

}  // extern "C"
