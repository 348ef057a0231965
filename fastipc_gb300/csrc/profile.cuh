// Optional per-kernel timing for the roofline report: when enabled for one kernel id, the
// launcher records a CUDA event pair around every launch of that kernel on its stream and
// adds the launch's algorithmic bytes and flops; fipc_profile_read sums the event times.
#pragma once

#include <cuda_runtime.h>

namespace fipc {

enum ProfKernel : int { PK_NONE = 0, PK_PCG_SPMV = 1, PK_PCG_UPDATE = 2, PK_ELASTICITY = 3, PK_BARRIER = 4, PK_ASSEMBLE = 5 };

// the kernel id being timed (PK_NONE when off)
int profile_kernel();

struct ProfScope {
    int id;
    cudaStream_t s;
    cudaEvent_t a = nullptr, b = nullptr;
    double bytes, flops;
    ProfScope(int kernel, cudaStream_t stream, double bytes_, double flops_);
    ~ProfScope();
};

}  // namespace fipc
