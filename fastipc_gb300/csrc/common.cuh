// Shared helpers for the FastIPC GB300 kernels: small FP64 vector algebra usable from host
// and device code (the headers are also compiled by g++ for CPU unit tests of the math).
#pragma once

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define FIPC_HD __host__ __device__ __forceinline__
#else
#define FIPC_HD inline
#endif

namespace fipc {

struct v3 {
    double x, y, z;
};

FIPC_HD v3 mk(double a, double b, double c) { return v3{a, b, c}; }
FIPC_HD v3 operator+(v3 a, v3 b) { return v3{a.x + b.x, a.y + b.y, a.z + b.z}; }
FIPC_HD v3 operator-(v3 a, v3 b) { return v3{a.x - b.x, a.y - b.y, a.z - b.z}; }
FIPC_HD v3 operator-(v3 a) { return v3{-a.x, -a.y, -a.z}; }
FIPC_HD v3 operator*(double s, v3 a) { return v3{s * a.x, s * a.y, s * a.z}; }
FIPC_HD double dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
FIPC_HD v3 cross(v3 a, v3 b) { return v3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
FIPC_HD double sq(v3 a) { return dot(a, a); }
FIPC_HD double comp(v3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
FIPC_HD v3 vmin(v3 a, v3 b) { return v3{fmin(a.x, b.x), fmin(a.y, b.y), fmin(a.z, b.z)}; }
FIPC_HD v3 vmax(v3 a, v3 b) { return v3{fmax(a.x, b.x), fmax(a.y, b.y), fmax(a.z, b.z)}; }

FIPC_HD v3 load3(const double* p, int i) { return v3{p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }

// status codes shared with the C ABI (include/fastipc.h)
enum : int {
    FIPC_OK = 0,
    FIPC_ERR_CAPACITY = 1,
    FIPC_ERR_ITERATION = 2,
    FIPC_ERR_NONFINITE = 3,
    FIPC_ERR_CUDA = 4,
    FIPC_ERR_ARGUMENT = 5,
    FIPC_ERR_IO = 6,
};

// constraint lists, in the reference's order (NEWTON_IPC.py:349)
enum : int { T_PP = 0, T_PE = 1, T_PT = 2, T_EE = 3, T_EEM = 4, T_PPM = 5, T_PEM = 6, N_TYPES = 7 };

FIPC_HD int type_nverts(int t) { return t == T_PP ? 2 : (t == T_PE ? 3 : 4); }

}  // namespace fipc
