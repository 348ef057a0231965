// Per-vertex MLP of the learned Newton warm start: forward, backward, MSE loss, Adam, FP32.
//
// Network: 55 inputs (padded to 64) -> 128 -> 128 -> 128 -> 3 (padded to 4), GELU after each
// hidden layer.  Rows are vertices; parameters are one flat FP32 array:
//   W1 [128][64], b1 [128], W2 [128][128], b2 [128], W3 [128][128], b3 [128], W4 [4][128], b4 [4].
// The layer products run on a tiled FP32 SGEMM (64x64 output tiles, 16-deep K slices in shared
// memory, 4x4 outputs per thread); every output element sums its K range in a fixed order, so
// forward and backward results are reproducible.  No counterpart in the reference: this is the
// learned warm start the task adds beside the drop-in path.
#include <cuda_runtime.h>

#include "ctx.cuh"

namespace fipc {

constexpr int MLP_IN = 64, MLP_H = 128, MLP_OUT = 4;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + MLP_H * MLP_IN, OFF_W2 = OFF_B1 + MLP_H, OFF_B2 = OFF_W2 + MLP_H * MLP_H,
              OFF_W3 = OFF_B2 + MLP_H, OFF_B3 = OFF_W3 + MLP_H * MLP_H, OFF_W4 = OFF_B3 + MLP_H,
              OFF_B4 = OFF_W4 + MLP_OUT * MLP_H, MLP_NPARAM = OFF_B4 + MLP_OUT;

// C[M][N] (ldc) = alpha * op(A)[M][K] * op(B)[K][N] + beta * C.  op(A) = A[M][K] (lda) or, when
// ta, A stored [K][M]; op(B) = B[K][N] (ldb) or, when tb, B stored [N][K].
constexpr int TM = 64, TN = 64, TK = 16;
__global__ void __launch_bounds__(256) k_sgemm(int M, int N, int K, float alpha, const float* __restrict__ A, int lda, int ta,
                                               const float* __restrict__ B, int ldb, int tb, float beta, float* __restrict__ C,
                                               int ldc) {
    __shared__ float As[TK][TM + 4];
    __shared__ float Bs[TK][TN + 4];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += TK) {
        // 64 x 16 tile of op(A) and 16 x 64 tile of op(B), 4 elements per thread each
        for (int e = threadIdx.x; e < TM * TK; e += 256) {
            const int mm = e / TK, kk = e % TK;
            const int gm = m0 + mm, gk = k0 + kk;
            float va = 0.f;
            if (gm < M && gk < K) va = ta ? A[(size_t)gk * lda + gm] : A[(size_t)gm * lda + gk];
            As[kk][mm] = va;
        }
        for (int e = threadIdx.x; e < TK * TN; e += 256) {
            const int kk = e / TN, nn = e % TN;
            const int gk = k0 + kk, gn = n0 + nn;
            float vb = 0.f;
            if (gk < K && gn < N) vb = tb ? B[(size_t)gn * ldb + gk] : B[(size_t)gk * ldb + gn];
            Bs[kk][nn] = vb;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < TK; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int gm = m0 + ty * 4 + i, gn = n0 + tx * 4 + j;
            if (gm < M && gn < N) {
                float* c = C + (size_t)gm * ldc + gn;
                *c = alpha * acc[i][j] + (beta != 0.f ? beta * *c : 0.f);
            }
        }
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
    return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// Z += bias (row broadcast); A = gelu(Z) when act, else A = Z
__global__ void k_bias_act(int rows, int cols, float* __restrict__ Z, const float* __restrict__ bias, float* __restrict__ A, int act) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)rows * cols) return;
    const float z = Z[i] + bias[i % cols];
    Z[i] = z;
    A[i] = act ? gelu(z) : z;
}

// dZ = dA * gelu'(Z), in place on dA
__global__ void k_gelu_back(int rows, int cols, const float* __restrict__ Z, float* __restrict__ dA) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)rows * cols) return;
    dA[i] *= gelu_grad(Z[i]);
}

// db[c] = sum over rows of dZ[r][c]: one block per column, fixed-order strides + tree
__global__ void k_bias_grad(int rows, int cols, const float* __restrict__ dZ, float* __restrict__ db) {
    __shared__ float sh[256];
    const int c = blockIdx.x;
    float a = 0.f;
    for (int r = threadIdx.x; r < rows; r += blockDim.x) a += dZ[(size_t)r * cols + c];
    sh[threadIdx.x] = a;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[c] = sh[0];
}

// mean squared error over the first 3 outputs: dout = 2 (out - target) / (3 n), loss partials
__global__ void k_mse(int n, const float* __restrict__ out, const float* __restrict__ target, float* __restrict__ dout,
                      float* __restrict__ part) {
    __shared__ float sh[256];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (i < n) {
        const float s = 2.f / (3.f * (float)n);
        for (int d = 0; d < MLP_OUT; ++d) {
            const float e = d < 3 ? out[4 * (size_t)i + d] - target[4 * (size_t)i + d] : 0.f;
            dout[4 * (size_t)i + d] = s * e;
            l += e * e;
        }
    }
    sh[threadIdx.x] = l;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}
__global__ void k_mse_finish(int nb, int n, const float* __restrict__ part, float* __restrict__ loss) {
    __shared__ float sh[256];
    float a = 0.f;
    for (int i = threadIdx.x; i < nb; i += 256) a += part[i];
    sh[threadIdx.x] = a;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *loss = sh[0] / (3.f * (float)n);
}

// Adam with bias correction (step t >= 1)
__global__ void k_adam(int n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

}  // namespace fipc

// ---------------------------------------------------------------- host side
namespace fipc {
static inline int nblk(long long n, int b) { return (int)((n + b - 1) / b); }

static void sgemm(cudaStream_t s, int M, int N, int K, const float* A, int lda, int ta, const float* B, int ldb, int tb, float beta,
                  float* C, int ldc) {
    dim3 grid(nblk(N, TN), nblk(M, TM));
    k_sgemm<<<grid, 256, 0, s>>>(M, N, K, 1.f, A, lda, ta, B, ldb, tb, beta, C, ldc);
    FIPC_LAUNCHED();
}
static void bias_act(cudaStream_t s, int rows, int cols, float* Z, const float* b, float* A, int act) {
    k_bias_act<<<nblk((long long)rows * cols, 256), 256, 0, s>>>(rows, cols, Z, b, A, act);
    FIPC_LAUNCHED();
}
}  // namespace fipc

using namespace fipc;

extern "C" {

int fipc_mlp_param_count(void) { return MLP_NPARAM; }

// out [n][4] for inputs X [n][64]; Z and A: scratch [3][n][128] (pre- and post-activations,
// kept for the backward pass)
int fipc_mlp_forward(int n, const float* X, const float* params, float* Z, float* A, float* out, void* stream) {
    if (n < 0 || !X || !params || !Z || !A || !out) return FIPC_ERR_ARGUMENT;
    if (n == 0) return FIPC_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t L = (size_t)n * MLP_H;
    const float* P = params;
    sgemm(s, n, MLP_H, MLP_IN, X, MLP_IN, 0, P + OFF_W1, MLP_IN, 1, 0.f, Z, MLP_H);
    bias_act(s, n, MLP_H, Z, P + OFF_B1, A, 1);
    sgemm(s, n, MLP_H, MLP_H, A, MLP_H, 0, P + OFF_W2, MLP_H, 1, 0.f, Z + L, MLP_H);
    bias_act(s, n, MLP_H, Z + L, P + OFF_B2, A + L, 1);
    sgemm(s, n, MLP_H, MLP_H, A + L, MLP_H, 0, P + OFF_W3, MLP_H, 1, 0.f, Z + 2 * L, MLP_H);
    bias_act(s, n, MLP_H, Z + 2 * L, P + OFF_B3, A + 2 * L, 1);
    sgemm(s, n, MLP_OUT, MLP_H, A + 2 * L, MLP_H, 0, P + OFF_W4, MLP_H, 1, 0.f, out, MLP_OUT);
    bias_act(s, n, MLP_OUT, out, P + OFF_B4, out, 0);
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

// parameter gradients (grads, same layout as params) of sum(dout . out) for the forward pass
// that produced Z, A; dA: scratch [2][n][128]
int fipc_mlp_backward(int n, const float* X, const float* params, const float* Z, const float* A, const float* dout, float* grads,
                      float* dA, void* stream) {
    if (n <= 0 || !X || !params || !Z || !A || !dout || !grads || !dA) return FIPC_ERR_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t L = (size_t)n * MLP_H;
    const float* P = params;
    float* G = grads;
    float *d0 = dA, *d1 = dA + L;
    // layer 4 (linear)
    sgemm(s, MLP_OUT, MLP_H, n, dout, MLP_OUT, 1, A + 2 * L, MLP_H, 0, 0.f, G + OFF_W4, MLP_H);
    k_bias_grad<<<MLP_OUT, 256, 0, s>>>(n, MLP_OUT, dout, G + OFF_B4);
    FIPC_LAUNCHED();
    sgemm(s, n, MLP_H, MLP_OUT, dout, MLP_OUT, 0, P + OFF_W4, MLP_H, 0, 0.f, d0, MLP_H);
    // layers 3, 2, 1 (GELU)
    const int offW[3] = {OFF_W3, OFF_W2, OFF_W1}, offB[3] = {OFF_B3, OFF_B2, OFF_B1};
    for (int l = 2; l >= 0; --l) {
        const int k = 2 - l;
        k_gelu_back<<<nblk((long long)L, 256), 256, 0, s>>>(n, MLP_H, Z + l * L, d0);
        FIPC_LAUNCHED();
        const float* in = l > 0 ? A + (l - 1) * L : X;
        const int din = l > 0 ? MLP_H : MLP_IN;
        sgemm(s, MLP_H, din, n, d0, MLP_H, 1, in, din, 0, 0.f, G + offW[k], din);
        k_bias_grad<<<MLP_H, 256, 0, s>>>(n, MLP_H, d0, G + offB[k]);
        FIPC_LAUNCHED();
        if (l > 0) {
            sgemm(s, n, MLP_H, MLP_H, d0, MLP_H, 0, P + offW[k], MLP_H, 0, 0.f, d1, MLP_H);
            float* t = d0;
            d0 = d1;
            d1 = t;
        }
    }
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

// loss = mean over n rows and 3 outputs of (out - target)^2 into *loss (device); dout its gradient;
// part: scratch of ceil(n / 256) floats
int fipc_mlp_mse(int n, const float* out, const float* target, float* dout, float* part, float* loss, void* stream) {
    if (n <= 0 || !out || !target || !dout || !part || !loss) return FIPC_ERR_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    const int nb = nblk(n, 256);
    k_mse<<<nb, 256, 0, s>>>(n, out, target, dout, part);
    FIPC_LAUNCHED();
    k_mse_finish<<<1, 256, 0, s>>>(nb, n, part, loss);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

// one Adam step (t counts from 1)
int fipc_mlp_adam(int n_params, float* params, const float* grads, float* m, float* v, float lr, float beta1, float beta2, float eps,
                  int t, void* stream) {
    if (n_params <= 0 || !params || !grads || !m || !v || t < 1) return FIPC_ERR_ARGUMENT;
    const float c1 = 1.f - powf(beta1, (float)t), c2 = 1.f - powf(beta2, (float)t);
    k_adam<<<nblk(n_params, 256), 256, 0, (cudaStream_t)stream>>>(n_params, params, grads, m, v, lr, beta1, beta2, eps, c1, c2);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- per-vertex features
#include "geometry.cuh"

namespace fipc {

constexpr int MLP_NBR = 16;

__global__ void k_fill_u32(int n, unsigned* __restrict__ a, unsigned v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}

// distance of each constraint row (square root of its squared distance), min'd into its vertices
// (non-negative floats order like their bit patterns, so atomicMin on the bits is exact)
__global__ void k_row_dist(int type, int n, const int4* __restrict__ rows, const double* __restrict__ x, unsigned* __restrict__ dmin) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int4 q = rows[r];
    double d2;
    switch (type) {
        case T_PP: d2 = d_PP(ld3(x, q.x), ld3(x, q.y)); break;
        case T_PE: d2 = d_PE(ld3(x, q.x), ld3(x, q.y), ld3(x, q.z)); break;
        case T_PT: d2 = d_PT(ld3(x, q.x), ld3(x, q.y), ld3(x, q.z), ld3(x, q.w)); break;
        case T_EE: case T_EEM: d2 = d_EE(ld3(x, q.x), ld3(x, q.y), ld3(x, q.z), ld3(x, q.w)); break;
        case T_PPM: d2 = d_PP(ld3(x, q.x), ld3(x, q.z)); break;
        default: d2 = d_PE(ld3(x, q.x), ld3(x, q.z), ld3(x, q.w)); break;
    }
    const unsigned bits = __float_as_uint((float)sqrt(fmax(d2, 0.0)));
    const int nv = type_nverts(type);
    const int id[4] = {q.x, q.y, q.z, q.w};
    for (int k = 0; k < nv; ++k) atomicMin(dmin + id[k], bits);
}

// X[i] = (16 one-ring relative positions / h, v dt / h, dx_prev / h, min(dist / dhat, 1), 0 pad);
// relative positions are x_j - x_i, or (x_j - x_i) - (X_j - X_i) against the rest shape X when
// x0 is given (the one-ring's deformation)
__global__ void k_features(int nV, const int* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ x,
                           const double* __restrict__ x0, const double* __restrict__ v, const double* __restrict__ dxp, double dt,
                           double inv_h, double inv_dhat, const unsigned* __restrict__ dmin, float* __restrict__ X) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nV) return;
    float* f = X + (size_t)i * MLP_IN;
    const v3 xi = ld3(x, i);
    const v3 Xi = x0 ? ld3(x0, i) : mk(0, 0, 0);
    int k = 0;
    for (int e = rp[i]; e < rp[i + 1] && k < MLP_NBR; ++e) {
        const int j = ci[e];
        if (j == i) continue;
        v3 d = ld3(x, j) - xi;
        if (x0) d = d - (ld3(x0, j) - Xi);
        f[3 * k] = (float)(d.x * inv_h);
        f[3 * k + 1] = (float)(d.y * inv_h);
        f[3 * k + 2] = (float)(d.z * inv_h);
        ++k;
    }
    for (; k < MLP_NBR; ++k) f[3 * k] = f[3 * k + 1] = f[3 * k + 2] = 0.f;
    const v3 vi = ld3(v, i), pi = ld3(dxp, i);
    f[48] = (float)(vi.x * dt * inv_h);
    f[49] = (float)(vi.y * dt * inv_h);
    f[50] = (float)(vi.z * dt * inv_h);
    f[51] = (float)(pi.x * inv_h);
    f[52] = (float)(pi.y * inv_h);
    f[53] = (float)(pi.z * inv_h);
    const float dm = __uint_as_float(dmin[i]);
    f[54] = fminf(dm * (float)inv_dhat, 1.f);
    for (int q = 55; q < MLP_IN; ++q) f[q] = 0.f;
}

}  // namespace fipc

extern "C" int fipc_mlp_features(fipc_ctx* c, const double* x, const double* v, const double* dx_prev, double h, int rest_relative,
                                 float* X, void* stream) {
    if (!c || !x || !v || !dx_prev || !X || !(h > 0)) return FIPC_ERR_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    if (c->mlp_dist.ensure(4ll * c->nV)) return FIPC_ERR_CUDA;
    unsigned* dmin = c->mlp_dist.as<unsigned>();
    k_fill_u32<<<nblk(c->nV, 256), 256, 0, s>>>(c->nV, dmin, 0x7f800000u);   // +inf
    FIPC_LAUNCHED();
    for (int t = 0; t < N_TYPES; ++t) {
        if (c->h_counts[t] <= 0) continue;
        k_row_dist<<<nblk(c->h_counts[t], 128), 128, 0, s>>>(t, c->h_counts[t], c->rows[t].as<int4>(), x, dmin);
        FIPC_LAUNCHED();
    }
    k_features<<<nblk(c->nV, 128), 128, 0, s>>>(c->nV, c->row_ptr, c->col_idx, x, rest_relative ? c->x0 : nullptr, v, dx_prev, c->dt,
                                                1.0 / h, 1.0 / c->dhat, dmin, X);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

// ---------------------------------------------------------------- smoothing of a displacement
namespace fipc {
// out_i = mean of d_j over the one-ring of i including i (the elastic block pattern); 0 on
// Dirichlet vertices
__global__ void k_ring_mean(int nV, const int* __restrict__ rp, const int* __restrict__ ci, const unsigned char* __restrict__ fixed,
                            const double* __restrict__ d, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nV) return;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    if (!fixed[i]) {
        for (int e = rp[i]; e < rp[i + 1]; ++e) {
            const int j = ci[e];
            s0 += d[3 * (size_t)j];
            s1 += d[3 * (size_t)j + 1];
            s2 += d[3 * (size_t)j + 2];
        }
        const double inv = 1.0 / (double)(rp[i + 1] - rp[i]);
        s0 *= inv;
        s1 *= inv;
        s2 *= inv;
    }
    out[3 * (size_t)i] = s0;
    out[3 * (size_t)i + 1] = s1;
    out[3 * (size_t)i + 2] = s2;
}
}  // namespace fipc

// passes of one-ring averaging of d [V][3] (in place, tmp: scratch [V][3]); the learned
// correction is smoothed so that its vertex-to-vertex noise does not load the elastic energy
extern "C" int fipc_mlp_smooth(fipc_ctx* c, const unsigned char* fixed, double* d, double* tmp, int passes, void* stream) {
    if (!c || !fixed || !d || !tmp || passes < 0) return FIPC_ERR_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    for (int k = 0; k < passes; ++k) {
        k_ring_mean<<<nblk(c->nV, 128), 128, 0, s>>>(c->nV, c->row_ptr, c->col_idx, fixed, d, tmp);
        FIPC_LAUNCHED();
        FIPC_CUDA(cudaMemcpyAsync(d, tmp, 24ll * c->nV, cudaMemcpyDeviceToDevice, s));
    }
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}
