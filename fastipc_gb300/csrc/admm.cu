// ADMM-IPC: the alternating-direction variant of the IPC time step
// (projects/FastIPC/ADMM_IPC.py), on the GPU.
//
// Per time step (ADMM_IPC.py:1471-1526) the variables are
//   * per tet:            W (weight), z (3x3 local deformation gradient), u (3x3 scaled dual);
//   * per constraint row: y (the row's relative vectors x_c0 - x_ck, k = 1..nv-1), r (their
//                         scaled duals) and Q (weight), stored in the constraint lists' order
//                         (the seven lists concatenated, rows [nv-1] vectors padded to 3).
// One ADMM iteration (the caller's loop) is: constraint finding, reuse of the previous rows'
// variables (fipc_admm_reuse), the global step (fipc_admm_global: one sparse SPD solve for x),
// the CCD / intersection filter of the new x, the local steps (fipc_admm_local: per tet a Newton
// solve in singular values, per row a Newton solve in its relative vectors) and the dual step
// (fipc_admm_dual).
//
// The reference script calls its barrier helpers as functions of the relative vectors with the
// row's first vertex at the origin (PP_gradient(op, pos), ...), while common/math/ipc.py
// defines them on all the row's points (its PP_gradient returns the 6-vector of both points).
// The relative-coordinate derivatives are taken here: the gradient with respect to the
// vertices at pos_1..pos_{nv-1} and the Hessian block among them, of the row energy at
// (0, pos_1, ..., pos_{nv-1}).  The Q weights use the whole row Hessian there, as the reference's
// reuse step computes it.  Elasticity is fixed-corotated (common/physics/fixed_corotated.py,
// the model the script imports).
#include <cuda_runtime.h>

#include "barrier.cuh"
#include "ctx.cuh"
#include "ldlt.cuh"
#include "nh.cuh"

namespace fipc {

int contact_prepare(fipc_ctx* c, TypeTable* tt, int* nrows_out, long long* nent_out, cudaStream_t s);
int contact_reduce(fipc_ctx* c, const TypeTable& tt, int nrows, long long nent, cudaStream_t s);
int assemble_elastic(fipc_ctx* c, cudaStream_t s);
int cs_offsets(fipc_ctx* c, const double* x, cudaStream_t s);
int pcg_solve(fipc_ctx* c, const unsigned char* fixed, const int* diag_pos, double rtol, int maxit, double* sol, int* iters,
              cudaStream_t s);

// The reference's local loops run until the step is small.  A row whose Hessian (unprojected,
// as the reference takes it) is indefinite gets a huge regularised step that the halving cuts
// to almost nothing, and the loop never meets its tolerance; here it stops at the bound and the
// local step reports which bound was reached (the oracle stops the same way).
constexpr int ADMM_MAX_NEWTON = 256;   // local Newton iterations
constexpr int ADMM_MAX_HALVINGS = 64;  // line-search halvings per local Newton iteration
// bits of the local step's detail status
constexpr int ADMM_ELASTIC_NEWTON = 1, ADMM_ELASTIC_HALVING = 2, ADMM_ROW_NEWTON = 4, ADMM_ROW_HALVING = 8, ADMM_NONFINITE = 16;

// ---------------------------------------------------------------- fixed-corotated in sigma
// common/physics/fixed_corotated.py:6-80, 3D branch
FIPC_HD double fc3_psi(const double* s, double la, double mu) {
    const double a = s[0] - 1, b = s[1] - 1, c = s[2] - 1, p = s[0] * s[1] * s[2] - 1;
    return mu * (a * a + b * b + c * c) + la / 2 * p * p;
}
FIPC_HD void fc3_grad(const double* s, double la, double mu, double* g) {
    const double pl = la * (s[0] * s[1] * s[2] - 1);
    const double n0 = s[1] * s[2], n1 = s[2] * s[0], n2 = s[0] * s[1];
    const double m2 = mu * 2;
    g[0] = m2 * (s[0] - 1) + n0 * pl;
    g[1] = m2 * (s[1] - 1) + n1 * pl;
    g[2] = m2 * (s[2] - 1) + n2 * pl;
}
FIPC_HD void fc3_hess(const double* s, double la, double mu, double* H) {
    const double P = s[0] * s[1] * s[2];
    const double n0 = s[1] * s[2], n1 = s[2] * s[0], n2 = s[0] * s[1];
    const double m2 = mu * 2;
    const double h01 = la * (s[2] * (P - 1) + n0 * n1), h02 = la * (s[1] * (P - 1) + n0 * n2), h12 = la * (s[0] * (P - 1) + n1 * n2);
    H[0] = m2 + la * n0 * n0;
    H[4] = m2 + la * n1 * n1;
    H[8] = m2 + la * n2 * n2;
    H[1] = H[3] = h01;
    H[2] = H[6] = h02;
    H[5] = H[7] = h12;
}

// shape-function gradients G[p][j] of a tet from its rest-shape inverse A = Dm^-1
// (ADMM_IPC.py:315-336 X2F): rows 1..3 of A, and minus their sum for vertex 0
FIPC_HD void shape_grads(const double* A, double G[4][3]) {
    for (int j = 0; j < 3; ++j) {
        G[1][j] = A[0 * 3 + j];
        G[2][j] = A[1 * 3 + j];
        G[3][j] = A[2 * 3 + j];
        G[0][j] = -A[0 * 3 + j] - A[1 * 3 + j] - A[2 * 3 + j];
    }
}

// ---------------------------------------------------------------- per tet
// initial_guess (ADMM_IPC.py:296-313): W = sqrt((la + 2 mu / 3) dt^2 vol0), z = F(xTilde), u = 0
__global__ void k_admm_init(int nT, const int4* __restrict__ tets, const double* __restrict__ xt, const double* __restrict__ dminv,
                            const double* __restrict__ vol, const double* __restrict__ lam, const double* __restrict__ mu, double dt2,
                            double* __restrict__ W, double* __restrict__ z, double* __restrict__ u) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nT) return;
    const int4 t = tets[e];
    const v3 X[4] = {ld3(xt, t.x), ld3(xt, t.y), ld3(xt, t.z), ld3(xt, t.w)};
    double IB[9], F[9];
    for (int i = 0; i < 9; ++i) IB[i] = dminv[9 * (size_t)e + i];
    deformation_gradient(X, IB, F);
    W[e] = sqrt((lam[e] + mu[e] * 2 / 3) * dt2 * vol[e]);
    for (int i = 0; i < 9; ++i) {
        z[9 * (size_t)e + i] = F[i];
        u[9 * (size_t)e + i] = 0.0;
    }
}

// global_step, element part (ADMM_IPC.py:388-411): the element's scalar stiffness
// K = W^2 G G^T as 3x3 blocks K[v][w] I into the tiled element-block layout of the context's
// elastic assembly, and its right-hand side W^2 (z - u) G[p] per vertex into eg [T][12]
__global__ void k_admm_global_elem(int nT, const double* __restrict__ dminv, const double* __restrict__ W, const double* __restrict__ z,
                                   const double* __restrict__ u, double* __restrict__ Hu, double* __restrict__ eg) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nT) return;
    double A[9], G[4][3], Fz[9];
    for (int i = 0; i < 9; ++i) {
        A[i] = dminv[9 * (size_t)e + i];
        Fz[i] = z[9 * (size_t)e + i] - u[9 * (size_t)e + i];
    }
    shape_grads(A, G);
    const double w2 = W[e] * W[e];
    double* tile = Hu + (size_t)(e >> 5) * 2880 + (e & 31) * 9;
    int b = 0;
    for (int v = 0; v < 4; ++v)
        for (int w = v; w < 4; ++w, ++b) {
            const double k = (G[v][0] * G[w][0] + G[v][1] * G[w][1] + G[v][2] * G[w][2]) * w2;
            double* blk = tile + b * 288;
            for (int i = 0; i < 9; ++i) blk[i] = (i % 4 == 0) ? k : 0.0;
        }
    for (int p = 0; p < 4; ++p)
        for (int q = 0; q < 3; ++q)
            eg[12 * (size_t)e + 3 * p + q] = (G[p][0] * Fz[q * 3 + 0] + G[p][1] * Fz[q * 3 + 1] + G[p][2] * Fz[q * 3 + 2]) * w2;
}

// right-hand side m xTilde + sum of the element parts (global_step, ADMM_IPC.py:391-411)
__global__ void k_admm_rhs(int nV, const int* __restrict__ vt_ptr, const int* __restrict__ vt_list, const double* __restrict__ eg,
                           const double* __restrict__ mass, const double* __restrict__ xt, double* __restrict__ rhs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nV) return;
    const double m = mass[i];
    double r0 = m * xt[3 * i], r1 = m * xt[3 * i + 1], r2 = m * xt[3 * i + 2];
    for (int k = vt_ptr[i]; k < vt_ptr[i + 1]; ++k) {
        const int c = vt_list[k];   // tet * 4 + local vertex
        const double* g = eg + 12 * (size_t)(c >> 2) + 3 * (c & 3);
        r0 += g[0];
        r1 += g[1];
        r2 += g[2];
    }
    rhs[3 * i] = r0;
    rhs[3 * i + 1] = r1;
    rhs[3 * i + 2] = r2;
}

// local_elasticity (ADMM_IPC.py:633-666): per tet, F + u = U diag(s0) V^T; Newton in sigma on
// dt^2 vol0 psi(sigma) + W^2 / 2 |sigma - s0|^2 with the projected sigma Hessian, halving while
// the energy rises; z = U diag(sigma) V^T.  status: 2 when a loop reached its bound
__global__ void k_admm_local_elastic(int nT, const int4* __restrict__ tets, const double* __restrict__ x, const double* __restrict__ dminv,
                                     const double* __restrict__ vol, const double* __restrict__ lam, const double* __restrict__ mu,
                                     double dt2, const double* __restrict__ W, double* __restrict__ z, const double* __restrict__ u,
                                     int* __restrict__ status) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nT) return;
    const int4 t = tets[e];
    const v3 X[4] = {ld3(x, t.x), ld3(x, t.y), ld3(x, t.z), ld3(x, t.w)};
    double IB[9], F[9];
    for (int i = 0; i < 9; ++i) IB[i] = dminv[9 * (size_t)e + i];
    deformation_gradient(X, IB, F);
    for (int i = 0; i < 9; ++i) F[i] += u[9 * (size_t)e + i];
    double U[9], s0[3], V[9];
    svd3(F, U, s0, V);
    const double la = lam[e], m = mu[e], wv = dt2 * vol[e], W2 = W[e] * W[e];
    auto energy = [&](const double* sg) {
        const double a = sg[0] - s0[0], b = sg[1] - s0[1], c = sg[2] - s0[2];
        return fc3_psi(sg, la, m) * wv + (a * a + b * b + c * c) * W2 / 2;
    };
    double sg[3] = {s0[0], s0[1], s0[2]};
    bool converged = false;
    int it = 0;
    while (!converged) {
        if (++it > ADMM_MAX_NEWTON) {
            atomicOr(status, ADMM_ELASTIC_NEWTON);
            break;
        }
        double g[3], H[9];
        fc3_grad(sg, la, m, g);
        fc3_hess(sg, la, m, H);
        psd_project3(H);
        for (int i = 0; i < 3; ++i) g[i] = g[i] * wv + (sg[i] - s0[i]) * W2;
        for (int i = 0; i < 9; ++i) H[i] = H[i] * wv + ((i % 4 == 0) ? W2 : 0.0);
        // p = -P^-1 g (cofactor inverse, as a 3x3 matrix inverse)
        const double c00 = H[4] * H[8] - H[5] * H[7], c01 = H[5] * H[6] - H[3] * H[8], c02 = H[3] * H[7] - H[4] * H[6];
        const double id = 1.0 / (H[0] * c00 + H[1] * c01 + H[2] * c02);
        const double I[9] = {c00 * id, (H[2] * H[7] - H[1] * H[8]) * id, (H[1] * H[5] - H[2] * H[4]) * id,
                             c01 * id, (H[0] * H[8] - H[2] * H[6]) * id, (H[2] * H[3] - H[0] * H[5]) * id,
                             c02 * id, (H[1] * H[6] - H[0] * H[7]) * id, (H[0] * H[4] - H[1] * H[3]) * id};
        double p[3];
        for (int i = 0; i < 3; ++i) p[i] = -(I[i * 3] * g[0] + I[i * 3 + 1] * g[1] + I[i * 3 + 2] * g[2]);
        if (p[0] * p[0] + p[1] * p[1] + p[2] * p[2] < 1e-6) converged = true;
        double alpha = 1.0;
        const double q0[3] = {sg[0], sg[1], sg[2]};
        const double E0 = energy(q0);
        for (int i = 0; i < 3; ++i) sg[i] = q0[i] + p[i];
        double E = energy(sg);
        int k = 0;
        while (E > E0) {
            if (++k > ADMM_MAX_HALVINGS) {
                atomicOr(status, ADMM_ELASTIC_HALVING);
                break;
            }
            alpha *= 0.5;
            for (int i = 0; i < 3; ++i) sg[i] = q0[i] + alpha * p[i];
            E = energy(sg);
        }
        // a step that left sigma exactly where it was repeats itself in every later iteration:
        // the loop would run to its bound without moving, so stop here with the same result
        if (!converged && sg[0] == q0[0] && sg[1] == q0[1] && sg[2] == q0[2]) {
            atomicOr(status, ADMM_ELASTIC_NEWTON);
            break;
        }
    }
    bool finite = true;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const double v = U[i * 3 + 0] * sg[0] * V[j * 3 + 0] + U[i * 3 + 1] * sg[1] * V[j * 3 + 1] + U[i * 3 + 2] * sg[2] * V[j * 3 + 2];
            finite = finite && isfinite(v);
            z[9 * (size_t)e + i * 3 + j] = v;
        }
    if (!finite) atomicOr(status, ADMM_NONFINITE);
}

// dual_step, element part (ADMM_IPC.py:963-967): u += F(x) - z
__global__ void k_admm_dual_elem(int nT, const int4* __restrict__ tets, const double* __restrict__ x, const double* __restrict__ dminv,
                                 const double* __restrict__ z, double* __restrict__ u) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nT) return;
    const int4 t = tets[e];
    const v3 X[4] = {ld3(x, t.x), ld3(x, t.y), ld3(x, t.z), ld3(x, t.w)};
    double IB[9], F[9];
    for (int i = 0; i < 9; ++i) IB[i] = dminv[9 * (size_t)e + i];
    deformation_gradient(X, IB, F);
    for (int i = 0; i < 9; ++i) u[9 * (size_t)e + i] += F[i] - z[9 * (size_t)e + i];
}

// ---------------------------------------------------------------- per constraint row
__device__ __forceinline__ int row_type(const TypeTable& tt, int r) {
    int t = 0;
    while (t < N_TYPES - 1 && r >= tt.row0[t + 1]) ++t;
    return t;
}

// the row's energy at (0, pos_1, .., pos_{nv-1}): E, the gradient with respect to pos (gp, 3
// (nv-1)) and the unprojected Hessian block among them (Hp, n x n row-major, n = 3 (nv-1)), or
// with full, the Frobenius norm of the whole row Hessian in *fro
__device__ void rel_row(int type, const double* pos, const v3* X0, double dh2, double kappa, double* E, double* gp, double* Hp,
                        double* fro) {
    const int nv = type_nverts(type), n = 3 * (nv - 1);
    v3 X[4] = {mk(0, 0, 0), mk(0, 0, 0), mk(0, 0, 0), mk(0, 0, 0)};
    for (int k = 1; k < nv; ++k) X[k] = mk(pos[3 * (k - 1)], pos[3 * (k - 1) + 1], pos[3 * (k - 1) + 2]);
    double g[12], Hb[144];
    barrier_row(type, X, X0, dh2, kappa, (gp || Hp || fro) ? 2 : 0, E, g, Hb);
    if (gp)
        for (int i = 0; i < n; ++i) gp[i] = g[3 + i];
    if (Hp)
        for (int v = 1; v < nv; ++v)
            for (int w = 1; w < nv; ++w)
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) Hp[(3 * (v - 1) + i) * n + 3 * (w - 1) + j] = Hb[(v * 4 + w) * 9 + i * 3 + j];
    if (fro) {
        double s = 0.0;
        for (int v = 0; v < nv; ++v)
            for (int w = 0; w < nv; ++w)
                for (int i = 0; i < 9; ++i) s += Hb[(v * 4 + w) * 9 + i] * Hb[(v * 4 + w) * 9 + i];
        *fro = sqrt(s);
    }
}

__device__ __forceinline__ bool row_less(int4 a, int4 b) {
    if (a.x != b.x) return a.x < b.x;
    if (a.y != b.y) return a.y < b.y;
    if (a.z != b.z) return a.z < b.z;
    return a.w < b.w;
}
__device__ __forceinline__ bool row_eq(int4 a, int4 b) { return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w; }

// reuse_admm_variables (ADMM_IPC.py:1230-1388): every current row starts from y = the relative
// vectors of xTilde alpha + x (1 - alpha), r = 0 and Q = clamp(sqrt(|H_row(x)|), min_Q, max_Q);
// a row that was in the previous iteration's list (the lists are sorted, so a binary search
// finds it) takes its previous y, r and Q instead
__global__ void k_admm_reuse(int n, const int4* __restrict__ rows, TypeTable tt, const double* __restrict__ x, const double* __restrict__ xt,
                             const double* __restrict__ x0, double alpha, double dh2, double kappa, double minQ, double maxQ,
                             const int4* __restrict__ old_rows, TypeTable ot, const double* __restrict__ old_y,
                             const double* __restrict__ old_r, const double* __restrict__ old_Q, double* __restrict__ y,
                             double* __restrict__ r, double* __restrict__ Q) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const int t = row_type(tt, c);
    const int nv = type_nverts(t);
    const int4 q = rows[c];
    const int id[4] = {q.x, q.y, q.z, q.w};
    // a previous row with the same vertices?
    int lo = ot.row0[t], hi = ot.row0[t + 1];
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (row_less(old_rows[mid], q)) lo = mid + 1;
        else hi = mid;
    }
    if (lo < ot.row0[t + 1] && row_eq(old_rows[lo], q)) {
        for (int i = 0; i < 9; ++i) {
            y[9 * (size_t)c + i] = old_y[9 * (size_t)lo + i];
            r[9 * (size_t)c + i] = old_r[9 * (size_t)lo + i];
        }
        Q[c] = old_Q[lo];
        return;
    }
    const v3 b0 = alpha * ld3(xt, id[0]) + (1 - alpha) * ld3(x, id[0]);
    double pos[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = 1; k < nv; ++k) {
        const v3 bk = alpha * ld3(xt, id[k]) + (1 - alpha) * ld3(x, id[k]);
        const v3 d = b0 - bk;
        y[9 * (size_t)c + 3 * (k - 1)] = d.x;
        y[9 * (size_t)c + 3 * (k - 1) + 1] = d.y;
        y[9 * (size_t)c + 3 * (k - 1) + 2] = d.z;
        const v3 dx = ld3(x, id[0]) - ld3(x, id[k]);
        pos[3 * (k - 1)] = dx.x;
        pos[3 * (k - 1) + 1] = dx.y;
        pos[3 * (k - 1) + 2] = dx.z;
    }
    for (int k = 3 * (nv - 1); k < 9; ++k) y[9 * (size_t)c + k] = 0.0;
    for (int k = 0; k < 9; ++k) r[9 * (size_t)c + k] = 0.0;
    v3 X0[4];
    for (int k = 0; k < 4; ++k) X0[k] = t >= T_EEM ? ld3(x0, id[k]) : mk(0, 0, 0);
    double E, fro;
    rel_row(t, pos, X0, dh2, kappa, &E, nullptr, nullptr, &fro);
    Q[c] = fmin(fmax(sqrt(fro), minQ), maxQ);
}

// global_step, constraint part (ADMM_IPC.py:413-547): Q^2 E^T E in 3x3 blocks (E maps the row's
// vertices to its relative vectors) and the right-hand side Q^2 E^T (y - r), as the gradient
// slot the contact reduction subtracts
__global__ void k_admm_global_rows(int n, TypeTable tt, const double* __restrict__ y, const double* __restrict__ r,
                                   const double* __restrict__ Q, double* __restrict__ cg, double* __restrict__ cH) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const int nv = type_nverts(row_type(tt, c));
    const double q2 = Q[c] * Q[c];
    double* H = cH + 144 * (size_t)c;
    for (int v = 0; v < nv; ++v)
        for (int w = 0; w < nv; ++w) {
            const double k = (v == 0 && w == 0) ? (nv - 1) : ((v == 0 || w == 0) ? -1.0 : (v == w ? 1.0 : 0.0));
            for (int i = 0; i < 9; ++i) H[(v * 4 + w) * 9 + i] = (i % 4 == 0) ? k * q2 : 0.0;
        }
    double* g = cg + 12 * (size_t)c;
    for (int d = 0; d < 3; ++d) {
        double s = 0.0;
        for (int k = 1; k < nv; ++k) {
            const double yr = (y[9 * (size_t)c + 3 * (k - 1) + d] - r[9 * (size_t)c + 3 * (k - 1) + d]) * q2;
            g[3 * k + d] = yr;   // the reduction subtracts: vertex k gets -Q^2 (y_k - r_k)
            s += yr;
        }
        g[d] = -s;               // vertex 0 gets +Q^2 sum (y_k - r_k)
    }
}

// local_PP .. local_PEM (ADMM_IPC.py:668-960): per row, Newton in the relative vectors pos on
// barrier(pos) + Q^2 / 2 |pos - (x-relative + r)|^2, regularised solve_N steps, halving while
// the energy rises; y = pos.  One warp per row: lane 0 forms the Newton step, then the lanes
// evaluate the energy at the step sizes 2^-k for k = lane, 32 + lane and 64 at once, and the
// smallest k whose energy does not rise is taken -- the step size, and every bit of the new
// point, the sequential halving loop would reach.
__global__ void __launch_bounds__(64) k_admm_local_rows(int n, const int4* __restrict__ rows, TypeTable tt, const double* __restrict__ x,
                                                        const double* __restrict__ x0, double dh2, double kappa, const double* __restrict__ Q,
                                                        const double* __restrict__ r, double* __restrict__ y, int* __restrict__ status) {
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (c >= n) return;
    const unsigned full = 0xffffffffu;
    const int t = row_type(tt, c);
    const int nv = type_nverts(t), m = 3 * (nv - 1);
    const int4 q = rows[c];
    const int id[4] = {q.x, q.y, q.z, q.w};
    double pos[9], tgt[9];
    for (int k = 0; k < 9; ++k) pos[k] = tgt[k] = 0.0;
    for (int k = 1; k < nv; ++k) {
        const v3 d = ld3(x, id[0]) - ld3(x, id[k]);
        const double dd[3] = {d.x, d.y, d.z};
        for (int j = 0; j < 3; ++j) {
            pos[3 * (k - 1) + j] = dd[j];
            tgt[3 * (k - 1) + j] = dd[j] + r[9 * (size_t)c + 3 * (k - 1) + j];
        }
    }
    v3 X0[4];
    for (int k = 0; k < 4; ++k) X0[k] = t >= T_EEM ? ld3(x0, id[k]) : mk(0, 0, 0);
    const double q2 = Q[c] * Q[c];
    auto energy = [&](const double* ps) {
        double E;
        rel_row(t, ps, X0, dh2, kappa, &E, nullptr, nullptr, nullptr);
        double s = 0.0;
        for (int i = 0; i < m; ++i) s += (ps[i] - tgt[i]) * (ps[i] - tgt[i]);
        return E + s * q2 / 2;
    };
    int stat = 0;
    bool converged = false;
    int it = 0;
    while (!converged) {
        if (++it > ADMM_MAX_NEWTON) {
            stat |= ADMM_ROW_NEWTON;
            break;
        }
        double p[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, E0 = 0.0;
        int conv = 0;
        if (lane == 0) {
            double E, g[9], P[81];
            rel_row(t, pos, X0, dh2, kappa, &E, g, P, nullptr);
            for (int i = 0; i < m; ++i) {
                g[i] += (pos[i] - tgt[i]) * q2;
                P[i * m + i] += q2;
            }
            solve_n(m, P, g, p);
            double pp = 0.0;
            for (int i = 0; i < m; ++i) {
                p[i] = -p[i];
                pp += p[i] * p[i];
            }
            conv = pp < 1e-6;
            E0 = energy(pos);
        }
        for (int i = 0; i < 9; ++i) p[i] = __shfl_sync(full, p[i], 0);
        E0 = __shfl_sync(full, E0, 0);
        converged = __shfl_sync(full, conv, 0) != 0;
        double p0[9];
        for (int i = 0; i < 9; ++i) p0[i] = pos[i];
        // step sizes 2^-k, k = 0 .. ADMM_MAX_HALVINGS: the first whose energy does not rise
        int kstar = -1;
        for (int base = 0; base <= ADMM_MAX_HALVINGS && kstar < 0; base += 32) {
            const int k = base + lane;
            bool ok = false;
            if (k <= ADMM_MAX_HALVINGS) {
                double alpha = 1.0, ps[9];
                for (int h = 0; h < k; ++h) alpha *= 0.5;
                for (int i = 0; i < m; ++i) ps[i] = k == 0 ? p0[i] + p[i] : p0[i] + alpha * p[i];
                ok = !(energy(ps) > E0);
            }
            const unsigned bal = __ballot_sync(full, ok);
            if (bal) kstar = base + __ffs(bal) - 1;
        }
        if (kstar < 0) {
            kstar = ADMM_MAX_HALVINGS;
            stat |= ADMM_ROW_HALVING;
        }
        double alpha = 1.0;
        for (int h = 0; h < kstar; ++h) alpha *= 0.5;
        for (int i = 0; i < m; ++i) pos[i] = kstar == 0 ? p0[i] + p[i] : p0[i] + alpha * p[i];
        // a step that left pos exactly where it was repeats itself in every later iteration:
        // the loop would run to its bound without moving, so stop here with the same result
        bool same = true;
        for (int i = 0; i < m; ++i) same = same && pos[i] == p0[i];
        if (!converged && same) {
            stat |= ADMM_ROW_NEWTON;
            break;
        }
    }
    if (lane != 0) return;
    bool finite = true;
    for (int i = 0; i < m; ++i) {
        finite = finite && isfinite(pos[i]);
        y[9 * (size_t)c + i] = pos[i];
    }
    if (!finite) stat |= ADMM_NONFINITE;
    if (stat) atomicOr(status, stat);
}

// dual_step, constraint part (ADMM_IPC.py:968-994): r_k += (x_c0 - x_ck) - y_k
__global__ void k_admm_dual_rows(int n, const int4* __restrict__ rows, TypeTable tt, const double* __restrict__ x,
                                 const double* __restrict__ y, double* __restrict__ r) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const int nv = type_nverts(row_type(tt, c));
    const int4 q = rows[c];
    const int id[4] = {q.x, q.y, q.z, q.w};
    for (int k = 1; k < nv; ++k) {
        const v3 d = ld3(x, id[0]) - ld3(x, id[k]);
        const double dd[3] = {d.x, d.y, d.z};
        for (int j = 0; j < 3; ++j) r[9 * (size_t)c + 3 * (k - 1) + j] += dd[j] - y[9 * (size_t)c + 3 * (k - 1) + j];
    }
}

static inline int nblk_a(long long n, int b) { return (int)((n + b - 1) / b); }

// the current lists concatenated (rows_tmp) with their type table
static int current_rows(fipc_ctx* c, TypeTable* tt, int* n, cudaStream_t s) {
    long long nent = 0;
    return contact_prepare(c, tt, n, &nent, s);
}

static TypeTable table_of(const int* counts_h) {
    TypeTable t;
    int off = 0;
    long long eoff = 0;
    for (int k = 0; k < N_TYPES; ++k) {
        t.row0[k] = off;
        t.ent0[k] = eoff;
        off += counts_h[k];
        eoff += (long long)counts_h[k] * type_nverts(k) * type_nverts(k);
    }
    t.row0[N_TYPES] = off;
    t.ent0[N_TYPES] = eoff;
    return t;
}

// Frobenius norm of the PP row Hessian at relative vector (d, d, d) (the reuse step's Q bounds)
static double pp_hessian_norm(double d, double dh2, double kappa) {
    const v3 X[4] = {mk(0, 0, 0), mk(d, d, d), mk(0, 0, 0), mk(0, 0, 0)};
    double E, g[12], Hb[144];
    barrier_row(T_PP, X, X, dh2, kappa, 2, &E, g, Hb);
    double s = 0.0;
    for (int v = 0; v < 2; ++v)
        for (int w = 0; w < 2; ++w)
            for (int i = 0; i < 9; ++i) s += Hb[(v * 4 + w) * 9 + i] * Hb[(v * 4 + w) * 9 + i];
    return sqrt(s);
}

}  // namespace fipc

using namespace fipc;

extern "C" {

int fipc_admm_init(fipc_ctx* c, const double* xtilde, double* W, double* z, double* u, void* stream) {
    if (!c || !xtilde || (c->nT && (!W || !z || !u))) return FIPC_ERR_ARGUMENT;
    if (c->nT == 0) return FIPC_OK;
    k_admm_init<<<nblk_a(c->nT, 128), 128, 0, (cudaStream_t)stream>>>(c->nT, (const int4*)c->tets, xtilde, c->dminv, c->vol, c->lam, c->mu,
                                                                      c->dt * c->dt, W, z, u);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc_admm_reuse(fipc_ctx* c, double alpha, const double* x, const double* xtilde, const int* old_counts_h, const int* old_rows,
                    const double* old_y, const double* old_r, const double* old_Q, double* y, double* r, double* Q, void* stream) {
    if (!c || !x || !xtilde || !old_counts_h) return FIPC_ERR_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    TypeTable tt;
    int n = 0;
    int st = current_rows(c, &tt, &n, s);
    if (st) return st;
    const TypeTable ot = table_of(old_counts_h);
    if (n == 0) return FIPC_OK;
    if (!y || !r || !Q || (ot.row0[N_TYPES] > 0 && (!old_rows || !old_y || !old_r || !old_Q))) return FIPC_ERR_ARGUMENT;
    const double dhat = sqrt(c->dhat2);
    const double minQ = sqrt(pp_hessian_norm(9e-1 * dhat, c->dhat2, c->kappa)) / 10;
    const double maxQ = sqrt(pp_hessian_norm(1e-4 * dhat, c->dhat2, c->kappa)) * 10;
    k_admm_reuse<<<nblk_a(n, 128), 128, 0, s>>>(n, c->rows_tmp.as<int4>(), tt, x, xtilde, c->x0, alpha, c->dhat2, c->kappa, minQ, maxQ,
                                                (const int4*)old_rows, ot, old_y, old_r, old_Q, y, r, Q);
    FIPC_LAUNCHED();
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

int fipc_admm_global(fipc_ctx* c, const double* xtilde, const double* W, const double* z, const double* u, const double* y,
                     const double* r, const double* Q, const unsigned char* fixed, double rtol, int maxit, double* x, int* iters_h,
                     void* stream) {
    if (!c || !xtilde || !fixed || !x || (c->nT && (!W || !z || !u)) || rtol <= 0 || maxit <= 0) return FIPC_ERR_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    int st = cs_offsets(c, x, s);
    if (st) return st;
    if (c->nT) {
        k_admm_global_elem<<<nblk_a(c->nT, 128), 128, 0, s>>>(c->nT, c->dminv, W, z, u, c->elem_H, c->elem_g);
        FIPC_LAUNCHED();
    }
    st = assemble_elastic(c, s);
    if (st) return st;
    k_admm_rhs<<<nblk_a(c->nV, 128), 128, 0, s>>>(c->nV, c->vt_ptr, c->vt_list, c->elem_g, c->mass, xtilde, c->rhs);
    FIPC_LAUNCHED();
    TypeTable tt;
    int n = 0;
    long long nent = 0;
    st = contact_prepare(c, &tt, &n, &nent, s);
    if (st) return st;
    if (n > 0) {
        if (!y || !r || !Q) return FIPC_ERR_ARGUMENT;
        k_admm_global_rows<<<nblk_a(n, 128), 128, 0, s>>>(n, tt, y, r, Q, c->c_g.as<double>(), c->c_H.as<double>());
        FIPC_LAUNCHED();
        st = contact_reduce(c, tt, n, nent, s);
        if (st) return st;
    }
    FIPC_CUDA(cudaGetLastError());
    return pcg_solve(c, fixed, nullptr, rtol, maxit, x, iters_h, s);
}

int fipc_admm_local(fipc_ctx* c, const double* x, const double* W, double* z, const double* u, double* y, const double* r,
                    const double* Q, int* detail_h, void* stream) {
    if (!c || !x || (c->nT && (!W || !z || !u))) return FIPC_ERR_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    if (c->scal.ensure(64)) return FIPC_ERR_CUDA;
    int* status = (int*)(c->scal.as<char>() + 40);
    FIPC_CUDA(cudaMemsetAsync(status, 0, sizeof(int), s));
    if (c->nT) {
        k_admm_local_elastic<<<nblk_a(c->nT, 128), 128, 0, s>>>(c->nT, (const int4*)c->tets, x, c->dminv, c->vol, c->lam, c->mu,
                                                                c->dt * c->dt, W, z, u, status);
        FIPC_LAUNCHED();
    }
    TypeTable tt;
    int n = 0;
    int st = current_rows(c, &tt, &n, s);
    if (st) return st;
    if (n > 0) {
        if (!y || !r || !Q) return FIPC_ERR_ARGUMENT;
        k_admm_local_rows<<<nblk_a(32ll * n, 64), 64, 0, s>>>(n, c->rows_tmp.as<int4>(), tt, x, c->x0, c->dhat2, c->kappa, Q, r, y, status);
        FIPC_LAUNCHED();
    }
    int h = 0;
    FIPC_CUDA(cudaMemcpyAsync(&h, status, sizeof(int), cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaStreamSynchronize(s));
    if (detail_h) *detail_h = h;
    return (h & ADMM_NONFINITE) ? FIPC_ERR_NONFINITE : FIPC_OK;
}

int fipc_admm_dual(fipc_ctx* c, const double* x, const double* z, double* u, const double* y, double* r, void* stream) {
    if (!c || !x || (c->nT && (!z || !u))) return FIPC_ERR_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    if (c->nT) {
        k_admm_dual_elem<<<nblk_a(c->nT, 128), 128, 0, s>>>(c->nT, (const int4*)c->tets, x, c->dminv, z, u);
        FIPC_LAUNCHED();
    }
    TypeTable tt;
    int n = 0;
    int st = current_rows(c, &tt, &n, s);
    if (st) return st;
    if (n > 0) {
        if (!y || !r) return FIPC_ERR_ARGUMENT;
        k_admm_dual_rows<<<nblk_a(n, 128), 128, 0, s>>>(n, c->rows_tmp.as<int4>(), tt, x, y, r);
        FIPC_LAUNCHED();
    }
    FIPC_CUDA(cudaGetLastError());
    return FIPC_OK;
}

}  // extern "C"
