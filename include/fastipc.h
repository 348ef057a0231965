/*
 * libfastipc — C ABI of the GB300 (sm_103a) implementation of FastIPC's IPC Newton inner loop.
 *
 * Each entry point replaces one Taichi kernel (or one piece of the native a.so) of the
 * reference, cited as file:line relative to the FastIPC checkout.  All array arguments are
 * DEVICE pointers unless the name ends in _h (host).  Positions are vertex-major [V][3] FP64;
 * constraint rows are [n][4] int32 (unused trailing ids zero); tets [T][4] int32.  `stream`
 * is a cudaStream_t (NULL for the legacy default stream).  Every function returns a status:
 * 0 ok, 1 capacity exceeded, 2 iteration limit, 3 non-finite value, 4 CUDA error,
 * 5 invalid argument, 6 file I/O error.  The library allocates its own scratch inside a
 * context and never frees caller memory.  Calls on one context are not reentrant.
 */
#ifndef FASTIPC_H
#define FASTIPC_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fipc_ctx_impl fipc_ctx;

/* constraint list ids, in the reference's list order (NEWTON_IPC.py:349) */
enum { FIPC_PP = 0, FIPC_PE = 1, FIPC_PT = 2, FIPC_EE = 3, FIPC_EEM = 4, FIPC_PPM = 5, FIPC_PEM = 6 };

/* ---- stateless element kernels ------------------------------------------------------------ */

/* Neo-Hookean tets: gradient g [T][12] and the 10 upper 3x3 blocks Hu [T][90]
 * ((0,0)(0,1)(0,2)(0,3)(1,1)(1,2)(1,3)(2,2)(2,3)(3,3)) of dt^2 vol0 psi(Ds Dm^-1), energy E [T]
 * (may be NULL).  Replaces compute_elasticity, NEWTON_IPC.py:568-691, with the material of
 * common/physics/neo_hookean.py:6-131. */
int fipc_elasticity(int n_tets, const int* tets, const double* x, const double* dm_inv, const double* vol,
                    const double* lam, const double* mu, double dt, double* E, double* g, double* Hu, void* stream);

/* Barrier energy E [n], gradient g [n][12] and PSD-projected Hessian H [n][16][9] (3x3 vertex
 * blocks v*4+w) of n rows of one constraint list; x0 = rest positions (mollified lists).
 * Replaces PP/PE/PT/EE/EEM/PPM/PEM_g_and_H, common/math/ipc.py:67-329, and the a.so
 * project_pd_{6,9,12} calls of common/math/math_tools.py:101-128. */
int fipc_barrier_rows(int type, int n_rows, const int* rows, const double* x, const double* x0, double dhat2,
                      double kappa, double* E, double* g, double* H, void* stream);

/* Time of impact of explicit primitive pairs xq/pq [n][4][3] (kind 0: point-triangle,
 * 1: edge-edge) with the current-distance argument computed as NEWTON_IPC.py:404/:438 do.
 * Replaces a.so point_triangle_ccd / edge_edge_ccd (common/math/wrapper/wrapper.cpp:254-328). */
int fipc_ccd_pairs(int kind, int n, const double* xq, const double* pq, double eta, double* toc, void* stream);

/* Inversion-free step per tet, xs/ps [n][4][3].  Replaces
 * get_smallest_positive_real_cubic_root, common/math/math_tools.py:161-181. */
int fipc_inversion_free_pairs(int n, const double* xs, const double* ps, double eta, double* out, void* stream);

/* ---- vector updates of the Newton loop ---------------------------------------------------- */
int fipc_compute_xn_and_xtilde(int n_verts, const double* x, const double* v, double dt, double gravity, double* xn,
                               double* xtilde, void* stream);                 /* NEWTON_IPC.py:497-502 */
int fipc_move_nodes(int n_verts, const unsigned char* fixed, const double* target, double* x, double* xtilde,
                    void* stream);                                             /* NEWTON_IPC.py:505-511 */
/* Dirichlet schedule settings['dirichlet'](t) (projects/FastIPC/reader.py:154-357, consumed by
 * move_nodes and solve_system, NEWTON_IPC.py:505-511, 758-763) evaluated on the device when it
 * is a rigid motion of vertex groups.  group [V] int32 (< 0: free); motion [n_groups][10] =
 * (centre c[3], unit axis a[3], omega rad/s, velocity u[3]); vertex i of group g gets
 * target = c + R(a, omega t)(x_rest_i - c) + u t and fixed = 1.  Free vertices get fixed = 0 and
 * target = x_rest.  Covers the reference's static masks (omega = 0, u = 0: target = x_rest
 * exactly when c = 0), mat twist (reader.py:170-185) and translating faces (reader.py:336-345). */
int fipc_dirichlet_script(int n_verts, const double* x_rest, const int* group, int n_groups, const double* motion, double t,
                          unsigned char* fixed, double* target, void* stream);
int fipc_apply_sol(int n_verts, const double* xprev, const double* sol, double alpha, double* x,
                   void* stream);                                              /* NEWTON_IPC.py:792-796 */
int fipc_compute_v(int n_verts, const double* x, const double* xn, double dt, double* v,
                   void* stream);                                              /* NEWTON_IPC.py:799-802 */

/* ---- scene context: the module state of NEWTON_IPC.py -------------------------------------- */

/* Host inputs.  Computes rest shapes, volumes and lumped mass (NEWTON_IPC.py:485-494), the
 * adaptive kappa x10 (:116-124, :943), inv_dx = 1/mean boundary edge (:127-134, :944; the hash
 * itself uses the median edge, which finds the same lists)
 * and the static block pattern.  x_rest is also the mollifier rest shape (save_x0, :780-783). */
int fipc_ctx_create(fipc_ctx** ctx, int n_verts, int n_tets, const int* tets_h, const double* x_rest_h,
                    const double* lam_h, const double* mu_h, double rho, int n_bp, const int* bp_h, int n_be,
                    const int* be_h, int n_bt, const int* bt_h, double dhat2, double dt);
int fipc_ctx_destroy(fipc_ctx* ctx);
int fipc_ctx_params(fipc_ctx* ctx, double* kappa_h, double* inv_dx_h, int* nnzb_h);
int fipc_ctx_set_params(fipc_ctx* ctx, double kappa, double inv_dx);
int fipc_ctx_mass(fipc_ctx* ctx, double* mass_h);
int fipc_ctx_set_x0(fipc_ctx* ctx, const double* x0, void* stream);
/* Preconditioner of fipc_solve_system: agg_rows = 0 selects block-Jacobi; a positive multiple of
 * 128 adds the coarse correction on the six rigid-body modes of every run of agg_rows
 * consecutive vertices (at most 1024 runs).  Either switches the multigrid preconditioner below
 * off.  The solution satisfies the same tolerance with every preconditioner. */
int fipc_ctx_set_preconditioner(fipc_ctx* ctx, int agg_rows);
int fipc_ctx_preconditioner(fipc_ctx* ctx, int* agg_rows, int* n_coarse);
/* Multigrid preconditioner of fipc_solve_system (no counterpart in the reference, which solves
 * directly): geometric aggregation of the rest shape into boxes (the first three cells h wide,
 * each coarser level's twice the last, never across two bodies), six rigid-body modes per
 * aggregate, Galerkin coarse matrices rebuilt every Newton iteration (contact blocks included),
 * one symmetric V(1,1)-cycle with damped block-Jacobi smoothing per PCG iteration, dense inverse
 * at the coarsest level.  When in use it replaces the coarse correction selected above.  on = 0
 * switches it off; h <= 0 takes the spatial hash's cell.  Created on by default for
 * single-scene contexts of at least 1000 vertices.  fipc_ctx_multigrid: levels in use (0:
 * off) and nodes per level (nodes_h: 8 ints, may be NULL). */
int fipc_ctx_set_multigrid(fipc_ctx* ctx, int on, double h);
int fipc_ctx_multigrid(fipc_ctx* ctx, int* levels, int* nodes_h);
/* Precision of the V-cycle's two level-0 smoothing products (the residual after pre-smoothing
 * and the post-smoothing product): 1 = FP32 copies of the values and of the iterate with FP32
 * sums, the residuals and the smoother updates in FP64 (the default); 0 = FP64.  The PCG's own
 * product, its recurrences and the coarser levels are FP64 either way; the solve's tolerance is
 * unchanged. */
int fipc_ctx_set_multigrid_fp32(fipc_ctx* ctx, int on);
/* In-place inverse of a dense SPD matrix on the device (n a multiple of 32, row-major; work: 1024
 * + 64 n doubles): the symmetric block sweep (Gauss-Jordan sweep operator on the lower triangle's
 * 32 x 32 tiles) used for the coarse matrices, one cooperative launch; the result is exactly
 * symmetric. */
int fipc_dense_spd_inverse(int n, double* a, double* work, void* stream);

/* find_constraints, NEWTON_IPC.py:337-357 (spatial hash :213-334, dedup :348-356): the seven
 * lists, sorted lexicographically and de-duplicated; counts_h [7] receives their sizes. */
int fipc_find_constraints(fipc_ctx* ctx, const double* x, int* counts_h, void* stream);
int fipc_get_constraints(fipc_ctx* ctx, int type, int* rows, void* stream);

/* compute_hessian_and_gradient, NEWTON_IPC.py:736-747 (inertia :558-567, elasticity
 * :568-691, barriers :692-733): block-sparse system and right-hand side -grad. */
int fipc_compute_hessian_and_gradient(fipc_ctx* ctx, const double* x, const double* xtilde, void* stream);
int fipc_system_sizes(fipc_ctx* ctx, int* nnzb_elastic_h, int* nnzb_contact_h);
int fipc_export_system(fipc_ctx* ctx, int* row_ptr, int* col_idx, double* val, int* c_row_ptr, int* c_col_idx,
                       double* c_val, double* rhs, void* stream);

/* solve_system, NEWTON_IPC.py:750-777: Newton direction with Dirichlet vertices (fixed [V])
 * held at zero, by block-Jacobi PCG to relative residual rtol (iters_h: iterations used).
 * use_guess = 0 starts from zero (the reference's semantics); otherwise sol holds the
 * initial guess on entry. */
int fipc_solve_system(fipc_ctx* ctx, const unsigned char* fixed, double rtol, int maxit, int use_guess, double* sol,
                      int* iters_h, void* stream);

/* output_residual, NEWTON_IPC.py:805-812: max |sol| */
/* solve_system by a sparse Cholesky factorisation instead of PCG: the reference's CHOLMOD solve
 * (NEWTON_IPC.py:758-776) for the assembled system with its Dirichlet edit, for iterations
 * where fipc_solve_system reaches its iteration limit.  A multifrontal factorisation on the GPU
 * (nested-dissection ordering on the host); status 3 when the system is not positive definite,
 * 1 when its fronts do not fit in free device memory.  nnz_h (may be NULL): entries stored in
 * the factor's fronts (lower triangles), saturated at INT_MAX. */
int fipc_solve_system_direct(fipc_ctx* ctx, const unsigned char* fixed, double* sol, int* nnz_h, void* stream);
/* the last direct solve (no counterpart in the reference): fronts of its assembly tree, doubles
 * of front storage, dense factorisation flops, host analysis time in ms (each may be NULL) */
int fipc_direct_stats(const fipc_ctx* ctx, int* fronts_h, long long* front_doubles_h, double* flops_h, double* analyse_ms_h);
int fipc_output_residual(fipc_ctx* ctx, const double* sol, double* res_h, void* stream);

/* compute_energy, NEWTON_IPC.py:514-542, over the lists of the last find_constraints */
int fipc_compute_energy(fipc_ctx* ctx, const double* x, const double* xtilde, double* e_h, void* stream);

/* Allocation-free compute_energy for callers that cannot allocate device memory while running
 * (a host application that reserves all device memory in one arena at start-up and forbids
 * cudaMalloc afterwards, since it synchronises the device and can fail against the arena).  No
 * counterpart in the reference.  Stateless: the caller passes mass [V], tets [T][4], dm_inv
 * [T][9], vol/lam/mu [T], counts_h [7] (host) and rows_h [7] (host array of device row
 * pointers), and receives the total in *energy (device).  It covers one scene with one kappa:
 * for the concatenated scenes of a batch context (whose energy takes kappa per scene) it does
 * not reproduce fipc_batch_compute_energy.  tets and every rows_h[t] with counts_h[t] > 0 must
 * be 16-byte aligned and the double arrays 8-byte aligned (status 5 otherwise, before anything
 * runs).  The reduction's partial sums live in a fixed file-scope device array of 65,536 doubles
 * (512 KiB per GPU that loads the library, held until exit): one partial per 256 vertices, tets
 * or rows, so requests needing more (about 16.7M elements in total) return status 1.  The first
 * call on a device looks up that array and loads the kernels it launches, which can allocate
 * and synchronise: make it at start-up, before the arena takes the memory and before any stream
 * capture (a call with all sizes zero is enough).  The lookup is not redone after
 * cudaDeviceReset.  Calls that overlap on the GPU share the array and race. */
int fipc_compute_energy_noalloc(int n_verts, const double* x, const double* xtilde, const double* mass, int n_tets,
                                const int* tets, const double* dm_inv, const double* vol, const double* lam,
                                const double* mu, double dt, const int* counts_h, const int* const* rows_h,
                                const double* x0, double dhat2, double kappa, double* energy, void* stream);

/* compute_intersection_free_step_size, NEWTON_IPC.py:456-468 (PT :377-406, EE :409-440,
 * inversion :443-453 when `inversion` is nonzero) */
int fipc_compute_intersection_free_step_size(fipc_ctx* ctx, const double* x, const double* p, double eta, int inversion,
                                             double* alpha_h, void* stream);

/* check_collision, NEWTON_IPC.py:855-886 */
int fipc_check_collision(fipc_ctx* ctx, const double* x, int* hit_h, void* stream);

/* ---- ADMM-IPC (projects/FastIPC/ADMM_IPC.py) ----------------------------------------------
 * The ADMM variant of the time step on a context (fixed-corotated elasticity, as the script
 * imports).  Per tet: W [T], z [T][9], u [T][9].  Per constraint row of the current lists, in
 * list order (the seven lists concatenated): y, r [n][9] (the row's nv-1 relative vectors
 * x_c0 - x_ck, padded to 3) and Q [n].  The caller runs the iteration loop (ADMM_IPC.py:
 * 1471-1526): fipc_find_constraints, fipc_admm_reuse, fipc_admm_global, the CCD filter
 * (fipc_compute_intersection_free_step_size without the inversion filter, and
 * fipc_check_collision), fipc_admm_local, fipc_admm_dual. */
/* initial_guess, ADMM_IPC.py:296-313: W, z = F(xtilde), u = 0 */
int fipc_admm_init(fipc_ctx* ctx, const double* xtilde, double* W, double* z, double* u, void* stream);
/* reuse_admm_variables, ADMM_IPC.py:1230-1388, for the lists of the last find_constraints:
 * old_counts_h [7] and old_rows [n_old][4] (the previous lists, concatenated in list order)
 * with their old_y, old_r, old_Q; fills y, r, Q of the current rows. */
int fipc_admm_reuse(fipc_ctx* ctx, double alpha, const double* x, const double* xtilde, const int* old_counts_h,
                    const int* old_rows, const double* old_y, const double* old_r, const double* old_Q, double* y, double* r,
                    double* Q, void* stream);
/* global_step + global_PP..PEM + solve_system, ADMM_IPC.py:388-631: assembles the SPD system
 * (mass, W^2 G G^T per tet, Q^2 E^T E per row) and solves it by PCG to relative residual rtol;
 * x holds the guess on entry with the Dirichlet targets at the fixed vertices, which keep them,
 * and the solution on return. */
int fipc_admm_global(fipc_ctx* ctx, const double* xtilde, const double* W, const double* z, const double* u, const double* y,
                     const double* r, const double* Q, const unsigned char* fixed, double rtol, int maxit, double* x,
                     int* iters_h, void* stream);
/* local_elasticity + local_PP..PEM, ADMM_IPC.py:633-960: updates z and y.  The reference's
 * local loops are unbounded; here each stops after 256 Newton iterations or 64 halvings (a row
 * with an indefinite Hessian can take steps that never fall below the tolerance).  detail_h
 * (may be null) receives the bits: 1 / 2 a tet reached its Newton / halving bound, 4 / 8 a row,
 * 16 a non-finite z or y.  Status 3 when a result is not finite. */
int fipc_admm_local(fipc_ctx* ctx, const double* x, const double* W, double* z, const double* u, double* y, const double* r,
                    const double* Q, int* detail_h, void* stream);
/* dual_step, ADMM_IPC.py:962-994: u += F(x) - z, r += (x_c0 - x_ck) - y */
int fipc_admm_dual(fipc_ctx* ctx, const double* x, const double* z, double* u, const double* y, double* r, void* stream);

/* ---- learned Newton warm start (no counterpart in the reference) ----------------------------
 * A per-vertex MLP 55 (padded 64) -> 128 -> 128 -> 128 -> 3 (padded 4), GELU, FP32, parameters
 * in one flat array (W1 [128][64], b1, W2 [128][128], b2, W3, b3, W4 [4][128], b4). */
int fipc_mlp_param_count(void);
/* out [n][4] = MLP(X [n][64]); Z, A: scratch [3][n][128] kept for the backward pass */
int fipc_mlp_forward(int n, const float* X, const float* params, float* Z, float* A, float* out, void* stream);
/* grads (params layout) of sum(dout . out) for that forward pass; dA: scratch [2][n][128] */
int fipc_mlp_backward(int n, const float* X, const float* params, const float* Z, const float* A, const float* dout,
                      float* grads, float* dA, void* stream);
/* mean squared error over the first 3 outputs into *loss (device) and its gradient dout [n][4];
 * part: scratch of ceil(n/256) floats */
int fipc_mlp_mse(int n, const float* out, const float* target, float* dout, float* part, float* loss, void* stream);
/* one Adam step, t >= 1 */
int fipc_mlp_adam(int n_params, float* params, const float* grads, float* m, float* v, float lr, float beta1, float beta2,
                  float eps, int t, void* stream);
/* per-vertex inputs X [V][64] at positions x: 16 one-ring relative positions / h (x_j - x_i, or
 * with rest_relative (x_j - x_i) - (X_j - X_i) against the rest shape), v dt / h, dx_prev / h
 * (the Python driver passes the displacement of the step before the last one), min(nearest
 * constraint distance / d-hat, 1) over the lists of the last fipc_find_constraints */
int fipc_mlp_features(fipc_ctx* ctx, const double* x, const double* v, const double* dx_prev, double h, int rest_relative,
                      float* X, void* stream);
/* passes of one-ring averaging of a displacement d [V][3] over the elastic block pattern, zero on
 * Dirichlet vertices (in place; tmp: scratch [V][3]) */
int fipc_mlp_smooth(fipc_ctx* ctx, const unsigned char* fixed, double* d, double* tmp, int passes, void* stream);

/* ---- batched scenes ---------------------------------------------------------------------- *
 * S independent scenes (1 <= S <= 1024) in one context, each stepping its own Newton loop of
 * NEWTON_IPC.py:955-999.  The arrays are the concatenation of the scenes' arrays with global
 * vertex ids: scene s owns vertices [vert_off[s], vert_off[s+1]), tets [tet_off[s],
 * tet_off[s+1]) and boundary edges [be_off[s], be_off[s+1]); boundary points and triangles
 * each lie in one scene.  Every single-scene entry point above accepts a batch context and
 * then works per scene where the reference's quantity is per scene (hash cell size and kappa
 * per scene, NEWTON_IPC.py:116-134; keys of different scenes never meet).  The entries below
 * return one value per scene into device arrays of S. */
int fipc_batch_create(fipc_ctx** out, int n_scenes, const int* vert_off, const int* tet_off, const int* be_off, int n_verts,
                      int n_tets, const int* tets, const double* x_rest, const double* lam, const double* mu, double rho,
                      int n_bp, const int* bp, int n_be, const int* be, int n_bt, const int* bt, double dhat2, double dt);
/* host copies of the per-scene kappa and inverse hash cell size (arrays of S) */
int fipc_batch_params(fipc_ctx* ctx, int* n_scenes, double* kappa, double* inv_dx);
/* compute_energy (NEWTON_IPC.py:515-542) per scene */
int fipc_batch_compute_energy(fipc_ctx* ctx, const double* x, const double* xtilde, double* energy, void* stream);
/* output_residual (NEWTON_IPC.py:806-812) per scene: max |sol| over the scene's DOFs */
int fipc_batch_output_residual(fipc_ctx* ctx, const double* sol, double* residual, void* stream);
/* compute_intersection_free_step_size (NEWTON_IPC.py:456-468) per scene */
int fipc_batch_step_size(fipc_ctx* ctx, const double* x, const double* sol, double eta, int inversion, double* alpha,
                         void* stream);
/* check_collision (NEWTON_IPC.py:881-886) per scene: hit[s] = 1 when scene s intersects */
int fipc_batch_check_collision(fipc_ctx* ctx, const double* x, int* hit, void* stream);
/* apply_sol (NEWTON_IPC.py:792-796) with alpha[scene] */
int fipc_batch_apply_sol(fipc_ctx* ctx, const double* x_prev, const double* sol, const double* alpha, double* x, void* stream);
/* solve_system (NEWTON_IPC.py:750-777) for every scene with active[s] != 0 (null: all); the
 * others get sol = 0.  PCG with per-scene scalars and tolerance (relative to the scene's |rhs|),
 * persistent kernels over a tile table, iterations replayed as a captured CUDA graph; the
 * tile shape and grid are chosen by timing at the first call.  iters: device int[S] or null;
 * *n_failed (host): scenes that hit maxit (status 2 when any did). */
int fipc_batch_solve_system(fipc_ctx* ctx, const unsigned char* fixed, const unsigned char* active, double rtol, int maxit,
                            int use_guess, double* sol, int* iters, int* n_failed, void* stream);
/* the PCG shape the timing picked: rows per tile (= threads per block), grid, tiles, SpMV ms */
int fipc_batch_pcg_shape(fipc_ctx* ctx, int* tile_rows, int* grid, int* n_tiles, float* spmv_ms);

/* ---- the 2D path (NEWTON_IPC.py with dim == 2) ---------------------------------------------- */
/* Positions [V][2] FP64, triangles [T][3] int32; fixed-corotated material (the reference's
 * default import, common/physics/fixed_corotated.py); constraints between boundary points and
 * boundary edges only: list 0 = PP rows (a, b), list 1 = PE rows (p, e0, e1), as [n][4] int32. */
typedef struct fipc2d_ctx_impl fipc2d_ctx;

/* compute_restT_and_m (NEWTON_IPC.py:485-494), adaptive kappa x10 (:116-124, :943), mean
 * boundary edge (:127-134).  n_verts < 2^21.  Status 5 on an inverted or degenerate rest
 * triangle. */
int fipc2d_ctx_create(fipc2d_ctx** ctx, int n_verts, int n_tris, const int* tris_h, const double* x_rest_h,
                      const double* lam_h, const double* mu_h, double rho, int n_bp, const int* bp_h, int n_be,
                      const int* be_h, double dhat2, double dt);
int fipc2d_ctx_destroy(fipc2d_ctx* ctx);
int fipc2d_ctx_params(fipc2d_ctx* ctx, double* kappa_h, double* mean_edge_h);
int fipc2d_ctx_set_kappa(fipc2d_ctx* ctx, double kappa);
int fipc2d_ctx_mass(fipc2d_ctx* ctx, double* mass_h);
int fipc2d_compute_xn_and_xtilde(int n_verts, const double* x, const double* v, double dt, double gravity, double* xn,
                                 double* xtilde, void* stream);               /* NEWTON_IPC.py:497-502 */
int fipc2d_move_nodes(int n_verts, const unsigned char* fixed, const double* target, double* x, double* xtilde,
                      void* stream);                                           /* NEWTON_IPC.py:505-511 */
int fipc2d_apply_sol(int n_verts, const double* xprev, const double* sol, double alpha, double* x,
                     void* stream);                                            /* NEWTON_IPC.py:792-796 */
int fipc2d_compute_v(int n_verts, const double* x, const double* xn, double dt, double* v,
                     void* stream);                                            /* NEWTON_IPC.py:799-802 */
/* Stateless kernels (tests): fixed-corotated triangles (NEWTON_IPC.py:577-624) -> energy E [T],
 * gradient g [T][6], Hessian [T][6][6]; barrier rows of list type 0/1 (common/math/ipc.py:67-136,
 * dim 2) -> E [n], g [n][2 nv], H [n][nv*nv][2][2]; point-edge CCD of explicit pairs
 * xq/pq [n][3][2] (common/math/ipc.py:415-481). */
int fipc2d_elements(int n_tris, const int* tris, const double* x, const double* ib, const double* vol, const double* lam,
                    const double* mu, double dt, double* E, double* g, double* H, void* stream);
int fipc2d_barrier_rows(int type, int n_rows, const int* rows, const double* x, double dhat2, double kappa, double* E,
                        double* g, double* H, void* stream);
int fipc2d_ccd_pairs(int n, const double* xq, const double* pq, double eta, double* toc, void* stream);
/* find_constraints_2D_PE + dedup (NEWTON_IPC.py:159-179, 337-357): counts_h [2] */
int fipc2d_find_constraints(fipc2d_ctx* ctx, const double* x, int* counts_h, void* stream);
int fipc2d_get_constraints(fipc2d_ctx* ctx, int type, int* rows, void* stream);
/* compute_hessian_and_gradient (NEWTON_IPC.py:736-747, dim 2): 2x2-block CSR and rhs -grad */
int fipc2d_compute_hessian_and_gradient(fipc2d_ctx* ctx, const double* x, const double* xtilde, void* stream);
int fipc2d_system_nnzb(fipc2d_ctx* ctx, int* nnzb_h);
int fipc2d_export_system(fipc2d_ctx* ctx, int* row_ptr, int* col_idx, double* val, double* rhs, void* stream);
/* solve_system (NEWTON_IPC.py:750-777) by block-Jacobi PCG to |r| <= rtol |b| */
int fipc2d_solve_system(fipc2d_ctx* ctx, const unsigned char* fixed, double rtol, int maxit, double* sol, int* iters_h,
                        void* stream);
int fipc2d_output_residual(fipc2d_ctx* ctx, const double* sol, double* res_h, void* stream);    /* :805-812 */
int fipc2d_compute_energy(fipc2d_ctx* ctx, const double* x, const double* xtilde, double* e_h, void* stream);  /* :514-542 */
/* compute_filter_2D_PE (NEWTON_IPC.py:361-374, 456-468) */
int fipc2d_compute_intersection_free_step_size(fipc2d_ctx* ctx, const double* x, const double* sol, double eta,
                                               double* alpha_h, void* stream);
/* check_collision_2D (NEWTON_IPC.py:843-854) */
int fipc2d_check_collision(fipc2d_ctx* ctx, const double* x, int* hit_h, void* stream);

/* ---- per-frame output ---------------------------------------------------------------------- */
/* write_image for 3D scenes (NEWTON_IPC.py:926-931): the OBJ file at path with one
 * "v %.6f %.6f %.6f" line per vertex and one "f %d %d %d" line (1-based ids) per boundary
 * triangle, byte for byte as the reference's Python formatting writes it.  HOST arrays
 * x_h [V][3] and tris_h [F][3]; host code only (no GPU needed).  Status 6 on a file error. */
int fipc_write_obj(const char* path, int n_verts, const double* x_h, int n_tris, const int* tris_h);

/* ---- diagnostics -------------------------------------------------------------------------- */
/* Time every launch of one kernel with CUDA events on its stream (1 PCG SpMV, 2 PCG update,
 * 3 Neo-Hookean element, 4 barrier rows, 5 elastic assembly; 0 off) and read back the summed
 * milliseconds, launch count and the launches' algorithmic bytes and flops. */
int fipc_profile_enable(int kernel_id);
int fipc_profile_read(double* total_ms_h, long long* launches_h, double* bytes_h, double* flops_h);
/* FP64 throughput probe for the FP64 roofline's denominator (no counterpart in the reference):
 * one launch of blocks x 256 threads, each running 8 independent FMA chains for iters rounds
 * (blocks x 256 x iters x 16 flops); out [blocks * 256] doubles (device) receives the sums. */
int fipc_fp64_fma_probe(int blocks, int iters, double* out, void* stream);
long long fipc_launch_count(void);           /* kernels launched by this library so far */
const char* fipc_status_string(int status);

#ifdef __cplusplus
}
#endif

#endif
