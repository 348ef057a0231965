// C ABI of libfastipc.so: scene context and the Newton-loop entry points that replace the
// Taichi kernels of projects/FastIPC/NEWTON_IPC.py.  Declarations and per-function reference
// citations are in include/fastipc.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "barrier.cuh"
#include "ctx.cuh"

namespace fipc {
int find_constraints(fipc_ctx* c, const double* x, cudaStream_t s);
int ensure_row_capacity(fipc_ctx* c, int cap);
int ccd_step(fipc_ctx* c, const double* x, const double* p, double eta, bool inversion, double* alpha_h, cudaStream_t s);
int check_collision(fipc_ctx* c, const double* x, int* hit_h, cudaStream_t s);
int assemble_system(fipc_ctx* c, const double* x, const double* xt, cudaStream_t s);
int pcg_solve(fipc_ctx* c, const unsigned char* fixed, const int* diag_pos, double rtol, int maxit, double* sol, int* iters,
              cudaStream_t s);
int sell_to_bsr(fipc_ctx* c, double* out, cudaStream_t s);
int launch_energy(const fipc_ctx* c, const double* x, const double* xt, const int* const* rows, const int* counts, double* part,
                  double* out, cudaStream_t s);
int launch_absmax(int n, const double* p, double* part, double* out, cudaStream_t s);
void free_batch(fipc_ctx* c);
int cs_setup(fipc_ctx* c, int agg_rows, const int* row_ptr_h, const int* col_idx_h);
int mg_setup(fipc_ctx* c, double h);
void mg_free(fipc_ctx* c);
void cs_free(fipc_ctx* c);
// 1 / median length of boundary edges [e0, e1) (fallback when there are none)
double median_edge_inv(const double* x, const int* be, int e0, int e1, double fallback) {
    if (e1 <= e0) return fallback;
    std::vector<double> len(e1 - e0);
    for (int i = e0; i < e1; ++i) {
        const int a = be[2 * i], b = be[2 * i + 1];
        const double dx = x[3 * a] - x[3 * b], dy = x[3 * a + 1] - x[3 * b + 1], dz = x[3 * a + 2] - x[3 * b + 2];
        len[i - e0] = std::sqrt(dx * dx + dy * dy + dz * dz);
    }
    std::nth_element(len.begin(), len.begin() + len.size() / 2, len.end());
    const double m = len[len.size() / 2];
    return m > 0 ? 1.0 / m : fallback;
}
// default aggregate size of the two-level preconditioner: 2048 vertices, larger when needed to
// keep the dense coarse matrix at most 6 x 512 square
int default_agg_rows(int n_verts) {
    const int per = (n_verts + 511) / 512;
    const int a = ((per + 127) / 128) * 128;
    return a > 2048 ? a : 2048;
}
}  // namespace fipc

using namespace fipc;

namespace {

template <class T>
int upload(T** dst, const T* src, size_t n) {
    *dst = nullptr;
    if (n == 0) return FIPC_OK;
    if (cudaMalloc((void**)dst, sizeof(T) * n) != cudaSuccess) return FIPC_ERR_CUDA;
    if (cudaMemcpy(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice) != cudaSuccess) return FIPC_ERR_CUDA;
    return FIPC_OK;
}

double det3h(const double* A) {
    return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) + A[2] * (A[3] * A[7] - A[4] * A[6]);
}

void free_ctx(fipc_ctx* c) {
    if (c->pcg3_exec) cudaGraphExecDestroy((cudaGraphExec_t)c->pcg3_exec);
    c->pcg3_exec = nullptr;
    free_batch(c);
    cs_free(c);
    mg_free(c);
    void* ptrs[] = {c->tets, c->bp, c->be, c->bt, c->dminv, c->vol, c->lam, c->mu, c->mass, c->x0, c->row_ptr, c->col_idx,
                    c->up_pos, c->up_tpos, c->up_row, c->up_cptr, c->up_contrib, c->vt_ptr, c->vt_list, c->elem_g, c->elem_H,
                    c->bsr_val, c->rhs, c->d_counts, c->diag_pos, c->sell_off, c->sell_col, c->row_len, c->bsr2sell,
                    c->up_spos, c->up_tspos, c->diag_spos, c->sell_val, c->prim_off};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    for (int t = 0; t < N_TYPES; ++t) c->rows[t].release();
    DBuf* bufs[] = {&c->rows_tmp, &c->sort_keys, &c->sort_keys_alt, &c->sort_vals, &c->sort_vals_alt, &c->flags, &c->scan,
                    &c->cub_tmp, &c->big_flags, &c->big_list, &c->ccd_work, &c->c_g, &c->c_H, &c->c_keys, &c->c_keys_alt, &c->c_vals, &c->c_vals_alt, &c->c_ukeys,
                    &c->c_ucount, &c->c_ustart, &c->c_val, &c->c_rowptr, &c->c_col, &c->pcg_vec, &c->pcg_part, &c->scal, &c->red, &c->mlp_dist};
    for (DBuf* b : bufs) b->release();
    Grid* gs[] = {&c->gp, &c->ge};
    for (Grid* g : gs) {
        DBuf* gb[] = {&g->keys, &g->ids, &g->keys_alt, &g->ids_alt, &g->ukeys, &g->ustart, &g->counts, &g->offsets, &g->ncells, &g->tmp,
                      &g->hkeys, &g->hvals, &g->cell4, &g->box4};
        for (DBuf* b : gb) b->release();
    }
    delete c;
}

}  // namespace

extern "C" {

int fipc_ctx_create(fipc_ctx** out, int n_verts, int n_tets, const int* tets, const double* x_rest, const double* lam,
                    const double* mu, double rho, int n_bp, const int* bp, int n_be, const int* be, int n_bt, const int* bt,
                    double dhat2, double dt) {
    if (!out || n_verts <= 0 || n_verts >= (1 << 21) || n_tets < 0 || (n_tets && (!tets || !lam || !mu)) || !x_rest || n_bp < 0 ||
        n_be < 0 || n_bt < 0 || dhat2 <= 0 || dt <= 0)
        return FIPC_ERR_ARGUMENT;
    for (long long i = 0; i < 4ll * n_tets; ++i)
        if (tets[i] < 0 || tets[i] >= n_verts) return FIPC_ERR_ARGUMENT;
    fipc_ctx* c = new fipc_ctx();
    *out = nullptr;
    c->nV = n_verts;
    c->nT = n_tets;
    c->nBP = n_bp;
    c->nBE = n_be;
    c->nBT = n_bt;
    c->dhat2 = dhat2;
    c->dhat = std::sqrt(dhat2);
    c->dt = dt;
    // rest shape, volume and lumped mass (NEWTON_IPC.py:485-494)
    std::vector<double> dminv(9ull * n_tets), vol(n_tets), mass(n_verts, 0.0);
    for (int e = 0; e < n_tets; ++e) {
        const int* t = tets + 4 * e;
        double Dm[9];
        for (int i = 0; i < 3; ++i)
            for (int m = 0; m < 3; ++m) Dm[i * 3 + m] = x_rest[3 * t[m + 1] + i] - x_rest[3 * t[0] + i];
        const double det = det3h(Dm);
        if (!(det > 0.0)) {
            free_ctx(c);
            return FIPC_ERR_ARGUMENT;   // inverted or degenerate rest element
        }
        vol[e] = det / 3.0 / 2.0;
        const double A[9] = {Dm[0], Dm[1], Dm[2], Dm[3], Dm[4], Dm[5], Dm[6], Dm[7], Dm[8]};
        const double c00 = A[4] * A[8] - A[5] * A[7], c01 = A[5] * A[6] - A[3] * A[8], c02 = A[3] * A[7] - A[4] * A[6];
        const double id = 1.0 / det;
        double* R = dminv.data() + 9ull * e;
        R[0] = c00 * id;
        R[1] = (A[2] * A[7] - A[1] * A[8]) * id;
        R[2] = (A[1] * A[5] - A[2] * A[4]) * id;
        R[3] = c01 * id;
        R[4] = (A[0] * A[8] - A[2] * A[6]) * id;
        R[5] = (A[2] * A[3] - A[0] * A[5]) * id;
        R[6] = c02 * id;
        R[7] = (A[1] * A[6] - A[0] * A[7]) * id;
        R[8] = (A[0] * A[4] - A[1] * A[3]) * id;
        const double mt = vol[e] * rho / 4.0;
        for (int k = 0; k < 4; ++k) mass[t[k]] += mt;
    }
    // adaptive kappa (NEWTON_IPC.py:116-124, x10 at :943) and hash cell (:127-134, :944)
    {
        double total = 0.0;
        for (int i = 0; i < n_verts; ++i) total += mass[i];
        const double Hb = barrier_H(1.0e-16, dhat2, 1.0);
        c->kappa = 1.0e13 * total / n_verts / (4.0e-16 * Hb) * 10.0;
        double len = 0.0;
        for (int i = 0; i < n_be; ++i) {
            const int a = be[2 * i], b = be[2 * i + 1];
            const double dx = x_rest[3 * a] - x_rest[3 * b], dy = x_rest[3 * a + 1] - x_rest[3 * b + 1],
                         dz = x_rest[3 * a + 2] - x_rest[3 * b + 2];
            len += std::sqrt(dx * dx + dy * dy + dz * dz);
        }
        c->inv_dx = n_be ? 1.0 / (len / (double)n_be) : 1.0;
        c->hash_inv_dx = median_edge_inv(x_rest, be, 0, n_be, c->inv_dx);
    }
    // static block pattern: all (tet[v], tet[w]) pairs plus every diagonal
    std::vector<unsigned long long> pairs;
    pairs.reserve(16ull * n_tets + n_verts);
    for (int e = 0; e < n_tets; ++e)
        for (int v = 0; v < 4; ++v)
            for (int w = 0; w < 4; ++w)
                pairs.push_back(((unsigned long long)tets[4 * e + v] << 32) | (unsigned)tets[4 * e + w]);
    for (int i = 0; i < n_verts; ++i) pairs.push_back(((unsigned long long)i << 32) | (unsigned)i);
    std::sort(pairs.begin(), pairs.end());
    pairs.erase(std::unique(pairs.begin(), pairs.end()), pairs.end());
    const long long nnzb = (long long)pairs.size();
    std::vector<int> row_ptr(n_verts + 1, 0), col_idx(nnzb);
    for (long long k = 0; k < nnzb; ++k) {
        row_ptr[(pairs[k] >> 32) + 1]++;
        col_idx[k] = (int)(pairs[k] & 0xffffffffu);
    }
    for (int i = 0; i < n_verts; ++i) row_ptr[i + 1] += row_ptr[i];
    auto pos_of = [&](int i, int j) -> int {
        const unsigned long long key = ((unsigned long long)i << 32) | (unsigned)j;
        return (int)(std::lower_bound(pairs.begin(), pairs.end(), key) - pairs.begin());
    };
    // upper blocks and their contribution lists
    std::vector<int> up_pos, up_tpos, up_row;
    std::vector<long long> up_index(nnzb, -1);
    for (int i = 0; i < n_verts; ++i)
        for (int k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
            const int j = col_idx[k];
            if (j < i) continue;
            up_index[k] = (long long)up_pos.size();
            up_pos.push_back(k);
            up_tpos.push_back(pos_of(j, i));
            up_row.push_back(i);
        }
    const int n_upper = (int)up_pos.size();
    std::vector<int> cnt(n_upper + 1, 0), cptr(n_upper + 1, 0), contrib(10ull * n_tets);
    std::vector<int> which(10ull * n_tets);
    {
        int blk_v[10], blk_w[10], b = 0;
        for (int v = 0; v < 4; ++v)
            for (int w = v; w < 4; ++w, ++b) {
                blk_v[b] = v;
                blk_w[b] = w;
            }
        for (int e = 0; e < n_tets; ++e)
            for (b = 0; b < 10; ++b) {
                int i = tets[4 * e + blk_v[b]], j = tets[4 * e + blk_w[b]];
                int tr = 0;
                if (i > j) {
                    std::swap(i, j);
                    tr = 1;
                }
                const int u = (int)up_index[pos_of(i, j)];
                which[10ull * e + b] = u;
                // the block's place in the element kernel's tiled layout (32 tets per tile)
                contrib[10ull * e + b] = ((((e >> 5) * 10 + b) * 32 + (e & 31)) << 1) | tr;
                cnt[u + 1]++;
            }
        for (int u = 0; u < n_upper; ++u) cptr[u + 1] = cptr[u] + cnt[u + 1];
        std::vector<int> fill(cptr.begin(), cptr.end() - 1), sorted(10ull * n_tets);
        for (long long k = 0; k < 10ll * n_tets; ++k) sorted[fill[which[k]]++] = contrib[k];   // tet order within a block
        contrib.swap(sorted);
    }
    // vertex -> (tet, local) incidence for the gradient gather
    std::vector<int> vt_ptr(n_verts + 1, 0), vt_list(4ull * n_tets);
    for (long long k = 0; k < 4ll * n_tets; ++k) vt_ptr[tets[k] + 1]++;
    for (int i = 0; i < n_verts; ++i) vt_ptr[i + 1] += vt_ptr[i];
    {
        std::vector<int> fill(vt_ptr.begin(), vt_ptr.end() - 1);
        for (int e = 0; e < n_tets; ++e)
            for (int v = 0; v < 4; ++v) vt_list[fill[tets[4 * e + v]]++] = e * 4 + v;
    }
    std::vector<int> diag_pos(n_verts);
    for (int i = 0; i < n_verts; ++i) diag_pos[i] = pos_of(i, i);
    // sliced-ELL layout of the same pattern
    const int n_slices = (n_verts + 31) / 32;
    std::vector<int> sell_off(n_slices + 1, 0), row_len(32ull * n_slices, 0);
    for (int i = 0; i < n_verts; ++i) row_len[i] = row_ptr[i + 1] - row_ptr[i];
    for (int sl = 0; sl < n_slices; ++sl) {
        int mx = 0;
        for (int l = 0; l < 32; ++l) mx = std::max(mx, row_len[32 * sl + l]);
        sell_off[sl + 1] = sell_off[sl] + mx;
    }
    const long long n_slots = sell_off[n_slices];
    std::vector<int> sell_col(32ull * n_slots, 0), bsr2sell(nnzb);
    for (int i = 0; i < n_verts; ++i) {
        const int sl = i >> 5, lane = i & 31;
        for (int k = 0; k < row_len[i]; ++k) {
            const long long slot = sell_off[sl] + k;
            sell_col[slot * 32 + lane] = col_idx[row_ptr[i] + k];
            bsr2sell[row_ptr[i] + k] = (int)(slot * 32 + lane);
        }
        for (int k = row_len[i]; k < sell_off[sl + 1] - sell_off[sl]; ++k) sell_col[(sell_off[sl] + k) * 32 + lane] = i;
    }
    if (32ll * n_slots >= (1ll << 31)) {
        free_ctx(c);
        return FIPC_ERR_CAPACITY;
    }
    std::vector<int> up_spos(n_upper), up_tspos(n_upper), diag_spos(n_verts);
    for (int u = 0; u < n_upper; ++u) {
        up_spos[u] = bsr2sell[up_pos[u]];
        up_tspos[u] = bsr2sell[up_tpos[u]];
    }
    for (int i = 0; i < n_verts; ++i) diag_spos[i] = bsr2sell[diag_pos[i]];

    int st = FIPC_OK;
    st |= upload(&c->tets, tets, 4ull * n_tets);
    st |= upload(&c->bp, bp, (size_t)n_bp);
    st |= upload(&c->be, be, 2ull * n_be);
    st |= upload(&c->bt, bt, 3ull * n_bt);
    st |= upload(&c->dminv, dminv.data(), dminv.size());
    st |= upload(&c->vol, vol.data(), vol.size());
    st |= upload(&c->lam, lam, (size_t)n_tets);
    st |= upload(&c->mu, mu, (size_t)n_tets);
    st |= upload(&c->mass, mass.data(), mass.size());
    st |= upload(&c->x0, x_rest, 3ull * n_verts);
    st |= upload(&c->row_ptr, row_ptr.data(), row_ptr.size());
    st |= upload(&c->col_idx, col_idx.data(), col_idx.size());
    st |= upload(&c->up_pos, up_pos.data(), up_pos.size());
    st |= upload(&c->up_tpos, up_tpos.data(), up_tpos.size());
    st |= upload(&c->up_row, up_row.data(), up_row.size());
    st |= upload(&c->up_cptr, cptr.data(), cptr.size());
    st |= upload(&c->up_contrib, contrib.data(), contrib.size());
    st |= upload(&c->vt_ptr, vt_ptr.data(), vt_ptr.size());
    st |= upload(&c->vt_list, vt_list.data(), vt_list.size());
    st |= upload(&c->diag_pos, diag_pos.data(), diag_pos.size());
    st |= upload(&c->sell_off, sell_off.data(), sell_off.size());
    st |= upload(&c->sell_col, sell_col.data(), sell_col.size());
    st |= upload(&c->row_len, row_len.data(), row_len.size());
    st |= upload(&c->bsr2sell, bsr2sell.data(), bsr2sell.size());
    st |= upload(&c->up_spos, up_spos.data(), up_spos.size());
    st |= upload(&c->up_tspos, up_tspos.data(), up_tspos.size());
    st |= upload(&c->diag_spos, diag_spos.data(), diag_spos.size());
    {
        const int off[6] = {0, n_bp, 0, n_be, 0, n_bt};   // one scene: whole boundary lists
        st |= upload(&c->prim_off, off, 6);
    }
    c->n_slices = n_slices;
    c->n_slots = n_slots;
    c->nnzb = (int)nnzb;
    c->n_upper = n_upper;
    if (st == FIPC_OK) {
        if (cudaMalloc((void**)&c->elem_g, sizeof(double) * 12ull * (n_tets > 0 ? n_tets : 1)) != cudaSuccess ||
            cudaMalloc((void**)&c->elem_H, sizeof(double) * 2880ull * ((n_tets + 31) / 32 + 1)) != cudaSuccess ||
            cudaMalloc((void**)&c->bsr_val, sizeof(double) * 9ull * nnzb) != cudaSuccess ||
            cudaMalloc((void**)&c->sell_val, sizeof(double) * 288ull * (n_slots > 0 ? n_slots : 1)) != cudaSuccess ||
            cudaMemset(c->sell_val, 0, sizeof(double) * 288ull * (n_slots > 0 ? n_slots : 1)) != cudaSuccess ||
            cudaMalloc((void**)&c->rhs, sizeof(double) * 3ull * n_verts) != cudaSuccess ||
            cudaMalloc((void**)&c->d_counts, sizeof(int) * (N_TYPES + 1)) != cudaSuccess)
            st = FIPC_ERR_CUDA;
    }
    if (st == FIPC_OK) st = ensure_row_capacity(c, 4096);
    if (st == FIPC_OK) st = cs_setup(c, default_agg_rows(n_verts), row_ptr.data(), col_idx.data());
    if (st == FIPC_OK) st = mg_setup(c, 0.0);
    if (st != FIPC_OK) {
        free_ctx(c);
        return FIPC_ERR_CUDA;
    }
    *out = c;
    return FIPC_OK;
}

int fipc_ctx_destroy(fipc_ctx* c) {
    if (!c) return FIPC_ERR_ARGUMENT;
    cudaDeviceSynchronize();
    free_ctx(c);
    return FIPC_OK;
}

int fipc_ctx_set_preconditioner(fipc_ctx* c, int agg_rows) {
    if (!c || agg_rows < 0 || agg_rows % 128) return FIPC_ERR_ARGUMENT;
    mg_free(c);   // an explicit choice of the one- or two-level preconditioner
    std::vector<int> rp(c->nV + 1), ci(c->nnzb);
    if (cudaMemcpy(rp.data(), c->row_ptr, 4ll * (c->nV + 1), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(ci.data(), c->col_idx, 4ll * c->nnzb, cudaMemcpyDeviceToHost) != cudaSuccess)
        return FIPC_ERR_CUDA;
    return cs_setup(c, agg_rows, rp.data(), ci.data());
}

int fipc_ctx_set_multigrid(fipc_ctx* c, int on, double h) {
    if (!c) return FIPC_ERR_ARGUMENT;
    if (!on) {
        mg_free(c);
        return FIPC_OK;
    }
    return mg_setup(c, h);
}

int fipc_ctx_preconditioner(fipc_ctx* c, int* agg_rows, int* n_coarse) {
    if (!c) return FIPC_ERR_ARGUMENT;
    if (agg_rows) *agg_rows = c->cs_agg_rows;
    if (n_coarse) *n_coarse = 6 * c->cs_n_agg;
    return FIPC_OK;
}

int fipc_ctx_params(fipc_ctx* c, double* kappa, double* inv_dx, int* nnzb) {
    if (!c) return FIPC_ERR_ARGUMENT;
    if (kappa) *kappa = c->kappa;
    if (inv_dx) *inv_dx = c->inv_dx;
    if (nnzb) *nnzb = c->nnzb;
    return FIPC_OK;
}

int fipc_ctx_set_params(fipc_ctx* c, double kappa, double inv_dx) {
    if (!c || !(kappa > 0) || !(inv_dx > 0)) return FIPC_ERR_ARGUMENT;
    c->kappa = kappa;
    c->inv_dx = inv_dx;
    return FIPC_OK;
}

int fipc_ctx_mass(fipc_ctx* c, double* mass_h) {
    if (!c || !mass_h) return FIPC_ERR_ARGUMENT;
    FIPC_CUDA(cudaMemcpy(mass_h, c->mass, sizeof(double) * c->nV, cudaMemcpyDeviceToHost));
    return FIPC_OK;
}

int fipc_ctx_set_x0(fipc_ctx* c, const double* x0, void* stream) {
    if (!c || !x0) return FIPC_ERR_ARGUMENT;
    FIPC_CUDA(cudaMemcpyAsync(c->x0, x0, sizeof(double) * 3ull * c->nV, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
    return FIPC_OK;
}

int fipc_find_constraints(fipc_ctx* c, const double* x, int* counts_h, void* stream) {
    if (!c || !x) return FIPC_ERR_ARGUMENT;
    const int st = find_constraints(c, x, (cudaStream_t)stream);
    if (st) return st;
    if (counts_h)
        for (int t = 0; t < N_TYPES; ++t) counts_h[t] = c->h_counts[t];
    return FIPC_OK;
}

int fipc_get_constraints(fipc_ctx* c, int type, int* rows, void* stream) {
    if (!c || type < 0 || type >= N_TYPES || !rows) return FIPC_ERR_ARGUMENT;
    if (c->h_counts[type] == 0) return FIPC_OK;
    FIPC_CUDA(cudaMemcpyAsync(rows, c->rows[type].p, 16ll * c->h_counts[type], cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
    return FIPC_OK;
}

int fipc_compute_hessian_and_gradient(fipc_ctx* c, const double* x, const double* xtilde, void* stream) {
    if (!c || !x || !xtilde) return FIPC_ERR_ARGUMENT;
    return assemble_system(c, x, xtilde, (cudaStream_t)stream);
}

int fipc_system_sizes(fipc_ctx* c, int* nnzb_elastic, int* nnzb_contact) {
    if (!c) return FIPC_ERR_ARGUMENT;
    if (nnzb_elastic) *nnzb_elastic = c->nnzb;
    if (nnzb_contact) *nnzb_contact = c->c_nnzb;
    return FIPC_OK;
}

int fipc_export_system(fipc_ctx* c, int* row_ptr, int* col_idx, double* val, int* c_row_ptr, int* c_col_idx, double* c_val,
                       double* rhs, void* stream) {
    if (!c) return FIPC_ERR_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    if (row_ptr) FIPC_CUDA(cudaMemcpyAsync(row_ptr, c->row_ptr, 4ll * (c->nV + 1), cudaMemcpyDeviceToDevice, s));
    if (col_idx) FIPC_CUDA(cudaMemcpyAsync(col_idx, c->col_idx, 4ll * c->nnzb, cudaMemcpyDeviceToDevice, s));
    if (val) {
        const int st = sell_to_bsr(c, val, s);
        if (st) return st;
    }
    if (c_row_ptr) {
        if (c->c_nnzb) FIPC_CUDA(cudaMemcpyAsync(c_row_ptr, c->c_rowptr.p, 4ll * (c->nV + 1), cudaMemcpyDeviceToDevice, s));
        else FIPC_CUDA(cudaMemsetAsync(c_row_ptr, 0, 4ll * (c->nV + 1), s));
    }
    if (c_col_idx && c->c_nnzb) FIPC_CUDA(cudaMemcpyAsync(c_col_idx, c->c_col.p, 4ll * c->c_nnzb, cudaMemcpyDeviceToDevice, s));
    if (c_val && c->c_nnzb) FIPC_CUDA(cudaMemcpyAsync(c_val, c->c_val.p, 72ll * c->c_nnzb, cudaMemcpyDeviceToDevice, s));
    if (rhs) FIPC_CUDA(cudaMemcpyAsync(rhs, c->rhs, 24ll * c->nV, cudaMemcpyDeviceToDevice, s));
    return FIPC_OK;
}

int fipc_solve_system(fipc_ctx* c, const unsigned char* fixed, double rtol, int maxit, int use_guess, double* sol, int* iters_h,
                      void* stream) {
    if (!c || !fixed || !sol || maxit <= 0 || !(rtol >= 0)) return FIPC_ERR_ARGUMENT;
    if (!use_guess) FIPC_CUDA(cudaMemsetAsync(sol, 0, sizeof(double) * 3ull * c->nV, (cudaStream_t)stream));
    return pcg_solve(c, fixed, c->diag_pos, rtol, maxit, sol, iters_h, (cudaStream_t)stream);
}

int fipc_output_residual(fipc_ctx* c, const double* sol, double* res_h, void* stream) {
    if (!c || !sol || !res_h) return FIPC_ERR_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    if (c->red.ensure(8ull * (RED_BLOCKS * (2 + N_TYPES) + 8))) return FIPC_ERR_CUDA;
    double* part = c->red.as<double>();
    double* outv = part + RED_BLOCKS * (2 + N_TYPES);
    const int st = launch_absmax(3 * c->nV, sol, part, outv, s);
    if (st) return st;
    FIPC_CUDA(cudaMemcpyAsync(res_h, outv, 8, cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaStreamSynchronize(s));
    return FIPC_OK;
}

int fipc_compute_energy(fipc_ctx* c, const double* x, const double* xtilde, double* e_h, void* stream) {
    if (!c || !x || !xtilde || !e_h) return FIPC_ERR_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    if (c->red.ensure(8ull * (RED_BLOCKS * (2 + N_TYPES) + 8))) return FIPC_ERR_CUDA;
    double* part = c->red.as<double>();
    double* outv = part + RED_BLOCKS * (2 + N_TYPES);
    const int* rows[N_TYPES];
    for (int t = 0; t < N_TYPES; ++t) rows[t] = c->rows[t].as<int>();
    const int st = launch_energy(c, x, xtilde, rows, c->h_counts, part, outv, s);
    if (st) return st;
    FIPC_CUDA(cudaMemcpyAsync(e_h, outv, 8, cudaMemcpyDeviceToHost, s));
    FIPC_CUDA(cudaStreamSynchronize(s));
    return FIPC_OK;
}

int fipc_compute_intersection_free_step_size(fipc_ctx* c, const double* x, const double* p, double eta, int inversion,
                                             double* alpha_h, void* stream) {
    if (!c || !x || !p || !alpha_h || !(eta >= 0 && eta < 1)) return FIPC_ERR_ARGUMENT;
    return ccd_step(c, x, p, eta, inversion != 0, alpha_h, (cudaStream_t)stream);
}

int fipc_check_collision(fipc_ctx* c, const double* x, int* hit_h, void* stream) {
    if (!c || !x || !hit_h) return FIPC_ERR_ARGUMENT;
    return check_collision(c, x, hit_h, (cudaStream_t)stream);
}

}  // extern "C"
