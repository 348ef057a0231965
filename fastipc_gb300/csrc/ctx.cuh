// Scene context shared by the translation units of libfastipc.so: the device-resident state
// that projects/FastIPC/NEWTON_IPC.py keeps in module-global Taichi fields (mesh, rest shape,
// mass, constraint lists, the assembled system, scratch), plus device-buffer bookkeeping.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <atomic>
#include <vector>

#include "common.cuh"

namespace fipc {

// number of kernels this library launched (reported by fipc_launch_count)
extern std::atomic<long long> g_launches;

#define FIPC_CUDA(call)                                  \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return FIPC_ERR_CUDA;     \
    } while (0)

#define FIPC_LAUNCHED() (g_launches.fetch_add(1, std::memory_order_relaxed))

// Grow-only device buffer.  Contents are not preserved across growth.
struct DBuf {
    void* p = nullptr;
    size_t bytes = 0;
    int ensure(size_t need) {
        if (need <= bytes) return FIPC_OK;
        if (p) cudaFree(p);
        p = nullptr;
        size_t nb = need + need / 4 + 256;
        if (cudaMalloc(&p, nb) != cudaSuccess) {
            bytes = 0;
            return FIPC_ERR_CUDA;
        }
        bytes = nb;
        return FIPC_OK;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T>
    T* as() const { return (T*)p; }
};

// sorted spatial-hash grid over primitives: (cell key, primitive id) pairs sorted by key,
// unique keys and the start of each key's run
struct Grid {
    DBuf keys, ids, keys_alt, ids_alt, ukeys, ustart, counts, offsets, ncells, tmp, hkeys, hvals;
    DBuf cell4, box4;   // per stored primitive: first cell of its pair de-duplication, FP32 box
    int n_entries = 0, n_unique = 0;
    unsigned long long hmask = 0;   // cell table size - 1 (a power of two >= 2 x entries)
};

struct fipc_ctx_impl {
    int nV = 0, nT = 0, nBP = 0, nBE = 0, nBT = 0;
    // mesh (device)
    int *tets = nullptr, *bp = nullptr, *be = nullptr, *bt = nullptr;
    double *dminv = nullptr, *vol = nullptr, *lam = nullptr, *mu = nullptr, *mass = nullptr, *x0 = nullptr;
    double dhat2 = 0, dhat = 0, kappa = 0, inv_dx = 0, dt = 0;
    // cell size of the spatial hash: the median boundary edge.  The reference's cell is the mean
    // (inv_dx above, kept for callers); the lists found do not depend on it, but a few long
    // edges (a ground plane) inflate the mean until one cell holds a whole body.
    double hash_inv_dx = 0;
    // static elastic + inertia BSR pattern (full, both triangles)
    int nnzb = 0, n_upper = 0;
    int *row_ptr = nullptr, *col_idx = nullptr;
    int *up_pos = nullptr, *up_tpos = nullptr, *up_row = nullptr, *up_cptr = nullptr, *up_contrib = nullptr;
    int *vt_ptr = nullptr, *vt_list = nullptr;   // vertex -> (tet*4 + local) for the gradient gather
    int* diag_pos = nullptr;                     // BSR position of each vertex's diagonal block
    // the same matrix in sliced-ELL form (32 rows per slice, blocks of a slice stored
    // column-major so that each of the 9 block entries loads as one coalesced 256-byte row):
    // slot (slice s, k) = sell_off[s] + k; its column ids at sell_col[slot*32 + lane] and its
    // values at sell_val[slot*288 + entry*32 + lane]; padding slots have row_len <= k
    int n_slices = 0;
    long long n_slots = 0;
    int *sell_off = nullptr, *sell_col = nullptr, *row_len = nullptr, *bsr2sell = nullptr;
    int *up_spos = nullptr, *up_tspos = nullptr, *diag_spos = nullptr;
    double* sell_val = nullptr;
    // per-iteration element data and the system
    double *elem_g = nullptr, *elem_H = nullptr, *bsr_val = nullptr, *rhs = nullptr;
    // constraint lists (capacity rows of 4 ints each) and counts
    DBuf rows[N_TYPES], rows_tmp, sort_keys, sort_keys_alt, sort_vals, sort_vals_alt, flags, scan, cub_tmp;
    int *d_counts = nullptr;     // [N_TYPES + 1] device (last: overflow flag)
    int h_counts[N_TYPES] = {0};
    int cap = 0;
    // contact system
    DBuf c_g, c_H, c_keys, c_keys_alt, c_vals, c_vals_alt, c_ukeys, c_ucount, c_ustart, c_val, c_rowptr, c_col;
    int c_rows = 0, c_nnzb = 0;
    // PCG
    DBuf pcg_vec, pcg_part;
    // two-level preconditioner: block-Jacobi plus a coarse space of the six rigid-body modes of
    // each aggregate of cs_agg_rows consecutive vertices (0: block-Jacobi only)
    int cs_agg_rows = 0, cs_n_agg = 0, cs_n_pairs = 0;
    int* cs_pairs = nullptr;              // [cs_n_pairs][2] aggregate pairs coupled by the pattern
    DBuf cs_d, cs_Ac, cs_tick, cs_buf, cs_part, cs_gbuf;
    // grids
    Grid gp, ge;
    // small device scalars: [0] alpha bits, [1] hit flag, reductions ...
    DBuf scal, red;
    // learned warm start: per-vertex nearest-constraint distance
    DBuf mlp_dist;
    // batched scenes (n_scenes > 1): scene s owns vertices [voff[s], voff[s+1]) and tets
    // [toff[s], toff[s+1]); its own kappa and hash cell; null tables for a single scene
    int n_scenes = 1;
    int *v_scene = nullptr, *voff_d = nullptr, *toff_d = nullptr;
    double *s_kappa = nullptr, *s_inv_dx = nullptr, *s_hash_inv_dx = nullptr;
    std::vector<int> h_voff, h_toff;
    // boundary lists of scene s: points [prim_off[0][s], prim_off[0][s+1]), edges [1], triangles
    // [2] (device, 3 x (n_scenes + 1)); big-primitive flags and lists of the spatial hash
    int* prim_off = nullptr;
    DBuf big_flags, big_list;
    DBuf ccd_work;                        // step filter: pairs left to the exact test, and their counts
    std::vector<double> h_kappa, h_inv_dx;
    // batched PCG: tiles of consecutive rows inside one scene
    int n_tiles = 0, tile_rows = 0, pcg_grid = 0;
    DBuf tile_scene, tile_row0, scene_tile0, bpcg_vec, bpcg_sc, bpcg_part, bpcg_flag, s_red, s_rowoff;
    void* graph_exec = nullptr;           // captured PCG chunk (cudaGraphExec_t)
    void* cap_stream = nullptr;           // private stream used only for capturing it
    std::vector<unsigned char> graph_sig; // the kernel arguments it was captured with
    float tune_ms = 0.f;                  // time of one SpMV launch in the chosen shape
    // single-scene PCG: a captured chunk of iterations and the kernel arguments it holds
    void* pcg3_exec = nullptr;
    std::vector<unsigned char> pcg3_sig;
    // multigrid preconditioner of the PCG (mg_levels >= 2: in use, replacing the coarse space
    // above); an MgState owned by the context
    void* mg = nullptr;
    int mg_levels = 0;
    int mg_fp32 = 1;                      // FP32 level-0 smoothing products in the V-cycle (the default)
    // the last direct solve: fronts, their storage (doubles), factorisation flops, host analysis time
    int mf_fronts = 0;
    long long mf_front_doubles = 0;
    double mf_flops = 0.0, mf_analyse_ms = 0.0;
};

// scene lookup for the spatial hash: one scene (null table) or per-vertex scene ids with
// per-scene cell sizes; keys of different scenes never coincide
struct SceneGeo {
    const int* vscene = nullptr;
    const double* inv_dx_s = nullptr;
    double inv_dx = 1.0;
    // primitives whose query box covers more than BIG_CELLS cells: tested against every
    // primitive of their scene instead of through the grid (null: none)
    const unsigned char* big_tri = nullptr;
    const unsigned char* big_edge = nullptr;
#if defined(__CUDACC__)
    __device__ __forceinline__ int scene(int v) const { return vscene ? __ldg(vscene + v) : 0; }
    __device__ __forceinline__ double idx(int s) const { return vscene ? __ldg(inv_dx_s + s) : inv_dx; }
#endif
};

// ---------------------------------------------------------------- shared device helpers
#if defined(__CUDACC__)
__device__ __forceinline__ v3 ld3(const double* __restrict__ x, int i) {
    return v3{__ldg(x + 3 * i), __ldg(x + 3 * i + 1), __ldg(x + 3 * i + 2)};
}
#endif

// row ranges of the concatenated lists: rows [row0[t], row0[t+1]) are of type t and their
// nv(t)^2 blocks start at ent0[t] + (r - row0[t]) nv(t)^2
struct TypeTable {
    int row0[N_TYPES + 1];
    long long ent0[N_TYPES + 1];
};

constexpr int RED_BLOCKS = 304;     // 2 x 152 SMs: fixed reduction grid (deterministic sums)
constexpr int RED_THREADS = 256;

// cell key of integer cell coordinates (21 bits per axis, offset 2^20)
FIPC_HD unsigned long long cell_key(long long i, long long j, long long k) {
    const long long off = 1ll << 20;
    auto c = [](long long v) { return v < 0 ? 0ll : (v > (1ll << 21) - 1 ? (1ll << 21) - 1 : v); };
    return ((unsigned long long)c(i + off) << 42) | ((unsigned long long)c(j + off) << 21) | (unsigned long long)c(k + off);
}
// batched scenes: 10 bits of scene id above 18 bits per axis (offset 2^17; the top coordinate
// value is never used, so no key is all ones)
FIPC_HD unsigned long long cell_key_scene(int s, long long i, long long j, long long k) {
    const long long off = 1ll << 17;
    auto c = [](long long v) { return v < 0 ? 0ll : (v > (1ll << 18) - 2 ? (1ll << 18) - 2 : v); };
    return ((unsigned long long)s << 54) | ((unsigned long long)c(i + off) << 36) | ((unsigned long long)c(j + off) << 18) |
           (unsigned long long)c(k + off);
}

}  // namespace fipc

using fipc_ctx = fipc::fipc_ctx_impl;
