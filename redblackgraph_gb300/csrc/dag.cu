// dag.cu -- closure of a DAG by levels, on sm_103a.
//
// Reference: transitive_closure_dag_sparse_cython, redblackgraph/sparse/csgraph/
// _transitive_closure_dag.pyx:168-351 (and the level-parallel transitive_closure_dag_gpu,
// redblackgraph/gpu/transitive_closure.py:474-652).  Row v of the closure is v's stored entries
// (+) A[v][w] (x) C[w][.] over v's parents w != v, with the Cython int32 product and sum; the
// diameter source is the largest magnitude of any stored entry or candidate.
//
// Design: the vertices are put in topological levels on the device (Kahn's algorithm, one launch
// per level: a vertex joins the next level when its last parent is placed).  A level's rows only
// read rows of earlier levels, so each level is one batch of independent rows: a count pass (one
// warp per row folds its candidates into a shared-memory table keyed by column and counts the
// distinct columns), a scan that places the rows in a caller-provided row pool, and a fill pass
// that folds again and writes each row sorted.  Rows with more distinct columns than the warp
// table holds are done by a 512-thread block with a larger table; a row wider than that makes the
// call return RBG_ERR_CAPACITY with *nnz = -1.  A pool too small for the closure returns
// RBG_ERR_CAPACITY with *nnz set to a larger size to retry with.  A cycle (vertices never placed)
// returns RBG_ERR_CYCLE.
#include <cuda_runtime.h>
#include <cub/cub.cuh>
#include <algorithm>
#include <vector>
#include "rbg_internal.cuh"

namespace rbg {

constexpr int DG_WSLOTS = 256;          // warp table slots (distinct columns of a row)
constexpr int DG_WARPS = 8;             // warps per CTA
constexpr int DG_BSLOTS = 8192;         // block table slots
constexpr int DG_BTHREADS = 512;
constexpr unsigned DG_NOKEY = 0xffffffffu;
constexpr int DG_NOVAL = 0x7fffffff;    // (+) identity of the table (no non-zero candidate yet)

template <int SLOTS> struct DagTable {
    unsigned key[SLOTS];
    int val[SLOTS];                     // signed minimum of the non-zero candidates
    unsigned char has[SLOTS];           // 1: some non-zero candidate landed here
    unsigned long long list[SLOTS];     // (column << 32 | slot) of the occupied slots
};

template <int SLOTS>
__device__ __forceinline__ int dag_slot(DagTable<SLOTS> &H, unsigned j, int mask) {
    int h = (int)((j * 2654435761u) >> 8) & mask;
    for (int probe = 0; probe <= mask; ++probe) {
        const unsigned k = H.key[h];
        if (k == j) return h;
        if (k == DG_NOKEY) {
            const unsigned old = atomicCAS(&H.key[h], DG_NOKEY, j);
            if (old == DG_NOKEY || old == j) return h;
        }
        h = (h + 1) & mask;
    }
    return -1;
}

__device__ __forceinline__ int dag_abs(int v) { return v > 0 ? v : (int)(0u - (unsigned)v); }

// Fold candidate (column j, value p) into the table; returns false when the table is full.
template <int SLOTS>
__device__ __forceinline__ bool dag_fold(DagTable<SLOTS> &H, unsigned j, int p, int mask) {
    const int s = dag_slot(H, j, mask);
    if (s < 0) return false;
    if (p != 0) {
        if (p < H.val[s]) atomicMin(&H.val[s], p);
        H.has[s] = 1;
    }
    return true;
}

struct DagArgs {
    int64_t n;
    const int64_t *ap; const int *aj; const int *av;     // A (int32 values)
    const int *order;                                   // vertices by level
    int64_t *row_off; int *row_len;                     // pool position / length of each row
    const int *pcols; const int *pvals;                 // the pool (rows of earlier levels)
    int *wcols; int *wvals;                             // the pool, written by the fill pass
    int64_t capacity;
    int *lvl_len;                                       // count pass output (level order)
    const int64_t *lvl_off;                             // fill pass input (level order)
    int *wide; int *nwide;                              // rows for the block tier (level order)
    unsigned long long *max_abs;
    int *flags;                                         // [0] row wider than the block table
};

// The candidates of row v, folded by `nthreads` threads of the calling group (lane = rank in it).
template <int SLOTS>
__device__ __forceinline__ bool dag_gather(const DagArgs &a, int v, DagTable<SLOTS> &H, int mask, int lane,
                                           int nthreads, int &best) {
    bool ok = true;
    for (int64_t e = a.ap[v] + lane; e < a.ap[v + 1]; e += nthreads) {   // the stored entries
        const int w = a.aj[e], val = a.av[e];
        best = max(best, dag_abs(val));
        ok &= dag_fold(H, (unsigned)w, val, mask);
    }
    for (int64_t e = a.ap[v]; e < a.ap[v + 1]; ++e) {                   // each parent's closed row
        const int w = a.aj[e];
        if (w == v || w < 0 || w >= a.n) continue;
        const int vw = a.av[e];
        const int64_t o = a.row_off[w];
        const int len = a.row_len[w];
        for (int f = lane; f < len; f += nthreads) {
            const int p = cy_product(vw, a.pvals[o + f]);
            if (p == 0) continue;
            best = max(best, dag_abs(p));
            ok &= dag_fold(H, (unsigned)a.pcols[o + f], p, mask);
        }
    }
    return ok;
}

template <int SLOTS>
__device__ __forceinline__ void dag_clear(DagTable<SLOTS> &H, int S, int lane, int nthreads) {
    for (int s = lane; s < S; s += nthreads) {
        H.key[s] = DG_NOKEY;
        H.val[s] = DG_NOVAL;
        H.has[s] = 0;
    }
}

// Count pass, one warp per row of the level (k = position in the level).
__global__ void __launch_bounds__(DG_WARPS * 32) dag_count_kernel(DagArgs a, int64_t ls, int nl) {
    extern __shared__ __align__(16) unsigned char dg_smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    DagTable<DG_WSLOTS> &H = reinterpret_cast<DagTable<DG_WSLOTS> *>(dg_smem)[w];
    int best = 0;
    for (int k = blockIdx.x * DG_WARPS + w; k < nl; k += gridDim.x * DG_WARPS) {
        const int v = a.order[ls + k];
        dag_clear(H, DG_WSLOTS, lane, 32);
        __syncwarp();
        const bool ok = dag_gather(a, v, H, DG_WSLOTS - 1, lane, 32, best);
        __syncwarp();
        if (!__all_sync(0xffffffffu, ok)) {
            if (lane == 0) a.wide[atomicAdd(a.nwide, 1)] = k;
            continue;
        }
        int nd = 0;
        for (int s0 = 0; s0 < DG_WSLOTS; s0 += 32)
            nd += __popc(__ballot_sync(0xffffffffu, H.key[s0 + lane] != DG_NOKEY));
        if (lane == 0) a.lvl_len[k] = nd;
        __syncwarp();
    }
    best = __reduce_max_sync(0xffffffffu, best);
    if (lane == 0 && best > 0) atomicMax(a.max_abs, (unsigned long long)best);
}

// Count pass for the wide rows, one block per row.
__global__ void __launch_bounds__(DG_BTHREADS) dag_count_block_kernel(DagArgs a, int64_t ls) {
    extern __shared__ __align__(16) unsigned char dg_smem[];
    DagTable<DG_BSLOTS> &H = *reinterpret_cast<DagTable<DG_BSLOTS> *>(dg_smem);
    __shared__ int s_cnt, s_ok;
    const int nw = *a.nwide;
    int best = 0;
    for (int b = blockIdx.x; b < nw; b += gridDim.x) {
        const int k = a.wide[b];
        const int v = a.order[ls + k];
        dag_clear(H, DG_BSLOTS, threadIdx.x, DG_BTHREADS);
        if (threadIdx.x == 0) { s_cnt = 0; s_ok = 1; }
        __syncthreads();
        const bool ok = dag_gather(a, v, H, DG_BSLOTS - 1, threadIdx.x, DG_BTHREADS, best);
        if (!ok) s_ok = 0;
        __syncthreads();
        int c = 0;
        for (int s = threadIdx.x; s < DG_BSLOTS; s += DG_BTHREADS) c += H.key[s] != DG_NOKEY;
        c = __reduce_add_sync(0xffffffffu, c);
        if ((threadIdx.x & 31) == 0) atomicAdd(&s_cnt, c);
        __syncthreads();
        if (threadIdx.x == 0) {
            if (!s_ok) atomicOr(a.flags, 1);
            a.lvl_len[k] = s_ok ? s_cnt : 0;
        }
        __syncthreads();
    }
    best = __reduce_max_sync(0xffffffffu, best);
    if ((threadIdx.x & 31) == 0 && best > 0) atomicMax(a.max_abs, (unsigned long long)best);
}

// Place the level's rows in the pool (base = rows placed so far, kept on the device).
__global__ void dag_place_kernel(DagArgs a, int64_t ls, int nl, int64_t *base) {
    const int64_t b = *base;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nl; k += gridDim.x * blockDim.x) {
        const int v = a.order[ls + k];
        a.row_off[v] = b + a.lvl_off[k];
        a.row_len[v] = a.lvl_len[k];
    }
}

__global__ void dag_advance_kernel(const int64_t *lvl_off, const int *lvl_len, int nl, int64_t *base) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && nl > 0) *base += lvl_off[nl - 1] + lvl_len[nl - 1];
}

// Write the occupied slots of a table as a sorted row at `dst` (warp: register sort for up to 64
// columns, shared-memory bitonic otherwise).
template <int SLOTS>
__device__ __forceinline__ int dag_collect(DagTable<SLOTS> &H, int S, int lane, int nthreads) {
    // compaction of the occupied slots into list (warp-synchronous when nthreads == 32)
    __shared__ int s_nd;
    int nd = 0;
    if (nthreads == 32) {
        for (int s0 = 0; s0 < S; s0 += 32) {
            const int s = s0 + lane;
            const bool occ = H.key[s] != DG_NOKEY;
            const unsigned bal = __ballot_sync(0xffffffffu, occ);
            if (occ) H.list[nd + __popc(bal & ((1u << lane) - 1u))] = ((unsigned long long)H.key[s] << 32) | (unsigned)s;
            nd += __popc(bal);
        }
        __syncwarp();
        return nd;
    }
    if (lane == 0) s_nd = 0;
    __syncthreads();
    for (int s = lane; s < S; s += nthreads)
        if (H.key[s] != DG_NOKEY) H.list[atomicAdd(&s_nd, 1)] = ((unsigned long long)H.key[s] << 32) | (unsigned)s;
    __syncthreads();
    return s_nd;
}

template <int SLOTS, typename Sync>
__device__ __forceinline__ void dag_sort(DagTable<SLOTS> &H, int nd, int lane, int nthreads, Sync sync) {
    int P = 1;
    while (P < nd) P <<= 1;
    for (int q = nd + lane; q < P; q += nthreads) H.list[q] = ~0ull;
    sync();
    for (int k = 2; k <= P; k <<= 1) {
        for (int jj = k >> 1; jj > 0; jj >>= 1) {
            for (int q = lane; q < P; q += nthreads) {
                const int qx = q ^ jj;
                if (qx > q) {
                    const unsigned long long x = H.list[q], y = H.list[qx];
                    if ((x > y) == ((q & k) == 0)) { H.list[q] = y; H.list[qx] = x; }
                }
            }
            sync();
        }
    }
}

struct DgWarpSync { __device__ void operator()() const { __syncwarp(); } };
struct DgBlockSync { __device__ void operator()() const { __syncthreads(); } };

// Fill pass, one warp per (not wide) row.
__global__ void __launch_bounds__(DG_WARPS * 32) dag_fill_kernel(DagArgs a, int64_t ls, int nl) {
    extern __shared__ __align__(16) unsigned char dg_smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    DagTable<DG_WSLOTS> &H = reinterpret_cast<DagTable<DG_WSLOTS> *>(dg_smem)[w];
    int best = 0;
    for (int k = blockIdx.x * DG_WARPS + w; k < nl; k += gridDim.x * DG_WARPS) {
        const int v = a.order[ls + k];
        const int64_t o = a.row_off[v];
        const int len = a.row_len[v];
        if (len > DG_WSLOTS || o + len > a.capacity) continue;   // wide rows: block pass
        dag_clear(H, DG_WSLOTS, lane, 32);
        __syncwarp();
        const bool ok = dag_gather(a, v, H, DG_WSLOTS - 1, lane, 32, best);
        if (!__all_sync(0xffffffffu, ok)) continue;              // counted wide: block pass
        const int nd = dag_collect(H, DG_WSLOTS, lane, 32);
        dag_sort(H, nd, lane, 32, DgWarpSync());
        for (int q = lane; q < nd; q += 32) {
            const unsigned long long e = H.list[q];
            const int s = (int)(e & 0xffffffffu);
            a.wcols[o + q] = (int)(e >> 32);
            a.wvals[o + q] = H.has[s] ? H.val[s] : 0;
        }
        __syncwarp();
    }
}

// Fill pass for the wide rows, one block per row.
__global__ void __launch_bounds__(DG_BTHREADS) dag_fill_block_kernel(DagArgs a, int64_t ls) {
    extern __shared__ __align__(16) unsigned char dg_smem[];
    DagTable<DG_BSLOTS> &H = *reinterpret_cast<DagTable<DG_BSLOTS> *>(dg_smem);
    const int nw = *a.nwide;
    int best = 0;
    for (int b = blockIdx.x; b < nw; b += gridDim.x) {
        const int k = a.wide[b];
        const int v = a.order[ls + k];
        const int64_t o = a.row_off[v];
        const int len = a.row_len[v];
        if (o + len > a.capacity) continue;                      // uniform across the block
        dag_clear(H, DG_BSLOTS, threadIdx.x, DG_BTHREADS);
        __syncthreads();
        dag_gather(a, v, H, DG_BSLOTS - 1, threadIdx.x, DG_BTHREADS, best);
        __syncthreads();
        const int nd = dag_collect(H, DG_BSLOTS, threadIdx.x, DG_BTHREADS);
        dag_sort(H, nd, threadIdx.x, DG_BTHREADS, DgBlockSync());
        for (int q = threadIdx.x; q < nd; q += DG_BTHREADS) {
            const unsigned long long e = H.list[q];
            const int s = (int)(e & 0xffffffffu);
            a.wcols[o + q] = (int)(e >> 32);
            a.wvals[o + q] = H.has[s] ? H.val[s] : 0;
        }
        __syncthreads();
    }
}

// ----------------------------------------------------------------------------- levels (Kahn)
__global__ void dag_indeg_kernel(int64_t n, const int64_t *ap, const int *aj, int *remaining, int *ccount) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        int c = 0;
        for (int64_t e = ap[v]; e < ap[v + 1]; ++e) {
            const int w = aj[e];
            if (w != (int)v && w >= 0 && w < n) {
                ++c;
                atomicAdd(&ccount[w], 1);
            }
        }
        remaining[v] = c;
    }
}

__global__ void dag_children_kernel(int64_t n, const int64_t *ap, const int *aj, const int64_t *coff, int *cursor,
                                    int *children) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        for (int64_t e = ap[v]; e < ap[v + 1]; ++e) {
            const int w = aj[e];
            if (w != (int)v && w >= 0 && w < n) children[coff[w] + atomicAdd(&cursor[w], 1)] = (int)v;
        }
    }
}

__global__ void dag_roots_kernel(int64_t n, const int *remaining, int *order, int *tail) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        if (remaining[v] == 0) order[atomicAdd(tail, 1)] = (int)v;
}

// place the children whose last parent is in [ls, le)
__global__ void dag_level_kernel(const int *order, int64_t ls, int64_t le, const int64_t *coff,
                                 const int *children, int *remaining, int *order_out, int *tail) {
    for (int64_t k = ls + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < le;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int w = order[k];
        for (int64_t e = coff[w]; e < coff[w + 1]; ++e) {
            const int c = children[e];
            if (atomicSub(&remaining[c], 1) == 1) order_out[atomicAdd(tail, 1)] = c;
        }
    }
}

__global__ void dag_gather_rows_kernel(int64_t n, const int64_t *row_off, const int *pcols, const int *pvals,
                                       const int64_t *indptr, int *cj, int *cx) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t v = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); v < n; v += warps) {
        const int64_t src = row_off[v], dst = indptr[v], len = indptr[v + 1] - dst;
        for (int64_t e = lane; e < len; e += 32) {
            cj[dst + e] = pcols[src + e];
            cx[dst + e] = pvals[src + e];
        }
    }
}

__global__ void dag_len64_kernel(int64_t n, const int *row_len, int64_t *len64) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v <= n; v += (int64_t)gridDim.x * blockDim.x)
        len64[v] = v < n ? row_len[v] : 0;
}

}  // namespace rbg

using namespace rbg;

namespace {

struct DagWs {
    int *remaining, *ccount, *cursor, *children, *order, *tail, *lvl_len, *wide, *nwide, *flags;
    int64_t *coff, *lvl_off, *base;
    unsigned long long *max_abs;
    void *tmp;
    size_t tmp_bytes;
};

size_t dag_tmp_bytes(int64_t n) {
    size_t a = 0, b = 0, c = 0;
    const int m = (int)std::max<int64_t>(n + 1, 1);
    cub::DeviceScan::ExclusiveSum(nullptr, a, (int *)nullptr, (int64_t *)nullptr, m);
    cub::DeviceScan::ExclusiveSum(nullptr, b, (int64_t *)nullptr, (int64_t *)nullptr, m);
    cub::DeviceScan::ExclusiveSum(nullptr, c, (int *)nullptr, (int64_t *)nullptr, m);
    return std::max(a, std::max(b, c));
}

size_t dag_layout(int64_t n, int64_t nnz, unsigned char *base, DagWs *w) {
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o = align_up(o + bytes, 256); return base ? base + at : nullptr; };
    const size_t ni = (size_t)(n + 1) * 4, nl = (size_t)(n + 1) * 8;
    unsigned char *p;
    p = take(ni); if (w) w->remaining = (int *)p;
    p = take(ni); if (w) w->ccount = (int *)p;
    p = take(ni); if (w) w->cursor = (int *)p;
    p = take((size_t)std::max<int64_t>(nnz, 1) * 4); if (w) w->children = (int *)p;
    p = take(ni); if (w) w->order = (int *)p;
    p = take(ni); if (w) w->lvl_len = (int *)p;
    p = take(ni); if (w) w->wide = (int *)p;
    p = take(64); if (w) { w->tail = (int *)p; w->nwide = (int *)p + 1; w->flags = (int *)p + 2; }
    p = take(nl); if (w) w->coff = (int64_t *)p;
    p = take(nl); if (w) w->lvl_off = (int64_t *)p;
    p = take(64); if (w) { w->base = (int64_t *)p; w->max_abs = (unsigned long long *)((int64_t *)p + 1); }
    const size_t tb = dag_tmp_bytes(n);
    p = take(tb); if (w) { w->tmp = p; w->tmp_bytes = tb; }
    return o;
}

}  // namespace

extern "C" int32_t rbg_dag_workspace_bytes(int64_t n, int64_t nnz, int64_t *bytes) {
    if (!bytes || n < 0 || nnz < 0 || n >= (1ll << 31) - 1) return RBG_ERR_INVALID;
    *bytes = (int64_t)dag_layout(n, nnz, nullptr, nullptr);
    return RBG_OK;
}

extern "C" int32_t rbg_dag_closure(const rbg_csr_t *A, void *workspace, int64_t workspace_bytes, int32_t *pool_cols,
                                   int32_t *pool_vals, int64_t pool_capacity, int64_t *row_off, int32_t *row_len,
                                   int64_t *nnz, int64_t *max_abs, int64_t *levels, rbg_stream_t stream) {
    if (!A || !A->indptr || A->n_rows != A->n_cols || A->n_rows < 0 || !workspace || !row_off || !row_len ||
        !nnz || !max_abs || !levels || pool_capacity < 0 || (pool_capacity > 0 && (!pool_cols || !pool_vals)))
        return RBG_ERR_INVALID;
    const int64_t n = A->n_rows;
    *nnz = 0; *max_abs = 0; *levels = 0;
    if (n == 0) return RBG_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int64_t annz = 0;
    RBG_CUDA_TRY(cudaMemcpyAsync(&annz, A->indptr + n, 8, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    if (workspace_bytes < (int64_t)dag_layout(n, annz, nullptr, nullptr)) return RBG_ERR_NOMEM;
    DagWs w;
    dag_layout(n, annz, reinterpret_cast<unsigned char *>(workspace), &w);
    const int *aj = reinterpret_cast<const int *>(A->indices);
    const int *av = reinterpret_cast<const int *>(A->data);
    const int g = grid_for(n, 256);
    // ---- levels
    RBG_CUDA_TRY(cudaMemsetAsync(w.ccount, 0, (size_t)(n + 1) * 4, s));
    RBG_CUDA_TRY(cudaMemsetAsync(w.cursor, 0, (size_t)(n + 1) * 4, s));
    RBG_CUDA_TRY(cudaMemsetAsync(w.tail, 0, 64, s));
    RBG_CUDA_TRY(cudaMemsetAsync(w.base, 0, 64, s));
    note_launches(2);
    dag_indeg_kernel<<<g, 256, 0, s>>>(n, A->indptr, aj, w.remaining, w.ccount);
    size_t tb = w.tmp_bytes;
    RBG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(w.tmp, tb, w.ccount, w.coff, (int)(n + 1), s));
    dag_children_kernel<<<g, 256, 0, s>>>(n, A->indptr, aj, w.coff, w.cursor, w.children);
    note_launches(1);
    dag_roots_kernel<<<g, 256, 0, s>>>(n, w.remaining, w.order, w.tail);
    std::vector<int64_t> bounds{0};
    int tail = 0;
    RBG_CUDA_TRY(cudaMemcpyAsync(&tail, w.tail, 4, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    while (tail > bounds.back()) {
        const int64_t ls = bounds.back(), le = tail;
        bounds.push_back(le);
        note_launches(1);
        dag_level_kernel<<<grid_for(le - ls, 256), 256, 0, s>>>(w.order, ls, le, w.coff, w.children, w.remaining,
                                                                w.order, w.tail);
        RBG_CUDA_TRY(cudaMemcpyAsync(&tail, w.tail, 4, cudaMemcpyDeviceToHost, s));
        RBG_CUDA_TRY(cudaStreamSynchronize(s));
    }
    *levels = (int64_t)bounds.size() - 1;
    if (tail < n) return RBG_ERR_CYCLE;          // vertices on (or below) a cycle were never placed
    // ---- rows, level by level
    static const int configured = [] {
        RBG_CUDA_TRY(cudaFuncSetAttribute(dag_count_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)(sizeof(DagTable<DG_WSLOTS>) * DG_WARPS)));
        RBG_CUDA_TRY(cudaFuncSetAttribute(dag_fill_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)(sizeof(DagTable<DG_WSLOTS>) * DG_WARPS)));
        RBG_CUDA_TRY(cudaFuncSetAttribute(dag_count_block_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)sizeof(DagTable<DG_BSLOTS>)));
        RBG_CUDA_TRY(cudaFuncSetAttribute(dag_fill_block_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)sizeof(DagTable<DG_BSLOTS>)));
        return (int)RBG_OK;
    }();
    if (configured) return configured;
    DagArgs a;
    a.n = n; a.ap = A->indptr; a.aj = aj; a.av = av; a.order = w.order;
    a.row_off = row_off; a.row_len = row_len;
    a.pcols = pool_cols; a.pvals = pool_vals; a.wcols = pool_cols; a.wvals = pool_vals;
    a.capacity = pool_capacity; a.lvl_len = w.lvl_len; a.lvl_off = w.lvl_off;
    a.wide = w.wide; a.nwide = w.nwide; a.max_abs = w.max_abs; a.flags = w.flags;
    const size_t wsm = sizeof(DagTable<DG_WSLOTS>) * DG_WARPS, bsm = sizeof(DagTable<DG_BSLOTS>);
    int64_t placed = 0;
    for (size_t L = 0; L + 1 < bounds.size(); ++L) {
        const int64_t ls = bounds[L];
        const int nl = (int)(bounds[L + 1] - ls);
        RBG_CUDA_TRY(cudaMemsetAsync(w.nwide, 0, 4, s));
        note_launches(6);
        const int cg = grid_for((int64_t)nl * 32, DG_WARPS * 32);
        dag_count_kernel<<<cg, DG_WARPS * 32, wsm, s>>>(a, ls, nl);
        dag_count_block_kernel<<<grid_for(304, 1), DG_BTHREADS, bsm, s>>>(a, ls);   // wide rows are rare
        tb = w.tmp_bytes;
        RBG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(w.tmp, tb, w.lvl_len, w.lvl_off, nl, s));
        dag_place_kernel<<<grid_for(nl, 256), 256, 0, s>>>(a, ls, nl, w.base);
        dag_advance_kernel<<<1, 32, 0, s>>>(w.lvl_off, w.lvl_len, nl, w.base);
        int fl[3] = {0, 0, 0};
        RBG_CUDA_TRY(cudaMemcpyAsync(&placed, w.base, 8, cudaMemcpyDeviceToHost, s));
        RBG_CUDA_TRY(cudaMemcpyAsync(fl, w.tail, 12, cudaMemcpyDeviceToHost, s));
        RBG_CUDA_TRY(cudaStreamSynchronize(s));
        if (fl[2]) { *nnz = -1; return RBG_ERR_CAPACITY; }          // a row wider than the block table
        if (placed > pool_capacity) {                               // rows of later levels need these
            *nnz = std::max<int64_t>(2 * pool_capacity, placed + placed / 2 + 1024);
            return RBG_ERR_CAPACITY;
        }
        dag_fill_kernel<<<cg, DG_WARPS * 32, wsm, s>>>(a, ls, nl);
        dag_fill_block_kernel<<<grid_for(304, 1), DG_BTHREADS, bsm, s>>>(a, ls);
        RBG_CUDA_TRY(cudaGetLastError());
    }
    unsigned long long mx = 0;
    RBG_CUDA_TRY(cudaMemcpyAsync(&mx, w.max_abs, 8, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    *nnz = placed;
    *max_abs = (int64_t)mx;
    return RBG_OK;
}

extern "C" int32_t rbg_dag_gather(int64_t n, const int32_t *pool_cols, const int32_t *pool_vals,
                                  const int64_t *row_off, const int32_t *row_len, void *workspace,
                                  int64_t workspace_bytes, int64_t *indptr, int32_t *indices, int32_t *data,
                                  rbg_stream_t stream) {
    if (n < 0 || !indptr || !workspace) return RBG_ERR_INVALID;
    size_t tb = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tb, (int64_t *)nullptr, (int64_t *)nullptr, (int)(n + 1));
    const size_t need = align_up((size_t)(n + 1) * 8, 256) + tb;
    if ((size_t)workspace_bytes < need) return RBG_ERR_NOMEM;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int64_t *len64 = reinterpret_cast<int64_t *>(workspace);
    void *tmp = reinterpret_cast<unsigned char *>(workspace) + align_up((size_t)(n + 1) * 8, 256);
    note_launches(2);
    dag_len64_kernel<<<grid_for(n + 1, 256), 256, 0, s>>>(n, row_len, len64);
    RBG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(tmp, tb, len64, indptr, (int)(n + 1), s));
    if (n > 0)
        dag_gather_rows_kernel<<<grid_for(n * 32, 256), 256, 0, s>>>(n, row_off, pool_cols, pool_vals, indptr,
                                                                     indices, data);
    RBG_CUDA_TRY(cudaGetLastError());
    return RBG_OK;
}

extern "C" int32_t rbg_dag_gather_workspace_bytes(int64_t n, int64_t *bytes) {
    if (!bytes || n < 0) return RBG_ERR_INVALID;
    size_t tb = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tb, (int64_t *)nullptr, (int64_t *)nullptr, (int)(n + 1));
    *bytes = (int64_t)(align_up((size_t)(n + 1) * 8, 256) + tb);
    return RBG_OK;
}
