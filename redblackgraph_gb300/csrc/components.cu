// components.cu -- component-wise closure support on sm_103a: connected components, grouping,
// densification into the batched-closure layout, and compaction of the closed components back
// into one merged CSR matrix.
//
// References (paths within rappdw/redblackgraph):
//   find_components_sparse     redblackgraph/sparse/csgraph/_components.pyx:86-177 (components of
//                              the graph with edges taken in both directions)
//   get_component_vertices     _components.pyx:326-344 (vertices of a component, ascending)
//   extract_submatrix          _components.pyx:180-252 (renumbering 0..len-1 in that order)
//   merge_component_matrices   _components.pyx:254-324 (global indices, rows sorted)
//   component_wise_closure     redblackgraph/sparse/csgraph/transitive_closure.py:85-195
//
// Components: union by atomicMin hooking of roots (the root of a component ends as its least
// vertex) alternating with pointer-jumping compression, until no hook changes a parent.  The
// loop has a fixed iteration bound (log2 n + 64 rounds of hooking); if it were ever reached the
// call reports RBG_ERR_TIMEOUT instead of spinning.
#include <cuda_runtime.h>
#include <cub/cub.cuh>
#include <algorithm>
#include "rbg_internal.cuh"
#include "dag_rows.cuh"

namespace rbg {

__device__ __forceinline__ int cc_find(const int *parent, int v) {
    int p = parent[v];
    while (p != v) {
        v = p;
        p = parent[v];
    }
    return v;
}

// The root of v, pointing every vertex on the way at its grandparent (path splitting).  A link
// only ever points at a smaller vertex of the same tree, so the shortcut keeps every tree; a
// shortcut stored over a concurrent hook of the same vertex undoes that hook, which the hooking
// thread then sees (its atomicMin did not find a root) and redoes from the new roots.
__device__ __forceinline__ int cc_find_split(int *parent, int v) {
    int p = parent[v];
    while (p != v) {
        const int gp = parent[p];
        if (gp != p) parent[v] = gp;
        v = p;
        p = gp;
    }
    return v;
}

__global__ void cc_init_kernel(int n, int *parent) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) parent[v] = v;
}

// one thread per stored entry (u, v): hook the larger root under the smaller
__global__ void cc_hook_kernel(int64_t n, const int64_t *indptr, const int *indices, int *parent, int *changed) {
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
        for (int64_t e = indptr[u]; e < indptr[u + 1]; ++e) {
            const int v = indices[e];
            if (v < 0 || v >= n) continue;            // malformed column index: ignored
            int ru = cc_find_split(parent, (int)u), rv = cc_find_split(parent, v);
            while (ru != rv) {
                const int hi = max(ru, rv), lo = min(ru, rv);
                const int old = atomicMin(&parent[hi], lo);
                if (old == hi) { *changed = 1; break; }
                // hi was hooked meanwhile: retry from the new roots
                ru = cc_find_split(parent, old);
                rv = cc_find_split(parent, lo);
            }
        }
    }
}

__global__ void cc_compress_kernel(int n, int *parent) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        parent[v] = cc_find(parent, v);
}

__global__ void cc_root_flag_kernel(int n, const int *parent, int *flag) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        flag[v] = parent[v] == v;
}

// label[v] = rank of its root among roots (components numbered by least vertex)
__global__ void cc_label_kernel(int n, const int *parent, const int *rank, int *label) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        label[v] = rank[parent[v]];
}

// after the stable sort by label: component starts, sizes, and each vertex's local index
__global__ void cc_layout_kernel(int n, const int *sorted_label, int64_t *start) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const int c = sorted_label[p];
        if (p == 0 || sorted_label[p - 1] != c) start[c] = p;
        if (p == n - 1 || sorted_label[p + 1] != c) start[c + 1] = p + 1;   // end marker
    }
}

__global__ void cc_local_kernel(int n, const int *sorted_label, const int *sorted_vertex, const int64_t *start,
                                int *local) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
        local[sorted_vertex[p]] = (int)(p - start[sorted_label[p]]);
}

// one warp per vertex row: zero the row of its block, then scatter the row's stored entries
// (__syncwarp orders the zeroing before the scatter).  Rows whose block would reach past
// flat_elems are skipped.
template <class T>
__global__ void cc_densify_kernel(int64_t n, const int64_t *indptr, const int *indices, const int *data,
                                  const int *label, const int *local, const int64_t *start,
                                  const int64_t *dense_off, T *flat, int64_t flat_elems) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t u = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); u < n; u += warps) {
        const int c = label[u];
        const int64_t nc = start[c + 1] - start[c];
        const int64_t row = dense_off[c] + (int64_t)local[u] * nc;
        if (dense_off[c] < 0 || dense_off[c] + nc * nc > flat_elems) continue;
        for (int64_t j = lane; j < nc; j += 32) flat[row + j] = (T)0;
        __syncwarp();
        for (int64_t e = indptr[u] + lane; e < indptr[u + 1]; e += 32) {
            const int v = indices[e];
            if (v >= 0 && v < n && label[v] == c) flat[row + local[v]] = (T)data[e];
        }
    }
}

// nonzeros of each closed row (warp per global row); optionally the largest value of each
// component (signed, floored at 0), which the final-value diameter needs
// Chunk masks: bit b of a row's mask words says whether columns [32 b, 32 b + 32) of the closed
// row hold a nonzero, so the fill reads only those chunks.  Component c keeps its rows' words
// (ceil(nc / 2048) each) from word ceil(dense_off[c] / 2048) + start[c] + c on.
__device__ __forceinline__ int64_t cc_mask_base(int c, const int64_t *start, const int64_t *dense_off) {
    return (dense_off[c] + 2047) / 2048 + start[c] + c;
}

__global__ void cc_rowcount_kernel(int64_t n, const int *label, const int *local, const int64_t *start,
                                   const int64_t *dense_off, const int *flat, int64_t *cnt, int *comp_max,
                                   unsigned long long *mask) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t u = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); u < n; u += warps) {
        const int c = label[u];
        const int64_t nc = start[c + 1] - start[c];
        const int *row = flat + dense_off[c] + (int64_t)local[u] * nc;
        const int64_t words = (nc + 2047) / 2048;
        unsigned long long *mrow = mask ? mask + cc_mask_base(c, start, dense_off) + (int64_t)local[u] * words : nullptr;
        int64_t k = 0;
        int mx = 0;
        unsigned long long word = 0;
        for (int64_t j0 = 0; j0 < nc; j0 += 256) {     // eight chunks of 32 columns in flight
            int v[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int64_t j = j0 + 32 * q + lane;
                v[q] = j < nc ? row[j] : 0;
            }
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int64_t c0 = j0 + 32 * q;
                if (c0 >= nc) break;                    // uniform
                mx = max(mx, v[q]);
                const unsigned bal = __ballot_sync(0xffffffffu, v[q] != 0);
                k += __popc(bal);
                const int64_t chunk = c0 >> 5;
                if (bal) word |= 1ull << (chunk & 63);
                if (mrow && ((chunk & 63) == 63 || c0 + 32 >= nc)) {
                    if (lane == 0) mrow[chunk >> 6] = word;
                    word = 0;
                }
            }
        }
        mx = __reduce_max_sync(0xffffffffu, mx);
        if (lane == 0) {
            cnt[u] = k;
            if (comp_max && mx > 0) atomicMax(comp_max + c, mx);
        }
    }
}

// write each closed row with global column indices (ascending: local order is vertex order)
__global__ void cc_fill_kernel(int64_t n, const int *label, const int *local, const int64_t *start,
                               const int64_t *dense_off, const int *flat, const int *sorted_vertex,
                               const int64_t *outptr, int *oj, int *ov, const unsigned long long *mask) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t u = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); u < n; u += warps) {
        const int c = label[u];
        const int64_t s = start[c], nc = start[c + 1] - s;
        const int *row = flat + dense_off[c] + (int64_t)local[u] * nc;
        int64_t out = outptr[u];
        if (mask) {
            const int64_t words = (nc + 2047) / 2048;
            const unsigned long long *mrow = mask + cc_mask_base(c, start, dense_off) + (int64_t)local[u] * words;
            for (int64_t wi = 0; wi < words; ++wi) {
                unsigned long long word = mrow[wi];
                while (word) {
                    const int b = __ffsll((long long)word) - 1;
                    word &= word - 1;
                    const int64_t j = (wi * 64 + b) * 32 + lane;
                    const int v = j < nc ? row[j] : 0;
                    const unsigned bal = __ballot_sync(0xffffffffu, v != 0);
                    if (v != 0) {
                        const int64_t pos = out + __popc(bal & ((1u << lane) - 1u));
                        oj[pos] = sorted_vertex[s + j];
                        ov[pos] = v;
                    }
                    out += __popc(bal);
                }
            }
            continue;
        }
        for (int64_t j0 = 0; j0 < nc; j0 += 32) {
            const int64_t j = j0 + lane;
            const int v = j < nc ? row[j] : 0;
            const unsigned bal = __ballot_sync(0xffffffffu, v != 0);
            if (v != 0) {
                const int64_t pos = out + __popc(bal & ((1u << lane) - 1u));
                oj[pos] = sorted_vertex[s + j];
                ov[pos] = v;
            }
            out += __popc(bal);
        }
    }
}

}  // namespace rbg

using namespace rbg;

namespace {

struct CcWs {
    int *parent, *flag, *rank, *changed, *keys_out;
    int *vid;
    int64_t *cnt;
    void *tmp;
    size_t tmp_bytes;
};

size_t cc_tmp_bytes(int64_t n) {
    const int m = (int)std::max<int64_t>(n + 1, 1);
    size_t a = 0, b = 0, c = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, a, (int *)nullptr, (int *)nullptr, m);
    cub::DeviceScan::ExclusiveSum(nullptr, b, (int64_t *)nullptr, (int64_t *)nullptr, m);
    cub::DeviceRadixSort::SortPairs(nullptr, c, (int *)nullptr, (int *)nullptr, (int *)nullptr, (int *)nullptr, m);
    return std::max(a, std::max(b, c));
}

size_t cc_layout(int64_t n, unsigned char *base, CcWs *w) {
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o = align_up(o + bytes, 256); return base ? base + at : nullptr; };
    const size_t ni = (size_t)(n + 1) * 4;
    unsigned char *p;
    p = take(ni); if (w) w->parent = (int *)p;
    p = take(ni); if (w) w->flag = (int *)p;
    p = take(ni); if (w) w->rank = (int *)p;
    p = take(64); if (w) w->changed = (int *)p;
    p = take(ni); if (w) w->keys_out = (int *)p;
    p = take(ni); if (w) w->vid = (int *)p;
    p = take((size_t)(n + 1) * 8); if (w) w->cnt = (int64_t *)p;
    const size_t tb = cc_tmp_bytes(n);
    p = take(tb); if (w) { w->tmp = p; w->tmp_bytes = tb; }
    return o;
}

__global__ void cc_iota_kernel(int n, int *v) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = i;
}

}  // namespace

extern "C" int32_t rbg_cc_workspace_bytes(int64_t n, int64_t *bytes) {
    if (!bytes || n < 0 || n >= (1ll << 31) - 1) return RBG_ERR_INVALID;
    *bytes = (int64_t)cc_layout(n, nullptr, nullptr);
    return RBG_OK;
}

extern "C" int32_t rbg_cc_label(int64_t n, const int64_t *indptr, const int32_t *indices, void *workspace,
                                int64_t workspace_bytes, int32_t *label, int32_t *sorted_vertex, int32_t *local,
                                int64_t *start, int64_t *ncomp, rbg_stream_t stream) {
    if (n < 0 || !indptr || !workspace || !label || !sorted_vertex || !local || !start || !ncomp)
        return RBG_ERR_INVALID;
    if (workspace_bytes < (int64_t)cc_layout(n, nullptr, nullptr)) return RBG_ERR_NOMEM;
    *ncomp = 0;
    if (n == 0) return RBG_OK;
    CcWs w;
    cc_layout(n, reinterpret_cast<unsigned char *>(workspace), &w);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int ni = (int)n;
    const int g = grid_for(n, 256);
    note_launches(1);
    cc_init_kernel<<<g, 256, 0, s>>>(ni, w.parent);
    int bound = 64;
    for (int64_t m = n; m > 1; m >>= 1) ++bound;
    int rounds = 0;
    for (;; ++rounds) {
        if (rounds >= bound) return RBG_ERR_TIMEOUT;
        int hc = 0;
        RBG_CUDA_TRY(cudaMemsetAsync(w.changed, 0, 4, s));
        note_launches(2);
        cc_hook_kernel<<<g, 256, 0, s>>>(n, indptr, indices, w.parent, w.changed);
        cc_compress_kernel<<<g, 256, 0, s>>>(ni, w.parent);
        RBG_CUDA_TRY(cudaMemcpyAsync(&hc, w.changed, 4, cudaMemcpyDeviceToHost, s));
        RBG_CUDA_TRY(cudaStreamSynchronize(s));
        if (!hc) break;
    }
    // number the components by their least vertex
    note_launches(4);
    cc_root_flag_kernel<<<g, 256, 0, s>>>(ni, w.parent, w.flag);
    RBG_CUDA_TRY(cudaMemsetAsync(w.flag + n, 0, 4, s));
    size_t tb = w.tmp_bytes;
    RBG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(w.tmp, tb, w.flag, w.rank, ni + 1, s));
    cc_label_kernel<<<g, 256, 0, s>>>(ni, w.parent, w.rank, label);
    // group vertices by component, ascending within each (radix sort is stable)
    cc_iota_kernel<<<g, 256, 0, s>>>(ni, w.vid);
    // the labels are below the component count: sort only their low bits
    int nc = 0;
    RBG_CUDA_TRY(cudaMemcpyAsync(&nc, w.rank + n, 4, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    int bits = 1;
    while (bits < 32 && ((int64_t)1 << bits) < (int64_t)nc) ++bits;
    tb = w.tmp_bytes;
    RBG_CUDA_TRY(cub::DeviceRadixSort::SortPairs(w.tmp, tb, label, w.keys_out, w.vid, sorted_vertex, ni, 0,
                                                 bits, s));
    note_launches(2);
    cc_layout_kernel<<<g, 256, 0, s>>>(ni, w.keys_out, start);
    cc_local_kernel<<<g, 256, 0, s>>>(ni, w.keys_out, sorted_vertex, start, local);
    RBG_CUDA_TRY(cudaGetLastError());
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    *ncomp = nc;
    return RBG_OK;
}

extern "C" int32_t rbg_cc_densify(int32_t dtype, int64_t n, const int64_t *indptr, const int32_t *indices,
                                  const int32_t *data, const int32_t *label, const int32_t *local,
                                  const int64_t *start, const int64_t *dense_off, void *flat, int64_t flat_elems,
                                  rbg_stream_t stream) {
    if (n < 0 || !flat || flat_elems < 0) return RBG_ERR_INVALID;
    if (dtype != RBG_DTYPE_INT32 && dtype != RBG_DTYPE_INT64) return RBG_ERR_INVALID;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (n > 0) {
        note_launches(1);
        const int g = grid_for(n * 32, 256);
        if (dtype == RBG_DTYPE_INT64)
            cc_densify_kernel<int64_t><<<g, 256, 0, s>>>(n, indptr, indices, data, label, local, start, dense_off,
                                                          reinterpret_cast<int64_t *>(flat), flat_elems);
        else
            cc_densify_kernel<int32_t><<<g, 256, 0, s>>>(n, indptr, indices, data, label, local, start, dense_off,
                                                          reinterpret_cast<int32_t *>(flat), flat_elems);
        RBG_CUDA_TRY(cudaGetLastError());
    }
    return RBG_OK;
}

extern "C" int32_t rbg_cc_chunk_mask_words(int64_t n, int64_t ncomp, int64_t flat_elems, int64_t *words) {
    if (!words || n < 0 || ncomp < 0 || flat_elems < 0) return RBG_ERR_INVALID;
    *words = (flat_elems + 2047) / 2048 + n + 2 * ncomp + 2;
    return RBG_OK;
}

extern "C" int32_t rbg_cc_compact_count(int64_t n, int64_t ncomp, const int32_t *label, const int32_t *local,
                                        const int64_t *start, const int64_t *dense_off, const int32_t *flat,
                                        void *workspace, int64_t workspace_bytes, int64_t *nnz,
                                        int32_t *comp_max, uint64_t *chunk_mask, rbg_stream_t stream) {
    if (n < 0 || ncomp < 0 || ncomp > n || !workspace || !nnz) return RBG_ERR_INVALID;
    if (workspace_bytes < (int64_t)cc_layout(n, nullptr, nullptr)) return RBG_ERR_NOMEM;
    CcWs w;
    cc_layout(n, reinterpret_cast<unsigned char *>(workspace), &w);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    RBG_CUDA_TRY(cudaMemsetAsync(w.cnt + n, 0, 8, s));
    if (comp_max && ncomp > 0) RBG_CUDA_TRY(cudaMemsetAsync(comp_max, 0, (size_t)ncomp * 4, s));
    if (n > 0) {
        note_launches(1);
        cc_rowcount_kernel<<<grid_for(n * 32, 256), 256, 0, s>>>(n, label, local, start, dense_off, flat, w.cnt,
                                                                 comp_max,
                                                                 reinterpret_cast<unsigned long long *>(chunk_mask));
    }
    size_t tb = w.tmp_bytes;
    RBG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(w.tmp, tb, w.cnt, w.cnt, (int)(n + 1), s));
    int64_t tot = 0;
    RBG_CUDA_TRY(cudaMemcpyAsync(&tot, w.cnt + n, 8, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    *nnz = tot;
    return RBG_OK;
}

extern "C" int32_t rbg_cc_compact_scan(int64_t n, const int64_t *row_count, void *workspace,
                                       int64_t workspace_bytes, int64_t *nnz, rbg_stream_t stream) {
    if (n < 0 || !workspace || !nnz || (n > 0 && !row_count)) return RBG_ERR_INVALID;
    if (workspace_bytes < (int64_t)cc_layout(n, nullptr, nullptr)) return RBG_ERR_NOMEM;
    CcWs w;
    cc_layout(n, reinterpret_cast<unsigned char *>(workspace), &w);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (n > 0) RBG_CUDA_TRY(cudaMemcpyAsync(w.cnt, row_count, (size_t)n * 8, cudaMemcpyDeviceToDevice, s));
    RBG_CUDA_TRY(cudaMemsetAsync(w.cnt + n, 0, 8, s));
    size_t tb = w.tmp_bytes;
    RBG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(w.tmp, tb, w.cnt, w.cnt, (int)(n + 1), s));
    int64_t tot = 0;
    RBG_CUDA_TRY(cudaMemcpyAsync(&tot, w.cnt + n, 8, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    *nnz = tot;
    return RBG_OK;
}

extern "C" int32_t rbg_cc_compact_fill(int64_t n, const int32_t *label, const int32_t *local, const int64_t *start,
                                       const int64_t *dense_off, const int32_t *flat, const int32_t *sorted_vertex,
                                       const void *workspace, int64_t *indptr, int32_t *indices, int32_t *data,
                                       const uint64_t *chunk_mask, rbg_stream_t stream) {
    if (n < 0 || !workspace || !indptr) return RBG_ERR_INVALID;
    CcWs w;
    cc_layout(n, const_cast<unsigned char *>(reinterpret_cast<const unsigned char *>(workspace)), &w);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    RBG_CUDA_TRY(cudaMemcpyAsync(indptr, w.cnt, (size_t)(n + 1) * 8, cudaMemcpyDeviceToDevice, s));
    if (n > 0) {
        note_launches(1);
        cc_fill_kernel<<<grid_for(n * 32, 256), 256, 0, s>>>(n, label, local, start, dense_off, flat, sorted_vertex,
                                                             w.cnt, indices, data,
                                                             reinterpret_cast<const unsigned long long *>(chunk_mask));
        RBG_CUDA_TRY(cudaGetLastError());
    }
    return RBG_OK;
}

// ------------------------------------------------------------------------------------------
// Component-wise closure straight from the CSR graph, for graphs whose components are all
// numbered in a topological order and in the clean regime: the DAG path of the batched dense
// closure (fw_tri.cu) without dense blocks.  Each component's closure is the DAG recurrence
// (rbg_dag_closure over the off-diagonal entries), its Floyd-Warshall diameter comes from each
// cell's first value (dag_rows.cuh), and the merged matrix is the closure rows with the
// diagonal put back.
// ------------------------------------------------------------------------------------------
namespace rbg {

constexpr unsigned CCD_UNCLEAN = 1u, CCD_BELOW = 2u, CCD_ABOVE = 4u;
constexpr int CCD_WARPS = 8;

// one thread per vertex, in the order of the components (position r of sorted_vertex): its row's
// diagonal value and off-diagonal nonzero count, and its component's flags (clean regime, side of
// the diagonal), ORed over the warp's lanes of each component into one atomic (a warp per
// component left the largest components' rows to one warp)
__global__ void __launch_bounds__(256) cc_dag_classify_kernel(int64_t n, int64_t ncomp,
                                       const int64_t *__restrict__ indptr,
                                       const int32_t *__restrict__ indices, const int32_t *__restrict__ data,
                                       const int32_t *__restrict__ sorted_vertex, const int64_t *__restrict__ start,
                                       unsigned *__restrict__ comp_flags, int32_t *__restrict__ diag,
                                       int64_t *__restrict__ cnt) {
    const int lane = threadIdx.x & 31;
    const int64_t step = (int64_t)gridDim.x * blockDim.x;
    for (int64_t rb = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); rb < n; rb += step) {
        const int64_t r = rb + lane;
        const bool in = r < n;
        int64_t c = 0;                               // the last component starting at or before rb
        if (lane == 0) {
            int64_t lo = 0, hi = ncomp - 1;
            while (lo < hi) {
                const int64_t mid = (lo + hi + 1) >> 1;
                if (start[mid] <= rb) lo = mid;
                else hi = mid - 1;
            }
            c = lo;
        }
        c = __shfl_sync(0xffffffffu, c, 0);
        unsigned f = 0;
        if (in) {
            while (c + 1 < ncomp && start[c + 1] <= r) ++c;
            const int64_t u = sorted_vertex[r];
            int32_t d = 0;
            int64_t k = 0;
            for (int64_t e = indptr[u]; e < indptr[u + 1]; ++e) {
                const int32_t v = data[e];
                const int64_t col = indices[e];
                if (col == u) {
                    d = v;
                    if (!(v == 0 || v == 1 || v == -1)) f |= CCD_UNCLEAN;
                } else if (v != 0) {
                    if (v == 1 || v < 0) f |= CCD_UNCLEAN;
                    f |= col < u ? CCD_BELOW : CCD_ABOVE;
                    ++k;
                }
            }
            diag[u] = d;
            cnt[u] = k;
        }
        unsigned todo = __ballot_sync(0xffffffffu, in);
        while (todo) {                               // each component of the warp's lanes
            const int leader = __ffs(todo) - 1;
            const int64_t cl = __shfl_sync(0xffffffffu, c, leader);
            const bool mine = in && c == cl;
            const unsigned fo = __reduce_or_sync(0xffffffffu, mine ? f : 0u);
            if (lane == leader && fo) atomicOr(comp_flags + cl, fo);
            todo &= ~__ballot_sync(0xffffffffu, mine);
        }
    }
}

// the off-diagonal nonzeros of every row, in column order
__global__ void cc_dag_edges_kernel(int64_t n, const int64_t *__restrict__ indptr, const int32_t *__restrict__ indices,
                                    const int32_t *__restrict__ data, const int64_t *__restrict__ edge_ptr,
                                    int32_t *__restrict__ edge_col, int32_t *__restrict__ edge_val) {
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
        int64_t o = edge_ptr[u];
        for (int64_t e = indptr[u]; e < indptr[u + 1]; ++e) {
            const int32_t v = data[e];
            if (indices[e] != u && v != 0) {
                edge_col[o] = indices[e];
                edge_val[o] = v;
                ++o;
            }
        }
    }
}

// the row statistics of dag_rows.cuh and the row's largest final value, reduced per component:
// a group of DAG_STATS_G lanes per vertex, runs of `run` vertices per group, one set of atomics
// per run and component (each group's bitmap takes 1 KB of shared memory)
constexpr int CCD_STATS_GROUPS = 32 * CCD_WARPS / DAG_STATS_G;
constexpr int CCD_STATS_CTAS = 5;
__global__ void __launch_bounds__(32 * CCD_WARPS, CCD_STATS_CTAS)
cc_dag_stats_kernel(int64_t n, const int32_t *__restrict__ label, const int32_t *__restrict__ local,
                    const int64_t *__restrict__ start, const int32_t *__restrict__ sorted_vertex,
                    const int32_t *__restrict__ comp_kind,
                    const int64_t *__restrict__ eptr, const int32_t *__restrict__ ecol, const int32_t *__restrict__ eval,
                    const int64_t *__restrict__ row_off, const int32_t *__restrict__ row_len,
                    const int32_t *__restrict__ ccol, const int32_t *__restrict__ cval,
                    const int32_t *__restrict__ diag, int *__restrict__ top, int *__restrict__ first,
                    int *__restrict__ cmax, int run) {
    constexpr int G = DAG_STATS_G;
    __shared__ __align__(16) unsigned bm_all[CCD_STATS_GROUPS][DAG_MAX_N / 32];
    const int grp = threadIdx.x / G, lane = threadIdx.x & (G - 1);
    const unsigned gmask = dag_group_mask<G>();
    int cur = -1, am = -1, fm = -1, mx = 0;  // the component of the run's current rows, its statistics
    int kind = DAG_KIND_NONE, lo = 0, hi = 0;  // and its kind, lowest and highest vertex, and the
    int lwords = 0;                            // bitmap words of its local indices
    unsigned long long prods = 0;
    auto flush = [&]() {                     // group-uniform
        const int am_r = __reduce_max_sync(gmask, am);
        const int fm_r = __reduce_max_sync(gmask, fm);
        const int mx_r = __reduce_max_sync(gmask, mx);
        if (lane == 0 && cur >= 0) {
            if (am_r >= 0) atomicMax(top + cur, am_r);
            if (fm_r >= 0) atomicMax(first + cur, fm_r);
            if (mx_r > 0) atomicMax(cmax + cur, mx_r);
        }
    };
    auto crow = [&](int64_t r, int64_t &off, int &len) { off = row_off[r]; len = row_len[r]; };
    const int64_t stride = (int64_t)gridDim.x * CCD_STATS_GROUPS * run;
    for (int64_t r0 = ((int64_t)blockIdx.x * CCD_STATS_GROUPS + grp) * run; r0 < n; r0 += stride) {
        const int64_t r1 = min(n, r0 + run);
        for (int64_t u = r0; u < r1; ++u) {
            const int c = label[u];
            const int64_t a0 = eptr[u];
            const int alen = (int)(eptr[u + 1] - a0);
            if (c != cur) {                          // group-uniform
                flush();
                cur = c;
                am = fm = -1;
                mx = 0;
                kind = comp_kind[c];
                // a component whose vertices span fewer than DAG_MAX_N numbers indexes its
                // bitmap by vertex - lowest vertex (no gather); otherwise by its local index
                const int64_t c0 = start[c], csize = start[c + 1] - c0;
                lo = sorted_vertex[c0];
                hi = sorted_vertex[c0 + csize - 1];
                lwords = (int)((min(csize, (int64_t)DAG_MAX_N + 32) + 31) >> 5);   // clamped by the rows
            }
            if (kind == DAG_KIND_NONE) continue;     // group-uniform
            if (hi - lo < DAG_MAX_N)
                dag_row_stats<G>(bm_all[grp], (hi - lo + 32) >> 5, kind, u, a0, alen, eptr, ecol, eval, crow, ccol,
                                 cval, [&](int32_t col) { return col - lo; }, lane, gmask, am, fm, prods);
            else
                dag_row_stats<G>(bm_all[grp], lwords, kind, u, a0, alen, eptr,
                                 ecol, eval, crow, ccol, cval, [&](int32_t col) { return local[col]; }, lane, gmask,
                                 am, fm, prods);
            const int64_t o = row_off[u];
            const int len = row_len[u];
            for (int q = lane; q < len; q += G) mx = max(mx, cval[o + q]);
            if (lane == 0) mx = max(mx, diag[u]);
        }
    }
    flush();
}

__global__ void cc_dag_merge_count_kernel(int64_t n, const int32_t *__restrict__ row_len, const int32_t *__restrict__ diag,
                                          int64_t *__restrict__ cnt) {
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x)
        cnt[u] = row_len[u] + (diag[u] != 0 ? 1 : 0);
}

// the closure row of each vertex with the diagonal value put in its place: a group of
// DAG_STATS_G lanes per vertex (a closure row holds about ten entries), runs of consecutive
// vertices per group
__global__ void __launch_bounds__(256) cc_dag_merge_fill_kernel(int64_t n, const int64_t *__restrict__ row_off,
                                         const int32_t *__restrict__ row_len, const int32_t *__restrict__ ccol,
                                         const int32_t *__restrict__ cval, const int32_t *__restrict__ diag,
                                         const int64_t *__restrict__ optr, int32_t *__restrict__ ocol,
                                         int32_t *__restrict__ oval, int run) {
    constexpr int G = DAG_STATS_G, GROUPS = 256 / G;
    const int grp = threadIdx.x / G, lane = threadIdx.x & (G - 1);
    const unsigned gmask = dag_group_mask<G>();
    const int64_t stride = (int64_t)gridDim.x * GROUPS * run;
    for (int64_t r0 = ((int64_t)blockIdx.x * GROUPS + grp) * run; r0 < n; r0 += stride) {
        const int64_t r1 = min(n, r0 + run);
        for (int64_t u = r0; u < r1; ++u) {
            const int64_t c0 = row_off[u], c1 = c0 + row_len[u], o = optr[u];
            const int32_t d = diag[u];
            const int shift = d != 0 ? 1 : 0;
            int below = 0;                           // closure entries left of the diagonal
            for (int64_t q = c0 + lane; q < c1; q += G) {
                const int32_t col = ccol[q];
                below += col < u;
                const int64_t at = o + (q - c0) + (col > u ? shift : 0);
                ocol[at] = col;
                oval[at] = cval[q];
            }
            below = __reduce_add_sync(gmask, below);
            if (lane == 0 && d != 0) {
                ocol[o + below] = (int32_t)u;
                oval[o + below] = d;
            }
        }
    }
}

}  // namespace rbg

extern "C" int32_t rbg_cc_dag_classify(int64_t n, const int64_t *indptr, const int32_t *indices, const int32_t *data,
                                       const int32_t *sorted_vertex, const int64_t *start, int64_t ncomp,
                                       void *workspace, int64_t workspace_bytes, uint32_t *comp_flags,
                                       int32_t *diag, int64_t *edge_ptr, int64_t *edges, rbg_stream_t stream) {
    if (n < 0 || ncomp < 0 || ncomp > n || (n > 0 && ncomp == 0) || !workspace || !edges ||
        (n > 0 && (!indptr || !sorted_vertex || !start || !comp_flags || !diag || !edge_ptr)))
        return RBG_ERR_INVALID;
    if (workspace_bytes < (int64_t)cc_layout(n, nullptr, nullptr)) return RBG_ERR_NOMEM;
    CcWs w;
    cc_layout(n, reinterpret_cast<unsigned char *>(workspace), &w);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    *edges = 0;
    if (n == 0) return RBG_OK;
    note_launches(1);
    RBG_CUDA_TRY(cudaMemsetAsync(comp_flags, 0, (size_t)ncomp * 4, s));
    cc_dag_classify_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, ncomp, indptr, indices, data, sorted_vertex, start,
                                                            comp_flags, diag, edge_ptr);
    RBG_CUDA_TRY(cudaGetLastError());
    RBG_CUDA_TRY(cudaMemsetAsync(edge_ptr + n, 0, 8, s));
    size_t tb = w.tmp_bytes;
    RBG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(w.tmp, tb, edge_ptr, edge_ptr, (int)(n + 1), s));
    RBG_CUDA_TRY(cudaMemcpyAsync(edges, edge_ptr + n, 8, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    return RBG_OK;
}

extern "C" int32_t rbg_cc_dag_edges(int64_t n, const int64_t *indptr, const int32_t *indices, const int32_t *data,
                                    const int64_t *edge_ptr, int32_t *edge_col, int32_t *edge_val,
                                    rbg_stream_t stream) {
    if (n < 0 || (n > 0 && (!indptr || !edge_ptr))) return RBG_ERR_INVALID;
    if (n == 0) return RBG_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    note_launches(1);
    cc_dag_edges_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, indptr, indices, data, edge_ptr, edge_col, edge_val);
    RBG_CUDA_TRY(cudaGetLastError());
    return RBG_OK;
}

extern "C" int32_t rbg_cc_dag_stats(int64_t n, int64_t ncomp, const int32_t *label, const int32_t *local,
                                    const int64_t *start, const int32_t *sorted_vertex, const int32_t *comp_kind,
                                    const rbg_csr_t *edges, const int64_t *row_off, const int32_t *row_len,
                                    const int32_t *pool_cols, const int32_t *pool_vals, const int32_t *diag,
                                    int32_t *top_msb, int32_t *first_msb, int32_t *comp_max, rbg_stream_t stream) {
    if (n < 0 || ncomp < 0 || !edges || (ncomp > 0 && (!top_msb || !first_msb || !comp_max)))
        return RBG_ERR_INVALID;
    if (edges->n_rows != n || (n > 0 && (!row_off || !row_len))) return RBG_ERR_INVALID;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (ncomp > 0) {
        RBG_CUDA_TRY(cudaMemsetAsync(top_msb, 0xff, (size_t)ncomp * 4, s));
        RBG_CUDA_TRY(cudaMemsetAsync(first_msb, 0xff, (size_t)ncomp * 4, s));
        RBG_CUDA_TRY(cudaMemsetAsync(comp_max, 0, (size_t)ncomp * 4, s));
    }
    if (n == 0) return RBG_OK;
    note_launches(1);
    const int64_t ctas = (int64_t)sm_count() * CCD_STATS_CTAS;
    const int run = dag_stats_run(n, ctas * CCD_STATS_GROUPS);
    const int64_t need = (n + (int64_t)run * CCD_STATS_GROUPS - 1) / ((int64_t)run * CCD_STATS_GROUPS);
    cc_dag_stats_kernel<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(need, ctas)), 32 * CCD_WARPS, 0, s>>>(
        n, label, local, start, sorted_vertex, comp_kind, edges->indptr, edges->indices, static_cast<const int32_t *>(edges->data),
        row_off, row_len, pool_cols, pool_vals, diag, top_msb, first_msb, comp_max, run);
    RBG_CUDA_TRY(cudaGetLastError());
    return RBG_OK;
}

extern "C" int32_t rbg_cc_dag_merge_count(int64_t n, const int32_t *row_len, const int32_t *diag, void *workspace,
                                          int64_t workspace_bytes, int64_t *out_indptr, int64_t *nnz,
                                          rbg_stream_t stream) {
    if (n < 0 || !workspace || !nnz || !out_indptr || (n > 0 && (!row_len || !diag))) return RBG_ERR_INVALID;
    if (workspace_bytes < (int64_t)cc_layout(n, nullptr, nullptr)) return RBG_ERR_NOMEM;
    CcWs w;
    cc_layout(n, reinterpret_cast<unsigned char *>(workspace), &w);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (n > 0) {
        note_launches(1);
        cc_dag_merge_count_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, row_len, diag, out_indptr);
        RBG_CUDA_TRY(cudaGetLastError());
    }
    RBG_CUDA_TRY(cudaMemsetAsync(out_indptr + n, 0, 8, s));
    size_t tb = w.tmp_bytes;
    RBG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(w.tmp, tb, out_indptr, out_indptr, (int)(n + 1), s));
    RBG_CUDA_TRY(cudaMemcpyAsync(nnz, out_indptr + n, 8, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    return RBG_OK;
}

extern "C" int32_t rbg_cc_dag_merge_fill(int64_t n, const int64_t *row_off, const int32_t *row_len,
                                         const int32_t *pool_cols, const int32_t *pool_vals, const int32_t *diag,
                                         const int64_t *out_indptr, int32_t *out_indices, int32_t *out_data,
                                         rbg_stream_t stream) {
    if (n < 0 || (n > 0 && (!row_off || !row_len || !diag || !out_indptr))) return RBG_ERR_INVALID;
    if (n == 0) return RBG_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    note_launches(1);
    const int64_t ctas = (int64_t)sm_count() * 8;
    const int run = dag_stats_run(n, ctas * 32);
    const int64_t need = (n + (int64_t)run * 32 - 1) / ((int64_t)run * 32);
    cc_dag_merge_fill_kernel<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(need, ctas)), 256, 0, s>>>(
        n, row_off, row_len, pool_cols, pool_vals, diag, out_indptr, out_indices, out_data, run);
    RBG_CUDA_TRY(cudaGetLastError());
    return RBG_OK;
}
