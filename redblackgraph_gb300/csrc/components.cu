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

namespace rbg {

__device__ __forceinline__ int cc_find(const int *parent, int v) {
    int p = parent[v];
    while (p != v) {
        v = p;
        p = parent[v];
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
            int ru = cc_find(parent, (int)u), rv = cc_find(parent, v);
            while (ru != rv) {
                const int hi = max(ru, rv), lo = min(ru, rv);
                const int old = atomicMin(&parent[hi], lo);
                if (old == hi) { *changed = 1; break; }
                // hi was hooked meanwhile: retry from the new roots
                ru = cc_find(parent, old);
                rv = cc_find(parent, lo);
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
    tb = w.tmp_bytes;
    RBG_CUDA_TRY(cub::DeviceRadixSort::SortPairs(w.tmp, tb, label, w.keys_out, w.vid, sorted_vertex, ni, 0,
                                                 32, s));
    int nc = 0;
    RBG_CUDA_TRY(cudaMemcpyAsync(&nc, w.rank + n, 4, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
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
