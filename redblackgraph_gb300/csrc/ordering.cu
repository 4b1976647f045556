// ordering.cu -- canonical ordering and permutation of closed matrices on sm_103a.
//
// References: avos_canonical_ordering with _get_permutation / _get_permutation_sparse /
// _compute_ordering_metrics_sparse (redblackgraph/sparse/csgraph/_ordering.pyx:15-177),
// permute / _permute_dense / permute_sparse (redblackgraph/sparse/csgraph/_permutation.pyx:11-205),
// and topological_sort / is_upper_triangular (_topological_sort.pyx:30-265).  The reference sorts
// topologically by an iterative depth-first search (reverse post-order); here the order comes
// from Kahn levels (deepest level first, vertex id ascending within a level): the same contract
// (every edge points to a later position, so the permuted matrix is upper triangular), another
// permutation where several orders qualify.
//
// The canonical order sorts the vertices by (component size descending, component id ascending,
// ancestor count descending, largest value in the vertex's column ascending, diagonal value
// descending, vertex id ascending); the ancestor count of a vertex is the sum of the Cython MSB
// of its row's non-zero values, the column maximum starts at zero.  Here the per-vertex metrics
// come from one pass over the matrix (a warp per row; column maxima by atomicMax), and the order
// from three stable radix sorts of 64-bit keys, least significant first, starting from the
// identity (which supplies the vertex-id tie break).  Permutation: dense B[i][j] = A[p[i]][p[j]]
// (a block of threads per output row); sparse: new row i is old row p[i] with columns mapped
// through the inverse permutation, counted, scattered and sorted per row (CUB segmented sort).
#include <cuda_runtime.h>
#include <cub/cub.cuh>
#include <algorithm>
#include <vector>
#include "rbg_internal.cuh"

namespace rbg {
namespace {

__device__ __forceinline__ int cy_msb_dev(int32_t x) {   // _rbg_math.pxi:1-11: `while x > 1`
    return x > 1 ? 31 - __clz(x) : 0;
}

__global__ void ord_metrics_csr_kernel(int64_t n, const int64_t *ip, const int32_t *ij, const int32_t *x, int64_t *anc,
                                       int32_t *maxrel, int32_t *diag) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
        long long a = 0;
        int64_t dpos = -1;
        for (int64_t e = ip[i] + lane; e < ip[i + 1]; e += 32) {
            const int32_t v = x[e];
            const int32_t c = ij[e];
            if (v != 0) {
                a += cy_msb_dev(v);
                if (v > 0) atomicMax(maxrel + c, v);
            }
            if (c == (int32_t)i) dpos = max(dpos, e);           // the row's last diagonal entry
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            dpos = max(dpos, (int64_t)__shfl_xor_sync(0xffffffffu, (long long)dpos, o));
        }
        if (lane == 0) {
            anc[i] = a;
            diag[i] = dpos >= 0 ? x[dpos] : 0;
        }
    }
}

__global__ void ord_metrics_dense_kernel(int64_t n, const int32_t *A, int64_t lda, int64_t *anc, int32_t *maxrel,
                                         int32_t *diag) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
        long long a = 0;
        for (int64_t j = lane; j < n; j += 32) {
            const int32_t v = A[i * lda + j];
            if (v != 0) {
                a += cy_msb_dev(v);
                if (v > 0) atomicMax(maxrel + j, v);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) {
            anc[i] = a;
            diag[i] = A[i * lda + i];
        }
    }
}

// keys of the three stable passes (least significant first)
__global__ void ord_keys_kernel(int64_t n, int pass, const int32_t *label, const int64_t *comp_start,
                                const int64_t *anc, const int32_t *maxrel, const int32_t *diag, const int32_t *vals,
                                unsigned long long *keys) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = vals[k];
        unsigned long long key;
        if (pass == 0) {        // column maximum ascending (>= 0), then diagonal descending
            const unsigned d = ~((unsigned)diag[v] ^ 0x80000000u);
            key = ((unsigned long long)(unsigned)maxrel[v] << 32) | d;
        } else if (pass == 1) { // ancestor count descending
            key = ~(unsigned long long)anc[v];
        } else {                // component size descending, then component id ascending
            const int32_t c = label[v];
            const int64_t size = comp_start[c + 1] - comp_start[c];
            key = ((unsigned long long)(n - size) << 32) | (unsigned)c;
        }
        keys[k] = key;
    }
}

__global__ void ord_iota_kernel(int64_t n, int32_t *v) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        v[k] = (int32_t)k;
}

template <typename T>
__global__ void ord_permute_dense_kernel(int64_t n, const T *A, int64_t lda, const int32_t *p, T *B, int64_t ldb,
                                         int upper) {
    for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
        const T *src = A + (int64_t)p[i] * lda;
        for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
            // the reference leaves B[i][j] = 0 below the diagonal in the triangular mode
            B[i * ldb + j] = (upper && j < i) ? T(0) : src[p[j]];
        }
    }
}

__global__ void ord_inverse_kernel(int64_t n, const int32_t *p, int32_t *pinv) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        pinv[p[k]] = (int32_t)k;
}

// entries of each new row (upper: only new columns >= the row)
__global__ void ord_csr_count_kernel(int64_t n, const int64_t *ip, const int32_t *ij, const int32_t *p,
                                     const int32_t *pinv, int upper, int64_t *cnt) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i <= n; i += warps) {
        if (i == n) { if (lane == 0) cnt[n] = 0; continue; }
        const int64_t r = p[i];
        long long c = 0;
        for (int64_t e = ip[r] + lane; e < ip[r + 1]; e += 32) c += (!upper || pinv[ij[e]] >= i) ? 1 : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        if (lane == 0) cnt[i] = c;
    }
}

__global__ void ord_csr_fill_kernel(int64_t n, const int64_t *ip, const int32_t *ij, const int32_t *x, const int32_t *p,
                                    const int32_t *pinv, int upper, const int64_t *op, int32_t *oj, int32_t *ox) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
        const int64_t r = p[i];
        int64_t base = op[i];
        for (int64_t e0 = ip[r]; e0 < ip[r + 1]; e0 += 32) {
            const int64_t e = e0 + lane;
            bool keep = false;
            int32_t c = 0;
            if (e < ip[r + 1]) {
                c = pinv[ij[e]];
                keep = !upper || c >= i;
            }
            const unsigned bal = __ballot_sync(0xffffffffu, keep);
            if (keep) {
                const int64_t q = base + __popc(bal & ((1u << lane) - 1u));
                oj[q] = c;
                ox[q] = x[e];
            }
            base += __popc(bal);
        }
    }
}

// ---------------------------------------------------------------------------- topological order
// Edges v -> w for the stored entries (v, w), w != v (w an ancestor of v).  Kahn's algorithm
// from the vertices without parents: level 0; a vertex joins level L + 1 when its last parent
// was placed at level L.  Every level is one launch reading its bounds lb[L], lb[L + 1] from
// device memory; a one-thread launch then records where the next level ends.
__global__ void topo_count_kernel(int64_t n, const int64_t *ip, const int32_t *ij, int32_t *remaining,
                                  int32_t *ccount, int32_t *level) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        int c = 0;
        for (int64_t e = ip[v]; e < ip[v + 1]; ++e) {
            const int32_t w = ij[e];
            if (w != (int32_t)v && w >= 0 && w < n) {
                ++c;
                atomicAdd(ccount + w, 1);
            }
        }
        remaining[v] = c;
        level[v] = -1;
    }
}

__global__ void topo_children_kernel(int64_t n, const int64_t *ip, const int32_t *ij, const int64_t *coff,
                                     int32_t *cursor, int32_t *children) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        for (int64_t e = ip[v]; e < ip[v + 1]; ++e) {
            const int32_t w = ij[e];
            if (w != (int32_t)v && w >= 0 && w < n) children[coff[w] + atomicAdd(cursor + w, 1)] = (int32_t)v;
        }
}

__device__ __forceinline__ void topo_append(bool ready, int32_t v, int32_t lvl, int32_t *order, int32_t *tail,
                                            int32_t *level) {
    const unsigned bal = __ballot_sync(0xffffffffu, ready);
    if (!bal) return;
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == 0) base = atomicAdd(tail, __popc(bal));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (ready) {
        order[base + __popc(bal & ((1u << lane) - 1u))] = v;
        level[v] = lvl;
    }
}

__global__ void topo_roots_kernel(int64_t n, const int32_t *remaining, int32_t *order, int32_t *tail, int32_t *level) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t v0 = ((int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; v0 < n; v0 += warps * 32) {
        const int64_t v = v0 + lane;
        topo_append(v < n && remaining[v] == 0, (int32_t)v, 0, order, tail, level);
    }
}

__global__ void topo_expand_kernel(int64_t L, const int64_t *lb, const int64_t *coff, const int32_t *children,
                                   int32_t *remaining, int32_t *order, int32_t *tail, int32_t *level) {
    const int64_t s = lb[L], e = lb[L + 1];
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t k0 = s + ((int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; k0 < e; k0 += warps * 32) {
        const int64_t k = k0 + lane;
        int64_t c0 = 0, c1 = 0;
        if (k < e) {
            const int32_t w = order[k];
            c0 = coff[w];
            c1 = coff[w + 1];
        }
        for (int64_t i = 0; __any_sync(0xffffffffu, c0 + i < c1); ++i) {
            bool ready = false;
            int32_t c = 0;
            if (c0 + i < c1) {
                c = children[c0 + i];
                ready = atomicSub(remaining + c, 1) == 1;
            }
            topo_append(ready, c, (int32_t)(L + 1), order, tail, level);
        }
    }
}

__global__ void topo_close_kernel(int64_t slot, int64_t *lb, const int32_t *tail) {
    if (threadIdx.x == 0 && blockIdx.x == 0) lb[slot] = *tail;
}

// On a cycle: from the least unplaced vertex follow unplaced parents (one always exists) until a
// vertex repeats; that vertex lies on a cycle.  At most n + 1 steps.
__global__ void topo_cycle_kernel(int64_t n, const int64_t *ip, const int32_t *ij, const int32_t *level,
                                  int32_t *seen, int64_t *out) {
    __shared__ int first;
    if (threadIdx.x == 0) first = INT_MAX;
    __syncthreads();
    for (int64_t v = threadIdx.x; v < n; v += blockDim.x)
        if (level[v] < 0) atomicMin(&first, (int)v);
    __syncthreads();
    if (threadIdx.x != 0) return;
    *out = -1;
    if (first == INT_MAX) return;
    int64_t cur = first;
    for (int64_t step = 0; step <= n; ++step) {
        if (seen[cur]) { *out = cur; return; }
        seen[cur] = 1;
        int64_t nxt = -1;
        for (int64_t e = ip[cur]; e < ip[cur + 1]; ++e) {
            const int32_t w = ij[e];
            if (w != (int32_t)cur && w >= 0 && w < n && level[w] < 0) { nxt = w; break; }
        }
        if (nxt < 0) return;
        cur = nxt;
    }
}

__global__ void topo_keys_kernel(int64_t n, const int32_t *level, uint32_t *keys, int32_t *vals) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        keys[v] = 0xffffffffu - (uint32_t)level[v];   // deepest level first
        vals[v] = (int32_t)v;
    }
}

size_t perm_sort_bytes(int64_t n) {
    size_t b = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, b, (unsigned long long *)nullptr, (unsigned long long *)nullptr,
                                    (int32_t *)nullptr, (int32_t *)nullptr, (int)std::max<int64_t>(n, 1));
    return b;
}

}  // namespace
}  // namespace rbg

using namespace rbg;

extern "C" int32_t rbg_ordering_metrics_csr(int64_t n, const int64_t *indptr, const int32_t *indices,
                                            const int32_t *data, int64_t *anc, int32_t *maxrel, int32_t *diag,
                                            rbg_stream_t stream) {
    if (n < 0 || (n > 0 && (!indptr || !anc || !maxrel || !diag))) return RBG_ERR_INVALID;
    if (n == 0) return RBG_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    RBG_CUDA_TRY(cudaMemsetAsync(maxrel, 0, (size_t)n * 4, s));
    note_launches(1);
    ord_metrics_csr_kernel<<<grid_for(n * 32, 256), 256, 0, s>>>(n, indptr, indices, data, anc, maxrel, diag);
    RBG_CUDA_TRY(cudaGetLastError());
    return RBG_OK;
}

extern "C" int32_t rbg_ordering_metrics_dense(int64_t n, const int32_t *A, int64_t lda, int64_t *anc, int32_t *maxrel,
                                              int32_t *diag, rbg_stream_t stream) {
    if (n < 0 || lda < n || (n > 0 && (!A || !anc || !maxrel || !diag))) return RBG_ERR_INVALID;
    if (n == 0) return RBG_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    RBG_CUDA_TRY(cudaMemsetAsync(maxrel, 0, (size_t)n * 4, s));
    note_launches(1);
    ord_metrics_dense_kernel<<<grid_for(n * 32, 256), 256, 0, s>>>(n, A, lda, anc, maxrel, diag);
    RBG_CUDA_TRY(cudaGetLastError());
    return RBG_OK;
}

extern "C" int32_t rbg_canonical_permutation_workspace_bytes(int64_t n, int64_t *bytes) {
    if (!bytes || n < 0 || n >= (1ll << 31) - 1) return RBG_ERR_INVALID;
    const size_t m = (size_t)std::max<int64_t>(n, 1);
    *bytes = (int64_t)(align_up(m * 8, 256) * 2 + align_up(m * 4, 256) + perm_sort_bytes(n) + 256);
    return RBG_OK;
}

extern "C" int32_t rbg_canonical_permutation(int64_t n, const int32_t *label, const int64_t *comp_start,
                                             const int64_t *anc, const int32_t *maxrel, const int32_t *diag,
                                             int32_t *perm, void *workspace, int64_t workspace_bytes,
                                             rbg_stream_t stream) {
    if (n < 0 || n >= (1ll << 31) - 1 || (n > 0 && (!label || !comp_start || !anc || !maxrel || !diag || !perm)))
        return RBG_ERR_INVALID;
    if (n == 0) return RBG_OK;
    int64_t need = 0;
    rbg_canonical_permutation_workspace_bytes(n, &need);
    if (!workspace || workspace_bytes < need) return RBG_ERR_NOMEM;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const size_t m = (size_t)n;
    unsigned char *w = reinterpret_cast<unsigned char *>(workspace);
    unsigned long long *k0 = reinterpret_cast<unsigned long long *>(w);
    unsigned long long *k1 = reinterpret_cast<unsigned long long *>(w + align_up(m * 8, 256));
    int32_t *v1 = reinterpret_cast<int32_t *>(w + 2 * align_up(m * 8, 256));
    void *tmp = w + 2 * align_up(m * 8, 256) + align_up(m * 4, 256);
    size_t tb = perm_sort_bytes(n);
    const int g = grid_for(n, 256);
    note_launches(1);
    ord_iota_kernel<<<g, 256, 0, s>>>(n, perm);
    for (int pass = 0; pass < 3; ++pass) {           // stable passes, least significant key first
        note_launches(1);
        ord_keys_kernel<<<g, 256, 0, s>>>(n, pass, label, comp_start, anc, maxrel, diag, perm, k0);
        size_t t = tb;
        RBG_CUDA_TRY(cub::DeviceRadixSort::SortPairs(tmp, t, k0, k1, perm, v1, (int)n, 0, 64, s));
        RBG_CUDA_TRY(cudaMemcpyAsync(perm, v1, m * 4, cudaMemcpyDeviceToDevice, s));
    }
    RBG_CUDA_TRY(cudaGetLastError());
    return RBG_OK;
}

extern "C" int32_t rbg_permute_dense(int32_t dtype, int64_t n, const void *A, int64_t lda, const int32_t *perm,
                                     void *B, int64_t ldb, int32_t upper, rbg_stream_t stream) {
    if (n < 0 || lda < n || ldb < n || dtype_bytes(dtype) == 0 || (n > 0 && (!A || !perm || !B)) || A == B)
        return RBG_ERR_INVALID;
    if (n == 0) return RBG_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int g = (int)std::min<int64_t>(n, (int64_t)grid_for(n * 256, 256));
    note_launches(1);
    RBG_DISPATCH_DTYPE(dtype, T,
        ord_permute_dense_kernel<T><<<g, 256, 0, s>>>(n, reinterpret_cast<const T *>(A), lda, perm,
                                                      reinterpret_cast<T *>(B), ldb, upper));
    RBG_CUDA_TRY(cudaGetLastError());
    return RBG_OK;
}

extern "C" int32_t rbg_permute_csr_workspace_bytes(int64_t n, int64_t nnz, int64_t *bytes) {
    if (!bytes || n < 0 || nnz < 0 || n >= (1ll << 31) - 1) return RBG_ERR_INVALID;
    const size_t m = (size_t)std::max<int64_t>(n, 1), z = (size_t)std::max<int64_t>(nnz, 1);
    size_t scan = 0, seg = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, scan, (int64_t *)nullptr, (int64_t *)nullptr, (int)(m + 1));
    cub::DeviceSegmentedSort::SortPairs(nullptr, seg, (int32_t *)nullptr, (int32_t *)nullptr, (int32_t *)nullptr,
                                        (int32_t *)nullptr, (int64_t)z, (int64_t)m, (int64_t *)nullptr,
                                        (int64_t *)nullptr);
    *bytes = (int64_t)(align_up(m * 4, 256) + align_up((m + 1) * 8, 256) + 2 * align_up(z * 4, 256) +
                       align_up(std::max(scan, seg), 256));
    return RBG_OK;
}

// Layout of the permute_csr workspace: inverse permutation, row counts, sort buffers, CUB scratch.
static void perm_csr_layout(int64_t n, int64_t nnz, unsigned char *w, int32_t **pinv, int64_t **cnt, int32_t **kj,
                            int32_t **kx, void **tmp, size_t *tmp_bytes) {
    const size_t m = (size_t)std::max<int64_t>(n, 1), z = (size_t)std::max<int64_t>(nnz, 1);
    *pinv = reinterpret_cast<int32_t *>(w);
    w += align_up(m * 4, 256);
    *cnt = reinterpret_cast<int64_t *>(w);
    w += align_up((m + 1) * 8, 256);
    *kj = reinterpret_cast<int32_t *>(w);
    w += align_up(z * 4, 256);
    *kx = reinterpret_cast<int32_t *>(w);
    w += align_up(z * 4, 256);
    *tmp = w;
    size_t scan = 0, seg = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, scan, (int64_t *)nullptr, (int64_t *)nullptr, (int)(m + 1));
    cub::DeviceSegmentedSort::SortPairs(nullptr, seg, (int32_t *)nullptr, (int32_t *)nullptr, (int32_t *)nullptr,
                                        (int32_t *)nullptr, (int64_t)z, (int64_t)m, (int64_t *)nullptr,
                                        (int64_t *)nullptr);
    *tmp_bytes = std::max(scan, seg);
}

extern "C" int32_t rbg_permute_csr_count(const rbg_csr_t *A, const int32_t *perm, int32_t upper, int64_t *indptr_out,
                                         void *workspace, int64_t workspace_bytes, int64_t *nnz_out,
                                         rbg_stream_t stream) {
    if (!A || !perm || !indptr_out || !nnz_out || A->n_rows != A->n_cols || A->n_rows < 0) return RBG_ERR_INVALID;
    const int64_t n = A->n_rows;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int64_t annz = 0;
    if (n > 0) {
        RBG_CUDA_TRY(cudaMemcpyAsync(&annz, A->indptr + n, 8, cudaMemcpyDeviceToHost, s));
        RBG_CUDA_TRY(cudaStreamSynchronize(s));
    }
    int64_t need = 0;
    rbg_permute_csr_workspace_bytes(n, annz, &need);
    if (!workspace || workspace_bytes < need) return RBG_ERR_NOMEM;
    *nnz_out = 0;
    if (n == 0) {
        RBG_CUDA_TRY(cudaMemsetAsync(indptr_out, 0, 8, s));
        return RBG_OK;
    }
    int32_t *pinv, *kj, *kx;
    int64_t *cnt;
    void *tmp;
    size_t tb;
    perm_csr_layout(n, annz, reinterpret_cast<unsigned char *>(workspace), &pinv, &cnt, &kj, &kx, &tmp, &tb);
    note_launches(2);
    ord_inverse_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, perm, pinv);
    ord_csr_count_kernel<<<grid_for((n + 1) * 32, 256), 256, 0, s>>>(n, A->indptr, A->indices, perm, pinv, upper, cnt);
    RBG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(tmp, tb, cnt, indptr_out, (int)(n + 1), s));
    RBG_CUDA_TRY(cudaMemcpyAsync(nnz_out, indptr_out + n, 8, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    return RBG_OK;
}

extern "C" int32_t rbg_permute_csr_fill(const rbg_csr_t *A, const int32_t *perm, int32_t upper,
                                        const int64_t *indptr_out, int32_t *indices_out, int32_t *data_out,
                                        void *workspace, int64_t workspace_bytes, rbg_stream_t stream) {
    if (!A || !perm || !indptr_out || A->n_rows != A->n_cols || A->n_rows < 0) return RBG_ERR_INVALID;
    const int64_t n = A->n_rows;
    if (n == 0) return RBG_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int64_t annz = 0, onnz = 0;
    RBG_CUDA_TRY(cudaMemcpyAsync(&annz, A->indptr + n, 8, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaMemcpyAsync(&onnz, indptr_out + n, 8, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    int64_t need = 0;
    rbg_permute_csr_workspace_bytes(n, annz, &need);
    if (!workspace || workspace_bytes < need) return RBG_ERR_NOMEM;
    if (onnz == 0) return RBG_OK;
    if (!indices_out || !data_out) return RBG_ERR_INVALID;
    int32_t *pinv, *kj, *kx;
    int64_t *cnt;
    void *tmp;
    size_t tb;
    perm_csr_layout(n, annz, reinterpret_cast<unsigned char *>(workspace), &pinv, &cnt, &kj, &kx, &tmp, &tb);
    note_launches(1);
    ord_csr_fill_kernel<<<grid_for(n * 32, 256), 256, 0, s>>>(n, A->indptr, A->indices,
                                                              reinterpret_cast<const int32_t *>(A->data), perm, pinv,
                                                              upper, indptr_out, kj, kx);
    RBG_CUDA_TRY(cub::DeviceSegmentedSort::SortPairs(tmp, tb, kj, indices_out, kx, data_out, onnz, n, indptr_out,
                                                     indptr_out + 1, s));
    RBG_CUDA_TRY(cudaGetLastError());
    return RBG_OK;
}

// ---------------------------------------------------------------------------- topological order
namespace rbg {
namespace {
struct TopoWs {
    int32_t *remaining, *ccount, *cursor, *children, *order, *level, *tail, *seen, *vals;
    uint32_t *keys, *keys2;
    int64_t *coff, *lb, *cyc;
    void *tmp;
    size_t tmp_bytes;
};
size_t topo_layout(int64_t n, int64_t nnz, unsigned char *base, TopoWs *w) {
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o = align_up(o + bytes, 256); return base ? base + at : nullptr; };
    const size_t m = (size_t)std::max<int64_t>(n, 1), ni = (m + 1) * 4, nl = (m + 2) * 8;
    unsigned char *p;
    p = take(ni); if (w) w->remaining = (int32_t *)p;
    p = take(ni); if (w) w->ccount = (int32_t *)p;
    p = take(ni); if (w) w->cursor = (int32_t *)p;
    p = take((size_t)std::max<int64_t>(nnz, 1) * 4); if (w) w->children = (int32_t *)p;
    p = take(ni); if (w) w->order = (int32_t *)p;
    p = take(ni); if (w) w->level = (int32_t *)p;
    p = take(ni); if (w) w->seen = (int32_t *)p;
    p = take(ni); if (w) w->vals = (int32_t *)p;
    p = take(ni); if (w) w->keys = (uint32_t *)p;
    p = take(ni); if (w) w->keys2 = (uint32_t *)p;
    p = take(nl); if (w) w->coff = (int64_t *)p;
    p = take(nl); if (w) w->lb = (int64_t *)p;
    p = take(64); if (w) { w->tail = (int32_t *)p; w->cyc = (int64_t *)(p + 8); }
    size_t a = 0, b = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, a, (int32_t *)nullptr, (int64_t *)nullptr, (int)(m + 1));
    cub::DeviceRadixSort::SortPairs(nullptr, b, (uint32_t *)nullptr, (uint32_t *)nullptr, (int32_t *)nullptr,
                                    (int32_t *)nullptr, (int)m);
    const size_t tb = std::max(a, b);
    p = take(tb); if (w) { w->tmp = p; w->tmp_bytes = tb; }
    return o;
}
}  // namespace
}  // namespace rbg

extern "C" int32_t rbg_topological_workspace_bytes(int64_t n, int64_t nnz, int64_t *bytes) {
    if (!bytes || n < 0 || nnz < 0 || n >= (1ll << 31) - 1) return RBG_ERR_INVALID;
    *bytes = (int64_t)topo_layout(n, nnz, nullptr, nullptr);
    return RBG_OK;
}

extern "C" int32_t rbg_topological_order(const rbg_csr_t *A, void *workspace, int64_t workspace_bytes, int32_t *perm,
                                         int64_t *levels, int64_t *cycle_vertex, rbg_stream_t stream) {
    if (!A || !levels || !cycle_vertex || A->n_rows != A->n_cols || A->n_rows < 0 || (A->n_rows > 0 && !perm))
        return RBG_ERR_INVALID;
    const int64_t n = A->n_rows;
    *levels = 0;
    *cycle_vertex = -1;
    if (n == 0) return RBG_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int64_t annz = 0;
    RBG_CUDA_TRY(cudaMemcpyAsync(&annz, A->indptr + n, 8, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    if (!workspace || workspace_bytes < (int64_t)topo_layout(n, annz, nullptr, nullptr)) return RBG_ERR_NOMEM;
    TopoWs w;
    topo_layout(n, annz, reinterpret_cast<unsigned char *>(workspace), &w);
    const int g = grid_for(n, 256);
    RBG_CUDA_TRY(cudaMemsetAsync(w.ccount, 0, (size_t)(n + 1) * 4, s));
    RBG_CUDA_TRY(cudaMemsetAsync(w.cursor, 0, (size_t)(n + 1) * 4, s));
    RBG_CUDA_TRY(cudaMemsetAsync(w.seen, 0, (size_t)(n + 1) * 4, s));
    RBG_CUDA_TRY(cudaMemsetAsync(w.tail, 0, 64, s));
    RBG_CUDA_TRY(cudaMemsetAsync(w.lb, 0, 8, s));
    note_launches(4);
    topo_count_kernel<<<g, 256, 0, s>>>(n, A->indptr, A->indices, w.remaining, w.ccount, w.level);
    size_t tb = w.tmp_bytes;
    RBG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(w.tmp, tb, w.ccount, w.coff, (int)(n + 1), s));
    topo_children_kernel<<<g, 256, 0, s>>>(n, A->indptr, A->indices, w.coff, w.cursor, w.children);
    topo_roots_kernel<<<g, 256, 0, s>>>(n, w.remaining, w.order, w.tail, w.level);
    topo_close_kernel<<<1, 32, 0, s>>>(1, w.lb, w.tail);
    int64_t L = 0;
    const int64_t chunk = 8;
    const int eg = grid_for(n, 256);
    while (true) {
        const int64_t Lend = std::min<int64_t>(L + chunk, n);
        for (; L < Lend; ++L) {
            note_launches(2);
            topo_expand_kernel<<<eg, 256, 0, s>>>(L, w.lb, w.coff, w.children, w.remaining, w.order, w.tail, w.level);
            topo_close_kernel<<<1, 32, 0, s>>>(L + 2, w.lb, w.tail);
        }
        RBG_CUDA_TRY(cudaGetLastError());
        int64_t range[2] = {0, 0};
        RBG_CUDA_TRY(cudaMemcpyAsync(range, w.lb + L, 16, cudaMemcpyDeviceToHost, s));
        RBG_CUDA_TRY(cudaStreamSynchronize(s));
        if (range[1] <= range[0] || L >= n) break;
    }
    int32_t placed = 0;
    RBG_CUDA_TRY(cudaMemcpyAsync(&placed, w.tail, 4, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    if (placed < n) {
        note_launches(1);
        topo_cycle_kernel<<<1, 256, 0, s>>>(n, A->indptr, A->indices, w.level, w.seen, w.cyc);
        RBG_CUDA_TRY(cudaMemcpyAsync(cycle_vertex, w.cyc, 8, cudaMemcpyDeviceToHost, s));
        RBG_CUDA_TRY(cudaStreamSynchronize(s));
        return RBG_ERR_CYCLE;
    }
    // levels: the last non-empty one
    std::vector<int64_t> lbh((size_t)std::min<int64_t>(L + 2, n + 2));
    RBG_CUDA_TRY(cudaMemcpyAsync(lbh.data(), w.lb, lbh.size() * 8, cudaMemcpyDeviceToHost, s));
    note_launches(1);
    topo_keys_kernel<<<g, 256, 0, s>>>(n, w.level, w.keys, w.vals);
    tb = w.tmp_bytes;
    RBG_CUDA_TRY(cub::DeviceRadixSort::SortPairs(w.tmp, tb, w.keys, w.keys2, w.vals, perm, (int)n, 0, 32, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    int64_t lv = 0;
    for (size_t k = 0; k + 1 < lbh.size(); ++k)
        if (lbh[k + 1] > lbh[k]) lv = (int64_t)k + 1;
    *levels = lv;
    return RBG_OK;
}

namespace rbg {
namespace {
__global__ void topo_upper_kernel(int64_t n, const int64_t *ip, const int32_t *ij, int strict, int32_t *bad) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        for (int64_t e = ip[i]; e < ip[i + 1]; ++e) {
            const int64_t c = ij[e];
            if (strict ? c <= i : c < i) { *bad = 1; break; }
        }
}
}  // namespace
}  // namespace rbg

extern "C" int32_t rbg_is_upper_triangular_csr(const rbg_csr_t *A, int32_t strict, int32_t *result, void *workspace,
                                               int64_t workspace_bytes, rbg_stream_t stream) {
    if (!A || !result || A->n_rows < 0) return RBG_ERR_INVALID;
    *result = 1;
    const int64_t n = A->n_rows;
    if (n == 0) return RBG_OK;
    if (!workspace || workspace_bytes < 4) return RBG_ERR_NOMEM;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int32_t *bad = reinterpret_cast<int32_t *>(workspace);
    RBG_CUDA_TRY(cudaMemsetAsync(bad, 0, 4, s));
    note_launches(1);
    topo_upper_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, A->indptr, A->indices, strict, bad);
    int32_t h = 0;
    RBG_CUDA_TRY(cudaMemcpyAsync(&h, bad, 4, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    *result = h ? 0 : 1;
    return RBG_OK;
}

// ---------------------------------------------------------------------------- row/column remap
// Output row row_map[k] (-1: dropped) receives input row k with its columns mapped through
// col_map (-1: dropped), columns ascending: extract_submatrix and merge_component_matrices
// (redblackgraph/sparse/csgraph/_components.pyx:178-323).  Each output row receives at most one
// input row.
namespace rbg {
namespace {
__global__ void remap_count_kernel(int64_t n_in, const int64_t *ip, const int32_t *ij, const int32_t *row_map,
                                   const int32_t *col_map, int64_t *cnt) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t k = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); k < n_in; k += warps) {
        const int32_t r = row_map[k];
        if (r < 0) continue;
        long long c = 0;
        for (int64_t e = ip[k] + lane; e < ip[k + 1]; e += 32) c += col_map[ij[e]] >= 0 ? 1 : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        if (lane == 0) cnt[r] = c;
    }
}

__global__ void remap_fill_kernel(int64_t n_in, const int64_t *ip, const int32_t *ij, const int32_t *x,
                                  const int32_t *row_map, const int32_t *col_map, const int64_t *op, int32_t *oj,
                                  int32_t *ox) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t k = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); k < n_in; k += warps) {
        const int32_t r = row_map[k];
        if (r < 0) continue;
        int64_t base = op[r];
        for (int64_t e0 = ip[k]; e0 < ip[k + 1]; e0 += 32) {
            const int64_t e = e0 + lane;
            int32_t c = -1;
            if (e < ip[k + 1]) c = col_map[ij[e]];
            const unsigned bal = __ballot_sync(0xffffffffu, c >= 0);
            if (c >= 0) {
                const int64_t q = base + __popc(bal & ((1u << lane) - 1u));
                oj[q] = c;
                ox[q] = x[e];
            }
            base += __popc(bal);
        }
    }
}

size_t remap_tmp_bytes(int64_t n_out, int64_t nnz) {
    size_t scan = 0, seg = 0;
    const size_t m = (size_t)std::max<int64_t>(n_out, 1), z = (size_t)std::max<int64_t>(nnz, 1);
    cub::DeviceScan::ExclusiveSum(nullptr, scan, (int64_t *)nullptr, (int64_t *)nullptr, (int)(m + 1));
    cub::DeviceSegmentedSort::SortPairs(nullptr, seg, (int32_t *)nullptr, (int32_t *)nullptr, (int32_t *)nullptr,
                                        (int32_t *)nullptr, (int64_t)z, (int64_t)m, (int64_t *)nullptr,
                                        (int64_t *)nullptr);
    return std::max(scan, seg);
}
}  // namespace
}  // namespace rbg

extern "C" int32_t rbg_csr_remap_workspace_bytes(int64_t n_out, int64_t nnz, int64_t *bytes) {
    if (!bytes || n_out < 0 || nnz < 0) return RBG_ERR_INVALID;
    const size_t m = (size_t)std::max<int64_t>(n_out, 1), z = (size_t)std::max<int64_t>(nnz, 1);
    *bytes = (int64_t)(align_up((m + 1) * 8, 256) + 2 * align_up(z * 4, 256) + align_up(remap_tmp_bytes(n_out, nnz), 256));
    return RBG_OK;
}

extern "C" int32_t rbg_csr_remap(const rbg_csr_t *A, const int32_t *row_map, const int32_t *col_map, int64_t n_out,
                                 int64_t *indptr_out, int32_t *indices_out, int32_t *data_out, int64_t capacity,
                                 void *workspace, int64_t workspace_bytes, int64_t *nnz_out, rbg_stream_t stream) {
    if (!A || !row_map || !col_map || !indptr_out || !nnz_out || A->n_rows < 0 || n_out < 0) return RBG_ERR_INVALID;
    const int64_t n_in = A->n_rows;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int64_t annz = 0;
    if (n_in > 0) {
        RBG_CUDA_TRY(cudaMemcpyAsync(&annz, A->indptr + n_in, 8, cudaMemcpyDeviceToHost, s));
        RBG_CUDA_TRY(cudaStreamSynchronize(s));
    }
    int64_t need = 0;
    rbg_csr_remap_workspace_bytes(n_out, annz, &need);
    if (!workspace || workspace_bytes < need) return RBG_ERR_NOMEM;
    unsigned char *w = reinterpret_cast<unsigned char *>(workspace);
    const size_t m = (size_t)std::max<int64_t>(n_out, 1), z = (size_t)std::max<int64_t>(annz, 1);
    int64_t *cnt = reinterpret_cast<int64_t *>(w);
    int32_t *kj = reinterpret_cast<int32_t *>(w + align_up((m + 1) * 8, 256));
    int32_t *kx = reinterpret_cast<int32_t *>(w + align_up((m + 1) * 8, 256) + align_up(z * 4, 256));
    void *tmp = w + align_up((m + 1) * 8, 256) + 2 * align_up(z * 4, 256);
    size_t tb = remap_tmp_bytes(n_out, annz);
    RBG_CUDA_TRY(cudaMemsetAsync(cnt, 0, (m + 1) * 8, s));
    if (n_in > 0) {
        note_launches(1);
        remap_count_kernel<<<grid_for(n_in * 32, 256), 256, 0, s>>>(n_in, A->indptr, A->indices, row_map, col_map,
                                                                     cnt);
    }
    RBG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(tmp, tb, cnt, indptr_out, (int)(n_out + 1), s));
    int64_t total = 0;
    RBG_CUDA_TRY(cudaMemcpyAsync(&total, indptr_out + n_out, 8, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    *nnz_out = total;
    if (total > capacity) return RBG_ERR_CAPACITY;
    if (total == 0) return RBG_OK;
    if (!indices_out || !data_out) return RBG_ERR_INVALID;
    note_launches(1);
    remap_fill_kernel<<<grid_for(n_in * 32, 256), 256, 0, s>>>(n_in, A->indptr, A->indices,
                                                                reinterpret_cast<const int32_t *>(A->data), row_map,
                                                                col_map, indptr_out, kj, kx);
    tb = remap_tmp_bytes(n_out, annz);
    RBG_CUDA_TRY(cub::DeviceSegmentedSort::SortPairs(tmp, tb, kj, indices_out, kx, data_out, total, n_out, indptr_out,
                                                     indptr_out + 1, s));
    RBG_CUDA_TRY(cudaGetLastError());
    return RBG_OK;
}
