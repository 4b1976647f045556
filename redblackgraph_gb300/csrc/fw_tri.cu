// fw_tri.cu -- dense closure of matrices numbered in a topological order, by the DAG closure.
//
// The reference's warshall (redblackgraph/core/src/redblackgraph/warshall.c.in:88-106) runs the
// sequential loop  for k, i, j: W(i, j) = W(i, j) (+) W(i, k) (x) W(k, j)  over the whole matrix.
// When every off-diagonal entry lies below the diagonal (an edge i -> k only for k < i, as in a
// pedigree whose vertices are numbered oldest first), a path from i to k passes only vertices
// numbered above k, none of which an earlier step has used: before step k, W(i, k) is still the
// input A(i, k), while row k is already final (every path from k descends through vertices
// below k).  Step k therefore adds A(i, k) (x) C(k, .) to the rows of k's children, and the
// closure is the DAG recurrence  C(i, .) = A(i, .) (+) sum over parents k of A(i, k) (x) C(k, .)
// that rbg_dag_closure computes level by level.  Above the diagonal (edges to higher numbers)
// it is the mirror image: before step k, W(i, k) = C(i, k) and W(k, j) = A(k, j).
//
// In the clean regime (off-diagonal values 0 or >= 2, diagonal in {-1, 0, 1}) products with the
// diagonal change nothing and a cell only decreases once it holds a value, so the largest value
// the loop ever writes -- the diameter's source -- is, per cell, its first value: A(i, j), else
// the product of the first step that reaches the cell.  Below the diagonal that is the smallest
// parent k of i with j in C(k); above it, the smallest k in C(i) with j a parent of k.  A
// product whose most significant bit may reach the top bit of the 32-bit value sends the
// matrix to the blocked kernels (which report the reference's overflow or wrap), as does
// anything outside the clean regime, a row of more than TRI_CAP entries or n > 8192.
//
// Pipeline (one call): scan the dense rows (clean-regime test, which side of the diagonal, up
// to TRI_CAP off-diagonal entries per row) -> CSR of the candidate matrices with batch-global
// row numbers -> rbg_dag_closure -> per-row statistics (largest product MSB, largest
// first-value MSB) -> the dense rows of the accepted matrices written from the closure rows.
#include <cuda_runtime.h>
#include <cub/cub.cuh>
#include <string.h>
#include <algorithm>
#include <mutex>
#include <vector>
#include "rbg_internal.cuh"
#include "dag_rows.cuh"

namespace rbg {
namespace {

constexpr int TRI_ROWS = 8;                  // rows per CTA, one warp each
constexpr int TRI_THREADS = 32 * TRI_ROWS;
constexpr int TRI_CAP = 16;                  // off-diagonal entries per row the scan keeps
constexpr int64_t TRI_MAX_N = DAG_MAX_N;     // rows of a matrix on this path (bitmap size)
constexpr int TRI_BM_WORDS = (int)(TRI_MAX_N / 32);
constexpr unsigned TF_UNCLEAN = 1u, TF_BELOW = 2u, TF_ABOVE = 4u, TF_WIDE = 8u;
constexpr int KIND_NONE = DAG_KIND_NONE, KIND_BELOW = DAG_KIND_BELOW, KIND_ABOVE = DAG_KIND_ABOVE;
constexpr int TRI_TOP = DAG_TOP_MSB;         // lbits - 1 for 32-bit values

struct TriComp {
    int64_t n, in_off, out_off, row_base;    // row_base: first batch-global row
};

__device__ __forceinline__ int tri_find(const int64_t *__restrict__ prefix, int count, int64_t cta) {
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(prefix + mid) <= cta) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Off-diagonal entries of four consecutive columns j0 .. j0 + 3 held by each lane (m of them
// valid): clean-regime flags, and the nonzeros appended to the row's slots in column order.
// Column numbers fit 32 bits (n <= 8192 on this path).
__device__ __forceinline__ void tri_take(int32_t (&v)[4], int j0, int m, int i, int lane, int64_t g,
                                         int32_t *__restrict__ slot_col, int32_t *__restrict__ slot_val,
                                         unsigned &flags, int &cnt) {
    int c4 = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int j = j0 + k;
        if (k >= m) {
            v[k] = 0;
        } else if (j == i) {
            if (!(v[k] == 0 || v[k] == 1 || v[k] == -1)) flags |= TF_UNCLEAN;
            v[k] = 0;                        // the diagonal is not an edge
        } else if (v[k] != 0) {
            if (v[k] == 1 || v[k] < 0) flags |= TF_UNCLEAN;
            flags |= j < i ? TF_BELOW : TF_ABOVE;
            ++c4;
        }
    }
    if (!__any_sync(0xffffffffu, c4 != 0)) return;
    int x = c4;                              // inclusive prefix over the lanes
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    int pos = cnt + x - c4;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (v[k] != 0) {
            if (pos < TRI_CAP) {
                slot_col[g * TRI_CAP + pos] = j0 + k;
                slot_val[g * TRI_CAP + pos] = v[k];
            }
            ++pos;
        }
    }
    cnt += __shfl_sync(0xffffffffu, x, 31);
}

// One warp per row: clean-regime test, side of the diagonal, the row's off-diagonal entries in
// column order into its TRI_CAP slots (the count may exceed TRI_CAP: then only flagged).  The
// row is read as 16-byte vectors from its first 16-byte boundary (scalar head and tail), four
// vectors per lane in flight; a vector of zeros (the common case) costs one vote.
__global__ void __launch_bounds__(TRI_THREADS, 5)
tri_scan_kernel(const int32_t *__restrict__ in, const TriComp *__restrict__ comps,
                const int64_t *__restrict__ pre, int count, int32_t *__restrict__ slot_col,
                int32_t *__restrict__ slot_val, int32_t *__restrict__ row_cnt, int32_t *__restrict__ row_comp,
                unsigned *__restrict__ cflags) {
    const int ci = tri_find(pre, count, blockIdx.x);
    const TriComp c = comps[ci];
    const int i = (int)(((int64_t)blockIdx.x - pre[ci]) * TRI_ROWS) + (threadIdx.x >> 5);
    if (i >= c.n) return;                    // warp-uniform
    const int lane = threadIdx.x & 31;
    const int n = (int)c.n;
    const int64_t g = c.row_base + i;
    const int32_t *row = in + c.in_off + (int64_t)i * n;
    const int lead = (int)(((16 - ((uintptr_t)row & 15)) & 15) / 4);   // to the first boundary
    const int head = lead < n ? lead : n;
    const int nv = (n - head) / 4;           // 16-byte vectors after the head
    const int tail = n - head - 4 * nv;
    unsigned flags = 0;
    int cnt = 0;
    int32_t v[4];
    if (head) {                              // columns 0 .. head - 1, one per lane
        v[0] = lane < head ? row[lane] : 0;
        tri_take(v, lane, lane < head ? 1 : 0, i, lane, g, slot_col, slot_val, flags, cnt);
    }
    // vectors s0 + 32 u + lane (u = 0..3), taken in column order (u ascending)
    for (int s0 = 0; s0 < nv; s0 += 128) {
        int4 x[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int q = s0 + 32 * u + lane;
            x[u] = q < nv ? *reinterpret_cast<const int4 *>(row + head + 4 * q) : make_int4(0, 0, 0, 0);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int q = s0 + 32 * u + lane;
            const int j0 = head + 4 * q;
            // all-zero vectors (a zero diagonal included) leave nothing to take
            if (__any_sync(0xffffffffu, (x[u].x | x[u].y | x[u].z | x[u].w) != 0)) {
                v[0] = x[u].x; v[1] = x[u].y; v[2] = x[u].z; v[3] = x[u].w;
                tri_take(v, j0, q < nv ? 4 : 0, i, lane, g, slot_col, slot_val, flags, cnt);
            }
        }
    }
    if (tail) {
        const int j = head + 4 * nv + lane;
        v[0] = lane < tail ? row[j] : 0;
        tri_take(v, j, lane < tail ? 1 : 0, i, lane, g, slot_col, slot_val, flags, cnt);
    }
    if (cnt > TRI_CAP) flags |= TF_WIDE;
    flags = __reduce_or_sync(0xffffffffu, flags);
    if (lane == 0) {
        row_cnt[g] = cnt;
        row_comp[g] = ci;
        if (flags) atomicOr(cflags + ci, flags);
    }
}

// which matrices are candidates, from the scan's flags (decided on the device: no host round
// trip before the CSR is built)
__global__ void tri_kind_kernel(int count, const TriComp *__restrict__ comps, const unsigned *__restrict__ cflags,
                                int32_t *__restrict__ ckind) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const unsigned f = cflags[i];
        int k = KIND_NONE;
        if (comps[i].n > 0 && !(f & (TF_UNCLEAN | TF_WIDE)) && !((f & TF_BELOW) && (f & TF_ABOVE)))
            k = (f & TF_ABOVE) ? KIND_ABOVE : KIND_BELOW;
        ckind[i] = k;
    }
}

// entries of each row in the CSR of the candidate matrices (rows of other matrices empty)
__global__ void tri_count_kernel(int64_t R, const int32_t *__restrict__ row_cnt, const int32_t *__restrict__ row_comp,
                                 const int32_t *__restrict__ ckind, int64_t *__restrict__ cnt64) {
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < R; g += (int64_t)gridDim.x * blockDim.x)
        cnt64[g] = ckind[row_comp[g]] != KIND_NONE ? row_cnt[g] : 0;
}

__global__ void tri_csr_fill_kernel(int64_t R, const int32_t *__restrict__ row_comp, const int32_t *__restrict__ ckind,
                                    const TriComp *__restrict__ comps, const int64_t *__restrict__ indptr,
                                    const int32_t *__restrict__ slot_col, const int32_t *__restrict__ slot_val,
                                    int32_t *__restrict__ a_col, int32_t *__restrict__ a_val) {
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < R; g += (int64_t)gridDim.x * blockDim.x) {
        const int ci = row_comp[g];
        if (ckind[ci] == KIND_NONE) continue;
        const int32_t base = (int32_t)comps[ci].row_base;
        const int64_t o = indptr[g];
        const int m = (int)(indptr[g + 1] - o);
        for (int p = 0; p < m; ++p) {
            a_col[o + p] = base + slot_col[g * TRI_CAP + p];
            a_val[o + p] = slot_val[g * TRI_CAP + p];
        }
    }
}

// One warp per row of a candidate matrix: the row statistics of dag_rows.cuh, reduced per
// matrix (largest product MSB, largest first-value MSB, products).
__global__ void __launch_bounds__(TRI_THREADS, 8)
tri_stats_kernel(int64_t R, const int32_t *__restrict__ row_comp, const int32_t *__restrict__ ckind,
                 const TriComp *__restrict__ comps, const int64_t *__restrict__ indptr,
                 const int32_t *__restrict__ a_col, const int32_t *__restrict__ a_val,
                 const int64_t *__restrict__ row_off, const int32_t *__restrict__ row_len,
                 const int32_t *__restrict__ p_col, const int32_t *__restrict__ p_val, int *__restrict__ cam,
                 int *__restrict__ cfm, unsigned long long *__restrict__ cprod) {
    __shared__ unsigned bm_all[TRI_ROWS][TRI_BM_WORDS];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * TRI_ROWS;
    for (int64_t g = (int64_t)blockIdx.x * TRI_ROWS + w; g < R; g += warps) {
        const int ci = row_comp[g];
        const int kind = ckind[ci];
        if (kind == KIND_NONE) continue;     // warp-uniform
        const int32_t base = (int32_t)comps[ci].row_base;
        const int words = (int)((comps[ci].n + 31) >> 5);
        int am = -1, fm = -1;
        unsigned long long prods = 0;
        dag_row_stats(bm_all[w], words, kind, g, indptr, a_col, a_val,
                      [&](int64_t r, int64_t &off, int &len) { off = row_off[r]; len = row_len[r]; },
                      p_col, p_val, [&](int32_t col) { return col - base; }, lane, am, fm, prods);
        am = __reduce_max_sync(0xffffffffu, am);
        fm = __reduce_max_sync(0xffffffffu, fm);
        if (lane == 0) {
            if (am >= 0) atomicMax(cam + ci, am);
            if (fm >= 0) atomicMax(cfm + ci, fm);
            if (prods) atomicAdd(cprod + ci, prods);
        }
    }
}

constexpr int TRI_SEG = 512;                 // columns per shared-memory segment of a row

// One warp per row of an accepted matrix.  Out of place, the whole dense row is written in
// segments of TRI_SEG columns built in shared memory (zeros, the closure row's entries, the
// diagonal) and stored as full 16-byte vectors on the row's 16-byte grid, so no DRAM line is
// written partially; in place, only the closure's entries (the other cells already hold the
// result).  The row statistics are recorded when asked for.
__global__ void __launch_bounds__(TRI_THREADS)
tri_write_kernel(const int32_t *__restrict__ in, int32_t *__restrict__ out, const TriComp *__restrict__ comps,
                 const int64_t *__restrict__ pre, int count, const int32_t *__restrict__ ckind,
                 const int *__restrict__ cam,
                 const int64_t *__restrict__ row_off, const int32_t *__restrict__ row_len,
                 const int32_t *__restrict__ p_col, const int32_t *__restrict__ p_val, RowStats rs) {
    __shared__ __align__(16) int32_t seg_all[TRI_ROWS][TRI_SEG];
    const int ci = tri_find(pre, count, blockIdx.x);
    if (ckind[ci] == KIND_NONE || cam[ci] >= TRI_TOP) return;   // not accepted (block-uniform)
    const TriComp c = comps[ci];
    const int i = (int)(((int64_t)blockIdx.x - pre[ci]) * TRI_ROWS) + (threadIdx.x >> 5);
    if (i >= c.n) return;                    // warp-uniform
    const int lane = threadIdx.x & 31;
    const int n = (int)c.n;
    const int64_t g = c.row_base + i;
    const int32_t *rin = in + c.in_off + (int64_t)i * n;
    int32_t *rout = out + c.out_off + (int64_t)i * n;
    const int32_t diag = rin[i];
    const int64_t c0 = row_off[g];
    const int clen = row_len[g];
    const int32_t base = (int32_t)c.row_base;
    // chunk masks of the row (n <= 8192: at most four 64-bit words), held in registers
    unsigned long long w0 = 0, w1 = 0, w2 = 0, w3 = 0;
    auto mark = [&](int chunk) {
        const unsigned long long bit = 1ull << (chunk & 63);
        const int t = chunk >> 6;
        w0 |= t == 0 ? bit : 0ull;
        w1 |= t == 1 ? bit : 0ull;
        w2 |= t == 2 ? bit : 0ull;
        w3 |= t == 3 ? bit : 0ull;
    };
    int mx = 0;
    if (rin == rout) {
        for (int q = lane; q < clen; q += 32) {
            const int j = p_col[c0 + q] - base;
            const int32_t v = p_val[c0 + q];
            rout[j] = v;
            mx = max(mx, v);
            mark(j >> 5);
        }
    } else {
        int32_t *seg = seg_all[threadIdx.x >> 5];
        // column j sits at j' = j + shift on the 16-byte grid; segment s0 holds j' in [s0, s0 + TRI_SEG)
        const int shift = (int)(((uintptr_t)rout & 15) >> 2);
        int e = 0;                           // first closure entry not yet placed (warp-uniform)
        for (int s0 = 0; s0 < n + shift; s0 += TRI_SEG) {
            for (int t = lane; t < TRI_SEG / 4; t += 32) reinterpret_cast<int4 *>(seg)[t] = make_int4(0, 0, 0, 0);
            __syncwarp();
            const int lim = s0 + TRI_SEG - shift;        // entries with j < lim belong to this segment
            for (;;) {                                   // batches of 32 entries, ascending
                const int q = e + lane;
                int j = INT_MAX;
                int32_t v = 0;
                if (q < clen) {
                    j = p_col[c0 + q] - base;
                    v = p_val[c0 + q];
                }
                const bool here = j < lim;
                if (here) {
                    seg[j + shift - s0] = v;
                    mx = max(mx, v);
                    mark(j >> 5);
                }
                const unsigned bal = __ballot_sync(0xffffffffu, here);
                e += __popc(bal);
                if (bal != 0xffffffffu) break;
            }
            if (lane == 0 && i + shift >= s0 && i + shift < s0 + TRI_SEG) seg[i + shift - s0] = diag;
            __syncwarp();
            for (int t = lane; t < TRI_SEG / 4; t += 32) {
                const int j0 = s0 + 4 * t - shift;
                if (j0 >= n) break;
                const int4 z = reinterpret_cast<const int4 *>(seg)[t];
                if (j0 >= 0 && j0 + 4 <= n) {
                    *reinterpret_cast<int4 *>(rout + j0) = z;
                } else {                                 // the row's ragged ends
                    const int zz[4] = {z.x, z.y, z.z, z.w};
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (j0 + k >= 0 && j0 + k < n) rout[j0 + k] = zz[k];
                }
            }
            __syncwarp();                                // before the next segment is zeroed
        }
    }
    if (rs.row_count) {
        if (lane == 0 && diag != 0) {
            mark(i >> 5);
            mx = max(mx, diag);
        }
        auto orw = [](unsigned long long x) {
            const unsigned lo = __reduce_or_sync(0xffffffffu, (unsigned)x);
            const unsigned hi = __reduce_or_sync(0xffffffffu, (unsigned)(x >> 32));
            return ((unsigned long long)hi << 32) | lo;
        };
        const unsigned long long wd[4] = {orw(w0), orw(w1), orw(w2), orw(w3)};
        mx = __reduce_max_sync(0xffffffffu, mx);
        if (lane == 0) {
            const int64_t at = rs.row_base[ci] + i;
            rs.row_count[rs.row_id ? (int64_t)rs.row_id[at] : at] = clen + (diag != 0 ? 1 : 0);
            if (rs.chunk_mask) {
                const int64_t words = (n + 2047) / 2048;
                unsigned long long *mrow = rs.chunk_mask + (c.in_off + 2047) / 2048 + rs.row_base[ci] + ci +
                                           (int64_t)i * words;
#pragma unroll
                for (int t = 0; t < 4; ++t)
                    if (t < words) mrow[t] = wd[t];
            }
            if (rs.comp_max && mx > 0) atomicMax(rs.comp_max + ci, mx);
        }
    }
}

// Device scratch kept between calls (grown when a batch needs more; one call at a time).
struct TriScratch {
    unsigned char *p = nullptr;
    size_t cap = 0;
    int device = -1;                         // the device the buffer lives on
};
std::mutex g_tri_mu;
TriScratch g_tri_a, g_tri_b;
// the matrix table and CTA prefix last uploaded into g_tri_a (a batch closed again skips the copy)
std::vector<TriComp> g_tri_last_comps;
const unsigned char *g_tri_last_buf = nullptr;

// A buffer on another device than the calling thread's current one is freed and allocated
// again on the current device (a process may drive several GPUs, one at a time per call).
int tri_reserve(TriScratch &s, size_t bytes, cudaStream_t st) {
    int dev = 0;
    RBG_CUDA_TRY(cudaGetDevice(&dev));
    if (bytes <= s.cap && dev == s.device) return RBG_OK;
    RBG_CUDA_TRY(cudaStreamSynchronize(st));
    if (s.p) {                               // freed on its own device, after its work
        if (s.device != dev) RBG_CUDA_TRY(cudaSetDevice(s.device));
        RBG_CUDA_TRY(cudaDeviceSynchronize());
        cudaFree(s.p);
        if (s.device != dev) RBG_CUDA_TRY(cudaSetDevice(dev));
    }
    s.p = nullptr;
    s.cap = 0;
    s.device = -1;
    g_tri_last_buf = nullptr;
    const size_t want = bytes + bytes / 4;
    RBG_CUDA_TRY(cudaMalloc(reinterpret_cast<void **>(&s.p), want));
    s.cap = want;
    s.device = dev;
    return RBG_OK;
}

struct Carve {
    unsigned char *p;
    size_t off = 0;
    template <typename X> X *take(size_t n) {
        off = align_up(off, 256);
        X *r = reinterpret_cast<X *>(p + off);
        off += n * sizeof(X);
        return r;
    }
};

}  // namespace

int tri_batch(int64_t count, const int64_t *sizes, const int64_t *offsets, const int32_t *in, int32_t *out,
              rbg_result_t *results, char *closed, cudaStream_t s, const RowStats &rs) {
    if (count <= 0 || count > INT32_MAX) return RBG_OK;
    std::vector<TriComp> hc((size_t)count);
    std::vector<int64_t> pre((size_t)count + 1, 0);
    int64_t R = 0;
    for (int64_t i = 0; i < count; ++i) {
        const int64_t n = (sizes[i] > 0 && sizes[i] <= TRI_MAX_N) ? sizes[i] : 0;
        hc[(size_t)i] = TriComp{n, offsets[i], offsets[i], R};
        R += n;
        pre[(size_t)i + 1] = pre[(size_t)i] + (n + TRI_ROWS - 1) / TRI_ROWS;
    }
    if (R == 0 || R > INT32_MAX) return RBG_OK;
    std::lock_guard<std::mutex> lk(g_tri_mu);
    size_t scan_tmp = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, scan_tmp, (int64_t *)nullptr, (int64_t *)nullptr, (int)(R + 1));
    const size_t C = (size_t)count, NR = (size_t)R;
    auto layout = [&](Carve &cv, TriComp *&dc, int64_t *&dpre, unsigned *&cflags, int32_t *&ckind,
                      int *&cam, int *&cfm, unsigned long long *&cprod, int32_t *&row_cnt,
                      int32_t *&row_comp, int32_t *&slot_col, int32_t *&slot_val, int64_t *&indptr, void *&tmp,
                      int32_t *&a_col, int32_t *&a_val) {
        dc = cv.take<TriComp>(C);
        dpre = cv.take<int64_t>(C + 1);
        cflags = cv.take<unsigned>(C);
        ckind = cv.take<int32_t>(C);
        cam = cv.take<int>(C);
        cfm = cv.take<int>(C);
        cprod = cv.take<unsigned long long>(C);
        row_cnt = cv.take<int32_t>(NR);
        row_comp = cv.take<int32_t>(NR);
        slot_col = cv.take<int32_t>(NR * TRI_CAP);
        slot_val = cv.take<int32_t>(NR * TRI_CAP);
        indptr = cv.take<int64_t>(NR + 1);
        tmp = cv.take<unsigned char>(scan_tmp);
        a_col = cv.take<int32_t>(NR * TRI_CAP);
        a_val = cv.take<int32_t>(NR * TRI_CAP);
    };
    TriComp *dc;
    int64_t *dpre, *indptr;
    unsigned *cflags;
    int32_t *ckind, *row_cnt, *row_comp, *slot_col, *slot_val, *a_col, *a_val;
    int *cam, *cfm;
    unsigned long long *cprod;
    void *tmp;
    {
        Carve dry{nullptr};
        layout(dry, dc, dpre, cflags, ckind, cam, cfm, cprod, row_cnt, row_comp, slot_col, slot_val, indptr,
               tmp, a_col, a_val);
        const int rc = tri_reserve(g_tri_a, dry.off + 256, s);
        if (rc) return rc;
    }
    Carve cv{g_tri_a.p};
    layout(cv, dc, dpre, cflags, ckind, cam, cfm, cprod, row_cnt, row_comp, slot_col, slot_val, indptr, tmp,
           a_col, a_val);
    const bool same = g_tri_last_buf == g_tri_a.p && g_tri_last_comps.size() == C &&
                      memcmp(g_tri_last_comps.data(), hc.data(), C * sizeof(TriComp)) == 0;
    if (!same) {
        RBG_CUDA_TRY(cudaMemcpyAsync(dc, hc.data(), C * sizeof(TriComp), cudaMemcpyHostToDevice, s));
        RBG_CUDA_TRY(cudaMemcpyAsync(dpre, pre.data(), (C + 1) * 8, cudaMemcpyHostToDevice, s));
        g_tri_last_comps = hc;
        g_tri_last_buf = g_tri_a.p;
    }
    RBG_CUDA_TRY(cudaMemsetAsync(cflags, 0, C * 4, s));

    // 1. scan
    {
        cudaEvent_t t = timer_begin(4, s);
        note_launches(1);
        tri_scan_kernel<<<(unsigned)pre[C], TRI_THREADS, 0, s>>>(in, dc, dpre, (int)count, slot_col, slot_val,
                                                                 row_cnt, row_comp, cflags);
        RBG_CUDA_TRY(cudaGetLastError());
        timer_end(4, t, s);
    }
    // 2. CSR of the candidates and their closure by levels
    cudaEvent_t tdag = timer_begin(5, s);
    note_launches(3);
    tri_kind_kernel<<<(unsigned)std::min<int64_t>((count + 255) / 256, 1024), 256, 0, s>>>((int)count, dc, cflags,
                                                                                          ckind);
    tri_count_kernel<<<grid_for(R, 256), 256, 0, s>>>(R, row_cnt, row_comp, ckind, indptr);
    RBG_CUDA_TRY(cudaMemsetAsync(indptr + R, 0, 8, s));
    size_t tb = scan_tmp;
    RBG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(tmp, tb, indptr, indptr, (int)(R + 1), s));
    int64_t nnz_a = 0;
    RBG_CUDA_TRY(cudaMemcpyAsync(&nnz_a, indptr + R, 8, cudaMemcpyDeviceToHost, s));
    tri_csr_fill_kernel<<<grid_for(R, 256), 256, 0, s>>>(R, row_comp, ckind, dc, indptr, slot_col, slot_val, a_col,
                                                        a_val);
    RBG_CUDA_TRY(cudaGetLastError());
    std::vector<int32_t> kind(C);
    RBG_CUDA_TRY(cudaMemcpyAsync(kind.data(), ckind, C * 4, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    int64_t candidates = 0;
    for (size_t i = 0; i < C; ++i) candidates += kind[i] != KIND_NONE;
    if (candidates == 0) {
        timer_end(5, tdag, s);
        return RBG_OK;
    }
    rbg_csr_t A{R, R, indptr, a_col, a_val};
    int64_t dws = 0;
    int rc = rbg_dag_workspace_bytes(R, nnz_a, &dws);
    if (rc) return rc;
    int64_t pool = std::max<int64_t>(16 * nnz_a + R, 1024);
    int32_t *p_col = nullptr, *p_val = nullptr, *row_len = nullptr;
    int64_t *row_off = nullptr;
    int64_t used = 0;
    for (int attempt = 0;; ++attempt) {
        Carve dry{nullptr};
        dry.take<unsigned char>((size_t)dws);
        dry.take<int32_t>((size_t)pool);
        dry.take<int32_t>((size_t)pool);
        dry.take<int64_t>(NR);
        dry.take<int32_t>(NR);
        rc = tri_reserve(g_tri_b, dry.off + 256, s);
        if (rc) return rc;
        Carve cb{g_tri_b.p};
        void *dw = cb.take<unsigned char>((size_t)dws);
        p_col = cb.take<int32_t>((size_t)pool);
        p_val = cb.take<int32_t>((size_t)pool);
        row_off = cb.take<int64_t>(NR);
        row_len = cb.take<int32_t>(NR);
        int64_t mx = 0, levels = 0;
        used = 0;
        rc = rbg_dag_closure(&A, dw, dws, p_col, p_val, pool, row_off, row_len, &used, &mx, &levels,
                             reinterpret_cast<rbg_stream_t>(s));
        if (rc == RBG_ERR_CAPACITY && used > pool && attempt < 4) {
            pool = used;
            continue;
        }
        break;
    }
    timer_end(5, tdag, s);
    if (rc == RBG_ERR_CAPACITY || rc == RBG_ERR_CYCLE) return RBG_OK;   // the blocked kernels decide
    if (rc) return rc;

    // 3. statistics
    {
        cudaEvent_t t = timer_begin(6, s);
        RBG_CUDA_TRY(cudaMemsetAsync(cam, 0xff, C * 4, s));
        RBG_CUDA_TRY(cudaMemsetAsync(cfm, 0xff, C * 4, s));
        RBG_CUDA_TRY(cudaMemsetAsync(cprod, 0, C * 8, s));
        note_launches(1);
        tri_stats_kernel<<<grid_for(R * 32, TRI_THREADS), TRI_THREADS, 0, s>>>(
            R, row_comp, ckind, dc, indptr, a_col, a_val, row_off, row_len, p_col, p_val, cam, cfm, cprod);
        RBG_CUDA_TRY(cudaGetLastError());
        timer_end(6, t, s);
    }
    // 4. dense rows of the accepted matrices (decided on the device from the statistics)
    {
        cudaEvent_t t = timer_begin(7, s);
        note_launches(1);
        tri_write_kernel<<<(unsigned)pre[C], TRI_THREADS, 0, s>>>(in, out, dc, dpre, (int)count, ckind, cam,
                                                                  row_off, row_len, p_col, p_val, rs);
        RBG_CUDA_TRY(cudaGetLastError());
        timer_end(7, t, s);
    }
    std::vector<int> ham(C), hfm(C);
    std::vector<unsigned long long> hprod(C);
    RBG_CUDA_TRY(cudaMemcpyAsync(ham.data(), cam, C * 4, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaMemcpyAsync(hfm.data(), cfm, C * 4, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaMemcpyAsync(hprod.data(), cprod, C * 8, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    for (size_t i = 0; i < C; ++i) {
        if (kind[i] == KIND_NONE || ham[i] >= TRI_TOP) continue;
        closed[i] = 1;
        rbg_result_t &r = results[i];
        r.status = RBG_OK;
        r.flags = 0;
        r.diameter = hfm[i] > 0 ? hfm[i] : 0;
        r.k = r.i = r.j = -1;
        r.path = RBG_PATH_DAG;
        r.executed = (int64_t)hprod[i];
    }
    return RBG_OK;
}

}  // namespace rbg

extern "C" int32_t rbg_release_scratch(void) {
    std::lock_guard<std::mutex> lk(rbg::g_tri_mu);
    for (rbg::TriScratch *t : {&rbg::g_tri_a, &rbg::g_tri_b}) {
        if (t->p) {
            int cur = 0;
            RBG_CUDA_TRY(cudaGetDevice(&cur));
            if (t->device != cur) RBG_CUDA_TRY(cudaSetDevice(t->device));
            RBG_CUDA_TRY(cudaDeviceSynchronize());
            RBG_CUDA_TRY(cudaFree(t->p));
            if (t->device != cur) RBG_CUDA_TRY(cudaSetDevice(cur));
        }
        t->p = nullptr;
        t->cap = 0;
        t->device = -1;
    }
    rbg::g_tri_last_buf = nullptr;
    return RBG_OK;
}
