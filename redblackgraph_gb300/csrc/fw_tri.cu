// fw_tri.cu -- dense closure of acyclic matrices by the DAG closure.
//
// The reference's warshall (redblackgraph/core/src/redblackgraph/warshall.c.in:88-106) runs the
// sequential loop  for k, i, j: W(i, j) = W(i, j) (+) W(i, k) (x) W(k, j)  over the whole matrix.
// When every off-diagonal entry lies below the diagonal (an edge i -> k only for k < i, as in a
// pedigree whose vertices are numbered oldest first), a path from i to k passes only vertices
// numbered above k, none of which an earlier step has used: before step k, W(i, k) is still the
// input A(i, k), while row k is already final (every path from k descends through vertices
// below k).  Step k therefore adds A(i, k) (x) C(k, .) to the rows of k's children, and the
// closure is the DAG recurrence  C(i, .) = A(i, .) (+) sum over parents k of A(i, k) (x) C(k, .)
// that the closure by levels computes.  Above the diagonal (edges to higher numbers) it is the
// mirror image: before step k, W(i, k) = C(i, k) and W(k, j) = A(k, j).
//
// In the clean regime (off-diagonal values 0 or >= 2, diagonal in {-1, 0, 1}) products with the
// diagonal change nothing and a cell only decreases once it holds a value, so the largest value
// the loop ever writes -- the diameter's source -- is, per cell, its first value: A(i, j), else
// the product of the first step that reaches the cell.  Below the diagonal that is the smallest
// parent k of i with j in C(k); above it, the smallest k in C(i) with j a parent of k.  A
// product whose most significant bit may reach bit 31 sends the matrix to the blocked kernels
// (which report the reference's overflow or wrap for 32-bit storage, and carry 64-bit values
// exactly), as does anything outside the clean regime or the 32-bit value range, a row of more
// than TRI_CAP entries or n > 8192.  For 64-bit storage no product below bit 31 can overflow, so
// the values, the diameter and the absence of errors are the reference's as well.  A matrix the
// closure went through whose loop does compute a product reaching bit 31 is reported as such
// (TRI_TOP_BIT): its caller skips the 32-bit lanes, which could only report that risk.
//
// A matrix with entries on both sides of the diagonal (an acyclic graph in any numbering) has the
// same closure values, but which product reaches a cell first depends on the numbering: its
// sequential loop is replayed on the closure's pattern (the triples (i, k, j) with (i, k) and
// (k, j) in the pattern, step by step), which gives the exact product MSBs and first values.  A
// vertex the closure by levels never places (a cycle, or below one) sends its matrix on.
//
// Pipeline (one call, every decision on the device): scan the dense rows (clean-regime test,
// which side of the diagonal, up to TRI_CAP off-diagonal entries per row) -> CSR of the
// candidate matrices with batch-global row numbers -> closure by levels -> for matrices in any
// numbering, the transposed pattern, the steps' triples and the replay -> per-row statistics
// (largest product MSB, largest first-value MSB) -> the dense rows of the accepted matrices
// written from the closure rows -> one result record per matrix, read back once.  Scratch is
// carved from the caller's workspace; with RBG_MODE_GRAPH the sequence, level loop included (a
// while node the device ends), is one CUDA graph replayed for the same layout.
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
constexpr int KIND_GENERAL = DAG_KIND_GENERAL;
constexpr int TRI_TOP = DAG_TOP_MSB;         // products reaching bit 31 leave the path

struct TriComp {
    int64_t n, in_off, out_off, row_base;    // row_base: first batch-global row
};

// Result of one matrix, written on the device and read back once per call.
struct TriOut {
    int32_t verdict, diameter;               // verdict: TRI_OPEN, TRI_CLOSED or TRI_TOP_BIT
    unsigned long long executed;
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

// A 16-byte vector of the storage type, unpacked.
template <typename T> struct TriVec {
    static constexpr int E = 16 / (int)sizeof(T);
    __device__ __forceinline__ static void split(const int4 &x, T (&v)[E]) {
        static_assert(sizeof(T) == 4 || sizeof(T) == 8, "int32 or int64 storage");
        if constexpr (sizeof(T) == 4) {
            v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
        } else {
            v[0] = (T)(((unsigned long long)(unsigned)x.y << 32) | (unsigned)x.x);
            v[1] = (T)(((unsigned long long)(unsigned)x.w << 32) | (unsigned)x.z);
        }
    }
};

// Off-diagonal entries of E consecutive columns j0 .. j0 + E - 1 held by each lane (m of them
// valid): clean-regime flags, and the nonzeros appended to the row's slots in column order.
// Column numbers fit 32 bits (n <= 8192 on this path); values outside [2, 2^31) are unclean.
template <typename T, int E>
__device__ __forceinline__ void tri_take(T (&v)[E], int j0, int m, int i, int lane, int64_t g,
                                         int32_t *__restrict__ slot_col, int32_t *__restrict__ slot_val,
                                         unsigned &flags, int &cnt) {
    int c4 = 0;
#pragma unroll
    for (int k = 0; k < E; ++k) {
        const int j = j0 + k;
        if (k >= m) {
            v[k] = 0;
        } else if (j == i) {
            if (!(v[k] == 0 || v[k] == 1 || v[k] == -1)) flags |= TF_UNCLEAN;
            v[k] = 0;                        // the diagonal is not an edge
        } else if (v[k] != 0) {
            if (v[k] == 1 || v[k] < 0 || (sizeof(T) == 8 && (long long)v[k] > (long long)INT32_MAX))
                flags |= TF_UNCLEAN;
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
    for (int k = 0; k < E; ++k) {
        if (v[k] != 0) {
            if (pos < TRI_CAP) {
                slot_col[g * TRI_CAP + pos] = j0 + k;
                slot_val[g * TRI_CAP + pos] = (int32_t)v[k];
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
template <typename T>
__global__ void __launch_bounds__(TRI_THREADS, 5)
tri_scan_kernel(const T *__restrict__ in, int64_t ld_in, const TriComp *__restrict__ comps,
                const int64_t *__restrict__ pre, int count, int32_t *__restrict__ slot_col,
                int32_t *__restrict__ slot_val, int32_t *__restrict__ row_cnt, int32_t *__restrict__ row_comp,
                unsigned *__restrict__ cflags) {
    constexpr int E = TriVec<T>::E;
    const int ci = tri_find(pre, count, blockIdx.x);
    const TriComp c = comps[ci];
    const int i = (int)(((int64_t)blockIdx.x - pre[ci]) * TRI_ROWS) + (threadIdx.x >> 5);
    if (i >= c.n) return;                    // warp-uniform
    const int lane = threadIdx.x & 31;
    const int n = (int)c.n;
    const int64_t g = c.row_base + i;
    const T *row = in + c.in_off + (int64_t)i * (ld_in ? ld_in : c.n);
    const int lead = (int)(((16 - ((uintptr_t)row & 15)) & 15) / sizeof(T));   // to the first boundary
    const int head = lead < n ? lead : n;
    const int nv = (n - head) / E;           // 16-byte vectors after the head
    const int tail = n - head - E * nv;
    unsigned flags = 0;
    int cnt = 0;
    T v1[1];
    if (head) {                              // columns 0 .. head - 1, one per lane
        v1[0] = lane < head ? row[lane] : (T)0;
        tri_take<T, 1>(v1, lane, lane < head ? 1 : 0, i, lane, g, slot_col, slot_val, flags, cnt);
    }
    // vectors s0 + 32 u + lane (u = 0..3), taken in column order (u ascending)
    for (int s0 = 0; s0 < nv; s0 += 128) {
        int4 x[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int q = s0 + 32 * u + lane;
            x[u] = q < nv ? *reinterpret_cast<const int4 *>(row + head + E * q) : make_int4(0, 0, 0, 0);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int q = s0 + 32 * u + lane;
            const int j0 = head + E * q;
            // all-zero vectors (a zero diagonal included) leave nothing to take
            if (__any_sync(0xffffffffu, (x[u].x | x[u].y | x[u].z | x[u].w) != 0)) {
                T v[E];
                TriVec<T>::split(x[u], v);
                tri_take<T, E>(v, j0, q < nv ? E : 0, i, lane, g, slot_col, slot_val, flags, cnt);
            }
        }
    }
    if (tail) {
        const int j = head + E * nv + lane;
        v1[0] = lane < tail ? row[j] : (T)0;
        tri_take<T, 1>(v1, j, lane < tail ? 1 : 0, i, lane, g, slot_col, slot_val, flags, cnt);
    }
    if (cnt > TRI_CAP) flags |= TF_WIDE;
    flags = __reduce_or_sync(0xffffffffu, flags);
    if (lane == 0) {
        row_cnt[g] = cnt;
        row_comp[g] = ci;
        if (flags) atomicOr(cflags + ci, flags);
    }
}

// Per matrix: candidate kind from the scan's flags, and the statistics' starting values.
__global__ void tri_kind_kernel(int count, const TriComp *__restrict__ comps, const unsigned *__restrict__ cflags,
                                int general, int32_t *__restrict__ ckind, int *__restrict__ cam, int *__restrict__ cfm,
                                unsigned long long *__restrict__ cprod, unsigned *__restrict__ cbad,
                                unsigned *__restrict__ any_gen) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const unsigned f = cflags[i];
        int k = KIND_NONE;
        if (comps[i].n > 0 && !(f & (TF_UNCLEAN | TF_WIDE)))
            k = ((f & TF_BELOW) && (f & TF_ABOVE)) ? (general ? KIND_GENERAL : KIND_NONE)
                                                  : (f & TF_ABOVE) ? KIND_ABOVE : KIND_BELOW;
        ckind[i] = k;
        cam[i] = -1;
        cfm[i] = -1;
        cprod[i] = 0;
        cbad[i] = 0;
        if (k == KIND_GENERAL) atomicOr(any_gen, 1u);
    }
}

// entries of each row in the CSR of the candidate matrices (rows of other matrices empty)
__global__ void tri_count_kernel(int64_t R, const int32_t *__restrict__ row_cnt, const int32_t *__restrict__ row_comp,
                                 const int32_t *__restrict__ ckind, int64_t *__restrict__ cnt64) {
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g <= R; g += (int64_t)gridDim.x * blockDim.x)
        cnt64[g] = g < R && ckind[row_comp[g]] != KIND_NONE ? row_cnt[g] : 0;
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

// The closure by levels kept every row in the pool (no pool overflow); otherwise nothing of this
// call's DAG path is used.  A matrix with a row never placed (a cycle: only matrices with entries
// on both sides of the diagonal can hold one) is marked in cbad.
__device__ __forceinline__ bool tri_dag_ok(const DagCounters *dc) { return !(dc->flags & 7); }

// A closure row entry outside its matrix (which a consistent closure never holds): the access is
// skipped and the call's DAG path rejected (flag 4), so the blocked kernels decide.
constexpr int TRI_BAD_ROW = 4;

// The row statistics of dag_rows.cuh, reduced per matrix (largest product MSB, largest
// first-value MSB, products): a group of DAG_STATS_G lanes per row, runs of `run` rows per
// group, one set of atomics per run and matrix.  Each group's bitmap takes 1 KB of shared
// memory, so TRI_STATS_CTAS CTAs of TRI_STATS_GROUPS groups fit on an SM.
constexpr int TRI_STATS_GROUPS = TRI_THREADS / DAG_STATS_G;
constexpr int TRI_STATS_CTAS = 5;
__global__ void __launch_bounds__(TRI_THREADS, TRI_STATS_CTAS)
tri_stats_kernel(int64_t R, const int32_t *__restrict__ row_comp, const int32_t *__restrict__ ckind,
                 const TriComp *__restrict__ comps, const int64_t *__restrict__ indptr,
                 const int32_t *__restrict__ a_col, const int32_t *__restrict__ a_val,
                 const int64_t *__restrict__ row_off, const int32_t *__restrict__ row_len,
                 const int32_t *__restrict__ p_col, const int32_t *__restrict__ p_val, const DagCounters *dc,
                 int *__restrict__ cam, int *__restrict__ cfm, unsigned long long *__restrict__ cprod, int run) {
    constexpr int G = DAG_STATS_G;
    __shared__ __align__(16) unsigned bm_all[TRI_STATS_GROUPS][TRI_BM_WORDS];
    if (!tri_dag_ok(dc)) return;             // block-uniform
    const int grp = threadIdx.x / G, lane = threadIdx.x & (G - 1);
    const unsigned gmask = dag_group_mask<G>();
    int cur = -1, am = -1, fm = -1;          // the matrix of the run's current rows, its statistics,
    int kind = KIND_NONE, base = 0, words = 0;   // its kind, first row and bitmap words
    unsigned long long prods = 0;
    auto flush = [&]() {                     // group-uniform
        const int am_r = __reduce_max_sync(gmask, am);
        const int fm_r = __reduce_max_sync(gmask, fm);
        if (lane == 0 && cur >= 0) {
            if (am_r >= 0) atomicMax(cam + cur, am_r);
            if (fm_r >= 0) atomicMax(cfm + cur, fm_r);
            if (prods) atomicAdd(cprod + cur, prods);
        }
    };
    auto crow = [&](int64_t r, int64_t &off, int &len) { off = row_off[r]; len = row_len[r]; };
    const int64_t stride = (int64_t)gridDim.x * TRI_STATS_GROUPS * run;
    for (int64_t r0 = ((int64_t)blockIdx.x * TRI_STATS_GROUPS + grp) * run; r0 < R; r0 += stride) {
        const int64_t r1 = min(R, r0 + run);
        for (int64_t g = r0; g < r1; ++g) {
            const int ci = row_comp[g];
            const int64_t a0 = indptr[g];
            const int alen = (int)(indptr[g + 1] - a0);
            if (ci != cur) {                     // group-uniform
                flush();
                cur = ci;
                am = fm = -1;
                prods = 0;
                kind = ckind[ci];
                base = (int32_t)comps[ci].row_base;
                words = (int)((comps[ci].n + 31) >> 5);
            }
            if (kind == KIND_NONE || kind == KIND_GENERAL) continue;   // group-uniform
            dag_row_stats<G>(bm_all[grp], words, kind, g, a0, alen, indptr, a_col, a_val, crow, p_col, p_val,
                             [&](int32_t col) { return col - base; }, lane, gmask, am, fm, prods);
        }
    }
    flush();
}


// ------------------------------------------------------------------------------------------
// Matrices in any numbering (entries on both sides of the diagonal): the sequential loop
// replayed on the closure's pattern.
// ------------------------------------------------------------------------------------------
// Before step k of the loop, W(i, k) and W(k, j) hold the values of paths whose intermediate
// vertices are all below k, and every cell the loop ever fills lies in the closure's pattern C
// (in the clean regime a cell never returns to zero).  Step k therefore touches only the triples
// (i, k, j) with (i, k) and (k, j) in C (the pattern holds no diagonal, and i != j in a DAG); a
// triple performs a product when both cells are non-zero at that time.  No triple of a step
// writes a cell another triple of the step reads ((i, j) = (i', k) would need j = k), so a step's
// triples run in parallel and the steps in order.  The replay keeps each cell's current value
// and the largest MSB of the products it performs (an overflow risk sends the matrix to the
// blocked kernels) and of the first value each cell receives (the diameter); the values the
// loop ends with are the closure's, which the closure by levels already holds.

// position of column c in the sorted closure row [o, o + len), or -1
__device__ __forceinline__ int64_t tri_find_col(const int32_t *__restrict__ p_col, int64_t o, int len, int32_t c) {
    int lo = 0, hi = len - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int32_t v = p_col[o + mid];
        if (v == c) return o + mid;
        if (v < c) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

__device__ __forceinline__ bool tri_gen_row(int ci, const int32_t *ckind, const unsigned *cbad, const DagCounters *dc,
                                            const unsigned *gflags) {
    return ckind[ci] == KIND_GENERAL && !cbad[ci] && tri_dag_ok(dc) && !*gflags;
}

// One warp per candidate row: a row never placed by the closure by levels (on or below a cycle)
// marks its matrix; the general matrices' closure rows count their columns.
__global__ void tri_gen_count_kernel(int64_t R, const int32_t *__restrict__ row_comp, const int32_t *__restrict__ ckind,
                                     const int64_t *__restrict__ row_off, const int32_t *__restrict__ row_len,
                                     const int32_t *__restrict__ p_col, const DagCounters *dc, const unsigned *any_gen,
                                     unsigned *__restrict__ cbad, int64_t *__restrict__ ccnt) {
    if (!tri_dag_ok(dc) || !*any_gen) return;
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t g = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); g < R; g += warps) {
        const int ci = row_comp[g];
        if (ckind[ci] != KIND_GENERAL) continue;   // warp-uniform
        const int len = row_len[g];
        if (len < 0) {
            if (lane == 0) atomicOr(cbad + ci, 1u);
            continue;
        }
        const int64_t o = row_off[g];
        for (int q = lane; q < len; q += 32)
            atomicAdd(reinterpret_cast<unsigned long long *>(ccnt + p_col[o + q]), 1ull);
    }
}

// The general matrices' closure pattern transposed: per column, the rows holding it and the pool
// position of each entry (in any order).
__global__ void tri_gen_csc_kernel(int64_t R, const int32_t *__restrict__ row_comp, const int32_t *__restrict__ ckind,
                                   const unsigned *__restrict__ cbad, const int64_t *__restrict__ row_off,
                                   const int32_t *__restrict__ row_len, const int32_t *__restrict__ p_col,
                                   const DagCounters *dc, const unsigned *any_gen, const int64_t *__restrict__ cptr,
                                   int32_t *__restrict__ ccur, int32_t *__restrict__ csc_row,
                                   int32_t *__restrict__ csc_pos, int64_t cap, unsigned *gflags) {
    if (!tri_dag_ok(dc) || !*any_gen) return;
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t g = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); g < R; g += warps) {
        const int ci = row_comp[g];
        if (ckind[ci] != KIND_GENERAL || cbad[ci]) continue;   // warp-uniform
        const int64_t o = row_off[g];
        const int len = row_len[g];
        for (int q = lane; q < len; q += 32) {
            const int32_t c = p_col[o + q];
            const int64_t at = cptr[c] + atomicAdd(ccur + c, 1);
            if (at < cap) {
                csc_row[at] = (int32_t)g;
                csc_pos[at] = (int32_t)(o + q);
            } else {
                atomicOr(gflags, 1u);
            }
        }
    }
}

// Triples of step k (batch-global vertex g): column g's entries times row g's entries.
// Also the pattern length of every general row (lcnt), whose exclusive scan lays each general
// matrix's current values out contiguously, row after row.
__global__ void tri_gen_tcount_kernel(int64_t R, const int32_t *__restrict__ row_comp, const int32_t *__restrict__ ckind,
                                      const unsigned *__restrict__ cbad, const int32_t *__restrict__ row_len,
                                      const int64_t *__restrict__ cptr, const DagCounters *dc, const unsigned *any_gen,
                                      const unsigned *gflags, int64_t *__restrict__ tcnt, int64_t *__restrict__ lcnt) {
    const bool on = tri_dag_ok(dc) && *any_gen && !*gflags;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g <= R; g += (int64_t)gridDim.x * blockDim.x) {
        int64_t c = 0, l = 0;
        if (on && g < R) {
            const int ci = row_comp[g];
            if (ckind[ci] == KIND_GENERAL && !cbad[ci]) {
                c = (cptr[g + 1] - cptr[g]) * (int64_t)row_len[g];
                l = row_len[g];
            }
        }
        tcnt[g] = c;
        lcnt[g] = l;
    }
}

// One warp per vertex k of a general matrix: its step's triples, as positions of (i, k), (k, j)
// and (i, j) among the matrix's current values (row g's entry q at lpos[g] - lpos[first row] + q).
__global__ void tri_gen_fill_kernel(int64_t R, const int32_t *__restrict__ row_comp, const int32_t *__restrict__ ckind,
                                    const unsigned *__restrict__ cbad, const TriComp *__restrict__ comps,
                                    const int64_t *__restrict__ row_off, const int32_t *__restrict__ row_len,
                                    const int32_t *__restrict__ p_col, const int64_t *__restrict__ cptr,
                                    const int32_t *__restrict__ csc_row, const int32_t *__restrict__ csc_pos,
                                    const int64_t *__restrict__ tpos, const int64_t *__restrict__ lpos,
                                    const DagCounters *dc, const unsigned *any_gen, int4 *__restrict__ trip,
                                    int64_t cap, unsigned *gflags) {
    if (!tri_dag_ok(dc) || !*any_gen || *gflags) return;
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t k = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); k < R; k += warps) {
        const int ci = row_comp[k];
        if (ckind[ci] != KIND_GENERAL || cbad[ci]) continue;   // warp-uniform
        const int64_t m0 = lpos[comps[ci].row_base];
        const int64_t c0 = cptr[k], r0 = row_off[k], base = tpos[k], lk = lpos[k] - m0;
        const int cn = (int)(cptr[k + 1] - c0), rn = row_len[k];
        const int64_t total = (int64_t)cn * rn;
        if (base + total > cap) {
            if (lane == 0 && total) atomicOr(gflags, 1u);
            continue;
        }
        for (int64_t t = lane; t < total; t += 32) {
            const int a = (int)(t / rn), b = (int)(t - (int64_t)a * rn);
            const int32_t i = csc_row[c0 + a];
            const int64_t oi = row_off[i], li = lpos[i] - m0;
            const int64_t qc = tri_find_col(p_col, oi, row_len[i], p_col[r0 + b]);
            if (qc < 0) {
                atomicOr(gflags, 2u);
                continue;
            }
            trip[base + t] = make_int4((int32_t)(li + (csc_pos[c0 + a] - oi)), (int32_t)(lk + b),
                                       (int32_t)(li + (qc - oi)), (int32_t)k);
        }
    }
}

// One warp per row of a general matrix: the current MSBs (row g's at lpos[g]) start as those of
// A's entries, zero (no value) elsewhere in the pattern; A's largest MSB starts the first-value
// maximum.
__global__ void tri_gen_init_kernel(int64_t R, const int32_t *__restrict__ row_comp, const int32_t *__restrict__ ckind,
                                    const unsigned *__restrict__ cbad, const int64_t *__restrict__ indptr,
                                    const int32_t *__restrict__ a_col, const int32_t *__restrict__ a_val,
                                    const int64_t *__restrict__ row_off, const int32_t *__restrict__ row_len,
                                    const int32_t *__restrict__ p_col, const int64_t *__restrict__ lpos,
                                    const DagCounters *dc, const unsigned *any_gen, unsigned *gflags,
                                    uint8_t *__restrict__ cur, int *__restrict__ cfm) {
    if (!tri_dag_ok(dc) || !*any_gen || *gflags) return;
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t g = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); g < R; g += warps) {
        const int ci = row_comp[g];
        if (ckind[ci] != KIND_GENERAL || cbad[ci]) continue;   // warp-uniform
        const int64_t o = row_off[g], l = lpos[g];
        const int len = row_len[g];
        for (int q = lane; q < len; q += 32) cur[l + q] = 0;
        __syncwarp();
        int fm = -1;
        for (int64_t e = indptr[g] + lane; e < indptr[g + 1]; e += 32) {
            const int64_t q = tri_find_col(p_col, o, len, a_col[e]);
            if (q < 0) {
                atomicOr(gflags, 2u);
                continue;
            }
            cur[l + (q - o)] = (uint8_t)msb_u32((uint32_t)a_val[e]);   // a clean value: 2 <= v < 2^31
            fm = max(fm, dag_row_msb(a_val[e]));
        }
        fm = __reduce_max_sync(0xffffffffu, fm);
        if (lane == 0 && fm >= 0) atomicMax(cfm + ci, fm);
    }
}

// One warp per general matrix: its triples (ordered by step) streamed in chunks of TRI_CHUNK,
// each chunk loaded TRI_PREFETCH chunks ahead so that no step waits for its triples; within a
// chunk the lanes take the chunk's steps in order (a warp barrier after each), so one step's
// stores come before the next step's loads.  A cell is tracked by the MSB of its current value alone
// (0: no value yet): msb(x (x) y) = msb(x) + msb(y) in the clean regime and msb(min(a, b)) =
// min(msb(a), msb(b)), so the products' MSBs and each cell's first value, all the replay decides
// from, come out exactly.  The matrix's P MSBs, one byte each, lie contiguously at
// curg + lpos[first row].  SMEM: one CTA of one warp per matrix with P <= TRI_SMEM_CELLS copies
// them into shared memory first (a step then costs a shared-memory round trip, not one to L2);
// otherwise a warp per matrix with P > TRI_SMEM_CELLS works on them in place.  The chain of steps
// of the largest matrices (~2,300 non-empty steps) sets the kernel's length.
constexpr int TRI_PER_LANE = 4;              // triples of a chunk per lane
constexpr int TRI_CHUNK = 32 * TRI_PER_LANE;
constexpr int TRI_PREFETCH = 4;              // chunks in flight
constexpr int64_t TRI_SMEM_CELLS = 57344;    // 56 KB of shared memory: four one-warp CTAs per SM

template <bool SMEM>
__global__ void __launch_bounds__(SMEM ? 32 : 256)
tri_gen_replay_kernel(int count, const TriComp *__restrict__ comps, const int32_t *__restrict__ ckind,
                      const unsigned *__restrict__ cbad, const int64_t *__restrict__ tpos,
                      const int64_t *__restrict__ lpos, const int4 *__restrict__ trip, const DagCounters *dc,
                      const unsigned *any_gen, const unsigned *gflags, uint8_t *curg, int *__restrict__ cam,
                      int *__restrict__ cfm, unsigned long long *__restrict__ cprod) {
    if (!tri_dag_ok(dc) || !*any_gen) return;
    extern __shared__ __align__(16) uint8_t tri_cells[];
    const int lane = threadIdx.x & 31;
    const int warps = SMEM ? gridDim.x : gridDim.x * (blockDim.x >> 5);
    const int first_ci = SMEM ? blockIdx.x : blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    for (int ci = first_ci; ci < count; ci += warps) {
        if (!tri_gen_row(ci, ckind, cbad, dc, gflags)) continue;   // warp-uniform
        const int64_t base = comps[ci].row_base, rows = comps[ci].n;
        const int64_t m0 = lpos[base], P = lpos[base + rows] - m0;
        if (SMEM ? P > TRI_SMEM_CELLS : P <= TRI_SMEM_CELLS) continue;
        uint8_t *val = curg + m0;
        if (SMEM) {
            for (int64_t q = lane; q < P; q += 32) tri_cells[q] = val[q];
            __syncwarp();
            val = tri_cells;
        }
        const int64_t T0 = tpos[base], T1 = tpos[base + rows];
        // chunks of TRI_CHUNK triples, triple j of a lane at chunk position 32 j + lane (coalesced
        // loads; a lane's triples ascend by step); a ring of TRI_PREFETCH chunks in flight, slot d
        // holding chunk c0 + d and refilled with chunk c0 + d + TRI_PREFETCH once taken (slots are
        // compile-time indices, so no register awaiting its load is read early)
        auto fetch = [&](int64_t c, int j) -> int4 {
            const int64_t t = T0 + c * TRI_CHUNK + 32 * j + lane;
            return t < T1 ? trip[t] : make_int4(0, 0, 0, INT_MAX);
        };
        int4 q[TRI_PREFETCH][TRI_PER_LANE];
#pragma unroll
        for (int d = 0; d < TRI_PREFETCH; ++d)
#pragma unroll
            for (int j = 0; j < TRI_PER_LANE; ++j) q[d][j] = fetch(d, j);
        int top = -1, first = -1;
        unsigned long long prods = 0;
        const int64_t chunks = (T1 - T0 + TRI_CHUNK - 1) / TRI_CHUNK;
        for (int64_t c0 = 0; c0 < chunks; c0 += TRI_PREFETCH)
#pragma unroll
        for (int d = 0; d < TRI_PREFETCH; ++d) {
            const int64_t c = c0 + d;
            if (c >= chunks) break;                                   // warp-uniform
            int4 tr[TRI_PER_LANE];
#pragma unroll
            for (int j = 0; j < TRI_PER_LANE; ++j) {
                tr[j] = q[d][j];
                q[d][j] = fetch(c + TRI_PREFETCH, j);
            }
            // the chunk's steps in order: each lane does all its triples of the step at once
            // (a step's triples are independent), then a warp barrier
            int next = 0;                                             // the lane's first pending triple
            while (true) {
                int mine = INT_MAX;
#pragma unroll
                for (int j = 0; j < TRI_PER_LANE; ++j)
                    if (j == next) mine = tr[j].w;
                const int k = __reduce_min_sync(0xffffffffu, next < TRI_PER_LANE ? mine : INT_MAX);
                if (k == INT_MAX) break;                              // warp-uniform
#pragma unroll
                for (int j = 0; j < TRI_PER_LANE; ++j) {
                    if (j < next || tr[j].w != k) continue;
                    ++next;
                    if ((uint64_t)(uint32_t)tr[j].x >= (uint64_t)P || (uint64_t)(uint32_t)tr[j].y >= (uint64_t)P ||
                        (uint64_t)(uint32_t)tr[j].z >= (uint64_t)P) {
                        atomicOr(const_cast<int *>(&dc->flags), TRI_BAD_ROW);
                        continue;
                    }
                    // the three cells are read together: one round trip per step
                    const int mx = val[tr[j].x], my = val[tr[j].y], old = val[tr[j].z];
                    if (mx != 0 && my != 0) {
                        const int pm = mx + my;              // the product's MSB
                        top = max(top, pm);
                        ++prods;
                        if (old == 0) {
                            first = max(first, pm);
                            val[tr[j].z] = (uint8_t)pm;
                        } else if (pm < old) {
                            val[tr[j].z] = (uint8_t)pm;
                        }
                    }
                }
                __syncwarp();
            }
        }
        top = __reduce_max_sync(0xffffffffu, top);
        first = __reduce_max_sync(0xffffffffu, first);
        for (int o = 16; o > 0; o >>= 1) prods += __shfl_xor_sync(0xffffffffu, prods, o);
        if (lane == 0) {
            if (top >= 0) atomicMax(cam + ci, top);
            if (first >= 0) atomicMax(cfm + ci, first);
            cprod[ci] += prods;
        }
    }
}

PerDeviceOnce g_tri_configured;
int tri_configure() {
    return g_tri_configured.run([] {
        RBG_CUDA_TRY(cudaFuncSetAttribute(tri_gen_replay_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)TRI_SMEM_CELLS));
        return (int)RBG_OK;
    });
}

// Recorded graphs: the IF node around the replay opens only when the closure by levels went
// through and some matrix needs the replay; the decision is also kept for the launch count.
__global__ void tri_gen_gate_kernel(const DagCounters *dc, const unsigned *any_gen, unsigned *ran,
                                    cudaGraphConditionalHandle h) {
    if (threadIdx.x != 0) return;
    const unsigned go = (tri_dag_ok(dc) && *any_gen) ? 1u : 0u;
    *ran = go;
    cudaGraphSetConditional(h, go);
}

// Inside the capture on `s`: `gate(h)` launches on s the kernel that sets the condition, then an
// IF node whose body `body(stream)` records from a second stream captured into it.
template <typename Gate, typename Body>
int tri_captured_if(cudaStream_t s, Gate gate, Body body) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    RBG_CUDA_TRY(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &ndeps));
    if (st != cudaStreamCaptureStatusActive || !g) return RBG_ERR_INVALID;
    cudaGraphConditionalHandle h;
    RBG_CUDA_TRY(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
    gate(h);
    RBG_CUDA_TRY(cudaGetLastError());
    RBG_CUDA_TRY(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &ndeps));
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeIf;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    RBG_CUDA_TRY(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &p));
    static thread_local cudaStream_t side = nullptr;
    if (!side) RBG_CUDA_TRY(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
    RBG_CUDA_TRY(cudaStreamBeginCaptureToGraph(side, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                               cudaStreamCaptureModeThreadLocal));
    const int rc = body(side);
    cudaGraph_t got = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(side, &got);
    if (rc) return rc;
    if (ee != cudaSuccess) return RBG_ERR_CUDA;
    RBG_CUDA_TRY(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    return RBG_OK;
}

constexpr int TRI_GEN_LAUNCHES = 10;         // launches of the replay block

__device__ __forceinline__ bool tri_accepted(int ci, const int32_t *ckind, const int *cam, const unsigned *cbad,
                                             const DagCounters *dc, const unsigned *gflags) {
    const int k = ckind[ci];
    return k != KIND_NONE && cam[ci] < TRI_TOP && !cbad[ci] && tri_dag_ok(dc) && !(k == KIND_GENERAL && *gflags);
}

// The statistics are complete and some product of the loop reaches bit 31 (the first such
// product is computed from exact operands, so the test is exact).
__device__ __forceinline__ bool tri_top_bit(int ci, const int32_t *ckind, const int *cam, const unsigned *cbad,
                                            const DagCounters *dc, const unsigned *gflags) {
    const int k = ckind[ci];
    return k != KIND_NONE && cam[ci] >= TRI_TOP && !cbad[ci] && tri_dag_ok(dc) && !(k == KIND_GENERAL && *gflags);
}

// One warp per row of an accepted matrix.  Out of place, the whole dense row is written in
// segments of SEG columns (2 KB) built in shared memory (zeros, the closure row's entries, the
// diagonal) and stored as full 16-byte vectors on the row's 16-byte grid, so no DRAM line is
// written partially; in place, only the closure's entries (the other cells already hold the
// result).  The row statistics are recorded when asked for (32-bit storage).
template <typename T>
__global__ void __launch_bounds__(TRI_THREADS)
tri_write_kernel(const T *__restrict__ in, int64_t ld_in, T *__restrict__ out, int64_t ld_out,
                 const TriComp *__restrict__ comps, const int64_t *__restrict__ pre, int count,
                 const int32_t *__restrict__ ckind, const int *__restrict__ cam, const unsigned *__restrict__ cbad,
                 const DagCounters *dc, const unsigned *gflags,
                 const int64_t *__restrict__ row_off, const int32_t *__restrict__ row_len,
                 const int32_t *__restrict__ p_col, const int32_t *__restrict__ p_val, RowStats rs) {
    constexpr int SEG = 2048 / (int)sizeof(T);
    constexpr int E = TriVec<T>::E;
    __shared__ __align__(16) T seg_all[TRI_ROWS][SEG];
    const int ci = tri_find(pre, count, blockIdx.x);
    if (!tri_accepted(ci, ckind, cam, cbad, dc, gflags)) return;   // block-uniform
    const TriComp c = comps[ci];
    const int i = (int)(((int64_t)blockIdx.x - pre[ci]) * TRI_ROWS) + (threadIdx.x >> 5);
    if (i >= c.n) return;                    // warp-uniform
    const int lane = threadIdx.x & 31;
    const int n = (int)c.n;
    const int64_t g = c.row_base + i;
    const T *rin = in + c.in_off + (int64_t)i * (ld_in ? ld_in : c.n);
    T *rout = out + c.out_off + (int64_t)i * (ld_out ? ld_out : c.n);
    const T diag = rin[i];
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
            if ((unsigned)j >= (unsigned)n) {
                atomicOr(const_cast<int *>(&dc->flags), TRI_BAD_ROW);
                continue;
            }
            rout[j] = (T)v;
            mx = max(mx, v);
            mark(j >> 5);
        }
    } else {
        T *seg = seg_all[threadIdx.x >> 5];
        // column j sits at j' = j + shift on the 16-byte grid; segment s0 holds j' in [s0, s0 + SEG)
        const int shift = (int)(((uintptr_t)rout & 15) / sizeof(T));
        int e = 0;                           // first closure entry not yet placed (warp-uniform)
        for (int s0 = 0; s0 < n + shift; s0 += SEG) {
            for (int t = lane; t < SEG / E; t += 32) reinterpret_cast<int4 *>(seg)[t] = make_int4(0, 0, 0, 0);
            __syncwarp();
            const int lim = s0 + SEG - shift;            // entries with j < lim belong to this segment
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
                    if (j < 0 || j >= n || j + shift < s0) {   // outside the matrix, or out of order
                        atomicOr(const_cast<int *>(&dc->flags), TRI_BAD_ROW);
                    } else {
                        seg[j + shift - s0] = (T)v;
                        mx = max(mx, v);
                        mark(j >> 5);
                    }
                }
                const unsigned bal = __ballot_sync(0xffffffffu, here);
                e += __popc(bal);
                if (bal != 0xffffffffu) break;
            }
            if (lane == 0 && i + shift >= s0 && i + shift < s0 + SEG) seg[i + shift - s0] = diag;
            __syncwarp();
            for (int t = lane; t < SEG / E; t += 32) {
                const int j0 = s0 + E * t - shift;
                if (j0 >= n) break;
                const int4 z = reinterpret_cast<const int4 *>(seg)[t];
                if (j0 >= 0 && j0 + E <= n) {
                    *reinterpret_cast<int4 *>(rout + j0) = z;
                } else {                                 // the row's ragged ends
                    T zz[E];
                    TriVec<T>::split(z, zz);
#pragma unroll
                    for (int k = 0; k < E; ++k)
                        if (j0 + k >= 0 && j0 + k < n) rout[j0 + k] = zz[k];
                }
            }
            __syncwarp();                                // before the next segment is zeroed
        }
    }
    if constexpr (sizeof(T) == 4) {
        if (rs.row_count) {
            if (lane == 0 && diag != 0) {
                mark(i >> 5);
                mx = max(mx, (int)diag);
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
}

__global__ void tri_result_kernel(int count, const int32_t *__restrict__ ckind, const int *__restrict__ cam,
                                  const int *__restrict__ cfm, const unsigned long long *__restrict__ cprod,
                                  const unsigned *__restrict__ cbad, const DagCounters *dc, const unsigned *gflags,
                                  TriOut *__restrict__ res) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        TriOut o;
        o.verdict = tri_accepted(i, ckind, cam, cbad, dc, gflags) ? TRI_CLOSED
                    : tri_top_bit(i, ckind, cam, cbad, dc, gflags) ? TRI_TOP_BIT : TRI_OPEN;
        o.diameter = cfm[i] > 0 ? cfm[i] : 0;
        o.executed = cprod[i];
        res[i] = o;
    }
}

struct Carve {
    unsigned char *p;
    size_t off = 0;
    template <typename X> X *take(size_t n) {
        off = align_up(off, 256);
        X *r = p ? reinterpret_cast<X *>(p + off) : nullptr;
        off += n * sizeof(X);
        return r;
    }
};

// The scratch of one call, carved from the caller's workspace: the matrix table, per-matrix
// flags and statistics, the scan's row slots, the candidates' CSR, the closure's workspace and
// row index, and the row pool in whatever remains.
struct TriLayout {
    TriComp *dc;
    int64_t *dpre, *indptr, *row_off, *ccnt, *cptr, *tcnt, *tpos, *lpos;
    unsigned *cflags, *cbad, *gflags;        // gflags[0]: the general path's scratch overflowed; [1]: any general;
                                             // [2]: the replay ran (recorded graphs: its IF node's decision)
    int32_t *ckind, *row_cnt, *row_comp, *slot_col, *slot_val, *a_col, *a_val, *row_len, *p_col, *p_val;
    int32_t *ccur, *csc_row, *csc_pos;
    uint8_t *cur;                            // the replay's current MSB per pattern entry
    int4 *trip;                              // (pool positions of (i, k), (k, j), (i, j); step k)
    int *cam, *cfm;
    unsigned long long *cprod;
    TriOut *res;
    void *tmp, *dag_ws;
    size_t scan_tmp;
    int64_t pool, csc_cap, trip_cap;
    size_t fixed;                            // bytes before the pool
};

void tri_layout(unsigned char *base, size_t ws_bytes, size_t C, size_t NR, TriLayout &L) {
    Carve cv{base};
    L.scan_tmp = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, L.scan_tmp, (int64_t *)nullptr, (int64_t *)nullptr, (int)(NR + 1));
    L.dc = cv.take<TriComp>(C);
    L.dpre = cv.take<int64_t>(C + 1);
    L.cflags = cv.take<unsigned>(C);
    L.ckind = cv.take<int32_t>(C);
    L.cam = cv.take<int>(C);
    L.cfm = cv.take<int>(C);
    L.cprod = cv.take<unsigned long long>(C);
    L.cbad = cv.take<unsigned>(C);
    L.gflags = cv.take<unsigned>(3);
    L.res = cv.take<TriOut>(C);
    L.row_cnt = cv.take<int32_t>(NR);
    L.row_comp = cv.take<int32_t>(NR);
    L.slot_col = cv.take<int32_t>(NR * TRI_CAP);
    L.slot_val = cv.take<int32_t>(NR * TRI_CAP);
    L.indptr = cv.take<int64_t>(NR + 1);
    L.tmp = cv.take<unsigned char>(L.scan_tmp);
    L.a_col = cv.take<int32_t>(NR * TRI_CAP);
    L.a_val = cv.take<int32_t>(NR * TRI_CAP);
    L.dag_ws = cv.take<unsigned char>(dag_workspace_for((int64_t)NR, (int64_t)(NR * TRI_CAP)));
    L.row_off = cv.take<int64_t>(NR);
    L.row_len = cv.take<int32_t>(NR);
    L.ccnt = cv.take<int64_t>(NR + 1);
    L.cptr = cv.take<int64_t>(NR + 1);
    L.ccur = cv.take<int32_t>(NR);
    L.tcnt = cv.take<int64_t>(NR + 1);
    L.tpos = cv.take<int64_t>(NR + 1);
    L.lpos = cv.take<int64_t>(NR + 1);
    L.fixed = align_up(cv.off, 256);
    // the rest: 40% for the row pool (column, value and the replay's current MSB per entry),
    // 15% for the transposed pattern, 45% for the replay's triples
    const size_t rest = ws_bytes > L.fixed + 2048 ? ws_bytes - L.fixed - 2048 : 0;
    L.pool = std::min<int64_t>((int64_t)(rest / 10 * 4 / 9 / 64 * 64), (int64_t)INT32_MAX / 64 * 64);
    L.csc_cap = (int64_t)(rest / 100 * 15 / 8);
    L.trip_cap = (int64_t)(rest / 100 * 45 / 16);
    Carve tail{base};
    tail.off = L.fixed;
    L.p_col = tail.take<int32_t>((size_t)L.pool);
    L.p_val = tail.take<int32_t>((size_t)L.pool);
    L.cur = tail.take<uint8_t>((size_t)L.pool);
    L.csc_row = tail.take<int32_t>((size_t)L.csc_cap);
    L.csc_pos = tail.take<int32_t>((size_t)L.csc_cap);
    L.trip = tail.take<int4>((size_t)L.trip_cap);
}

struct TriShape {
    int64_t count, R, ctas;
    int64_t ld_in, ld_out;
};

// Every launch of the DAG path, in stream order, with no host synchronisation when `captured`
// (the level loop then is a while node).  Returns the number of kernel launches issued.
template <typename T>
int tri_enqueue(const TriShape &sh, const TriLayout &L, const T *in, T *out, cudaStream_t s, bool captured,
                const RowStats &rs, DagCounters **dcount, int64_t *launches) {
    const int64_t R = sh.R;
    const int count = (int)sh.count;
    RBG_CUDA_TRY(cudaMemsetAsync(L.cflags, 0, (size_t)count * 4, s));
    RBG_CUDA_TRY(cudaMemsetAsync(L.gflags, 0, 12, s));
    // 1. scan
    {
        cudaEvent_t t = timer_begin(4, s);
        note_launches(1);
        tri_scan_kernel<T><<<(unsigned)sh.ctas, TRI_THREADS, 0, s>>>(in, sh.ld_in, L.dc, L.dpre, count, L.slot_col,
                                                                     L.slot_val, L.row_cnt, L.row_comp, L.cflags);
        RBG_CUDA_TRY(cudaGetLastError());
        timer_end(4, t, s);
    }
    // 2. CSR of the candidates and their closure by levels
    cudaEvent_t tdag = timer_begin(5, s);
    note_launches(4);
    tri_kind_kernel<<<(unsigned)std::min<int64_t>((count + 255) / 256, 1024), 256, 0, s>>>(
        count, L.dc, L.cflags, 1, L.ckind, L.cam, L.cfm, L.cprod, L.cbad, L.gflags + 1);
    tri_count_kernel<<<grid_for(R + 1, 256), 256, 0, s>>>(R, L.row_cnt, L.row_comp, L.ckind, L.indptr);
    size_t tb = L.scan_tmp;
    RBG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(L.tmp, tb, L.indptr, L.indptr, (int)(R + 1), s));
    tri_csr_fill_kernel<<<grid_for(R, 256), 256, 0, s>>>(R, L.row_comp, L.ckind, L.dc, L.indptr, L.slot_col,
                                                        L.slot_val, L.a_col, L.a_val);
    RBG_CUDA_TRY(cudaGetLastError());
    *launches += 5;
    rbg_csr_t A{R, R, L.indptr, L.a_col, L.a_val};
    RBG_CUDA_TRY(cudaMemsetAsync(L.row_len, 0xff, (size_t)R * 4, s));   // -1: never placed
    int rc = dag_enqueue(&A, R * TRI_CAP, L.dag_ws, L.p_col, L.p_val, L.pool, L.row_off, L.row_len, s, captured,
                         dcount, launches);
    if (rc) return rc;
    timer_end(5, tdag, s);
    // 2b. matrices in any numbering: the loop replayed on the closure's pattern (every kernel
    // returns at once when the batch holds none; a recorded graph skips the block by an IF node)
    {
        cudaEvent_t tg = timer_begin(8, s);
        const DagCounters *dcn = *dcount;
        const unsigned *any = L.gflags + 1;
        const int gw = grid_for(R * 32, 256);
        RBG_CUDA_TRY(cudaMemsetAsync(L.ccnt, 0, (size_t)(R + 1) * 8, s));
        RBG_CUDA_TRY(cudaMemsetAsync(L.ccur, 0, (size_t)R * 4, s));
        auto body = [&](cudaStream_t b) -> int {
            tri_gen_count_kernel<<<gw, 256, 0, b>>>(R, L.row_comp, L.ckind, L.row_off, L.row_len, L.p_col, dcn, any,
                                                    L.cbad, L.ccnt);
            size_t tb2 = L.scan_tmp;
            RBG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(L.tmp, tb2, L.ccnt, L.cptr, (int)(R + 1), b));
            tri_gen_csc_kernel<<<gw, 256, 0, b>>>(R, L.row_comp, L.ckind, L.cbad, L.row_off, L.row_len, L.p_col, dcn,
                                                  any, L.cptr, L.ccur, L.csc_row, L.csc_pos, L.csc_cap, L.gflags);
            // (the column counts are scanned already: ccnt now takes the rows' pattern lengths)
            tri_gen_tcount_kernel<<<grid_for(R + 1, 256), 256, 0, b>>>(R, L.row_comp, L.ckind, L.cbad, L.row_len,
                                                                      L.cptr, dcn, any, L.gflags, L.tcnt, L.ccnt);
            tb2 = L.scan_tmp;
            RBG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(L.tmp, tb2, L.tcnt, L.tpos, (int)(R + 1), b));
            tb2 = L.scan_tmp;
            RBG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(L.tmp, tb2, L.ccnt, L.lpos, (int)(R + 1), b));
            tri_gen_fill_kernel<<<gw, 256, 0, b>>>(R, L.row_comp, L.ckind, L.cbad, L.dc, L.row_off, L.row_len,
                                                   L.p_col, L.cptr, L.csc_row, L.csc_pos, L.tpos, L.lpos, dcn, any,
                                                   L.trip, L.trip_cap, L.gflags);
            tri_gen_init_kernel<<<gw, 256, 0, b>>>(R, L.row_comp, L.ckind, L.cbad, L.indptr, L.a_col, L.a_val,
                                                   L.row_off, L.row_len, L.p_col, L.lpos, dcn, any, L.gflags, L.cur,
                                                   L.cfm);
            tri_gen_replay_kernel<true><<<(unsigned)count, 32, (size_t)TRI_SMEM_CELLS, b>>>(
                count, L.dc, L.ckind, L.cbad, L.tpos, L.lpos, L.trip, dcn, any, L.gflags, L.cur, L.cam, L.cfm,
                L.cprod);
            tri_gen_replay_kernel<false><<<grid_for((int64_t)count * 32, 256), 256, 0, b>>>(
                count, L.dc, L.ckind, L.cbad, L.tpos, L.lpos, L.trip, dcn, any, L.gflags, L.cur, L.cam, L.cfm,
                L.cprod);
            RBG_CUDA_TRY(cudaGetLastError());
            return (int)RBG_OK;
        };
        if (captured) {
            rc = tri_captured_if(
                s, [&](cudaGraphConditionalHandle h) { tri_gen_gate_kernel<<<1, 32, 0, s>>>(dcn, any, L.gflags + 2, h); },
                body);
            *launches += 1;                  // the gate; the block is counted when it runs
        } else {
            note_launches(TRI_GEN_LAUNCHES);
            rc = body(s);
            *launches += TRI_GEN_LAUNCHES;
        }
        if (rc) return rc;
        timer_end(8, tg, s);
    }
    // 3. statistics
    {
        cudaEvent_t t = timer_begin(6, s);
        note_launches(1);
        const int64_t ctas = (int64_t)sm_count() * TRI_STATS_CTAS;
        const int run = dag_stats_run(R, ctas * TRI_STATS_GROUPS);
        const int64_t need = (R + (int64_t)run * TRI_STATS_GROUPS - 1) / ((int64_t)run * TRI_STATS_GROUPS);
        tri_stats_kernel<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(need, ctas)), TRI_THREADS, 0, s>>>(
            R, L.row_comp, L.ckind, L.dc, L.indptr, L.a_col, L.a_val, L.row_off, L.row_len, L.p_col, L.p_val, *dcount,
            L.cam, L.cfm, L.cprod, run);
        RBG_CUDA_TRY(cudaGetLastError());
        timer_end(6, t, s);
    }
    // 4. dense rows of the accepted matrices (decided on the device from the statistics)
    {
        cudaEvent_t t = timer_begin(7, s);
        note_launches(2);
        tri_write_kernel<T><<<(unsigned)sh.ctas, TRI_THREADS, 0, s>>>(in, sh.ld_in, out, sh.ld_out, L.dc, L.dpre,
                                                                      count, L.ckind, L.cam, L.cbad, *dcount,
                                                                      L.gflags, L.row_off, L.row_len, L.p_col,
                                                                      L.p_val, rs);
        tri_result_kernel<<<(unsigned)std::min<int64_t>((count + 255) / 256, 1024), 256, 0, s>>>(
            count, L.ckind, L.cam, L.cfm, L.cprod, L.cbad, *dcount, L.gflags, L.res);
        RBG_CUDA_TRY(cudaGetLastError());
        timer_end(7, t, s);
    }
    *launches += 3;
    return RBG_OK;
}

// ------------------------------------------------------------------------------------------
// RBG_MODE_GRAPH: the whole sequence recorded once per layout and replayed
// ------------------------------------------------------------------------------------------
struct TriGraphKey {
    int device, tbytes;
    const void *in;
    void *out;
    unsigned char *ws;
    size_t ws_bytes;
    int64_t ld_in, ld_out;
    std::vector<int64_t> sizes, in_off, out_off;
    RowStats rs;
    bool operator==(const TriGraphKey &o) const {
        return device == o.device && tbytes == o.tbytes && in == o.in && out == o.out && ws == o.ws &&
               ws_bytes == o.ws_bytes && ld_in == o.ld_in && ld_out == o.ld_out && sizes == o.sizes &&
               in_off == o.in_off && out_off == o.out_off && rs == o.rs;
    }
};
struct TriGraph {
    TriGraphKey key;
    cudaGraphExec_t exec;
    DagCounters *dcount;
    int64_t launches;                        // outside the level loop
    unsigned long long stamp;
};
std::mutex g_tri_graph_mu;
std::vector<TriGraph> g_tri_graphs;
unsigned long long g_tri_clock = 0;
constexpr size_t TRI_GRAPH_CACHE = 8;

// Record the sequence into a graph on a private stream (the caller's may be the legacy default
// stream, which cannot be captured); nothing runs while recording.
template <typename T>
int tri_record(const TriShape &sh, const TriLayout &L, const T *in, T *out, const RowStats &rs, TriGraph &g) {
    static thread_local cudaStream_t cap = nullptr;
    if (!cap) RBG_CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    RBG_CUDA_TRY(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    launch_recording(true);
    int64_t launches = 0;
    const int rc = tri_enqueue<T>(sh, L, in, out, cap, true, rs, &g.dcount, &launches);
    launch_recording(false);
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(cap, &graph);
    if (rc || ec != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return rc ? rc : RBG_ERR_CUDA;
    }
    const cudaError_t ei = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) return RBG_ERR_CUDA;
    g.launches = launches;
    return RBG_OK;
}

}  // namespace

template <typename T>
int tri_batch(int64_t count, const int64_t *sizes, const int64_t *in_off, const int64_t *out_off, int64_t ld_in,
              int64_t ld_out, const T *in, T *out, rbg_result_t *results, char *closed, unsigned char *ws,
              size_t ws_bytes, uint32_t mode, cudaStream_t s, const RowStats &rs) {
    if (count <= 0 || count > INT32_MAX || !ws) return RBG_OK;
    {
        const int rc = tri_configure();     // before any capture: kernel attributes per device
        if (rc) return rc;
    }
    std::vector<TriComp> hc((size_t)count);
    std::vector<int64_t> pre((size_t)count + 1, 0);
    int64_t R = 0;
    for (int64_t i = 0; i < count; ++i) {
        const int64_t n = (sizes[i] > 0 && sizes[i] <= TRI_MAX_N) ? sizes[i] : 0;
        hc[(size_t)i] = TriComp{n, in_off[i], out_off[i], R};
        R += n;
        pre[(size_t)i + 1] = pre[(size_t)i] + (n + TRI_ROWS - 1) / TRI_ROWS;
    }
    if (R == 0 || R * TRI_CAP > INT32_MAX) return RBG_OK;
    const size_t C = (size_t)count, NR = (size_t)R;
    TriLayout L;
    tri_layout(nullptr, ws_bytes, C, NR, L);
    if (L.pool < 4 * R) return RBG_OK;       // no room for a closure: the other paths decide
    tri_layout(ws, ws_bytes, C, NR, L);
    const TriShape sh{count, R, pre[C], ld_in, ld_out};
    {
        HostStaging hs(s, C * sizeof(TriComp) + (C + 1) * 8 + C * sizeof(TriOut) + sizeof(DagCounters) + 256);
        int rc = hs.up(L.dc, hc.data(), C * sizeof(TriComp));
        if (!rc) rc = hs.up(L.dpre, pre.data(), (C + 1) * 8);
        if (rc) return rc;
    }

    DagCounters *dcount = nullptr;
    int64_t fixed_launches = -1;             // >= 0: a graph ran; its level loop is counted below
    if ((mode & RBG_MODE_GRAPH) && !timer_on()) {
        int dev = 0;
        RBG_CUDA_TRY(cudaGetDevice(&dev));
        TriGraphKey key{dev, (int)sizeof(T), in, out, ws, ws_bytes, ld_in, ld_out,
                        std::vector<int64_t>(sizes, sizes + count), std::vector<int64_t>(in_off, in_off + count),
                        std::vector<int64_t>(out_off, out_off + count), rs};
        std::lock_guard<std::mutex> lk(g_tri_graph_mu);
        TriGraph *hit = nullptr;
        for (auto &e : g_tri_graphs)
            if (e.key == key) hit = &e;
        if (!hit) {
            TriGraph g;
            g.key = std::move(key);
            const int rc = tri_record<T>(sh, L, in, out, rs, g);
            if (rc) return rc;
            if (g_tri_graphs.size() >= TRI_GRAPH_CACHE) {
                size_t old = 0;
                for (size_t k = 1; k < g_tri_graphs.size(); ++k)
                    if (g_tri_graphs[k].stamp < g_tri_graphs[old].stamp) old = k;
                RBG_CUDA_TRY(cudaDeviceSynchronize());   // the evicted graph may still run on another stream
                cudaGraphExecDestroy(g_tri_graphs[old].exec);
                g_tri_graphs.erase(g_tri_graphs.begin() + (long)old);
            }
            g_tri_graphs.push_back(std::move(g));
            hit = &g_tri_graphs.back();
        }
        hit->stamp = ++g_tri_clock;
        RBG_CUDA_TRY(cudaGraphLaunch(hit->exec, s));
        dcount = hit->dcount;
        fixed_launches = hit->launches;
    } else {
        int64_t launches = 0;
        const int rc = tri_enqueue<T>(sh, L, in, out, s, false, rs, &dcount, &launches);
        if (rc) return rc;
    }
    std::vector<TriOut> h(C);
    DagCounters hd;
    unsigned gate_ran = 0;
    {
        HostStaging hs(s, C * sizeof(TriOut) + sizeof(DagCounters) + 128);
        int rc = hs.down(h.data(), L.res, C * sizeof(TriOut));
        if (!rc) rc = hs.down(&hd, dcount, sizeof(hd));
        if (!rc && fixed_launches >= 0) rc = hs.down(&gate_ran, L.gflags + 2, 4);
        if (!rc) rc = hs.finish();
        if (rc) return rc;
    }
    if (fixed_launches >= 0) {
        const int64_t iters = std::max<int64_t>(1, (hd.nlevels + DAG_GRAPH_CHUNK - 1) / DAG_GRAPH_CHUNK);
        note_launches(fixed_launches + iters * (3 * DAG_GRAPH_CHUNK + 1) + (gate_ran ? TRI_GEN_LAUNCHES : 0));
    }
    for (size_t i = 0; i < C; ++i) {
        closed[i] = (char)h[i].verdict;
        if (h[i].verdict != TRI_CLOSED) continue;
        rbg_result_t &r = results[i];
        r.status = RBG_OK;
        r.flags = 0;
        r.diameter = h[i].diameter;
        r.k = r.i = r.j = -1;
        r.path = RBG_PATH_DAG;
        r.executed = (int64_t)h[i].executed;
    }
    return RBG_OK;
}

template int tri_batch<int32_t>(int64_t, const int64_t *, const int64_t *, const int64_t *, int64_t, int64_t,
                                const int32_t *, int32_t *, rbg_result_t *, char *, unsigned char *, size_t, uint32_t,
                                cudaStream_t, const RowStats &);
template int tri_batch<int64_t>(int64_t, const int64_t *, const int64_t *, const int64_t *, int64_t, int64_t,
                                const int64_t *, int64_t *, rbg_result_t *, char *, unsigned char *, size_t, uint32_t,
                                cudaStream_t, const RowStats &);

}  // namespace rbg

// Frees the DAG path's cached CUDA graphs (device memory is never held by this library outside
// rbg_fw_dense_noalloc's fixed array).
extern "C" int32_t rbg_release_scratch(void) {
    std::lock_guard<std::mutex> lk(rbg::g_tri_graph_mu);
    if (!rbg::g_tri_graphs.empty()) RBG_CUDA_TRY(cudaDeviceSynchronize());
    for (auto &g : rbg::g_tri_graphs) cudaGraphExecDestroy(g.exec);
    rbg::g_tri_graphs.clear();
    return RBG_OK;
}
