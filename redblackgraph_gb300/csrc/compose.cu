// compose.cu -- relational composition on sm_103a: the closure of a closed graph after adding
// one vertex or one edge, without recomputing the closure.
//
// References:
//   vertex: {{name}}_vertex_relational_composition, redblackgraph/core/src/redblackgraph/
//           relational_composition.c.in:166-262 (C core algebra, all storage types), and
//           vertex_relational_composition, redblackgraph/sparse/csgraph/_relational_composition.pyx:
//           10-64 (Cython int32 algebra, no cycle check);
//   edge:   {{name}}_edge_relational_composition, relational_composition.c.in:72-139, and
//           edge_relational_composition, _relational_composition.pyx:67-113.
//
// Vertex composition of closed R (n x n) with row vector u, column vector v and colour c:
//   uc = u (x) R, vc = R (x) v (steps 1 and 2); a k with uc[k] != 0 and vc[k] != 0 is a cycle
//   (step 3, C core only); out = R (+) vc (x) uc, out[n][:] = uc, out[:][n] = vc, out[n][n] = c.
// Edge composition (alpha -> beta with relationship r): u' = row alpha of R with column beta
//   replaced by r (when r != 0); out[alpha][:] = u' (x) R; every other row m:
//   out[m][p] = R[m][p] (+) R[m][alpha] (x) out[alpha][p] where out[alpha][p] != 0, else R[m][p].
//
// Design.  A product with a zero operand is zero and raises nothing, so only the non-zero
// operands matter: step 1 reads the rows of R where u (u') is non-zero (one thread per column,
// rows split over blocks, ⊕ combined with an order-encoded atomicMin), step 2 the columns where
// v is non-zero (one warp per row), and the update touches only the rectangle
// {m : vc[m] != 0} x {p : uc[p] != 0} (ordered lists from CUB select).  With out == R (same
// pointer and leading dimension) the update is in place and nothing else is copied; otherwise R
// is first copied into out with one 2-D copy.  The C core reports errors through PyErr_Format
// and keeps looping, so the exception it finally raises is the last one set, unless its MSB
// loop never returns (a negative signed operand): every event is numbered by its position in
// the reference's loop order and the last overflow, first never-returning product and first
// cycle index are kept; one thread then decides the outcome in the reference's order and
// reads back the deciding operands.
#include <cuda_runtime.h>
#include <cub/cub.cuh>
#include <thrust/iterator/counting_iterator.h>
#include <climits>
#include "rbg_internal.cuh"

namespace rbg {

namespace {

struct CmpStatus {
    unsigned flags;                  // RBG_EV_* of every product
    unsigned pad;
    unsigned long long ovf_seq1;     // 1 + loop index of the last overflow event (0: none)
    unsigned long long hang_seq;     // loop index of the first never-returning product (~0: none)
    long long cycle;                 // first k with uc[k] != 0 and vc[k] != 0 (LLONG_MAX: none)
    // operands of the step 1/2 candidates, noted before an in-place update can change R
    unsigned long long pre_hang_seq, pre_ovf_seq1;
    long long pre_hang_a, pre_hang_b, pre_ovf_a, pre_ovf_b;
    // decided by the finishing thread
    int status;
    unsigned ev;
    long long step, i, j, lhs, rhs;
    long long n_rows, n_cols;        // rectangle sizes (counts from the selects)
};

// C core (+): all ones absorbs, zero is the identity, else the unsigned minimum -> keys with
// all ones first and zero last.
template <typename T> __device__ __forceinline__ unsigned long long core_key(T x) {
    typedef typename utype<T>::type U;
    const U u = (U)x;
    if (u == (U)~(U)0) return 0ull;
    if (u == 0) return ~0ull;
    return (unsigned long long)u;
}
template <typename T> __device__ __forceinline__ T core_unkey(unsigned long long k) {
    typedef typename utype<T>::type U;
    if (k == 0ull) return (T)(U)~(U)0;
    if (k == ~0ull) return (T)0;
    return (T)(U)k;
}
// Cython (+) on int32: signed minimum of the non-zero values.
__device__ __forceinline__ unsigned long long cy_key(int32_t x) {
    return x == 0 ? (1ull << 32) : (unsigned long long)((uint32_t)x ^ 0x80000000u);
}
__device__ __forceinline__ int32_t cy_unkey(unsigned long long k) {
    return k >= (1ull << 32) ? 0 : (int32_t)((uint32_t)k ^ 0x80000000u);
}

template <typename T, bool CY> __device__ __forceinline__ unsigned long long sum_key(T x) {
    if constexpr (CY) return cy_key((int32_t)x);
    else return core_key<T>(x);
}
template <typename T, bool CY> __device__ __forceinline__ T sum_unkey(unsigned long long k) {
    if constexpr (CY) return (T)cy_unkey(k);
    else return core_unkey<T>(k);
}
template <typename T, bool CY> __device__ __forceinline__ T sum2(T a, T b) {
    if constexpr (CY) return (T)cy_sum((int32_t)a, (int32_t)b);
    else return avos_sum<T>(a, b);
}

// Product with its events numbered `seq` in the reference's loop order.
template <typename T, bool CY>
__device__ __forceinline__ T cmp_product(T a, T b, unsigned long long seq, CmpStatus *st) {
    if constexpr (CY) {
        return (T)cy_product((int32_t)a, (int32_t)b);
    } else {
        unsigned ev = 0;
        const T p = (T)avos_product<T>(a, b, ev);
        if (ev) {
            atomicOr(&st->flags, ev);
            if (ev & RBG_EV_HANG) atomicMin(&st->hang_seq, seq);
            else atomicMax(&st->ovf_seq1, seq + 1);
        }
        return p;
    }
}

// ---------------------------------------------------------------------------- selections
template <typename T> struct NonZeroAt {
    const T *x;
    int64_t stride;
    __device__ __forceinline__ bool operator()(const int &i) const { return x[(int64_t)i * stride] != 0; }
};
// Edge step 1 left operand: row alpha with column beta replaced by r.  The C core replaces
// only a non-zero r and compares the loop index in the storage type ((T)i == beta); the Cython
// code assigns R[alpha][beta] = r whatever r is.
template <typename T> struct EdgeLhs {
    const T *row;
    int64_t beta;
    T np;
    bool cy;
    __device__ __forceinline__ T operator()(int64_t i) const {
        const bool hit = cy ? (i == beta) : (np != 0 && (T)i == (T)beta);
        return hit ? np : row[i];
    }
};
template <typename T> struct EdgeLhsNonZero {
    EdgeLhs<T> f;
    __device__ __forceinline__ bool operator()(const int &i) const { return f(i) != 0; }
};
// Rows other than alpha (the C core compares in the storage type, (T)m != alpha) whose
// column-alpha entry is non-zero.
template <typename T> struct EdgeRow {
    const T *col;
    int64_t ld;
    int64_t alpha;
    bool cy;
    __device__ __forceinline__ bool operator()(const int &m) const {
        const bool skip = cy ? (m == alpha) : ((T)m == (T)alpha);
        return !skip && col[(int64_t)m * ld] != 0;
    }
};
template <typename T> struct ColAt {
    const T *c;
    int64_t ld;
    __device__ __forceinline__ T operator()(int64_t m) const { return c[m * ld]; }
};
struct CmpAll {
    __device__ __forceinline__ bool operator()(const int &) const { return true; }
};

// values of the selected left operands (list order)
template <typename T, typename F>
__global__ void cmp_lhs_gather_kernel(const int *list, const int *count, F f, T *vals) {
    const int c = *count;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < c; k += gridDim.x * blockDim.x) vals[k] = f(list[k]);
}

template <typename T> struct VecAt {
    const T *x;
    __device__ __forceinline__ T operator()(int64_t i) const { return x[i]; }
};

// ---------------------------------------------------------------------------- step 1
// uc[p] = (+)_k lval[k] (x) R[list[k]][p]; sequence p * n + list[k].  One thread per column, the
// list split in chunks of CHUNK over blockIdx.y; partial sums meet in ukey by atomicMin.
// Cython edge composition reads R with R[alpha][beta] = r (the Cython code edits R in place).
constexpr int CMP_CHUNK = 64;
template <typename T, bool CY>
__global__ void cmp_colreduce_kernel(int64_t n, const T *R, int64_t ldr, const int *list, const int *count,
                                     const T *lval, unsigned long long *ukey, CmpStatus *st,
                                     int64_t sub_i, int64_t sub_j, T sub_v) {
    const int c = *count;
    for (int k0 = blockIdx.y * CMP_CHUNK; k0 < c; k0 += gridDim.y * CMP_CHUNK) {
        const int k1 = min(c, k0 + CMP_CHUNK);
        for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
            T acc = 0;
            for (int k = k0; k < k1; ++k) {
                const int64_t i = list[k];
                T r = R[i * ldr + p];
                if (CY && i == sub_i && p == sub_j) r = sub_v;
                if (r == 0) continue;
                acc = sum2<T, CY>(acc, cmp_product<T, CY>(lval[k], r, (unsigned long long)p * n + i, st));
            }
            if (acc != 0) atomicMin(ukey + p, sum_key<T, CY>(acc));
        }
    }
}

template <typename T, bool CY>
__global__ void cmp_unkey_kernel(int64_t n, const unsigned long long *ukey, T *uc) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
        uc[p] = sum_unkey<T, CY>(ukey[p]);
}

// ---------------------------------------------------------------------------- step 2
// vc[m] = (+)_k R[m][list[k]] (x) vval[k]; sequence n^2 + m n + list[k].  One warp per row.
template <typename T, bool CY>
__global__ void cmp_rowreduce_kernel(int64_t n, const T *R, int64_t ldr, const int *list, const int *count,
                                     const T *vval, T *vc, CmpStatus *st) {
    const int c = *count;
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const unsigned long long nn = (unsigned long long)n * n;
    for (int64_t m = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); m < n; m += warps) {
        unsigned long long key = sum_key<T, CY>((T)0);
        for (int k = lane; k < c; k += 32) {
            const int64_t j = list[k];
            const T r = R[m * ldr + j];
            if (r == 0) continue;
            const T pr = cmp_product<T, CY>(r, vval[k], nn + (unsigned long long)m * n + j, st);
            key = min(key, sum_key<T, CY>(pr));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) key = min(key, __shfl_xor_sync(0xffffffffu, key, o));
        if (lane == 0) vc[m] = sum_unkey<T, CY>(key);
    }
}

// ---------------------------------------------------------------------------- step 3
template <typename T>
__global__ void cmp_cycle_kernel(int64_t n, const T *uc, const T *vc, CmpStatus *st) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        if (uc[k] != 0 && vc[k] != 0) atomicMin(&st->cycle, (long long)k);
}

// ---------------------------------------------------------------------------- update
// out[m][p] = R[m][p] (+) lhs_m (x) uc[p] over rows m of `rows` (left operand rlhs[k] of
// row rows[k]) and columns p of `cols`; sequence base + m n + p.  One block per row.
template <typename T, bool CY>
__global__ void cmp_rect_kernel(int64_t n, const T *R, int64_t ldr, T *out, int64_t ldo, const int *rows,
                                const int *nrows, const T *rlhs, const int *cols, const int *ncols, const T *uc,
                                unsigned long long base, CmpStatus *st) {
    const int nr = *nrows, nc = *ncols;
    for (int k = blockIdx.x; k < nr; k += gridDim.x) {
        const int64_t m = rows[k];
        const T lhs = rlhs[k];
        for (int q = threadIdx.x; q < nc; q += blockDim.x) {
            const int64_t p = cols[q];
            const T pr = cmp_product<T, CY>(lhs, uc[p], base + (unsigned long long)m * n + p, st);
            out[m * ldo + p] = sum2<T, CY>(R[m * ldr + p], pr);
        }
    }
}

// new row n, column n and corner (vertex), or the new row alpha (edge)
template <typename T>
__global__ void cmp_vertex_border_kernel(int64_t n, const T *uc, const T *vc, T color, T *out, int64_t ldo) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k <= n; k += (int64_t)gridDim.x * blockDim.x) {
        out[n * ldo + k] = k < n ? uc[k] : color;
        if (k < n) out[k * ldo + n] = vc[k];
    }
}
template <typename T>
__global__ void cmp_row_write_kernel(int64_t n, const T *uc, T *out_row) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        out_row[k] = uc[k];
}

// ---------------------------------------------------------------------------- outcome
// Operands of a step 1 or step 2 product, numbered as in cmp_colreduce_kernel /
// cmp_rowreduce_kernel (vertex) or the edge update.
template <typename T>
__device__ __forceinline__ void cmp_operands12(unsigned long long seq, int64_t n, int vertex, const T *R,
                                               int64_t ldr, const T *u, const T *v, const T *uc, EdgeLhs<T> el,
                                               const int *rows, const int *nrows, const T *rlhs, T &a, T &b) {
    const unsigned long long nn = (unsigned long long)n * n;
    if (seq < nn) {                              // step 1: column p = seq / n, row i = seq % n
        const int64_t p = (int64_t)(seq / n), i = (int64_t)(seq % n);
        a = vertex ? u[i] : el(i);
        b = R[i * ldr + p];
    } else {                                     // step 2: row m, column j (vertex) / p (edge)
        const int64_t m = (int64_t)((seq - nn) / n), j = (int64_t)((seq - nn) % n);
        if (vertex) {
            a = R[m * ldr + j];
            b = v[j];
        } else {                                 // R[m][alpha] as it was: the sorted row list
            int lo = 0, hi = *nrows;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (rows[mid] < m) lo = mid + 1; else hi = mid;
            }
            a = rlhs[lo];
            b = uc[j];
        }
    }
}

// Before the update: note the operands of the first never-returning product and of the last
// overflowing one seen so far (steps 1 and 2 read R, which an in-place update then changes).
template <typename T>
__global__ void cmp_note_kernel(int64_t n, int vertex, const T *R, int64_t ldr, const T *u, const T *v,
                                EdgeLhs<T> el, CmpStatus *st) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    T a = 0, b = 0;
    st->pre_hang_seq = st->hang_seq;
    if (st->hang_seq != ~0ull) {
        cmp_operands12<T>(st->hang_seq, n, vertex, R, ldr, u, v, nullptr, el, nullptr, nullptr, nullptr, a, b);
        st->pre_hang_a = (long long)a;
        st->pre_hang_b = (long long)b;
    }
    st->pre_ovf_seq1 = st->ovf_seq1;
    if (st->ovf_seq1) {
        cmp_operands12<T>(st->ovf_seq1 - 1, n, vertex, R, ldr, u, v, nullptr, el, nullptr, nullptr, nullptr, a, b);
        st->pre_ovf_a = (long long)a;
        st->pre_ovf_b = (long long)b;
    }
}

// Decide the reference's outcome and read the deciding operands.  `vertex` selects the vertex
// loop structure (steps 1, 2, the cycle check, 4), else the edge one (steps 1, 2).
template <typename T>
__global__ void cmp_finish_kernel(int64_t n, int vertex, const T *uc, const T *vc, const int *rows,
                                  const int *nrows, const T *rlhs, const int *ncols, CmpStatus *st) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const unsigned long long nn = (unsigned long long)n * n;
    const bool hang = st->hang_seq != ~0ull;
    unsigned long long seq = 0;
    int status = RBG_OK;
    if (vertex && hang && st->hang_seq < 2 * nn) {
        status = RBG_ERR_OVERFLOW; seq = st->hang_seq;
    } else if (vertex && st->cycle != LLONG_MAX) {
        status = RBG_ERR_CYCLE;
    } else if (hang) {
        status = RBG_ERR_OVERFLOW; seq = st->hang_seq;
    } else if (st->ovf_seq1) {
        status = RBG_ERR_OVERFLOW; seq = st->ovf_seq1 - 1;
    }
    st->status = status;
    st->n_rows = *nrows;
    st->n_cols = *ncols;
    st->ev = 0;
    if (status == RBG_OK) return;
    if (status == RBG_ERR_CYCLE) {
        const long long k = st->cycle;
        st->step = 3; st->i = k; st->j = n;
        st->lhs = (long long)uc[k]; st->rhs = (long long)vc[k];
        return;
    }
    T a = 0, b = 0;
    long long step, i, j;
    const unsigned long long last = vertex ? 2 * nn : nn;   // loops whose operands were noted
    if (seq < nn) {
        step = 1; j = (long long)(seq / n); i = (long long)(seq % n);
    } else if (seq < 2 * nn) {
        step = 2; i = (long long)((seq - nn) / n); j = (long long)((seq - nn) % n);
    } else {
        step = 4; i = (long long)((seq - 2 * nn) / n); j = (long long)((seq - 2 * nn) % n);
    }
    if (seq < last) {
        if (hang && seq == st->pre_hang_seq) { a = (T)st->pre_hang_a; b = (T)st->pre_hang_b; }
        else { a = (T)st->pre_ovf_a; b = (T)st->pre_ovf_b; }
    } else if (vertex) {                         // step 4: vc[m] (x) uc[p]
        a = vc[i]; b = uc[j];
    } else {                                     // edge step 2: R[m][alpha] (x) out[alpha][p]
        int lo = 0, hi = *nrows;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (rows[mid] < i) lo = mid + 1; else hi = mid;
        }
        a = rlhs[lo]; b = uc[j];
    }
    unsigned ev = 0;
    avos_product<T>(a, b, ev);
    st->step = step; st->i = i; st->j = j;
    st->lhs = (long long)a; st->rhs = (long long)b;
    st->ev = ev;
}

struct CmpWs {
    CmpStatus *st;
    unsigned long long *ukey;
    void *uc, *vc, *lval, *vval, *rlhs;
    int *list_u, *list_v, *rows, *cols, *counts;  // counts: [0] list_u, [1] list_v, [2] rows, [3] cols
    void *tmp;
    size_t tmp_bytes;
};

size_t cmp_tmp_bytes(int64_t n) {
    size_t b = 0;
    cub::DeviceSelect::If(nullptr, b, thrust::counting_iterator<int>(0), (int *)nullptr, (int *)nullptr,
                          (int)std::max<int64_t>(n, 1), CmpAll());
    return b + 1024;                             // predicates differ in type, not in scratch need
}

size_t cmp_layout(int64_t n, int elem, unsigned char *base, CmpWs *w) {
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o = align_up(o + bytes, 256); return base ? base + at : nullptr; };
    const size_t nv = (size_t)std::max<int64_t>(n, 1) * elem, ni = (size_t)std::max<int64_t>(n, 1) * 4;
    unsigned char *p;
    p = take(sizeof(CmpStatus)); if (w) w->st = (CmpStatus *)p;
    p = take((size_t)std::max<int64_t>(n, 1) * 8); if (w) w->ukey = (unsigned long long *)p;
    p = take(nv); if (w) w->uc = p;
    p = take(nv); if (w) w->vc = p;
    p = take(nv); if (w) w->lval = p;
    p = take(nv); if (w) w->vval = p;
    p = take(nv); if (w) w->rlhs = p;
    p = take(ni); if (w) w->list_u = (int *)p;
    p = take(ni); if (w) w->list_v = (int *)p;
    p = take(ni); if (w) w->rows = (int *)p;
    p = take(ni); if (w) w->cols = (int *)p;
    p = take(64); if (w) w->counts = (int *)p;
    const size_t tb = cmp_tmp_bytes(n);
    p = take(tb); if (w) { w->tmp = p; w->tmp_bytes = tb; }
    return o;
}

int cmp_grid(int64_t work, int threads) { return grid_for(std::max<int64_t>(work, 1), threads); }

template <typename F>
int cmp_select(const CmpWs &w, int64_t n, F pred, int *out, int *count, cudaStream_t s) {
    size_t tb = w.tmp_bytes;
    RBG_CUDA_TRY(cub::DeviceSelect::If(w.tmp, tb, thrust::counting_iterator<int>(0), out, count, (int)n, pred, s));
    return RBG_OK;
}

void fill_result(const CmpStatus &h, rbg_compose_result_t *res) {
    const bool ok = h.status == RBG_OK;
    res->status = h.status;
    res->flags = h.flags;
    res->event = h.status == RBG_ERR_OVERFLOW ? h.ev : 0u;
    res->reserved = 0;
    res->step = ok ? -1 : h.step;
    res->i = ok ? -1 : h.i;
    res->j = ok ? -1 : h.j;
    res->lhs = ok ? 0 : h.lhs;
    res->rhs = ok ? 0 : h.rhs;
    res->updated = (int64_t)h.n_rows * h.n_cols;
}

int cmp_status_init(const CmpWs &w, cudaStream_t s) {
    CmpStatus h;
    memset(&h, 0, sizeof(h));
    h.hang_seq = ~0ull;
    h.cycle = LLONG_MAX;
    h.status = RBG_OK;
    RBG_CUDA_TRY(cudaMemcpyAsync(w.st, &h, sizeof(h), cudaMemcpyHostToDevice, s));
    RBG_CUDA_TRY(cudaMemsetAsync(w.counts, 0, 64, s));
    return RBG_OK;
}

int cmp_read_counts(const CmpWs &w, int *h, cudaStream_t s) {
    RBG_CUDA_TRY(cudaMemcpyAsync(h, w.counts, 4 * sizeof(int), cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    return RBG_OK;
}

dim3 cmp_colreduce_grid(int64_t n, int count) {
    const int64_t gx = std::min<int64_t>((n + 255) / 256, 1024);
    const int64_t gy = std::min<int64_t>(std::max<int64_t>((count + CMP_CHUNK - 1) / CMP_CHUNK, 1), 1024);
    return dim3((unsigned)std::max<int64_t>(gx, 1), (unsigned)gy);
}

template <typename T, bool CY>
int vertex_t(int64_t n, const T *R, int64_t ldr, const T *u, const T *v, T color, T *out, int64_t ldo,
             const CmpWs &w, rbg_compose_result_t *res, cudaStream_t s) {
    T *uc = reinterpret_cast<T *>(w.uc), *vc = reinterpret_cast<T *>(w.vc);
    T *lval = reinterpret_cast<T *>(w.lval), *vval = reinterpret_cast<T *>(w.vval);
    T *rlhs = reinterpret_cast<T *>(w.rlhs);
    int rc = cmp_status_init(w, s);
    if (rc) return rc;
    if (n > 0 && (out != R || ldo != ldr))
        RBG_CUDA_TRY(cudaMemcpy2DAsync(out, ldo * sizeof(T), R, ldr * sizeof(T), n * sizeof(T), n,
                                       cudaMemcpyDeviceToDevice, s));
    int hc[4] = {0, 0, 0, 0};
    if (n > 0) {
        RBG_CUDA_TRY(cudaMemsetAsync(w.ukey, 0xff, (size_t)n * 8, s));
        // steps 1 and 2 over the non-zero entries of u and v
        rc = cmp_select(w, n, NonZeroAt<T>{u, 1}, w.list_u, w.counts + 0, s); if (rc) return rc;
        rc = cmp_select(w, n, NonZeroAt<T>{v, 1}, w.list_v, w.counts + 1, s); if (rc) return rc;
        rc = cmp_read_counts(w, hc, s); if (rc) return rc;
        note_launches(5 + (CY ? 0 : 2));
        cmp_lhs_gather_kernel<<<cmp_grid(hc[0], 256), 256, 0, s>>>(w.list_u, w.counts + 0, VecAt<T>{u}, lval);
        cmp_lhs_gather_kernel<<<cmp_grid(hc[1], 256), 256, 0, s>>>(w.list_v, w.counts + 1, VecAt<T>{v}, vval);
        if (hc[0] > 0)
            cmp_colreduce_kernel<T, CY><<<cmp_colreduce_grid(n, hc[0]), 256, 0, s>>>(
                n, R, ldr, w.list_u, w.counts + 0, lval, w.ukey, w.st, -1, -1, T(0));
        cmp_unkey_kernel<T, CY><<<cmp_grid(n, 256), 256, 0, s>>>(n, w.ukey, uc);
        cmp_rowreduce_kernel<T, CY><<<cmp_grid(n * 32, 256), 256, 0, s>>>(n, R, ldr, w.list_v, w.counts + 1, vval,
                                                                         vc, w.st);
        if (!CY) {
            cmp_cycle_kernel<T><<<cmp_grid(n, 256), 256, 0, s>>>(n, uc, vc, w.st);
            cmp_note_kernel<T><<<1, 32, 0, s>>>(n, 1, R, ldr, u, v, EdgeLhs<T>{nullptr, 0, T(0), false}, w.st);
        }
        // step 4 on the rectangle {vc != 0} x {uc != 0}
        rc = cmp_select(w, n, NonZeroAt<T>{vc, 1}, w.rows, w.counts + 2, s); if (rc) return rc;
        rc = cmp_select(w, n, NonZeroAt<T>{uc, 1}, w.cols, w.counts + 3, s); if (rc) return rc;
        rc = cmp_read_counts(w, hc, s); if (rc) return rc;
        if (hc[2] > 0 && hc[3] > 0) {
            note_launches(2);
            cmp_lhs_gather_kernel<<<cmp_grid(hc[2], 256), 256, 0, s>>>(w.rows, w.counts + 2, VecAt<T>{vc}, rlhs);
            cmp_rect_kernel<T, CY><<<cmp_grid((int64_t)hc[2] * 256, 256), 256, 0, s>>>(
                n, R, ldr, out, ldo, w.rows, w.counts + 2, rlhs, w.cols, w.counts + 3, uc,
                2ull * (unsigned long long)n * n, w.st);
        }
    }
    note_launches(2);
    cmp_vertex_border_kernel<T><<<cmp_grid(n + 1, 256), 256, 0, s>>>(n, uc, vc, color, out, ldo);
    cmp_finish_kernel<T><<<1, 32, 0, s>>>(n, 1, uc, vc, w.rows, w.counts + 2, rlhs, w.counts + 3, w.st);
    RBG_CUDA_TRY(cudaGetLastError());
    CmpStatus h;
    RBG_CUDA_TRY(cudaMemcpyAsync(&h, w.st, sizeof(h), cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    fill_result(h, res);
    return RBG_OK;
}

template <typename T, bool CY>
int edge_t(int64_t n, const T *R, int64_t ldr, int64_t alpha, int64_t beta, T np, T *out, int64_t ldo,
           const CmpWs &w, rbg_compose_result_t *res, cudaStream_t s) {
    T *uc = reinterpret_cast<T *>(w.uc), *lval = reinterpret_cast<T *>(w.lval);
    T *rlhs = reinterpret_cast<T *>(w.rlhs);
    int rc = cmp_status_init(w, s);
    if (rc) return rc;
    if (out != R || ldo != ldr)
        RBG_CUDA_TRY(cudaMemcpy2DAsync(out, ldo * sizeof(T), R, ldr * sizeof(T), n * sizeof(T), n,
                                       cudaMemcpyDeviceToDevice, s));
    RBG_CUDA_TRY(cudaMemsetAsync(w.ukey, 0xff, (size_t)n * 8, s));
    const EdgeLhs<T> lhs{R + alpha * ldr, beta, np, CY};
    int hc[4] = {0, 0, 0, 0};
    rc = cmp_select(w, n, EdgeLhsNonZero<T>{lhs}, w.list_u, w.counts + 0, s); if (rc) return rc;
    rc = cmp_read_counts(w, hc, s); if (rc) return rc;
    note_launches(3 + (CY ? 0 : 1));
    cmp_lhs_gather_kernel<<<cmp_grid(hc[0], 256), 256, 0, s>>>(w.list_u, w.counts + 0, lhs, lval);
    // the Cython code reads R with R[alpha][beta] = r during the product
    if (hc[0] > 0)
        cmp_colreduce_kernel<T, CY><<<cmp_colreduce_grid(n, hc[0]), 256, 0, s>>>(
            n, R, ldr, w.list_u, w.counts + 0, lval, w.ukey, w.st, CY ? alpha : -1, CY ? beta : -1, np);
    cmp_unkey_kernel<T, CY><<<cmp_grid(n, 256), 256, 0, s>>>(n, w.ukey, uc);
    if (!CY) cmp_note_kernel<T><<<1, 32, 0, s>>>(n, 0, R, ldr, nullptr, nullptr, lhs, w.st);
    // rows m != alpha with R[m][alpha] != 0, columns p with out[alpha][p] != 0
    rc = cmp_select(w, n, EdgeRow<T>{R + alpha, ldr, alpha, CY}, w.rows, w.counts + 2, s); if (rc) return rc;
    rc = cmp_select(w, n, NonZeroAt<T>{uc, 1}, w.cols, w.counts + 3, s); if (rc) return rc;
    rc = cmp_read_counts(w, hc, s); if (rc) return rc;
    if (hc[2] > 0 && hc[3] > 0) {
        note_launches(2);
        cmp_lhs_gather_kernel<<<cmp_grid(hc[2], 256), 256, 0, s>>>(w.rows, w.counts + 2, ColAt<T>{R + alpha, ldr},
                                                                   rlhs);
        cmp_rect_kernel<T, CY><<<cmp_grid((int64_t)hc[2] * 256, 256), 256, 0, s>>>(
            n, R, ldr, out, ldo, w.rows, w.counts + 2, rlhs, w.cols, w.counts + 3, uc, (unsigned long long)n * n,
            w.st);
    }
    note_launches(2);
    cmp_finish_kernel<T><<<1, 32, 0, s>>>(n, 0, uc, nullptr, w.rows, w.counts + 2, rlhs, w.counts + 3, w.st);
    cmp_row_write_kernel<T><<<cmp_grid(n, 256), 256, 0, s>>>(n, uc, out + alpha * ldo);
    RBG_CUDA_TRY(cudaGetLastError());
    CmpStatus h;
    RBG_CUDA_TRY(cudaMemcpyAsync(&h, w.st, sizeof(h), cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    fill_result(h, res);
    return RBG_OK;
}

}  // namespace
}  // namespace rbg

using namespace rbg;

extern "C" int32_t rbg_compose_workspace_bytes(int32_t dtype, int64_t n, int64_t *bytes) {
    if (!bytes || n < 0 || n >= (1ll << 31) - 1 || dtype_bytes(dtype) == 0) return RBG_ERR_INVALID;
    *bytes = (int64_t)cmp_layout(n, dtype_bytes(dtype), nullptr, nullptr);
    return RBG_OK;
}

extern "C" int32_t rbg_vertex_compose(int32_t dtype, int64_t n, const void *R, int64_t ldr, const void *u,
                                      const void *v, int64_t color, void *out, int64_t ldo, uint32_t mode,
                                      void *workspace, int64_t workspace_bytes, rbg_compose_result_t *res,
                                      rbg_stream_t stream) {
    if (!res || n < 0 || n >= (1ll << 31) - 1 || dtype_bytes(dtype) == 0 || (n > 0 && (!R || !u || !v)) || !out ||
        ldr < n || ldo < n + 1 || ((mode & RBG_MODE_CYTHON) && dtype != RBG_DTYPE_INT32))
        return RBG_ERR_INVALID;
    if (out == R && ldo != ldr) return RBG_ERR_INVALID;
    if (!workspace || workspace_bytes < (int64_t)cmp_layout(n, dtype_bytes(dtype), nullptr, nullptr))
        return RBG_ERR_NOMEM;
    CmpWs w;
    cmp_layout(n, dtype_bytes(dtype), reinterpret_cast<unsigned char *>(workspace), &w);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int rc = RBG_ERR_INVALID;
    if (mode & RBG_MODE_CYTHON) {
        rc = vertex_t<int32_t, true>(n, (const int32_t *)R, ldr, (const int32_t *)u, (const int32_t *)v,
                                     (int32_t)color, (int32_t *)out, ldo, w, res, s);
    } else {
        RBG_DISPATCH_DTYPE(dtype, T,
            rc = (vertex_t<T, false>(n, (const T *)R, ldr, (const T *)u, (const T *)v, (T)color, (T *)out, ldo,
                                     w, res, s)));
    }
    return rc;
}

extern "C" int32_t rbg_edge_compose(int32_t dtype, int64_t n, const void *R, int64_t ldr, int64_t alpha,
                                    int64_t beta, int64_t relationship, void *out, int64_t ldo, uint32_t mode,
                                    void *workspace, int64_t workspace_bytes, rbg_compose_result_t *res,
                                    rbg_stream_t stream) {
    if (!res || n <= 0 || n >= (1ll << 31) - 1 || dtype_bytes(dtype) == 0 || !R || !out || ldr < n || ldo < n ||
        alpha < 0 || alpha >= n || beta < 0 || beta >= n || ((mode & RBG_MODE_CYTHON) && dtype != RBG_DTYPE_INT32))
        return RBG_ERR_INVALID;
    if (out == R && ldo != ldr) return RBG_ERR_INVALID;
    if (!workspace || workspace_bytes < (int64_t)cmp_layout(n, dtype_bytes(dtype), nullptr, nullptr))
        return RBG_ERR_NOMEM;
    CmpWs w;
    cmp_layout(n, dtype_bytes(dtype), reinterpret_cast<unsigned char *>(workspace), &w);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int rc = RBG_ERR_INVALID;
    if (mode & RBG_MODE_CYTHON) {
        rc = edge_t<int32_t, true>(n, (const int32_t *)R, ldr, alpha, beta, (int32_t)relationship, (int32_t *)out,
                                   ldo, w, res, s);
    } else {
        RBG_DISPATCH_DTYPE(dtype, T,
            rc = (edge_t<T, false>(n, (const T *)R, ldr, alpha, beta, (T)relationship, (T *)out, ldo, w, res, s)));
    }
    return rc;
}
