// spgemm.cu -- sparse AVOS product C = A (x) B (CSR) and the squaring-closure step, sm_103a.
//
// References (paths within rappdw/redblackgraph):
//   rb_matrix @      redblackgraph/sparse/rbm.py:39-122 -> rbm_matmat_pass1/pass2
//                    redblackgraph/sparse/sparsetools/rbm_math.h:117-222 (values upcast to 64 bit,
//                    C core scalar semantics, zero sums dropped, result cast back)
//   gpu spgemm       redblackgraph/gpu/spgemm.py:32-119, spgemm_numeric.py:104-176 (int32 values,
//                    the Cython scalar semantics, optional j >= i mask)
//   squaring merge   redblackgraph/sparse/csgraph/transitive_closure.py:272-357 and
//                    redblackgraph/gpu/transitive_closure.py:77-156 (R (+) R^2 taken per cell as
//                    the value of smallest magnitude, R's value on a tie, zeros dropped)
//
// Design: one pass per output row, no global sort and no global hash.  A warp takes a row,
// walks its candidates (every product A[i,k] (x) B[k,j], plus R[i,.] for a squaring step) in
// place and folds them into a shared-memory table keyed by column; the distinct columns are
// sorted and reduced: the (+) of the products of a column, then, for a squaring step, the
// magnitude merge with R's entry.  Rows with more distinct columns than the warp table holds
// are redone one per block with a sort of their candidates; rows of more than 8192 candidates
// use a dense per-block accumulator in the workspace.  The output of every row is written
// compacted (columns ascending) at the row's candidate offset; a scan of the row counts and a
// gather produce the final CSR.
#include <cuda_runtime.h>
#include <cub/cub.cuh>
#include <string.h>
#include <algorithm>
#include <vector>
#include "rbg_internal.cuh"

namespace rbg {

constexpr int SP_BLOCK_CAP = 8192;    // candidates per block row
constexpr int SP_BLOCK_THREADS = 512;
constexpr int SP_DENSE_BLOCKS = 8;    // concurrent dense-accumulator rows (one scratch slot each)

// semantics of the scalar algebra
constexpr int SEM_C64 = 0;   // C core on 64-bit compute values (rb_matrix @)
constexpr int SEM_CY32 = 1;  // Cython semantics on int32 (the gpu module)

// Products and sums: for SEM_C64 the compute values are the storage values widened to 64 bits
// (unsigned storage uses the unsigned 64-bit algebra with RED_ONE widened to all ones).
// NARROW: signed values of 4-byte storage (below 2^31), whose splice mostly fits 32 bits.
template <int SEM, bool UNS, bool NARROW = false>
__device__ __forceinline__ long long sp_mul(long long a, long long b, unsigned &ev) {
    if (SEM == SEM_CY32) return (long long)cy_product((int32_t)a, (int32_t)b);
    if (!UNS) {
        // signed storage, the cases of pedigree data without the general function's branches
        // (rbg_math.c.in:48-121): two plain values; a zero; the identities -1 (keeps an even
        // left value) and 1 (keeps an odd one) on the right; an identity on the left (gives the
        // right value); two identities (equal: itself, else 0)
        if (a >= 2 && b >= 2) {
            if (NARROW) {
                const unsigned x = (unsigned)a, y = (unsigned)b;
                const int bp = 31 - __clz((int)y), mx = 31 - __clz((int)x);
                if (mx + bp < 31) return (long long)((x << bp) | (y ^ (1u << bp)));
            }
            const unsigned long long x = (unsigned long long)a, y = (unsigned long long)b;
            const int bp = 63 - __clzll((long long)y), mx = 63 - __clzll((long long)x);
            if (mx + bp >= 64) ev |= RBG_EV_OVF_SIZE;
            const unsigned long long r = (x << bp) | (y ^ (1ull << bp));
            if (~r == 0) ev |= RBG_EV_OVF_ONES;
            return (long long)r;
        }
        if (a == 0 || b == 0) return 0;
        const bool ai = a == 1 || a == -1, bi = b == 1 || b == -1;
        if (bi && a >= 2) return ((a & 1) == (b == 1 ? 1 : 0)) ? a : 0;
        if (ai && b >= 2) return b;
        if (ai && bi) return a == b ? a : 0;
        return (long long)avos_product<int64_t>((int64_t)a, (int64_t)b, ev);   // negative: never returns there
    }
    // both operands plain values (neither 0, 1, the red one nor, signed, negative): the bit
    // splice with the C core's two overflow tests, without the identity and sign cases
    const unsigned long long x = (unsigned long long)a, y = (unsigned long long)b;
    const bool plain = UNS ? (x >= 2 && y >= 2 && ~x != 0 && ~y != 0) : (a >= 2 && b >= 2);
    if (plain) {
        const int bp = 63 - __clzll((long long)y), mx = 63 - __clzll((long long)x);
        if (mx + bp >= 64) ev |= RBG_EV_OVF_SIZE;
        const unsigned long long r = (x << bp) | (y ^ (1ull << bp));
        if (~r == 0) ev |= RBG_EV_OVF_ONES;
        return (long long)r;
    }
    if (UNS) return (long long)avos_product<uint64_t>((uint64_t)a, (uint64_t)b, ev);
    return (long long)avos_product<int64_t>((int64_t)a, (int64_t)b, ev);
}

// a stored value widened to the 64-bit compute value (compile-time storage width)
template <int BYTES, bool UNS>
__device__ __forceinline__ long long sp_load_t(const void *x, int64_t i) {
    if (BYTES == 8) return ((const long long *)x)[i];
    const int v = ((const int *)x)[i];
    if (UNS) return v == -1 ? -1ll : (long long)(unsigned)v;   // RED_ONE widens to all ones
    return (long long)v;
}
template <int SEM, bool UNS>
__device__ __forceinline__ long long sp_add(long long a, long long b) {
    if (SEM == SEM_CY32) return (long long)cy_sum((int32_t)a, (int32_t)b);
    if (UNS) return (long long)avos_sum<uint64_t>((uint64_t)a, (uint64_t)b);
    return (long long)avos_sum<int64_t>((int64_t)a, (int64_t)b);
}

// Value as the storage type holds it: C-core results are computed in 64 bits and cast back to
// the storage width (rbm.py:120-121), wrapping like numpy's astype.
__device__ __forceinline__ long long sp_trunc(long long v, int bytes, int uns) {
    if (bytes == 8) return v;
    return uns ? (long long)(unsigned)v : (long long)(int)v;
}

// Magnitude merge of the squaring step: the smaller |value| wins, R's value on a tie (R comes
// first in the reference's stable sort).  Magnitudes are taken in the storage type.
__device__ __forceinline__ long long sp_minabs(long long r, long long s, int uns) {
    unsigned long long ar = uns ? (unsigned long long)r : (r < 0 ? 0ull - (unsigned long long)r : (unsigned long long)r);
    unsigned long long as = uns ? (unsigned long long)s : (s < 0 ? 0ull - (unsigned long long)s : (unsigned long long)s);
    return as < ar ? s : r;
}

struct SpArgs {
    int64_t n_rows, n_cols;
    const int64_t *ap; const int *aj; const void *ax;   // A (CSR, int64 row pointers)
    const int64_t *bp; const int *bj; const void *bx;   // B
    const int64_t *rp; const int *rj; const void *rx;   // R for a squaring step (or null)
    int upper;                                          // keep only j >= i
    int elem_bytes;                                     // storage value bytes (4 or 8)
    int uns;                                            // unsigned storage
    int64_t *cand_off;                                  // exclusive scan of candidates (n+1)
    int *ocol; long long *oval;                         // per-row compacted output (temp)
    int64_t *rownnz;                                    // output count per row
    long long *dense_val; unsigned *dense_mark;         // dense accumulators (SP_DENSE_BLOCKS rows)
    int *big_rows; int *big_count;                      // rows for the block / dense kernels
    unsigned *flags;
    int2 *win;                                          // per row: first and last column it can reach
};

__device__ __forceinline__ long long sp_load(const void *x, int64_t i, int bytes, int uns) {
    if (bytes == 8) return ((const long long *)x)[i];
    const int v = ((const int *)x)[i];
    if (uns) return v == -1 ? -1ll : (long long)(unsigned)v;   // RED_ONE widens to all ones
    return (long long)v;
}

// ----------------------------------------------------------------------------- candidates
// cand[i] = sum over k in A[i] of nnz(B[k]) (+ nnz(R[i]) for a squaring step), and the row's
// column window win[i]: the first and last column of every B row it gathers and of R's row (the
// numeric pass folds rows whose window spans at most SP_WIN columns into a direct accumulator).
// Rows above the warp capacity are listed for the block / dense kernels.
__global__ void sp_count_kernel(SpArgs a, int64_t *cand) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= a.n_rows;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (i == a.n_rows) { cand[i] = 0; continue; }
        int64_t c = 0;
        int jlo = INT_MAX, jhi = -1;
        for (int64_t e = a.ap[i]; e < a.ap[i + 1]; ++e) {
            const int k = a.aj[e];
            const int64_t b0 = a.bp[k], b1 = a.bp[k + 1];
            if (b1 > b0) {
                c += b1 - b0;
                jlo = min(jlo, a.bj[b0]);
                jhi = max(jhi, a.bj[b1 - 1]);
            }
        }
        if (a.rp) {
            const int64_t r0 = a.rp[i], r1 = a.rp[i + 1];
            if (r1 > r0) {
                c += r1 - r0;
                jlo = min(jlo, a.rj[r0]);
                jhi = max(jhi, a.rj[r1 - 1]);
            }
        }
        a.win[i] = make_int2(jlo, jhi);
        cand[i] = c;
        if (c > SP_BLOCK_CAP) {      // the dense kernel's rows
            a.big_rows[atomicAdd(a.big_count, 1)] = (int)i;
            atomicAdd(a.big_count + 1, 1);
        }
    }
}

// Encoded candidate key: column << 1 | source (0 = R's own entry, 1 = a product), so that R's
// entry of a column sorts before the products of that column.
__device__ __forceinline__ unsigned sp_key(int col, int src) { return ((unsigned)col << 1) | (unsigned)src; }
constexpr unsigned SP_PAD = 0xffffffffu;

// Reduce the sorted run starting at `h` (keys[h] is the first key of its column) into one value;
// returns false when the column has no nonzero result.
template <int SEM, bool UNS>
__device__ __forceinline__ bool sp_reduce_run(const unsigned *keys, const long long *vals, int h, int cnt,
                                              bool merge, int bytes, long long &out) {
    const unsigned col = keys[h] >> 1;
    bool have_r = false;
    long long r = 0, s = 0;
    int e = h;
    if ((keys[e] & 1u) == 0) { have_r = true; r = vals[e]; ++e; }
    for (; e < cnt && (keys[e] >> 1) == col; ++e) s = sp_add<SEM, UNS>(s, vals[e]);
    if (!merge) {
        if (s == 0) return false;          // zero sums are dropped (rbm_math.h:207)
        out = (SEM == SEM_CY32) ? s : sp_trunc(s, bytes, UNS);
        return true;
    }
    long long v;
    if (s == 0) v = r;                     // no entry of R^2 in this column
    else {
        const long long s_t = (SEM == SEM_CY32) ? s : sp_trunc(s, bytes, UNS);
        v = have_r ? sp_minabs(r, s_t, UNS) : s_t;
    }
    v = (long long)(int)v;                 // the merged matrix is int32 (transitive_closure.py:327)
    if (v == 0) return false;
    out = v;
    return true;
}

// Append the candidates of row i to (keys, vals) at *cnt (shared), using the calling group of
// `nthreads` threads (a warp or a block); products use the group's lanes over each B row.
template <int SEM, bool UNS>
__device__ __forceinline__ void sp_gather(const SpArgs &a, int64_t i, bool merge, unsigned *keys, long long *vals,
                                          int *cnt, int lane, int nthreads, unsigned &ev) {
    if (merge && a.rp) {
        for (int64_t e = a.rp[i] + lane; e < a.rp[i + 1]; e += nthreads) {
            const int pos = atomicAdd(cnt, 1);
            keys[pos] = sp_key(a.rj[e], 0);
            vals[pos] = sp_load(a.rx, e, a.elem_bytes, a.uns);
        }
    }
    for (int64_t e = a.ap[i]; e < a.ap[i + 1]; ++e) {
        const int k = a.aj[e];
        const long long av = sp_load(a.ax, e, a.elem_bytes, a.uns);
        for (int64_t f = a.bp[k] + lane; f < a.bp[k + 1]; f += nthreads) {
            const int j = a.bj[f];
            if (a.upper && j < i) continue;
            const long long p = sp_mul<SEM, UNS>(av, sp_load(a.bx, f, a.elem_bytes, a.uns), ev);
            if (p == 0) continue;                    // a zero product adds nothing
            if (j == i && p != -1 && p != 1) ev |= RBG_EV_CYCLE;   // a vertex reaches itself
            const int pos = atomicAdd(cnt, 1);
            keys[pos] = sp_key(j, 1);
            vals[pos] = p;
        }
    }
}

struct WarpSync { __device__ void operator()() const { __syncwarp(); } };
struct BlockSync { __device__ void operator()() const { __syncthreads(); } };

// Bitonic sort of keys/vals[0, P) (P a power of two) by the calling group; sync() orders steps.
template <typename Sync>
__device__ __forceinline__ void sp_bitonic(unsigned *keys, long long *vals, int P, int lane, int nthreads, Sync sync) {
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int idx = lane; idx < P; idx += nthreads) {
                const int ixj = idx ^ j;
                if (ixj > idx) {
                    const bool up = (idx & k) == 0;
                    const unsigned ka = keys[idx], kb = keys[ixj];
                    if ((ka > kb) == up) {
                        keys[idx] = kb; keys[ixj] = ka;
                        const long long t = vals[idx]; vals[idx] = vals[ixj]; vals[ixj] = t;
                    }
                }
            }
            sync();
        }
    }
}

constexpr size_t SP_BLOCK_SMEM = (size_t)SP_BLOCK_CAP * 12 + 64;

// One row per block for the rows the warp kernel handed over (more distinct columns than its
// table holds) with at most SP_BLOCK_CAP candidates: gather, bitonic sort, reduce.
template <int SEM, bool UNS>
__global__ void __launch_bounds__(SP_BLOCK_THREADS)
sp_block_kernel(SpArgs a, int merge) {
    extern __shared__ __align__(16) unsigned char sp_smem[];
    long long *vals = reinterpret_cast<long long *>(sp_smem);
    unsigned *keys = reinterpret_cast<unsigned *>(vals + SP_BLOCK_CAP);
    __shared__ int scnt;
    __shared__ int wsum[SP_BLOCK_THREADS / 32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    unsigned ev = 0;
    const int nbig = *a.big_count;
    for (int b = blockIdx.x; b < nbig; b += gridDim.x) {
        const int64_t i = a.big_rows[b];
        const int64_t c = a.cand_off[i + 1] - a.cand_off[i];
        if (c > SP_BLOCK_CAP) continue;              // the dense kernel takes it
        if (tid == 0) scnt = 0;
        __syncthreads();
        sp_gather<SEM, UNS>(a, i, merge != 0, keys, vals, &scnt, tid, SP_BLOCK_THREADS, ev);
        __syncthreads();
        const int cnt = scnt;
        int P = 1;
        while (P < cnt) P <<= 1;
        for (int idx = cnt + tid; idx < P; idx += SP_BLOCK_THREADS) keys[idx] = SP_PAD;
        __syncthreads();
        sp_bitonic(keys, vals, P, tid, SP_BLOCK_THREADS, BlockSync());
        int64_t out = 0;
        const int64_t base = a.cand_off[i];
        for (int c0 = 0; c0 < cnt; c0 += SP_BLOCK_THREADS) {
            const int idx = c0 + tid;
            long long v = 0;
            bool keep = false;
            if (idx < cnt && (idx == 0 || (keys[idx] >> 1) != (keys[idx - 1] >> 1)))
                keep = sp_reduce_run<SEM, UNS>(keys, vals, idx, cnt, merge != 0, a.elem_bytes, v);
            const unsigned bal = __ballot_sync(0xffffffffu, keep);
            if (lane == 0) wsum[w] = __popc(bal);
            __syncthreads();
            int before = 0, total = 0;
            for (int q = 0; q < SP_BLOCK_THREADS / 32; ++q) {
                before += q < w ? wsum[q] : 0;
                total += wsum[q];
            }
            if (keep) {
                const int64_t pos = base + out + before + __popc(bal & ((1u << lane) - 1u));
                a.ocol[pos] = (int)(keys[idx] >> 1);
                a.oval[pos] = v;
            }
            out += total;
            __syncthreads();
        }
        if (tid == 0) a.rownnz[i] = out;
        __syncthreads();
    }
    for (int o = 16; o > 0; o >>= 1) ev |= __shfl_xor_sync(0xffffffffu, ev, o);
    if (lane == 0 && ev) atomicOr(a.flags, ev);
}

// Dense accumulator encoding for atomicMin: the (+) order becomes the unsigned (C core) or
// signed (Cython) order of the key; an empty slot holds the largest key.
template <int SEM>
__device__ __forceinline__ unsigned long long sp_enc(long long v) {
    if (SEM == SEM_CY32) return (unsigned long long)v;          // compared as signed below
    return v == -1 ? 0ull : (unsigned long long)v;
}
template <int SEM>
__device__ __forceinline__ long long sp_dec(unsigned long long k) {
    if (SEM == SEM_CY32) return (long long)k;
    return k == 0ull ? -1ll : (long long)k;
}
template <int SEM> __device__ __forceinline__ unsigned long long sp_empty() {
    return SEM == SEM_CY32 ? (unsigned long long)LLONG_MAX : ~0ull;
}

// ----------------------------------------------------------------------------- warp rows
// One row per warp for rows of at most SP_BLOCK_CAP candidates.  The candidates are never
// stored: the warp walks them in place -- the lanes take 32 entries (i, k) of A at a time, a
// warp scan of nnz(B[k]) flattens their products into one index range, and every lane finds
// the entry of its product by a shuffle binary search -- and folds each product into a small
// open-addressing table in shared memory keyed by column (atomicMin on the order-encoded (+)).
// A squaring step's own entries R[i, .] go into a second value per slot.  The table holds up to
// SP_HASH_SLOTS distinct columns; a row with more goes to the block kernel instead.  The
// distinct columns are then sorted (a bitonic sort of at most SP_HASH_SLOTS keys) and written
// ascending.
constexpr int SP_HASH_SLOTS = 128;
constexpr int SP_HWARPS = 8;          // warps per CTA
constexpr unsigned SP_NOKEY = 0xffffffffu;

// The (+) of a column's products is a minimum in an order encoding (sp_enc); keys below the
// 32-bit empty mark are folded with a native 32-bit shared atomicMin, larger ones (rare) with
// a 64-bit one, and the two halves are combined when the row is written.
struct SpHashWarp {
    unsigned key[SP_HASH_SLOTS];
    unsigned v32[SP_HASH_SLOTS];             // (+) of the products with small keys
    unsigned long long v64[SP_HASH_SLOTS];   // (+) of the products with large keys
    long long rv[SP_HASH_SLOTS];             // R's own entry (squaring step), 0 if none
    unsigned long long list[SP_HASH_SLOTS];  // (column << 32 | slot) of the occupied slots
};
constexpr unsigned SP_E32 = 0xffffffffu;     // empty mark of v32 (C core encoding)
constexpr int SP_E32S = 0x7fffffff;          // empty mark of v32 (Cython, signed)

// A row whose candidate columns all lie in a window of SP_WIN consecutive columns (the first
// and last column of every B row it gathers, and of R's row, bound it) folds its products into
// a dense accumulator over the window instead: no probing, and scanning the window in order
// writes the row already sorted.  A product outside the window (unsorted input rows) sends the
// row to the block kernel like a full table does.
constexpr int SP_WIN = 256;
struct SpWinWarp {
    unsigned v32[SP_WIN];
    unsigned long long v64[SP_WIN];
    long long rv[SP_WIN];
};
constexpr size_t SP_WARP_BYTES = sizeof(SpHashWarp) > sizeof(SpWinWarp) ? sizeof(SpHashWarp) : sizeof(SpWinWarp);
constexpr size_t SP_WARP_SMEM = SP_WARP_BYTES * SP_HWARPS;

// Slot of column j (inserted if new); -1 when the table is full.
__device__ __forceinline__ int sp_hash_slot(SpHashWarp &H, unsigned j, int mask) {
    int h = (int)((j * 2654435761u) >> 8) & mask;
    for (int probe = 0; probe <= mask; ++probe) {
        const unsigned k = H.key[h];
        if (k == j) return h;
        if (k == SP_NOKEY) {
            const unsigned old = atomicCAS(&H.key[h], SP_NOKEY, j);
            if (old == SP_NOKEY || old == j) return h;
        }
        h = (h + 1) & mask;
    }
    return -1;
}

template <int SEM, typename Tab>
__device__ __forceinline__ void sp_hash_fold(Tab &H, int slot, long long p) {
    if (SEM == SEM_CY32) {
        if (p < (long long)SP_E32S && p >= (long long)INT_MIN) {
            int *v = reinterpret_cast<int *>(&H.v32[slot]);
            if ((int)p < *v) atomicMin(v, (int)p);        // a larger value cannot lower the minimum
        } else {
            long long *v = reinterpret_cast<long long *>(&H.v64[slot]);
            if (p < *v) atomicMin(v, p);
        }
    } else {
        const unsigned long long e = sp_enc<SEM>(p);
        if (e < (unsigned long long)SP_E32) {
            if ((unsigned)e < H.v32[slot]) atomicMin(&H.v32[slot], (unsigned)e);
        } else if (e < H.v64[slot]) {
            atomicMin(&H.v64[slot], e);
        }
    }
}

// the folded (+) of slot s (0 when no product landed there)
template <int SEM, typename Tab>
__device__ __forceinline__ long long sp_hash_value(const Tab &H, int s) {
    if (SEM == SEM_CY32) {
        const long long a = (int)H.v32[s] == SP_E32S ? LLONG_MAX : (long long)(int)H.v32[s];
        const long long m = min(a, (long long)H.v64[s]);
        return m == LLONG_MAX ? 0 : m;
    }
    const unsigned long long a = H.v32[s] == SP_E32 ? ~0ull : (unsigned long long)H.v32[s];
    const unsigned long long m = min(a, H.v64[s]);
    return m == sp_empty<SEM>() ? 0 : sp_dec<SEM>(m);
}

// Sort the first nd (<= 64) keys of list ascending in registers (shuffle bitonic network over 64
// positions, two per lane, padded with the largest key); returns the two sorted keys of the lane.
__device__ __forceinline__ void sp_sort64(unsigned long long *list, int nd, int lane) {
    unsigned long long v[2];
    v[0] = lane < nd ? list[lane] : ~0ull;
    v[1] = lane + 32 < nd ? list[lane + 32] : ~0ull;
#pragma unroll
    for (int k = 2; k <= 64; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j == 32) {                           // partners in the same lane
                const unsigned long long lo = min(v[0], v[1]), hi = max(v[0], v[1]);
                v[0] = lo;                           // k == 64: the whole sequence ascends
                v[1] = hi;
            } else {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int i = lane + 32 * h;
                    const unsigned long long o = __shfl_xor_sync(0xffffffffu, v[h], j);
                    const bool up = (i & k) == 0, lower = (i & j) == 0;
                    v[h] = (lower == up) ? min(v[h], o) : max(v[h], o);
                }
            }
        }
    }
    __syncwarp();
    if (lane < nd) list[lane] = v[0];
    if (lane + 32 < nd) list[lane + 32] = v[1];
    __syncwarp();
}

template <int SEM, bool UNS, int BYTES>
__global__ void __launch_bounds__(SP_HWARPS * 32)
sp_warp_kernel(SpArgs a, int merge) {
    extern __shared__ __align__(16) unsigned char sp_smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    SpHashWarp &H = *reinterpret_cast<SpHashWarp *>(sp_smem + (size_t)w * SP_WARP_BYTES);
    SpWinWarp &Wn = *reinterpret_cast<SpWinWarp *>(sp_smem + (size_t)w * SP_WARP_BYTES);
    unsigned ev = 0;
    const int64_t warps = (int64_t)gridDim.x * SP_HWARPS;
    for (int64_t i = (int64_t)blockIdx.x * SP_HWARPS + w; i < a.n_rows; i += warps) {
        const int64_t c = a.cand_off[i + 1] - a.cand_off[i];
        if (c > SP_BLOCK_CAP) continue;              // the dense kernel takes it
        const bool sq = merge && a.rp;
        // the row's column window, from the count pass
        const int2 wnd = a.win[i];
        const int jlo = wnd.x, jhi = wnd.y;
        const long long width = jhi >= jlo ? (long long)jhi - jlo + 1 : 0;
        const int span = (int)(width < SP_WIN + 1 ? width : SP_WIN + 1);
        const bool win = span <= SP_WIN;             // warp-uniform
        int mask = 0;
        if (win) {
            for (int s = lane; s < span; s += 32) {
                Wn.v32[s] = SEM == SEM_CY32 ? (unsigned)SP_E32S : SP_E32;
                Wn.v64[s] = sp_empty<SEM>();
                Wn.rv[s] = 0;
            }
        } else {
            int S = 32;
            while (S < c && S < SP_HASH_SLOTS) S <<= 1;
            mask = S - 1;
            for (int s = lane; s < S; s += 32) {
                H.key[s] = SP_NOKEY;
                H.v32[s] = SEM == SEM_CY32 ? (unsigned)SP_E32S : SP_E32;
                H.v64[s] = sp_empty<SEM>();
                H.rv[s] = 0;
            }
        }
        __syncwarp();
        // slot of column j in the window or the table; -1: the row does not fit
        auto slot_of = [&](int j) -> int {
            if (win) return (unsigned)(j - jlo) < (unsigned)span ? j - jlo : -1;
            return sp_hash_slot(H, (unsigned)j, mask);
        };
        bool full = false;
        if (sq) {
            for (int64_t e = a.rp[i] + lane; e < a.rp[i + 1]; e += 32) {
                const int slot = slot_of(a.rj[e]);
                if (slot < 0) full = true;
                else if (win) Wn.rv[slot] = sp_load_t<BYTES, UNS>(a.rx, e);
                else H.rv[slot] = sp_load_t<BYTES, UNS>(a.rx, e);
            }
        }
        for (int64_t e0 = a.ap[i]; e0 < a.ap[i + 1]; e0 += 32) {
            const int64_t e = e0 + lane;
            const bool in = e < a.ap[i + 1];
            long long av = 0;
            int64_t b0 = 0;
            int len = 0;
            if (in) {
                const int k = a.aj[e];
                av = sp_load_t<BYTES, UNS>(a.ax, e);
                b0 = a.bp[k];
                len = (int)(a.bp[k + 1] - b0);
            }
            int incl = len;                           // warp scan of the B-row lengths
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            const int excl = incl - len;
            const int T = __shfl_sync(0xffffffffu, incl, 31);
            for (int base = 0; base < T; base += 32) {
                const int idx = base + lane;
                int lo = 0;                          // last entry whose range starts at or before idx
#pragma unroll
                for (int st = 16; st > 0; st >>= 1) {
                    const int v = __shfl_sync(0xffffffffu, excl, lo + st);
                    if (v <= idx) lo += st;
                }
                const long long aq = __shfl_sync(0xffffffffu, av, lo);
                const int64_t bq = __shfl_sync(0xffffffffu, b0, lo);
                const int xq = __shfl_sync(0xffffffffu, excl, lo);
                if (idx < T) {
                    const int64_t f = bq + (idx - xq);
                    const int j = a.bj[f];
                    if (!(a.upper && j < i)) {
                        const long long p = sp_mul<SEM, UNS, BYTES == 4 && !UNS>(aq, sp_load_t<BYTES, UNS>(a.bx, f), ev);
                        if (p != 0) {                // a zero product adds nothing
                            if (j == i && p != -1 && p != 1) ev |= RBG_EV_CYCLE;   // a vertex reaches itself
                            const int slot = slot_of(j);
                            if (slot < 0) full = true;
                            else if (win) sp_hash_fold<SEM>(Wn, slot, p);
                            else sp_hash_fold<SEM>(H, slot, p);
                        }
                    }
                }
            }
        }
        __syncwarp();
        if (__any_sync(0xffffffffu, full)) {         // too many distinct columns: the block kernel
            if (lane == 0) a.big_rows[atomicAdd(a.big_count, 1)] = (int)i;
            __syncwarp();
            continue;
        }
        // the value of a slot: the (+) of the products, then for a squaring step the magnitude
        // merge with R
        auto value_of = [&](long long sv, long long r) -> long long {
            const long long s_t = sv == 0 ? 0 : ((SEM == SEM_CY32) ? sv : sp_trunc(sv, BYTES, UNS));
            if (!merge) return s_t;
            const long long v = sv == 0 ? r : (r != 0 ? sp_minabs(r, s_t, UNS) : s_t);
            return (long long)(int)v;                // the merged matrix is int32 (transitive_closure.py:327)
        };
        int64_t out = 0;
        const int64_t base = a.cand_off[i];
        if (win) {                                   // the window in column order: already sorted
            for (int q0 = 0; q0 < span; q0 += 32) {
                const int q = q0 + lane;
                long long v = 0;
                if (q < span) v = value_of(sp_hash_value<SEM>(Wn, q), Wn.rv[q]);
                const bool keep = v != 0;
                const unsigned bal = __ballot_sync(0xffffffffu, keep);
                if (keep) {
                    const int64_t pos = base + out + __popc(bal & ((1u << lane) - 1u));
                    a.ocol[pos] = jlo + q;
                    a.oval[pos] = v;
                }
                out += __popc(bal);
            }
            if (lane == 0) a.rownnz[i] = out;
            __syncwarp();
            continue;
        }
        // the occupied slots, compacted, then sorted by column
        const int S = mask + 1;
        int nd = 0;
        for (int s0 = 0; s0 < S; s0 += 32) {
            const int s = s0 + lane;
            const bool occ = H.key[s] != SP_NOKEY;   // S is a multiple of 32
            const unsigned bal = __ballot_sync(0xffffffffu, occ);
            if (occ) H.list[nd + __popc(bal & ((1u << lane) - 1u))] = ((unsigned long long)H.key[s] << 32) | (unsigned)s;
            nd += __popc(bal);
        }
        int P = 1;
        while (P < nd) P <<= 1;
        if (nd <= 64) {
            __syncwarp();
            sp_sort64(H.list, nd, lane);
            P = 0;                                   // sorted: skip the shared-memory network
        }
        for (int q = nd + lane; q < P; q += 32) H.list[q] = ~0ull;
        __syncwarp();
        for (int k = 2; k <= P; k <<= 1) {
            for (int jj = k >> 1; jj > 0; jj >>= 1) {
                for (int q = lane; q < P; q += 32) {
                    const int qx = q ^ jj;
                    if (qx > q) {
                        const unsigned long long x = H.list[q], y = H.list[qx];
                        if ((x > y) == ((q & k) == 0)) { H.list[q] = y; H.list[qx] = x; }
                    }
                }
                __syncwarp();
            }
        }
        for (int q0 = 0; q0 < nd; q0 += 32) {
            const int q = q0 + lane;
            long long v = 0;
            unsigned col = 0;
            if (q < nd) {
                const unsigned long long e = H.list[q];
                const int s = (int)(e & 0xffffffffu);
                col = (unsigned)(e >> 32);
                v = value_of(sp_hash_value<SEM>(H, s), H.rv[s]);
            }
            const bool keep = v != 0;
            const unsigned bal = __ballot_sync(0xffffffffu, keep);
            if (keep) {
                const int64_t pos = base + out + __popc(bal & ((1u << lane) - 1u));
                a.ocol[pos] = (int)col;
                a.oval[pos] = v;
            }
            out += __popc(bal);
        }
        if (lane == 0) a.rownnz[i] = out;
        __syncwarp();
    }
    for (int o = 16; o > 0; o >>= 1) ev |= __shfl_xor_sync(0xffffffffu, ev, o);
    if (lane == 0 && ev) atomicOr(a.flags, ev);
}

// One row per block for rows beyond SP_BLOCK_CAP: a dense accumulator over all columns (one
// scratch slot per block, left empty again after each row), read back in column order.
template <int SEM, bool UNS>
__global__ void __launch_bounds__(SP_BLOCK_THREADS)
sp_dense_kernel(SpArgs a, int merge) {
    __shared__ int wsum[SP_BLOCK_THREADS / 32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int64_t nc = a.n_cols, nwords = (nc + 31) / 32;
    unsigned long long *dval = reinterpret_cast<unsigned long long *>(a.dense_val) + (int64_t)blockIdx.x * nc;
    long long *drv = a.dense_val + (int64_t)SP_DENSE_BLOCKS * nc + (int64_t)blockIdx.x * nc;
    unsigned *dmark = a.dense_mark + (int64_t)blockIdx.x * nwords;
    unsigned ev = 0;
    const int nbig = *a.big_count;
    for (int b = blockIdx.x; b < nbig; b += gridDim.x) {
        const int64_t i = a.big_rows[b];
        const int64_t c = a.cand_off[i + 1] - a.cand_off[i];
        if (c <= SP_BLOCK_CAP) continue;
        if (merge && a.rp) {
            for (int64_t e = a.rp[i] + tid; e < a.rp[i + 1]; e += SP_BLOCK_THREADS) {
                const int j = a.rj[e];
                drv[j] = sp_load(a.rx, e, a.elem_bytes, a.uns);
                atomicOr(&dmark[j >> 5], 1u << (j & 31));
            }
        }
        for (int64_t e = a.ap[i]; e < a.ap[i + 1]; ++e) {
            const int k = a.aj[e];
            const long long av = sp_load(a.ax, e, a.elem_bytes, a.uns);
            for (int64_t f = a.bp[k] + tid; f < a.bp[k + 1]; f += SP_BLOCK_THREADS) {
                const int j = a.bj[f];
                if (a.upper && j < i) continue;
                const long long p = sp_mul<SEM, UNS>(av, sp_load(a.bx, f, a.elem_bytes, a.uns), ev);
                if (p == 0) continue;
                if (j == i && p != -1 && p != 1) ev |= RBG_EV_CYCLE;
                if (SEM == SEM_CY32) atomicMin(reinterpret_cast<long long *>(&dval[j]), (long long)p);
                else atomicMin(&dval[j], sp_enc<SEM>(p));
                atomicOr(&dmark[j >> 5], 1u << (j & 31));
            }
        }
        __syncthreads();
        int64_t out = 0;
        const int64_t base = a.cand_off[i];
        for (int64_t w0 = 0; w0 < nwords; w0 += SP_BLOCK_THREADS) {
            const int64_t wi = w0 + tid;
            unsigned bits = wi < nwords ? dmark[wi] : 0u;
            // first pass: count this thread's outputs
            int mine = 0;
            for (unsigned bb = bits; bb; bb &= bb - 1) {
                const int64_t j = wi * 32 + __ffs(bb) - 1;
                const unsigned long long k = dval[j];
                const long long s = k == sp_empty<SEM>() ? 0 : sp_dec<SEM>(k);
                const long long r = merge ? drv[j] : 0;
                long long v;
                if (!merge) v = s == 0 ? 0 : ((SEM == SEM_CY32) ? s : sp_trunc(s, a.elem_bytes, UNS));
                else {
                    const long long s_t = s == 0 ? 0 : ((SEM == SEM_CY32) ? s : sp_trunc(s, a.elem_bytes, UNS));
                    v = s == 0 ? r : (r != 0 ? sp_minabs(r, s_t, UNS) : s_t);
                    v = (long long)(int)v;
                }
                mine += v != 0;
            }
            int incl = mine;
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            if (lane == 31) wsum[w] = incl;
            __syncthreads();
            int before = incl - mine, total = 0;
            for (int q = 0; q < SP_BLOCK_THREADS / 32; ++q) {
                before += q < w ? wsum[q] : 0;
                total += wsum[q];
            }
            // second pass: write in column order and leave the slot empty
            int k2 = 0;
            for (unsigned bb = bits; bb; bb &= bb - 1) {
                const int64_t j = wi * 32 + __ffs(bb) - 1;
                const unsigned long long k = dval[j];
                const long long s = k == sp_empty<SEM>() ? 0 : sp_dec<SEM>(k);
                const long long r = merge ? drv[j] : 0;
                long long v;
                if (!merge) v = s == 0 ? 0 : ((SEM == SEM_CY32) ? s : sp_trunc(s, a.elem_bytes, UNS));
                else {
                    const long long s_t = s == 0 ? 0 : ((SEM == SEM_CY32) ? s : sp_trunc(s, a.elem_bytes, UNS));
                    v = s == 0 ? r : (r != 0 ? sp_minabs(r, s_t, UNS) : s_t);
                    v = (long long)(int)v;
                }
                if (v != 0) {
                    a.ocol[base + out + before + k2] = (int)j;
                    a.oval[base + out + before + k2] = v;
                    ++k2;
                }
                dval[j] = sp_empty<SEM>();
                drv[j] = 0;
            }
            if (wi < nwords) dmark[wi] = 0;
            out += total;
            __syncthreads();
        }
        if (tid == 0) a.rownnz[i] = out;
        __syncthreads();
    }
    for (int o = 16; o > 0; o >>= 1) ev |= __shfl_xor_sync(0xffffffffu, ev, o);
    if (lane == 0 && ev) atomicOr(a.flags, ev);
}

template <int SEM>
__global__ void sp_dense_init_kernel(long long *dense_val, unsigned *dense_mark, int64_t nc) {
    const int64_t nwords = (nc + 31) / 32;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < (int64_t)SP_DENSE_BLOCKS * nc;
         e += (int64_t)gridDim.x * blockDim.x) {
        reinterpret_cast<unsigned long long *>(dense_val)[e] = sp_empty<SEM>();
        dense_val[(int64_t)SP_DENSE_BLOCKS * nc + e] = 0;
        if (e < (int64_t)SP_DENSE_BLOCKS * nwords) dense_mark[e] = 0;
    }
}

// Final CSR: row pointers from the scan of the row counts, entries gathered from the per-row
// compacted output and stored in the storage type.
__global__ void sp_gather_kernel(int64_t n_rows, const int64_t *cand_off, const int64_t *cptr,
                                 const int *ocol, const long long *oval, int *cj, void *cx, int bytes) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n_rows; i += warps) {
        const int64_t src = cand_off[i], dst = cptr[i], cnt = cptr[i + 1] - dst;
        for (int64_t e = lane; e < cnt; e += 32) {
            cj[dst + e] = ocol[src + e];
            if (bytes == 8) reinterpret_cast<long long *>(cx)[dst + e] = oval[src + e];
            else reinterpret_cast<int *>(cx)[dst + e] = (int)oval[src + e];
        }
    }
}

}  // namespace rbg

using namespace rbg;

namespace {

struct Head {   // workspace that lives from rbg_spgemm_count to rbg_spgemm_gather
    int64_t *cand_off;   // n+1
    int2 *win;           // n: each row's column window
    int *big_rows;       // n
    int *counters;       // [0] big rows, [1] dense rows, [2] flags
    void *scan_tmp;
    size_t scan_bytes;
};

size_t scan_bytes(int64_t n) {
    size_t b = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, b, (int64_t *)nullptr, (int64_t *)nullptr, (int)std::max<int64_t>(n + 1, 1));
    return b;
}

size_t head_layout(int64_t n, unsigned char *base, Head *h) {
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o = align_up(o + bytes, 256); return base ? base + at : nullptr; };
    unsigned char *p;
    p = take((size_t)(n + 1) * 8); if (h) h->cand_off = reinterpret_cast<int64_t *>(p);
    p = take((size_t)std::max<int64_t>(n, 1) * 8); if (h) h->win = reinterpret_cast<int2 *>(p);
    p = take((size_t)std::max<int64_t>(n, 1) * 4); if (h) h->big_rows = reinterpret_cast<int *>(p);
    p = take(64); if (h) h->counters = reinterpret_cast<int *>(p);
    const size_t sb = scan_bytes(n);
    p = take(sb); if (h) { h->scan_tmp = p; h->scan_bytes = sb; }
    return o;
}

struct Tail {
    int *ocol; long long *oval; int64_t *rownnz; int64_t *cptr;
    long long *dense_val; unsigned *dense_mark;
};

size_t tail_layout(int64_t n, int64_t nc, int64_t total, int64_t dense, unsigned char *base, Tail *t) {
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o = align_up(o + bytes, 256); return base ? base + at : nullptr; };
    unsigned char *p;
    p = take((size_t)std::max<int64_t>(total, 1) * 4); if (t) t->ocol = reinterpret_cast<int *>(p);
    p = take((size_t)std::max<int64_t>(total, 1) * 8); if (t) t->oval = reinterpret_cast<long long *>(p);
    p = take((size_t)(n + 1) * 8); if (t) t->rownnz = reinterpret_cast<int64_t *>(p);
    p = take((size_t)(n + 1) * 8); if (t) t->cptr = reinterpret_cast<int64_t *>(p);
    const int64_t nwords = (nc + 31) / 32;
    p = take(dense > 0 ? (size_t)SP_DENSE_BLOCKS * nc * 16 : 8); if (t) t->dense_val = reinterpret_cast<long long *>(p);
    p = take(dense > 0 ? (size_t)SP_DENSE_BLOCKS * nwords * 4 : 8); if (t) t->dense_mark = reinterpret_cast<unsigned *>(p);
    return o;
}

bool csr_ok(const rbg_csr_t *m) {
    return m && m->n_rows >= 0 && m->n_cols >= 0 && m->indptr && (m->n_cols < (1ll << 30));
}

void fill_args(SpArgs &a, const rbg_csr_t *A, const rbg_csr_t *B, const rbg_csr_t *R, int upper) {
    memset(&a, 0, sizeof(a));
    a.n_rows = A->n_rows; a.n_cols = B->n_cols;
    a.ap = A->indptr; a.aj = A->indices; a.ax = A->data;
    a.bp = B->indptr; a.bj = B->indices; a.bx = B->data;
    if (R) { a.rp = R->indptr; a.rj = R->indices; a.rx = R->data; }
    a.upper = upper;
}

int grid_of(int64_t work, int threads) { return grid_for(work, threads); }

}  // namespace

extern "C" int32_t rbg_spgemm_head_bytes(int64_t n_rows, int64_t *bytes) {
    if (!bytes || n_rows < 0) return RBG_ERR_INVALID;
    *bytes = (int64_t)head_layout(n_rows, nullptr, nullptr);
    return RBG_OK;
}

extern "C" int32_t rbg_spgemm_tail_bytes(int64_t n_rows, int64_t n_cols, int64_t total_candidates,
                                         int64_t dense_rows, int64_t *bytes) {
    if (!bytes || n_rows < 0 || n_cols < 0 || total_candidates < 0 || dense_rows < 0) return RBG_ERR_INVALID;
    *bytes = (int64_t)tail_layout(n_rows, n_cols, total_candidates, dense_rows, nullptr, nullptr);
    return RBG_OK;
}

extern "C" int32_t rbg_spgemm_count(const rbg_csr_t *A, const rbg_csr_t *B, const rbg_csr_t *R, int32_t upper,
                                    void *head, int64_t head_bytes, int64_t *total_candidates,
                                    int64_t *dense_rows, rbg_stream_t stream) {
    if (!csr_ok(A) || !csr_ok(B) || (R && !csr_ok(R)) || !head || !total_candidates || !dense_rows)
        return RBG_ERR_INVALID;
    if (A->n_cols != B->n_rows || (R && (R->n_rows != A->n_rows || R->n_cols != B->n_cols)))
        return RBG_ERR_INVALID;
    const int64_t n = A->n_rows;
    if (head_bytes < (int64_t)head_layout(n, nullptr, nullptr)) return RBG_ERR_NOMEM;
    Head h;
    head_layout(n, reinterpret_cast<unsigned char *>(head), &h);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    SpArgs a;
    fill_args(a, A, B, R, upper);
    a.big_rows = h.big_rows;
    a.big_count = h.counters;
    a.win = h.win;
    RBG_CUDA_TRY(cudaMemsetAsync(h.counters, 0, 64, s));
    note_launches(2);
    sp_count_kernel<<<grid_of(n + 1, 256), 256, 0, s>>>(a, h.cand_off);
    RBG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(h.scan_tmp, h.scan_bytes, h.cand_off, h.cand_off, (int)(n + 1), s));
    int64_t tot = 0;
    int hc[2] = {0, 0};
    RBG_CUDA_TRY(cudaMemcpyAsync(&tot, h.cand_off + n, 8, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaMemcpyAsync(hc, h.counters, 8, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    const int64_t dense = hc[1];
    *total_candidates = tot;
    *dense_rows = dense;
    return RBG_OK;
}

namespace {

template <int SEM, bool UNS>
int run_numeric(SpArgs &a, int merge, int64_t dense, int64_t nc, cudaStream_t s) {
    static PerDeviceOnce once;              // per instantiation, for every device
    const int configured = once.run([] {
        RBG_CUDA_TRY(cudaFuncSetAttribute(sp_warp_kernel<SEM, UNS, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)SP_WARP_SMEM));
        RBG_CUDA_TRY(cudaFuncSetAttribute(sp_warp_kernel<SEM, UNS, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)SP_WARP_SMEM));
        RBG_CUDA_TRY(cudaFuncSetAttribute(sp_block_kernel<SEM, UNS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)SP_BLOCK_SMEM));
        return (int)RBG_OK;
    });
    if (configured) return configured;
    const int64_t n = a.n_rows;
    note_launches(2 + (dense > 0 ? 2 : 0));
    const int wg = grid_of((n + SP_HWARPS - 1) / SP_HWARPS, 1);
    if (a.elem_bytes == 8) sp_warp_kernel<SEM, UNS, 8><<<wg, SP_HWARPS * 32, SP_WARP_SMEM, s>>>(a, merge);
    else sp_warp_kernel<SEM, UNS, 4><<<wg, SP_HWARPS * 32, SP_WARP_SMEM, s>>>(a, merge);
    sp_block_kernel<SEM, UNS><<<grid_of(1 << 20, 1), SP_BLOCK_THREADS, SP_BLOCK_SMEM, s>>>(a, merge);
    if (dense > 0) {
        sp_dense_init_kernel<SEM><<<grid_of((int64_t)SP_DENSE_BLOCKS * nc, 256), 256, 0, s>>>(a.dense_val,
                                                                                         a.dense_mark, nc);
        sp_dense_kernel<SEM, UNS><<<SP_DENSE_BLOCKS, SP_BLOCK_THREADS, 0, s>>>(a, merge);
    }
    RBG_CUDA_TRY(cudaGetLastError());
    return RBG_OK;
}

}  // namespace

extern "C" int32_t rbg_spgemm_numeric(int32_t sem, int32_t dtype, const rbg_csr_t *A, const rbg_csr_t *B,
                                      const rbg_csr_t *R, int32_t upper, void *head, void *tail,
                                      int64_t tail_bytes, int64_t total_candidates, int64_t dense_rows,
                                      int64_t *nnz, uint32_t *flags, rbg_stream_t stream) {
    if (!csr_ok(A) || !csr_ok(B) || (R && !csr_ok(R)) || !head || !tail || !nnz || !flags) return RBG_ERR_INVALID;
    if (sem != RBG_SEM_C64 && sem != RBG_SEM_CY32) return RBG_ERR_INVALID;
    if (sem == RBG_SEM_CY32 && dtype != RBG_DTYPE_INT32) return RBG_ERR_INVALID;
    if (dtype != RBG_DTYPE_INT32 && dtype != RBG_DTYPE_INT64 && dtype != RBG_DTYPE_UINT32 &&
        dtype != RBG_DTYPE_UINT64)
        return RBG_ERR_INVALID;
    const int64_t n = A->n_rows, nc = B->n_cols;
    if (tail_bytes < (int64_t)tail_layout(n, nc, total_candidates, dense_rows, nullptr, nullptr))
        return RBG_ERR_NOMEM;
    Head h;
    head_layout(n, reinterpret_cast<unsigned char *>(head), &h);
    Tail t;
    tail_layout(n, nc, total_candidates, dense_rows, reinterpret_cast<unsigned char *>(tail), &t);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    SpArgs a;
    fill_args(a, A, B, R, upper);
    a.elem_bytes = dtype_bytes(dtype);
    a.uns = (dtype == RBG_DTYPE_UINT32 || dtype == RBG_DTYPE_UINT64);
    a.cand_off = h.cand_off;
    a.ocol = t.ocol; a.oval = t.oval; a.rownnz = t.rownnz;
    a.dense_val = t.dense_val; a.dense_mark = t.dense_mark;
    a.big_rows = h.big_rows; a.big_count = h.counters;
    a.win = h.win;
    a.flags = reinterpret_cast<unsigned *>(h.counters + 2);
    RBG_CUDA_TRY(cudaMemsetAsync(h.counters + 2, 0, 4, s));
    RBG_CUDA_TRY(cudaMemsetAsync(t.rownnz, 0, (size_t)(n + 1) * 8, s));
    const int merge = R != nullptr;
    int rc;
    if (sem == RBG_SEM_CY32) rc = run_numeric<SEM_CY32, false>(a, merge, dense_rows, nc, s);
    else if (a.uns) rc = run_numeric<SEM_C64, true>(a, merge, dense_rows, nc, s);
    else rc = run_numeric<SEM_C64, false>(a, merge, dense_rows, nc, s);
    if (rc) return rc;
    size_t sb = h.scan_bytes;
    RBG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(h.scan_tmp, sb, t.rownnz, t.cptr, (int)(n + 1), s));
    int64_t tot = 0;
    unsigned hf = 0;
    RBG_CUDA_TRY(cudaMemcpyAsync(&tot, t.cptr + n, 8, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaMemcpyAsync(&hf, h.counters + 2, 4, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    *nnz = tot;
    *flags = hf;
    return (hf & (RBG_EV_OVF_SIZE | RBG_EV_OVF_ONES | RBG_EV_HANG)) ? RBG_ERR_OVERFLOW : RBG_OK;
}

extern "C" int32_t rbg_spgemm_gather(int32_t dtype, int64_t n_rows, int64_t n_cols, const void *head,
                                     const void *tail, int64_t total_candidates, int64_t dense_rows,
                                     int64_t *indptr, int32_t *indices, void *data, rbg_stream_t stream) {
    if (!head || !tail || !indptr || n_rows < 0 || dtype_bytes(dtype) < 4) return RBG_ERR_INVALID;
    Head h;
    head_layout(n_rows, const_cast<unsigned char *>(reinterpret_cast<const unsigned char *>(head)), &h);
    Tail t;
    tail_layout(n_rows, n_cols, total_candidates, dense_rows,
                const_cast<unsigned char *>(reinterpret_cast<const unsigned char *>(tail)), &t);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    RBG_CUDA_TRY(cudaMemcpyAsync(indptr, t.cptr, (size_t)(n_rows + 1) * 8, cudaMemcpyDeviceToDevice, s));
    if (n_rows > 0) {
        note_launches(1);
        sp_gather_kernel<<<grid_of(n_rows * 32, 256), 256, 0, s>>>(n_rows, h.cand_off, t.cptr, t.ocol, t.oval, indices,
                                                                  data, dtype_bytes(dtype));
        RBG_CUDA_TRY(cudaGetLastError());
    }
    return RBG_OK;
}

// ----------------------------------------------------------------------------- row merge
// Z = X (+) Y cell by cell with the squaring step's magnitude rule (redblackgraph/gpu/
// transitive_closure.py:77-156): the smaller |value| (X's on a tie), zero results dropped.
// int32 values, rows sorted.  One thread merges one row's two sorted lists.
namespace rbg {

__device__ __forceinline__ int mg_pick(int x, int y) {
    const unsigned ax = x < 0 ? 0u - (unsigned)x : (unsigned)x;
    const unsigned ay = y < 0 ? 0u - (unsigned)y : (unsigned)y;
    return ay < ax ? y : x;
}

template <bool FILL>
__global__ void mg_kernel(int64_t n, const int64_t *xp, const int *xj, const int *xv, const int64_t *yp,
                          const int *yj, const int *yv, int64_t *cnt, const int64_t *zp, int *zj, int *zv) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t a = xp[i], ae = xp[i + 1], b = yp[i], be = yp[i + 1];
        int64_t out = FILL ? zp[i] : 0;
        int64_t c = 0;
        while (a < ae || b < be) {
            int col, v;
            if (b >= be || (a < ae && xj[a] < yj[b])) { col = xj[a]; v = xv[a]; ++a; }
            else if (a >= ae || yj[b] < xj[a]) { col = yj[b]; v = yv[b]; ++b; }
            else { col = xj[a]; v = mg_pick(xv[a], yv[b]); ++a; ++b; }
            if (v == 0) continue;
            if (FILL) { zj[out + c] = col; zv[out + c] = v; }
            ++c;
        }
        if (!FILL) cnt[i] = c;
    }
}

}  // namespace rbg

extern "C" int32_t rbg_csr_merge_count(const rbg_csr_t *X, const rbg_csr_t *Y, void *head, int64_t head_bytes,
                                       int64_t *nnz, rbg_stream_t stream) {
    if (!csr_ok(X) || !csr_ok(Y) || !head || !nnz || X->n_rows != Y->n_rows || X->n_cols != Y->n_cols)
        return RBG_ERR_INVALID;
    const int64_t n = X->n_rows;
    if (head_bytes < (int64_t)head_layout(n, nullptr, nullptr)) return RBG_ERR_NOMEM;
    Head h;
    head_layout(n, reinterpret_cast<unsigned char *>(head), &h);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    RBG_CUDA_TRY(cudaMemsetAsync(h.cand_off + n, 0, 8, s));
    if (n > 0) {
        note_launches(1);
        mg_kernel<false><<<grid_of(n, 256), 256, 0, s>>>(n, X->indptr, X->indices, (const int *)X->data, Y->indptr,
                                                         Y->indices, (const int *)Y->data, h.cand_off, nullptr,
                                                         nullptr, nullptr);
    }
    RBG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(h.scan_tmp, h.scan_bytes, h.cand_off, h.cand_off, (int)(n + 1), s));
    int64_t tot = 0;
    RBG_CUDA_TRY(cudaMemcpyAsync(&tot, h.cand_off + n, 8, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    *nnz = tot;
    return RBG_OK;
}

extern "C" int32_t rbg_csr_merge_fill(const rbg_csr_t *X, const rbg_csr_t *Y, const void *head, int64_t *indptr,
                                      int32_t *indices, int32_t *data, rbg_stream_t stream) {
    if (!csr_ok(X) || !csr_ok(Y) || !head || !indptr) return RBG_ERR_INVALID;
    const int64_t n = X->n_rows;
    Head h;
    head_layout(n, const_cast<unsigned char *>(reinterpret_cast<const unsigned char *>(head)), &h);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    RBG_CUDA_TRY(cudaMemcpyAsync(indptr, h.cand_off, (size_t)(n + 1) * 8, cudaMemcpyDeviceToDevice, s));
    if (n > 0) {
        note_launches(1);
        mg_kernel<true><<<grid_of(n, 256), 256, 0, s>>>(n, X->indptr, X->indices, (const int *)X->data, Y->indptr,
                                                        Y->indices, (const int *)Y->data, nullptr, h.cand_off,
                                                        indices, data);
    }
    RBG_CUDA_TRY(cudaGetLastError());
    return RBG_OK;
}

// ------------------------------------------------------------------------------------------
// Entries that changed between two squarings (the semi-naive squaring's difference)
// ------------------------------------------------------------------------------------------
// Z = the entries of X whose column is absent from the same row of Y or holds another value
// there (values compared as integers, whatever the two storage types).  One warp per row: each
// lane looks its entry's column up in Y's row by binary search, a ballot packs the kept entries
// in column order.
namespace rbg {

__device__ __forceinline__ long long df_load(const void *v, int64_t e, int bytes, bool uns) {
    if (bytes == 8) return reinterpret_cast<const long long *>(v)[e];
    if (bytes == 4) return uns ? (long long)reinterpret_cast<const unsigned *>(v)[e]
                               : (long long)reinterpret_cast<const int *>(v)[e];
    if (bytes == 2) return uns ? (long long)reinterpret_cast<const unsigned short *>(v)[e]
                               : (long long)reinterpret_cast<const short *>(v)[e];
    return uns ? (long long)reinterpret_cast<const unsigned char *>(v)[e]
               : (long long)reinterpret_cast<const signed char *>(v)[e];
}

template <bool FILL>
__global__ void df_kernel(int64_t n, const int64_t *xp, const int *xj, const void *xv, int xb, bool xu,
                          const int64_t *yp, const int *yj, const void *yv, int yb, bool yu, int64_t *cnt,
                          const int64_t *zp, int *zj, void *zv) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
        const int64_t x0 = xp[i], x1 = xp[i + 1], y0 = yp[i];
        const int ylen = (int)(yp[i + 1] - y0);
        int64_t out = FILL ? zp[i] : 0;
        for (int64_t e0 = x0; e0 < x1; e0 += 32) {
            const int64_t e = e0 + lane;
            bool keep = false;
            int col = 0;
            if (e < x1) {
                col = xj[e];
                // when Y's row is a subset of X's (a squaring step only adds entries), entry q of
                // X sits at a position of Y in [q - (|X| - |Y|), q]: look there first, then in the
                // rest of the row
                const int q = (int)(e - x0), extra = (int)(x1 - x0) - ylen;
                auto find = [&](int lo, int hi) -> int {
                    while (lo <= hi) {
                        const int mid = (lo + hi) >> 1;
                        const int c = yj[y0 + mid];
                        if (c == col) return mid;
                        if (c < col) lo = mid + 1;
                        else hi = mid - 1;
                    }
                    return -1;
                };
                const int nlo = max(0, q - max(extra, 0)), nhi = min(q, ylen - 1);
                int f = find(nlo, nhi);
                if (f < 0) {
                    f = find(0, nlo - 1);
                    if (f < 0) f = find(nhi + 1, ylen - 1);
                }
                keep = f < 0 || df_load(yv, y0 + f, yb, yu) != df_load(xv, e, xb, xu);
            }
            const unsigned bal = __ballot_sync(0xffffffffu, keep);
            if (FILL && keep) {
                const int64_t q = out + __popc(bal & ((1u << lane) - 1u));
                zj[q] = col;
                if (xb == 8) {
                    reinterpret_cast<long long *>(zv)[q] = reinterpret_cast<const long long *>(xv)[e];
                } else if (xb == 4) {
                    reinterpret_cast<int *>(zv)[q] = reinterpret_cast<const int *>(xv)[e];
                } else {
                    unsigned char *d = reinterpret_cast<unsigned char *>(zv) + q * xb;
                    const unsigned char *s = reinterpret_cast<const unsigned char *>(xv) + e * xb;
                    for (int b = 0; b < xb; ++b) d[b] = s[b];
                }
            }
            out += __popc(bal);
        }
        if (!FILL && lane == 0) cnt[i] = out;
    }
}

bool df_dtype(int32_t dtype, int &bytes, bool &uns) {
    bytes = dtype_bytes(dtype);
    uns = dtype == RBG_DTYPE_UINT8 || dtype == RBG_DTYPE_UINT16 || dtype == RBG_DTYPE_UINT32 ||
          dtype == RBG_DTYPE_UINT64;
    return bytes > 0;
}

}  // namespace rbg

extern "C" int32_t rbg_csr_diff_count(int32_t x_dtype, const rbg_csr_t *X, int32_t y_dtype, const rbg_csr_t *Y,
                                      void *head, int64_t head_bytes, int64_t *nnz, rbg_stream_t stream) {
    int xb, yb;
    bool xu, yu;
    if (!csr_ok(X) || !csr_ok(Y) || !head || !nnz || X->n_rows != Y->n_rows || X->n_cols != Y->n_cols ||
        !df_dtype(x_dtype, xb, xu) || !df_dtype(y_dtype, yb, yu))
        return RBG_ERR_INVALID;
    const int64_t n = X->n_rows;
    if (head_bytes < (int64_t)head_layout(n, nullptr, nullptr)) return RBG_ERR_NOMEM;
    Head h;
    head_layout(n, reinterpret_cast<unsigned char *>(head), &h);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    RBG_CUDA_TRY(cudaMemsetAsync(h.cand_off + n, 0, 8, s));
    if (n > 0) {
        note_launches(1);
        df_kernel<false><<<grid_of(n * 32, 256), 256, 0, s>>>(n, X->indptr, X->indices, X->data, xb, xu, Y->indptr,
                                                              Y->indices, Y->data, yb, yu, h.cand_off, nullptr,
                                                              nullptr, nullptr);
    }
    RBG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(h.scan_tmp, h.scan_bytes, h.cand_off, h.cand_off, (int)(n + 1), s));
    int64_t tot = 0;
    {
        HostStaging hs(s, 64);
        int rc = hs.down(&tot, h.cand_off + n, 8);
        if (!rc) rc = hs.finish();
        if (rc) return rc;
    }
    *nnz = tot;
    return RBG_OK;
}

extern "C" int32_t rbg_csr_diff_fill(int32_t x_dtype, const rbg_csr_t *X, int32_t y_dtype, const rbg_csr_t *Y,
                                     const void *head, int64_t *indptr, int32_t *indices, void *data,
                                     rbg_stream_t stream) {
    int xb, yb;
    bool xu, yu;
    if (!csr_ok(X) || !csr_ok(Y) || !head || !indptr || X->n_rows != Y->n_rows || !df_dtype(x_dtype, xb, xu) ||
        !df_dtype(y_dtype, yb, yu))
        return RBG_ERR_INVALID;
    const int64_t n = X->n_rows;
    Head h;
    head_layout(n, const_cast<unsigned char *>(reinterpret_cast<const unsigned char *>(head)), &h);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    RBG_CUDA_TRY(cudaMemcpyAsync(indptr, h.cand_off, (size_t)(n + 1) * 8, cudaMemcpyDeviceToDevice, s));
    if (n > 0) {
        note_launches(1);
        df_kernel<true><<<grid_of(n * 32, 256), 256, 0, s>>>(n, X->indptr, X->indices, X->data, xb, xu, Y->indptr,
                                                             Y->indices, Y->data, yb, yu, nullptr, h.cand_off,
                                                             indices, data);
    }
    RBG_CUDA_TRY(cudaGetLastError());
    return RBG_OK;
}

// ------------------------------------------------------------------------------------------
// Operands of the semi-naive squaring step: A' = [D R] (n x 2n), B' = [R ; D] (2n x n), so that
// A' B' = D R (+) R D and one product with the merge of R forms R (+) D R (+) R D in one pass
// ------------------------------------------------------------------------------------------
namespace rbg {

// One warp per row: row i of A' is D's row, then R's row with its columns moved by n (so it
// stays sorted); A' row pointers are the sums of D's and R's.  The first n + 1 threads also
// write B''s row pointers (R's, then D's moved by nnz(R)).
__global__ void sn_operands_kernel(int64_t n, int eb, const int64_t *dp, const int *dj, const void *dv,
                                   const int64_t *rp, const int *rj, const void *rv, int64_t *ap, int *aj,
                                   void *av, int64_t *bp) {
    const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
    const int64_t rnnz = rp[n];
    for (int64_t i = gt; i <= 2 * n; i += nthreads) {
        if (i <= n) {
            ap[i] = dp[i] + rp[i];
            bp[i] = rp[i];
        } else {
            bp[i] = rnnz + dp[i - n];
        }
    }
    const int lane = threadIdx.x & 31;
    const int64_t warps = nthreads >> 5;
    auto copy = [&](void *dst, int64_t q, const void *src, int64_t e) {
        if (eb == 8) reinterpret_cast<long long *>(dst)[q] = reinterpret_cast<const long long *>(src)[e];
        else reinterpret_cast<int *>(dst)[q] = reinterpret_cast<const int *>(src)[e];
    };
    for (int64_t i = gt >> 5; i < n; i += warps) {
        const int64_t d0 = dp[i], d1 = dp[i + 1], r0 = rp[i], r1 = rp[i + 1];
        const int64_t o = d0 + r0;
        for (int64_t e = d0 + lane; e < d1; e += 32) {
            aj[o + (e - d0)] = dj[e];
            copy(av, o + (e - d0), dv, e);
        }
        const int64_t o2 = o + (d1 - d0);
        for (int64_t e = r0 + lane; e < r1; e += 32) {
            aj[o2 + (e - r0)] = rj[e] + (int)n;
            copy(av, o2 + (e - r0), rv, e);
        }
    }
}

}  // namespace rbg

extern "C" int32_t rbg_spgemm_seminaive_operands(int32_t dtype, const rbg_csr_t *D, const rbg_csr_t *R,
                                                 int64_t *a_indptr, int32_t *a_indices, void *a_data,
                                                 int64_t *b_indptr, int32_t *b_indices, void *b_data,
                                                 rbg_stream_t stream) {
    const int eb = dtype_bytes(dtype);
    if (!csr_ok(D) || !csr_ok(R) || D->n_rows != R->n_rows || D->n_cols != R->n_cols || R->n_rows != R->n_cols ||
        (eb != 4 && eb != 8) || !a_indptr || !b_indptr || R->n_rows >= (1ll << 29))
        return RBG_ERR_INVALID;
    const int64_t n = R->n_rows;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int64_t nnz[2] = {0, 0};
    {
        HostStaging hs(s, 64);
        int rc = hs.down(&nnz[0], D->indptr + n, 8);
        if (!rc) rc = hs.down(&nnz[1], R->indptr + n, 8);
        if (!rc) rc = hs.finish();
        if (rc) return rc;
    }
    const int64_t dn = nnz[0], rn = nnz[1];
    if ((dn + rn > 0) && (!a_indices || !a_data || !b_indices || !b_data)) return RBG_ERR_INVALID;
    // B' = [R ; D]: the entries of R, then those of D
    if (rn > 0) {
        RBG_CUDA_TRY(cudaMemcpyAsync(b_indices, R->indices, (size_t)rn * 4, cudaMemcpyDeviceToDevice, s));
        RBG_CUDA_TRY(cudaMemcpyAsync(b_data, R->data, (size_t)rn * eb, cudaMemcpyDeviceToDevice, s));
    }
    if (dn > 0) {
        RBG_CUDA_TRY(cudaMemcpyAsync(b_indices + rn, D->indices, (size_t)dn * 4, cudaMemcpyDeviceToDevice, s));
        RBG_CUDA_TRY(cudaMemcpyAsync(reinterpret_cast<unsigned char *>(b_data) + (size_t)rn * eb, D->data,
                                     (size_t)dn * eb, cudaMemcpyDeviceToDevice, s));
    }
    note_launches(1);
    sn_operands_kernel<<<grid_of(std::max<int64_t>(n, 1) * 32, 256), 256, 0, s>>>(
        n, eb, D->indptr, D->indices, D->data, R->indptr, R->indices, R->data, a_indptr, a_indices, a_data,
        b_indptr);
    RBG_CUDA_TRY(cudaGetLastError());
    return RBG_OK;
}

// ------------------------------------------------------------------------------------------
// Largest candidate of the DAG closure (the value its diameter is taken from)
// ------------------------------------------------------------------------------------------
// The reference's sparse DAG closure (redblackgraph/sparse/csgraph/_transitive_closure_dag.pyx:
// 262-305) builds row v from each parent w != v as A[v][w] (x) C[w][x] over w's closed row and
// keeps the largest magnitude of every such candidate, including those that lose the (+), and
// of every stored entry of A.  Given the closure C, one warp per row of A recomputes the
// candidates (Cython int32 product, magnitudes in int32) and keeps their maximum.
namespace rbg {
__global__ void dag_cand_max_kernel(int64_t n, const int64_t *ap, const int *aj, const int *ax,
                                    const int64_t *cp, const int *cj, const int *cx,
                                    unsigned long long *out) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    int best = 0;
    for (int64_t v = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); v < n; v += warps) {
        for (int64_t e = ap[v]; e < ap[v + 1]; ++e) {
            const int w = aj[e], a = ax[e];
            if (lane == 0) {                      // the stored entry itself
                const int m = a > 0 ? a : (int)(0u - (unsigned)a);
                best = max(best, m);
            }
            if (w == (int)v || w < 0 || w >= n) continue;
            for (int64_t f = cp[w] + lane; f < cp[w + 1]; f += 32) {
                const int p = cy_product(a, cx[f]);
                if (p == 0) continue;
                const int m = p > 0 ? p : (int)(0u - (unsigned)p);   // int32 magnitude, as -val
                best = max(best, m);
            }
        }
    }
    best = __reduce_max_sync(0xffffffffu, best);
    if (lane == 0 && best > 0) atomicMax(out, (unsigned long long)best);
}
}  // namespace rbg

extern "C" int32_t rbg_dag_candidate_max(const rbg_csr_t *A, const rbg_csr_t *C, void *workspace,
                                         int64_t workspace_bytes, int64_t *max_abs, rbg_stream_t stream) {
    if (!csr_ok(A) || !csr_ok(C) || !workspace || workspace_bytes < 8 || !max_abs) return RBG_ERR_INVALID;
    if (A->n_rows != A->n_cols || C->n_rows != A->n_rows) return RBG_ERR_INVALID;
    const int64_t n = A->n_rows;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    unsigned long long *d = reinterpret_cast<unsigned long long *>(workspace);
    RBG_CUDA_TRY(cudaMemsetAsync(d, 0, 8, s));
    if (n > 0) {
        note_launches(1);
        dag_cand_max_kernel<<<grid_of(n * 32, 256), 256, 0, s>>>(n, A->indptr, A->indices, (const int *)A->data,
                                                                C->indptr, C->indices, (const int *)C->data, d);
        RBG_CUDA_TRY(cudaGetLastError());
    }
    unsigned long long h = 0;
    RBG_CUDA_TRY(cudaMemcpyAsync(&h, d, 8, cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    *max_abs = (int64_t)h;
    return RBG_OK;
}
