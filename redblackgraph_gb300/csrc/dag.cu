// dag.cu -- closure of a DAG by levels, on sm_103a.
//
// Reference: transitive_closure_dag_sparse_cython, redblackgraph/sparse/csgraph/
// _transitive_closure_dag.pyx:168-351 (and the level-parallel transitive_closure_dag_gpu,
// redblackgraph/gpu/transitive_closure.py:474-652).  Row v of the closure is v's stored entries
// (+) A[v][w] (x) C[w][.] over v's parents w != v, with the Cython int32 product and sum; the
// diameter source is the largest magnitude of any stored entry or candidate.
//
// Design.  Vertices are put in topological levels on the device (Kahn's algorithm): a vertex
// joins the next level when its last parent's row is done.  The kernel that discovers a vertex
// also bounds its row (stored entries + the lengths of its parents' rows) and reserves that many
// slots of a caller-provided row pool (one atomic per warp), so each level then needs a single
// fill pass: one warp per row walks the row's candidates (a warp scan over the segment lengths and
// a shuffle binary search give every lane its candidate), and
//   - up to 128 candidates: orders (column, value) keys in registers and keeps the first of each
//     column (the signed minimum of the non-zero values, a stored zero when there is none), by
//     bitonic merges of the row's sorted runs (stored entries, each parent's row) when there are
//     few runs, else by a bitonic sort (up to 64); rows of up to 8 (16) candidates take 8 (16)
//     lanes each, so a warp fills four (two) at once;
//   - up to 256: folds them into a per-warp shared-memory table and sorts the occupied slots;
//   - more: the row goes to a 512-thread block with an 8192-slot table.
// The host launches levels in chunks without waiting (every kernel reads its level's bounds from
// device memory and exits at once on an empty level) and looks at the frontier once per chunk.
// A pool too small marks the rows past its end as skipped; the call then returns
// RBG_ERR_CAPACITY with *nnz = a larger pool to retry with.  A row with more distinct columns
// than the block table returns RBG_ERR_CAPACITY with *nnz = -1.  Vertices never placed (on or
// below a cycle) return RBG_ERR_CYCLE.
#include <cuda_runtime.h>
#include <cub/cub.cuh>
#include <algorithm>
#include "rbg_internal.cuh"

namespace rbg {

constexpr unsigned FULL = 0xffffffffu;
constexpr int DG_WSLOTS = 256;          // warp table slots (candidates per row)
constexpr int DG_WARPS = 8;             // warps per CTA of the fill pass
constexpr int DG_BSLOTS = 8192;         // block table slots (distinct columns)
constexpr int DG_BTHREADS = 512;
constexpr unsigned DG_NOKEY = 0xffffffffu;
constexpr int DG_NOVAL = 0x7fffffff;    // (+) identity of the table (no non-zero candidate yet)
constexpr unsigned long long DG_PAD = ~0ull;

template <int SLOTS> struct DagTable {
    unsigned key[SLOTS];
    int val[SLOTS];                     // signed minimum of the non-zero candidates
    unsigned char has[SLOTS];           // 1: some non-zero candidate landed here
    unsigned long long list[SLOTS];     // (column << 32 | slot) of the occupied slots
};

// The row at one position of the order, written when the vertex is discovered so that the fill
// pass starts from one coalesced record.
struct __align__(16) DagRec {
    long long off;                                       // pool position (-1: skipped)
    long long e0;                                        // first stored entry
    int v, ub, na, pad;
};
constexpr int DG_DESC_LEN_BITS = 24;

struct DagArgs {
    int64_t n;
    const int64_t *ap; const int *aj; const int *av;     // A (int32 values)
    int *order; int *tail;                               // vertices by level; vertices placed
    int64_t *lb;                                         // lb[L]: first position of level L in order
    const int64_t *coff; const int *children; int *remaining;
    int64_t *row_off; int *row_len;                      // pool position and length of each row
    int *pcols; int *pvals; int64_t capacity;            // the row pool
    unsigned long long *base;                            // pool slots reserved so far
    int *wide; int *nwide; int64_t *wlb;                 // block-tier rows; wlb[L]: first of level L
    unsigned long long *max_abs;
    unsigned long long *total;                           // entries written
    int *flags;                                          // 1: pool too small, 2: row past the block table
    int *nlevels;
    DagRec *rec;                                         // per order position: the row to fill
    unsigned long long *desc;                            // per stored entry: parent row (offset << 24 | length)
};


__device__ __forceinline__ int dag_abs(int v) { return v > 0 ? v : (int)(0u - (unsigned)v); }

// (column, value) sort key: ascending keys put a column's signed-minimum non-zero value first and
// a zero after every non-zero value.
__device__ __forceinline__ unsigned long long dag_key(int col, int v) {
    unsigned e = 0xffffffffu;
    if (v != 0) e = ((unsigned)v ^ 0x80000000u) - (v > 0 ? 1u : 0u);
    return ((unsigned long long)(unsigned)col << 32) | e;
}
__device__ __forceinline__ int dag_key_val(unsigned long long k) {
    const unsigned e = (unsigned)k;
    if (e == 0xffffffffu) return 0;
    return e >= 0x80000000u ? (int)((e + 1u) ^ 0x80000000u) : (int)(e ^ 0x80000000u);
}

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

template <int SLOTS>
__device__ __forceinline__ void dag_clear(DagTable<SLOTS> &H, int S, int lane, int nthreads) {
    for (int s = lane; s < S; s += nthreads) {
        H.key[s] = DG_NOKEY;
        H.val[s] = DG_NOVAL;
        H.has[s] = 0;
    }
}

// ----------------------------------------------------------------------------- candidate walk
// The candidates of a row, flattened: stored entry e of the row opens a segment of 1 + len(w)
// positions (the entry itself, then A[v][w] (x) C[w][f] for f < len(w); len = 0 when w == v).
// A group of G lanes (G = 8, 16 or 32; lane gl of the group) walks one row, one chunk of up to
// G stored entries at a time: lane gl holds chunk entry gl.
struct DagSeg {
    int w, avw, len, excl;
    int64_t off;
};

// Load chunk entry gl of a row (stored entries [e0, e1)) and scan the segment lengths over the
// group; returns the chunk's candidate count (all lanes of the group).
template <int G>
__device__ __forceinline__ int dag_seg_load(const DagArgs &a, int64_t e0, int64_t e1, int gl, DagSeg &sg) {
    const int64_t e = e0 + gl;
    sg.w = -1; sg.avw = 0; sg.len = 0; sg.off = 0;
    int cnt = 0;
    if (e < e1) {
        sg.w = a.aj[e];
        sg.avw = a.av[e];
        const unsigned long long d = a.desc[e];  // zero for the diagonal and invalid columns
        sg.len = (int)(d & ((1ull << DG_DESC_LEN_BITS) - 1));
        sg.off = (int64_t)(d >> DG_DESC_LEN_BITS);
        cnt = 1 + sg.len;
    }
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < G; o <<= 1) {
        const int t = __shfl_up_sync(FULL, incl, o, G);
        if (gl >= o) incl += t;
    }
    sg.excl = incl - cnt;
    return __shfl_sync(FULL, incl, G - 1, G);
}

// Candidate at chunk position idx (< the chunk's count when `in`): returns false for a zero
// product (no candidate); else its column and value.  Every lane must call it (shuffles).
template <int G>
__device__ __forceinline__ bool dag_candidate(const DagArgs &a, const DagSeg &sg, int idx, bool in, int &col,
                                              int &val) {
    int lo = 0;                                  // last segment starting at or before idx
#pragma unroll
    for (int st = G / 2; st > 0; st >>= 1) {
        const int x = __shfl_sync(FULL, sg.excl, lo + st, G);
        if (x <= idx) lo += st;
    }
    const int w = __shfl_sync(FULL, sg.w, lo, G);
    const int avw = __shfl_sync(FULL, sg.avw, lo, G);
    const int64_t off = __shfl_sync(FULL, sg.off, lo, G);
    const int x0 = __shfl_sync(FULL, sg.excl, lo, G);
    if (!in) return false;
    const int f = idx - x0;
    if (f == 0) {                                // the stored entry itself (a zero is kept)
        col = w;
        val = avw;
        return true;
    }
    col = a.pcols[off + f - 1];
    val = cy_product(avw, a.pvals[off + f - 1]);
    return val != 0;
}

// ----------------------------------------------------------------------------- register sorts
// Bitonic sort of G * H keys held H per lane of a G-lane group (element i = gl + G h).
template <int G, int H>
__device__ __forceinline__ void dag_sort(unsigned long long (&v)[H], int gl) {
#pragma unroll
    for (int k = 2; k <= G * H; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j >= G) {                        // partners in the same lane
                const int hj = j / G;
#pragma unroll
                for (int h = 0; h < H; ++h) {
                    if (h & hj) continue;
                    const bool up = ((gl + G * h) & k) == 0;
                    const unsigned long long x = v[h], y = v[h | hj];
                    const unsigned long long lo = min(x, y), hi = max(x, y);
                    v[h] = up ? lo : hi;
                    v[h | hj] = up ? hi : lo;
                }
            } else {
#pragma unroll
                for (int h = 0; h < H; ++h) {
                    const int i = gl + G * h;
                    const unsigned long long o = __shfl_xor_sync(FULL, v[h], j, G);
                    const bool up = (i & k) == 0, lower = (i & j) == 0;
                    v[h] = (lower == up) ? min(v[h], o) : max(v[h], o);
                }
            }
        }
    }
}

// One row per G-lane group (group g = lane / G) of at most G H candidates from at most G stored
// entries: keys sorted in registers, the first key of every column written at the row's pool
// position.  Every lane calls it; a group with act == false has no row.  Returns the row length.
template <int G, int H>
__device__ __forceinline__ int dag_group_row(const DagArgs &a, bool act, const DagRec &r, int lane, int &best) {
    const int gl = lane & (G - 1);
    DagSeg sg;
    const int T = dag_seg_load<G>(a, r.e0, act ? r.e0 + r.na : r.e0, gl, sg);
    unsigned long long key[H];
#pragma unroll
    for (int h = 0; h < H; ++h) {
        key[h] = DG_PAD;
        int col = 0, val = 0;
        if (dag_candidate<G>(a, sg, h * G + gl, h * G + gl < T, col, val)) {
            key[h] = dag_key(col, val);
            best = max(best, dag_abs(val));
        }
    }
    dag_sort<G, H>(key, gl);
    const unsigned lt = (1u << lane) - 1u;
    const unsigned gm = G == 32 ? FULL : ((1u << G) - 1u) << (lane & ~(G - 1));
    int nd = 0;
    unsigned long long carry = DG_PAD;            // the group's last key of the previous register
#pragma unroll
    for (int h = 0; h < H; ++h) {
        const unsigned long long up1 = __shfl_up_sync(FULL, key[h], 1, G);
        const unsigned long long prev = gl == 0 ? carry : up1;
        const bool head = key[h] != DG_PAD && ((gl == 0 && h == 0) || (prev >> 32) != (key[h] >> 32));
        const unsigned bal = __ballot_sync(FULL, head) & gm;
        if (head) {
            const int q = nd + __popc(bal & lt);
            a.pcols[r.off + q] = (int)(key[h] >> 32);
            a.pvals[r.off + q] = dag_key_val(key[h]);
        }
        nd += __popc(bal);
        carry = __shfl_sync(FULL, key[h], G - 1, G);
    }
    return nd;
}

// ----------------------------------------------------------------------------- merge of sorted runs
// A row's candidates are sorted runs: its stored entries (ascending columns) and each parent's
// closed row times the edge value (ascending columns).  With merge keys (column, zero-product
// flag, value code) a run stays sorted with its zero products in place.  The stored run goes to
// the front of a window of G H positions; each parent run then goes, descending, to the end of
// the window, which makes the window bitonic, and one bitonic merge (log2(G H) steps) sorts it.
// After the last merge the first key of a column carries the column's value, or the flag when
// the column has no candidate.
__device__ __forceinline__ unsigned long long dag_mkey(int col, int v) {
    unsigned e = 0xffffffffu;
    if (v != 0) e = ((unsigned)v ^ 0x80000000u) - (v > 0 ? 1u : 0u);
    return ((unsigned long long)(unsigned)col << 33) | e;
}
__device__ __forceinline__ unsigned long long dag_mkey_drop(int col) {
    return ((unsigned long long)(unsigned)col << 33) | (1ull << 32) | 0xffffffffull;
}

template <int G, int H>
__device__ __forceinline__ void dag_merge_asc(unsigned long long (&v)[H], int gl) {
#pragma unroll
    for (int j = G * H / 2; j > 0; j >>= 1) {
        if (j >= G) {
            const int hj = j / G;
#pragma unroll
            for (int h = 0; h < H; ++h) {
                if (h & hj) continue;
                const unsigned long long x = v[h], y = v[h | hj];
                v[h] = min(x, y);
                v[h | hj] = max(x, y);
            }
        } else {
#pragma unroll
            for (int h = 0; h < H; ++h) {
                const unsigned long long o = __shfl_xor_sync(FULL, v[h], j, G);
                v[h] = (gl & j) == 0 ? min(v[h], o) : max(v[h], o);
            }
        }
    }
}

__host__ __device__ constexpr int dag_log2(int x) { return x <= 1 ? 0 : 1 + dag_log2(x / 2); }

// One row per G-lane group, as dag_group_row, by merges of sorted runs.  Returns -1 (nothing
// written) when the warp should sort instead: a stored run that does not ascend strictly, more
// stored entries than lanes, or so many parent runs that the merges cost more than a sort.
template <int G, int H>
__device__ __forceinline__ int dag_group_row_runs(const DagArgs &a, bool act, const DagRec &r, int lane, int &best) {
    constexpr int P2 = G * H, LG = dag_log2(G * H);
    const int gl = lane & (G - 1);
    const bool has = act && gl < r.na;
    int w = -1, avw = 0, len = 0;
    int64_t off = 0;
    if (has) {
        w = a.aj[r.e0 + gl];
        avw = a.av[r.e0 + gl];
        const unsigned long long d = a.desc[r.e0 + gl];
        len = (int)(d & ((1ull << DG_DESC_LEN_BITS) - 1));
        off = (int64_t)(d >> DG_DESC_LEN_BITS);
    }
    const int wn = __shfl_down_sync(FULL, w, 1, G);
    const bool bad = (act && r.na > G) || (has && gl + 1 < r.na && wn <= w);
    const int runs = __popc(__ballot_sync(FULL, len > 0) & (G == 32 ? FULL : ((1u << G) - 1u) << (lane & ~(G - 1))));
    const int maxruns = __reduce_max_sync(FULL, (unsigned)runs);
    if (__any_sync(FULL, bad) || maxruns * LG >= LG * (LG + 1) / 2) return -1;
    unsigned long long key[H];
#pragma unroll
    for (int h = 0; h < H; ++h) key[h] = DG_PAD;
    if (has) {                                   // the stored run: positions [0, na)
        key[0] = dag_mkey(w, avw);
        best = max(best, dag_abs(avw));
    }
    const int nam = __reduce_max_sync(FULL, act ? (unsigned)r.na : 0u);
    for (int j = 0; j < nam; ++j) {
        const int lj = __shfl_sync(FULL, len, j, G);
        if (!__any_sync(FULL, lj > 0)) continue;
        const int64_t oj = __shfl_sync(FULL, off, j, G);
        const int vj = __shfl_sync(FULL, avw, j, G);
#pragma unroll
        for (int h = 0; h < H; ++h) {
            const int p = gl + G * h;
            if (p >= P2 - lj) {                  // element P2 - 1 - p of the run, descending
                const int64_t f = oj + (P2 - 1 - p);
                const int col = a.pcols[f];
                const int pv = cy_product(vj, a.pvals[f]);
                key[h] = pv != 0 ? dag_mkey(col, pv) : dag_mkey_drop(col);
                best = max(best, pv != 0 ? dag_abs(pv) : 0);
            }
        }
        dag_merge_asc<G, H>(key, gl);
    }
    const unsigned lt = (1u << lane) - 1u;
    const unsigned gm = G == 32 ? FULL : ((1u << G) - 1u) << (lane & ~(G - 1));
    int nd = 0;
    unsigned long long carry = DG_PAD;
#pragma unroll
    for (int h = 0; h < H; ++h) {
        const unsigned long long up1 = __shfl_up_sync(FULL, key[h], 1, G);
        const unsigned long long prev = gl == 0 ? carry : up1;
        const bool head = key[h] != DG_PAD && !((key[h] >> 32) & 1ull) &&
                          ((gl == 0 && h == 0) || (prev >> 33) != (key[h] >> 33));
        const unsigned bal = __ballot_sync(FULL, head) & gm;
        if (head) {
            const int q = nd + __popc(bal & lt);
            a.pcols[r.off + q] = (int)(key[h] >> 33);
            a.pvals[r.off + q] = dag_key_val(key[h]);
        }
        nd += __popc(bal);
        carry = __shfl_sync(FULL, key[h], G - 1, G);
    }
    return nd;
}

// ----------------------------------------------------------------------------- level discovery
// Append the lanes' ready vertices to the order, bound their rows and reserve their pool slots.
__device__ __forceinline__ void dag_append(const DagArgs &a, bool ready, int c, long long ub, int64_t e0, int lane) {
    const unsigned bal = __ballot_sync(FULL, ready);
    if (!bal) return;
    int pos0 = 0;
    if (lane == 0) pos0 = atomicAdd(a.tail, __popc(bal));
    pos0 = __shfl_sync(FULL, pos0, 0);
    const long long x = ready ? ub : 0;
    long long incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long t = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += t;
    }
    const long long tot = __shfl_sync(FULL, incl, 31);
    unsigned long long b0 = 0;
    if (lane == 0) b0 = atomicAdd(a.base, (unsigned long long)tot);
    b0 = __shfl_sync(FULL, b0, 0);
    if (ready) {
        const int pos = pos0 + __popc(bal & ((1u << lane) - 1u));
        a.order[pos] = c;
        long long off = (long long)b0 + incl - x;
        if (off + x > a.capacity) {              // past the pool: skipped, the call asks for more
            off = -1;
            a.row_len[c] = 0;
            atomicOr(a.flags, 1);
        } else if (x > DG_WSLOTS) {
            a.wide[atomicAdd(a.nwide, 1)] = c;
        }
        a.row_off[c] = off;
        DagRec r;
        r.off = off;
        r.e0 = e0;
        r.v = c;
        r.ub = (int)min(x, (long long)INT_MAX);
        r.na = (int)(a.ap[c + 1] - e0);
        r.pad = 0;
        a.rec[pos] = r;
    }
}

// Upper bound of row c's length (its stored entries plus its parents' rows, all done); records
// each stored entry's parent row for the fill pass.
__device__ __forceinline__ long long dag_bound(const DagArgs &a, int c, int64_t &e0) {
    long long ub = 0;
    e0 = a.ap[c];
    for (int64_t q = e0; q < a.ap[c + 1]; ++q) {
        const int x = a.aj[q];
        unsigned long long d = 0;
        if (x != c && x >= 0 && x < a.n) {
            const int len = a.row_len[x];
            const int64_t off = a.row_off[x];
            ub += len;
            if (len > 0) d = ((unsigned long long)off << DG_DESC_LEN_BITS) | (unsigned long long)len;
        }
        a.desc[q] = d;
        ub += 1;
    }
    return ub;
}

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

// Level 0: the vertices without parents.
__global__ void dag_roots_kernel(DagArgs a) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t v0 = ((int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; v0 < a.n; v0 += warps * 32) {
        const int64_t v = v0 + lane;
        const bool ready = v < a.n && a.remaining[v] == 0;
        int64_t e0 = 0;
        const long long ub = ready ? dag_bound(a, (int)v, e0) : 0;
        dag_append(a, ready, (int)v, ub, e0, lane);
    }
}

// The level a kernel works on: L itself, or L levels past the device-resident level counter *Lp
// (the level loop run as a CUDA-graph while node); false past the last possible level.
__device__ __forceinline__ bool dag_level(const DagArgs &a, int64_t &L, const int64_t *Lp) {
    if (Lp) L += *Lp;
    return L < a.n;
}

// Level L + 1 from level L: every child edge of the level's vertices, flattened over the warp.
__global__ void dag_discover_kernel(DagArgs a, int64_t L, const int64_t *Lp) {
    if (!dag_level(a, L, Lp)) return;
    const int lane = threadIdx.x & 31;
    const int64_t s = a.lb[L], e = a.lb[L + 1];
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t k0 = s + ((int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; k0 < e;
         k0 += warps * 32) {
        const int64_t k = k0 + lane;
        int64_t c0 = 0;
        int cnt = 0;
        if (k < e) {
            const int w = a.order[k];
            c0 = a.coff[w];
            cnt = (int)(a.coff[w + 1] - c0);
        }
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += t;
        }
        const int excl = incl - cnt;
        const int T = __shfl_sync(FULL, incl, 31);
        for (int b = 0; b < T; b += 32) {
            const int idx = b + lane;
            int lo = 0;
#pragma unroll
            for (int st = 16; st > 0; st >>= 1) {
                const int x = __shfl_sync(FULL, excl, lo + st);
                if (x <= idx) lo += st;
            }
            const int64_t cq = __shfl_sync(FULL, c0, lo);
            const int xq = __shfl_sync(FULL, excl, lo);
            bool ready = false;
            int c = 0;
            long long ub = 0;
            int64_t e0 = 0;
            if (idx < T) {
                c = a.children[cq + (idx - xq)];
                if (atomicSub(&a.remaining[c], 1) == 1) {
                    ready = true;
                    ub = dag_bound(a, c, e0);
                }
            }
            dag_append(a, ready, c, ub, e0, lane);
        }
    }
}

// ----------------------------------------------------------------------------- fill passes
// Write a warp's table (S slots) as a sorted row at pool position o; returns the row length.
// Up to 64 distinct columns sort in registers, more in shared memory.
__device__ __forceinline__ int dag_table_row(const DagArgs &a, DagTable<DG_WSLOTS> &H, int S, int64_t o, int lane) {
    int nd = 0;
    for (int s0 = 0; s0 < S; s0 += 32) {
        const int s = s0 + lane;
        const bool occ = H.key[s] != DG_NOKEY;
        const unsigned bal = __ballot_sync(FULL, occ);
        if (occ) H.list[nd + __popc(bal & ((1u << lane) - 1u))] = ((unsigned long long)H.key[s] << 32) | (unsigned)s;
        nd += __popc(bal);
    }
    __syncwarp();
    if (nd <= 64) {
        unsigned long long v[2];
        v[0] = lane < nd ? H.list[lane] : DG_PAD;
        v[1] = lane + 32 < nd ? H.list[lane + 32] : DG_PAD;
        dag_sort<32, 2>(v, lane);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int q = lane + 32 * h;
            if (q < nd) {
                const int sl = (int)(v[h] & 0xffffffffu);
                a.pcols[o + q] = (int)(v[h] >> 32);
                a.pvals[o + q] = H.has[sl] ? H.val[sl] : 0;
            }
        }
        __syncwarp();
        return nd;
    }
    int P = 32;
    while (P < nd) P <<= 1;
    for (int q = nd + lane; q < P; q += 32) H.list[q] = DG_PAD;
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
    for (int q = lane; q < nd; q += 32) {
        const unsigned long long e = H.list[q];
        const int s = (int)(e & 0xffffffffu);
        a.pcols[o + q] = (int)(e >> 32);
        a.pvals[o + q] = H.has[s] ? H.val[s] : 0;
    }
    __syncwarp();
    return nd;
}

// A row of up to 256 candidates through the warp's table (ub >= distinct columns, so a table of
// ub slots never fills).  Returns the row length.
__device__ __noinline__ int dag_table_fill(const DagArgs &a, DagTable<DG_WSLOTS> &H, const DagRec &r, int lane,
                                              int &best) {
    int S = 32;
    while (S < r.ub) S <<= 1;
    dag_clear(H, S, lane, 32);
    __syncwarp();
    for (int64_t c0 = r.e0; c0 < r.e0 + r.na; c0 += 32) {
        DagSeg sg;
        const int T = dag_seg_load<32>(a, c0, r.e0 + r.na, lane, sg);
        for (int b = 0; b < T; b += 32) {
            int col = 0, val = 0;
            if (dag_candidate<32>(a, sg, b + lane, b + lane < T, col, val)) {
                best = max(best, dag_abs(val));
                dag_fold(H, (unsigned)col, val, S - 1);
            }
        }
    }
    __syncwarp();
    return dag_table_row(a, H, S, r.off, lane);
}

__device__ __forceinline__ DagRec dag_shfl_rec(const DagRec &r, int src) {
    DagRec o;
    o.off = __shfl_sync(FULL, r.off, src);
    o.e0 = __shfl_sync(FULL, r.e0, src);
    o.v = __shfl_sync(FULL, r.v, src);
    o.ub = __shfl_sync(FULL, r.ub, src);
    o.na = __shfl_sync(FULL, r.na, src);
    o.pad = 0;
    return o;
}

// Level L's rows of up to 256 candidates, four consecutive rows per warp at a time, each by its
// own size: the rows of at most 8 candidates fill together (8 lanes each), then those of at most
// 16 two at a time, then the larger ones one after the other with the whole warp (deciding by the
// largest of the four sent three quarters of a pedigree forest's iterations down the slowest
// path).  Lanes 8i..8i+7 hold row i's record; the next four records are read before the current
// rows are filled.  Block 0 closes the level's range.
__global__ void __launch_bounds__(DG_WARPS * 32) dag_fill_kernel(DagArgs a, int64_t L, const int64_t *Lp) {
    if (!dag_level(a, L, Lp)) return;
    extern __shared__ __align__(16) unsigned char dg_smem[];
    const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
    DagTable<DG_WSLOTS> &H = reinterpret_cast<DagTable<DG_WSLOTS> *>(dg_smem)[wi];
    const int64_t s = a.lb[L], e = *a.tail;      // nothing appends to the order during the fill
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.lb[L + 1] = e;
        if (e > s) atomicAdd(a.nlevels, 1);
    }
    int best = 0;
    unsigned long long written = 0;
    const int64_t warps = (int64_t)gridDim.x * DG_WARPS;
    const int64_t nq = (e - s + 3) >> 2;
    const int sub = lane >> 3;
    int64_t q = (int64_t)blockIdx.x * DG_WARPS + wi;
    DagRec cur;
    bool cv = false;
    if (q < nq && s + 4 * q + sub < e) {
        cur = a.rec[s + 4 * q + sub];
        cv = true;
    }
    for (; q < nq; q += warps) {
        DagRec nxt;
        bool nv = false;
        const int64_t kn = s + 4 * (q + warps) + sub;
        if (q + warps < nq && kn < e) {
            nxt = a.rec[kn];
            nv = true;
        }
        const bool act = cv && cur.off >= 0 && cur.ub <= DG_WSLOTS;   // else skipped, or the block tier's
        const bool lead = (lane & 7) == 0;       // the lane that speaks for its group's row
        // rows of at most 8 candidates: each 8-lane group fills its own, all at once
        const bool a8 = act && cur.ub <= 8;
        if (__any_sync(FULL, a8)) {
            const int nd = dag_group_row<8, 1>(a, a8, cur, lane, best);
            if (lead && a8) {
                a.row_len[cur.v] = nd;
                written += (unsigned long long)nd;
            }
        }
        // rows of 9 to 16: two at a time, 16 lanes each
        unsigned b16 = __ballot_sync(FULL, lead && act && cur.ub > 8 && cur.ub <= 16);
        while (b16) {
            const int r0 = __ffs(b16) - 1;
            b16 &= b16 - 1;
            const int r1 = b16 ? __ffs(b16) - 1 : -1;
            if (b16) b16 &= b16 - 1;
            const bool upper = lane >= 16;
            const int src = upper ? (r1 >= 0 ? r1 : r0) : r0;
            const DagRec r = dag_shfl_rec(cur, src);
            const bool ra = !upper || r1 >= 0;
            const int nd = dag_group_row<16, 1>(a, ra, r, lane, best);
            if ((lane & 15) == 0 && ra) {
                a.row_len[r.v] = nd;
                written += (unsigned long long)nd;
            }
        }
        // larger rows: one after another with the whole warp
        unsigned bw = __ballot_sync(FULL, lead && act && cur.ub > 16);
        while (bw) {
            const int src = __ffs(bw) - 1;
            bw &= bw - 1;
            {
                const DagRec r = dag_shfl_rec(cur, src);
                int nd = -1;
                if (r.ub <= 32) {
                    nd = dag_group_row_runs<32, 1>(a, true, r, lane, best);
                    if (nd < 0) nd = dag_group_row<32, 1>(a, true, r, lane, best);
                } else if (r.ub <= 64 && r.na <= 32) {
                    nd = dag_group_row_runs<32, 2>(a, true, r, lane, best);
                    if (nd < 0) nd = dag_group_row<32, 2>(a, true, r, lane, best);
                } else if (r.ub <= 128 && r.na <= 32) {
                    nd = dag_group_row_runs<32, 4>(a, true, r, lane, best);
                }
                if (nd < 0) nd = dag_table_fill(a, H, r, lane, best);
                if (lane == 0) {
                    a.row_len[r.v] = nd;
                    written += (unsigned long long)nd;
                }
            }
        }
        cur = nxt;
        cv = nv;
    }
    best = __reduce_max_sync(FULL, best);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) written += __shfl_xor_sync(FULL, written, o);   // group leaders' counts
    if (lane == 0) {
        if (best > 0) atomicMax(a.max_abs, (unsigned long long)best);
        if (written) atomicAdd(a.total, written);
    }
}

// One 512-thread block per row of level L with more than 256 candidates.
__global__ void __launch_bounds__(DG_BTHREADS) dag_fill_block_kernel(DagArgs a, int64_t L, const int64_t *Lp) {
    if (!dag_level(a, L, Lp)) return;
    extern __shared__ __align__(16) unsigned char dg_smem[];
    DagTable<DG_BSLOTS> &H = *reinterpret_cast<DagTable<DG_BSLOTS> *>(dg_smem);
    __shared__ int s_nd, s_ok;
    const int64_t s = a.wlb[L], e = *a.nwide;
    if (blockIdx.x == 0 && threadIdx.x == 0) a.wlb[L + 1] = e;
    int best = 0;
    for (int64_t b = s + blockIdx.x; b < e; b += gridDim.x) {
        const int v = a.wide[b];
        const int64_t o = a.row_off[v];
        dag_clear(H, DG_BSLOTS, threadIdx.x, DG_BTHREADS);
        if (threadIdx.x == 0) { s_nd = 0; s_ok = 1; }
        __syncthreads();
        bool ok = true;
        for (int64_t q = a.ap[v] + threadIdx.x; q < a.ap[v + 1]; q += DG_BTHREADS) {   // stored entries
            const int val = a.av[q];
            best = max(best, dag_abs(val));
            ok &= dag_fold(H, (unsigned)a.aj[q], val, DG_BSLOTS - 1);
        }
        for (int64_t q = a.ap[v]; q < a.ap[v + 1]; ++q) {                              // parents' rows
            const int w = a.aj[q];
            if (w == v || w < 0 || w >= a.n) continue;
            const int avw = a.av[q];
            const int64_t po = a.row_off[w];
            const int len = a.row_len[w];
            for (int f = threadIdx.x; f < len; f += DG_BTHREADS) {
                const int p = cy_product(avw, a.pvals[po + f]);
                if (p == 0) continue;
                best = max(best, dag_abs(p));
                ok &= dag_fold(H, (unsigned)a.pcols[po + f], p, DG_BSLOTS - 1);
            }
        }
        if (!ok) s_ok = 0;
        __syncthreads();
        if (!s_ok) {                             // more distinct columns than the table
            if (threadIdx.x == 0) { atomicOr(a.flags, 2); a.row_len[v] = 0; }
            __syncthreads();
            continue;
        }
        for (int q = threadIdx.x; q < DG_BSLOTS; q += DG_BTHREADS)
            if (H.key[q] != DG_NOKEY) H.list[atomicAdd(&s_nd, 1)] = ((unsigned long long)H.key[q] << 32) | (unsigned)q;
        __syncthreads();
        const int nd = s_nd;
        int P = 1;
        while (P < nd) P <<= 1;
        for (int q = nd + threadIdx.x; q < P; q += DG_BTHREADS) H.list[q] = DG_PAD;
        __syncthreads();
        for (int k = 2; k <= P; k <<= 1) {
            for (int jj = k >> 1; jj > 0; jj >>= 1) {
                for (int q = threadIdx.x; q < P; q += DG_BTHREADS) {
                    const int qx = q ^ jj;
                    if (qx > q) {
                        const unsigned long long x = H.list[q], y = H.list[qx];
                        if ((x > y) == ((q & k) == 0)) { H.list[q] = y; H.list[qx] = x; }
                    }
                }
                __syncthreads();
            }
        }
        for (int q = threadIdx.x; q < nd; q += DG_BTHREADS) {
            const unsigned long long ek = H.list[q];
            const int sl = (int)(ek & 0xffffffffu);
            a.pcols[o + q] = (int)(ek >> 32);
            a.pvals[o + q] = H.has[sl] ? H.val[sl] : 0;
        }
        if (threadIdx.x == 0) {
            a.row_len[v] = nd;
            atomicAdd(a.total, (unsigned long long)nd);
        }
        __syncthreads();
    }
    best = __reduce_max_sync(FULL, best);
    if ((threadIdx.x & 31) == 0 && best > 0) atomicMax(a.max_abs, (unsigned long long)best);
}

// ----------------------------------------------------------------------------- pool -> CSR
// Eight lanes per row.
__global__ void dag_gather_rows_kernel(int64_t n, const int64_t *row_off, const int *pcols, const int *pvals,
                                       const int64_t *indptr, int *cj, int *cx) {
    const int sub = threadIdx.x & 7;
    const int64_t groups = (int64_t)gridDim.x * (blockDim.x >> 3);
    for (int64_t v = (int64_t)blockIdx.x * (blockDim.x >> 3) + (threadIdx.x >> 3); v < n; v += groups) {
        const int64_t dst = indptr[v], len = indptr[v + 1] - dst;
        if (len == 0) continue;
        const int64_t src = row_off[v];
        for (int64_t e = sub; e < len; e += 8) {
            cj[dst + e] = pcols[src + e];
            cx[dst + e] = pvals[src + e];
        }
    }
}

__global__ void dag_len64_kernel(int64_t n, const int *row_len, int64_t *len64) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v <= n; v += (int64_t)gridDim.x * blockDim.x)
        len64[v] = v < n ? row_len[v] : 0;
}

// One iteration of the graph's level loop has run DAG_GRAPH_CHUNK levels from *Lp: advance the
// counter and keep looping while the next level holds a vertex (fill(L - 1) wrote lb[L]).
__global__ void dag_advance_kernel(DagArgs a, int64_t *Lp, cudaGraphConditionalHandle h) {
    if (threadIdx.x != 0) return;
    const int64_t L = *Lp + DAG_GRAPH_CHUNK;
    *Lp = L;
    cudaGraphSetConditional(h, (L < a.n && (int64_t)*a.tail > a.lb[L]) ? 1u : 0u);
}

}  // namespace rbg

using namespace rbg;

namespace {

struct DagWs {
    int *remaining, *ccount, *cursor, *children, *order, *wide;
    int64_t *coff, *lb, *wlb;
    DagCounters *cnt;
    DagRec *rec;
    unsigned long long *desc;
    void *tmp;
    size_t tmp_bytes;
};

size_t dag_tmp_bytes(int64_t n) {
    size_t a = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, a, (int *)nullptr, (int64_t *)nullptr, (int)std::max<int64_t>(n + 1, 1));
    return a;
}

size_t dag_layout(int64_t n, int64_t nnz, unsigned char *base, DagWs *w) {
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o = align_up(o + bytes, 256); return base ? base + at : nullptr; };
    const size_t ni = (size_t)(n + 1) * 4, nl = (size_t)(n + 2) * 8;
    unsigned char *p;
    p = take(ni); if (w) w->remaining = (int *)p;
    p = take(ni); if (w) w->ccount = (int *)p;
    p = take(ni); if (w) w->cursor = (int *)p;
    p = take((size_t)std::max<int64_t>(nnz, 1) * 4); if (w) w->children = (int *)p;
    p = take(ni); if (w) w->order = (int *)p;
    p = take((size_t)(n + 1) * sizeof(DagRec)); if (w) w->rec = (DagRec *)p;
    p = take((size_t)std::max<int64_t>(nnz, 1) * 8); if (w) w->desc = (unsigned long long *)p;
    p = take(ni); if (w) w->wide = (int *)p;
    p = take(nl); if (w) w->coff = (int64_t *)p;
    p = take(nl); if (w) w->lb = (int64_t *)p;
    p = take(nl); if (w) w->wlb = (int64_t *)p;
    p = take(sizeof(DagCounters)); if (w) w->cnt = (DagCounters *)p;   // zeroed together
    const size_t tb = dag_tmp_bytes(n);
    p = take(tb); if (w) { w->tmp = p; w->tmp_bytes = tb; }
    return o;
}

PerDeviceOnce g_dag_configured;

int dag_configure() {
    return g_dag_configured.run([] {
        RBG_CUDA_TRY(cudaFuncSetAttribute(dag_fill_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)(sizeof(DagTable<DG_WSLOTS>) * DG_WARPS)));
        RBG_CUDA_TRY(cudaFuncSetAttribute(dag_fill_block_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)sizeof(DagTable<DG_BSLOTS>)));
        return (int)RBG_OK;
    });
}

DagArgs dag_args(int64_t n, const rbg_csr_t *A, const DagWs &w, int32_t *pool_cols, int32_t *pool_vals,
                 int64_t pool_capacity, int64_t *row_off, int32_t *row_len) {
    DagArgs a;
    a.n = n; a.ap = A->indptr; a.aj = reinterpret_cast<const int *>(A->indices);
    a.av = reinterpret_cast<const int *>(A->data);
    a.order = w.order; a.tail = &w.cnt->placed; a.lb = w.lb;
    a.coff = w.coff; a.children = w.children; a.remaining = w.remaining;
    a.row_off = row_off; a.row_len = row_len; a.rec = w.rec; a.desc = w.desc;
    a.pcols = pool_cols; a.pvals = pool_vals; a.capacity = pool_capacity;
    a.base = &w.cnt->reserved; a.wide = w.wide; a.nwide = &w.cnt->nwide; a.wlb = w.wlb;
    a.max_abs = &w.cnt->max_abs; a.total = &w.cnt->total; a.flags = &w.cnt->flags; a.nlevels = &w.cnt->nlevels;
    return a;
}

// parents -> children lists and level 0
int dag_front(const DagArgs &a, const DagWs &w, cudaStream_t s) {
    const int64_t n = a.n;
    const int g = grid_for(n, 256);
    RBG_CUDA_TRY(cudaMemsetAsync(w.ccount, 0, (size_t)(n + 1) * 4, s));
    RBG_CUDA_TRY(cudaMemsetAsync(w.cursor, 0, (size_t)(n + 1) * 4, s));
    RBG_CUDA_TRY(cudaMemsetAsync(w.cnt, 0, sizeof(DagCounters), s));
    RBG_CUDA_TRY(cudaMemsetAsync(w.lb, 0, 8, s));
    RBG_CUDA_TRY(cudaMemsetAsync(w.wlb, 0, 8, s));
    note_launches(4);
    dag_indeg_kernel<<<g, 256, 0, s>>>(n, a.ap, a.aj, w.remaining, w.ccount);
    size_t tb = w.tmp_bytes;
    RBG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(w.tmp, tb, w.ccount, w.coff, (int)(n + 1), s));
    dag_children_kernel<<<g, 256, 0, s>>>(n, a.ap, a.aj, w.coff, w.cursor, w.children);
    dag_roots_kernel<<<g, 256, 0, s>>>(a);
    RBG_CUDA_TRY(cudaGetLastError());
    return RBG_OK;
}

struct LevelLaunch {
    int fill_grid, disc_grid, block_grid;
    size_t wsm, bsm;
};

LevelLaunch level_launch() {
    LevelLaunch l;
    l.wsm = sizeof(DagTable<DG_WSLOTS>) * DG_WARPS;
    l.bsm = sizeof(DagTable<DG_BSLOTS>);
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, dag_fill_kernel, DG_WARPS * 32, l.wsm) != cudaSuccess || b < 1)
        b = 4;
    int bd = 0;                              // discovery: one wave of resident CTAs
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bd, dag_discover_kernel, 256, 0) != cudaSuccess || bd < 1)
        bd = 4;
    const int sms = sm_count();
    l.fill_grid = sms * b;
    l.disc_grid = sms * bd;
    l.block_grid = sms;
    return l;
}

void launch_level(const DagArgs &a, const LevelLaunch &l, int64_t L, const int64_t *Lp, cudaStream_t s) {
    dag_fill_kernel<<<l.fill_grid, DG_WARPS * 32, l.wsm, s>>>(a, L, Lp);
    dag_fill_block_kernel<<<l.block_grid, DG_BTHREADS, l.bsm, s>>>(a, L, Lp);
    dag_discover_kernel<<<l.disc_grid, 256, 0, s>>>(a, L, Lp);
}

// Levels launched in chunks of 8 without waiting (every kernel reads its level's bounds from
// device memory and exits at once on an empty level); the host looks at the frontier once per
// chunk.
int dag_levels_host(const DagArgs &a, const DagWs &w, cudaStream_t s, int64_t *launches) {
    const LevelLaunch l = level_launch();
    const int64_t chunk = 8;
    int64_t L = 0;
    while (true) {
        const int64_t Lend = std::min<int64_t>(L + chunk, a.n);
        for (; L < Lend; ++L) {
            note_launches(3);
            *launches += 3;
            launch_level(a, l, L, nullptr, s);
        }
        RBG_CUDA_TRY(cudaGetLastError());
        // level L is empty when the order has not grown past its start (written by fill(L - 1))
        int tail = 0;
        int64_t start = 0;
        HostStaging hs(s, 256);
        int rc = hs.down(&tail, &w.cnt->placed, 4);
        if (!rc) rc = hs.down(&start, w.lb + L, 8);
        if (!rc) rc = hs.finish();
        if (rc) return rc;
        if ((int64_t)tail <= start || L >= a.n) break;
    }
    return RBG_OK;
}

// The level loop inside the graph being captured on `s`: a while node whose body runs
// DAG_GRAPH_CHUNK levels from the device-resident counter and then lets dag_advance_kernel
// decide whether to go on.  Nothing is read back by the host.
int dag_levels_graph(const DagArgs &a, const DagWs &w, cudaStream_t s) {
    const LevelLaunch l = level_launch();
    int64_t *Lp = reinterpret_cast<int64_t *>(&w.cnt->level);
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    RBG_CUDA_TRY(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &ndeps));
    if (st != cudaStreamCaptureStatusActive || !g) return RBG_ERR_INVALID;
    cudaGraphConditionalHandle h;
    RBG_CUDA_TRY(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    RBG_CUDA_TRY(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &p));
    cudaGraph_t body = p.conditional.phGraph_out[0];
    // the body is recorded from a second stream captured into it
    static thread_local cudaStream_t side = nullptr;
    if (!side) RBG_CUDA_TRY(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
    RBG_CUDA_TRY(cudaStreamBeginCaptureToGraph(side, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    for (int t = 0; t < DAG_GRAPH_CHUNK; ++t) launch_level(a, l, t, Lp, side);
    dag_advance_kernel<<<1, 32, 0, side>>>(a, Lp, h);
    const cudaError_t le = cudaGetLastError();
    cudaGraph_t got = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(side, &got);
    if (le != cudaSuccess || ee != cudaSuccess) return RBG_ERR_CUDA;
    RBG_CUDA_TRY(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    return RBG_OK;
}

}  // namespace

namespace rbg {

int sm_count() {
    static int sms[PerDeviceOnce::kMaxDevices] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= PerDeviceOnce::kMaxDevices) return 152;
    if (sms[dev] <= 0) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        sms[dev] = v > 0 ? v : 152;   // every thread writes the same value
    }
    return sms[dev];
}

size_t dag_workspace_for(int64_t n, int64_t nnz_bound) { return dag_layout(n, nnz_bound, nullptr, nullptr); }

int dag_enqueue(const rbg_csr_t *A, int64_t nnz_bound, void *workspace, int32_t *pool_cols, int32_t *pool_vals,
                int64_t pool_capacity, int64_t *row_off, int32_t *row_len, cudaStream_t s, bool captured,
                DagCounters **counters, int64_t *launches) {
    const int64_t n = A->n_rows;
    DagWs w;
    dag_layout(n, nnz_bound, reinterpret_cast<unsigned char *>(workspace), &w);
    *counters = w.cnt;
    int rc = dag_configure();
    if (rc) return rc;
    const DagArgs a = dag_args(n, A, w, pool_cols, pool_vals, pool_capacity, row_off, row_len);
    rc = dag_front(a, w, s);
    if (rc) return rc;
    *launches += 4;
    if (n == 0) return RBG_OK;
    return captured ? dag_levels_graph(a, w, s) : dag_levels_host(a, w, s, launches);
}

}  // namespace rbg

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
    if (n >= (1ll << 31) - 1) return RBG_ERR_INVALID;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int64_t annz = 0;
    {
        HostStaging hs(s, 256);
        int rc = hs.down(&annz, A->indptr + n, 8);
        if (!rc) rc = hs.finish();
        if (rc) return rc;
    }
    if (workspace_bytes < (int64_t)dag_layout(n, annz, nullptr, nullptr)) return RBG_ERR_NOMEM;
    DagCounters *dc = nullptr;
    int64_t launched = 0;
    int rc = dag_enqueue(A, annz, workspace, pool_cols, pool_vals, pool_capacity, row_off, row_len, s, false, &dc,
                         &launched);
    if (rc) return rc;
    DagCounters c;
    {
        HostStaging hs(s, 256);
        rc = hs.down(&c, dc, sizeof(c));
        if (!rc) rc = hs.finish();
        if (rc) return rc;
    }
    *levels = c.nlevels;
    if (c.placed < n) return RBG_ERR_CYCLE;      // vertices on (or below) a cycle were never placed
    if (c.flags & 2) { *nnz = -1; return RBG_ERR_CAPACITY; }
    if (c.flags & 1) {
        const int64_t reserved = (int64_t)c.reserved;
        *nnz = std::max<int64_t>(2 * pool_capacity, reserved + reserved / 2 + 1024);
        return RBG_ERR_CAPACITY;
    }
    *nnz = (int64_t)c.total;
    *max_abs = (int64_t)c.max_abs;
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
        dag_gather_rows_kernel<<<grid_for(n * 8, 256), 256, 0, s>>>(n, row_off, pool_cols, pool_vals, indptr,
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
