// dag_rows.cuh -- per-row statistics of a closure computed by the DAG recurrence, measured
// against the sequential Floyd-Warshall loop it stands in for (warshall.c.in:88-106).
// Included by fw_tri.cu (dense batches) and components.cu (component-wise closure of a CSR
// graph).
//
// For a matrix whose vertices are numbered in a topological order, step k of the sequential
// loop adds A(i, k) (x) C(k, .) to the rows of k's children (entries below the diagonal) or
// C(i, k) (x) A(k, .) to the rows that reach k (entries above it); see fw_tri.cu.  Per row the
// statistics are the largest MSB of those products (a product whose MSB reaches the top bit of
// the 32-bit value may overflow: the matrix then leaves the DAG path) and the largest MSB of the
// row's first values (A(i, j), else the product of the first step that reaches the cell), whose
// maximum over the matrix is the loop's diameter.
//
// A row is handled by a group of G lanes of one warp (G = 8 for the closures of pedigrees,
// whose rows hold about ten entries).  The group's kernels give each group runs of up to
// DAG_STATS_RUN consecutive rows and keep the statistics of the current matrix in registers, so
// a run issues its atomics once per matrix instead of once per row.
#pragma once
#include "rbg_internal.cuh"

namespace rbg {

constexpr int DAG_KIND_NONE = 0, DAG_KIND_BELOW = 1, DAG_KIND_ABOVE = 2;
constexpr int DAG_KIND_GENERAL = 3;   // entries on both sides of the diagonal (any numbering)
constexpr int DAG_TOP_MSB = 31;   // lbits - 1 for 32-bit values
constexpr int DAG_MAX_N = 8192;   // columns of a matrix the per-group bitmap covers
constexpr int DAG_STATS_G = 8;    // lanes per row in the statistics kernels
constexpr int DAG_STATS_RUN = 16; // most consecutive rows a group takes at a time

// The run length for `rows` rows over `groups` resident groups: DAG_STATS_RUN, shorter when
// the runs would leave groups idle (one matrix of a few thousand rows).
inline int dag_stats_run(int64_t rows, int64_t groups) {
    const int64_t r = rows / (groups > 0 ? groups : 1);
    return (int)(r < 1 ? 1 : r > DAG_STATS_RUN ? DAG_STATS_RUN : r);
}

// MSB of an off-diagonal value; a value no clean product yields (zero, or negative after a
// wrap) counts as reaching the top bit
__device__ __forceinline__ int dag_row_msb(int32_t v) { return v > 0 ? msb_u32((uint32_t)v) : 99; }

// the lanes of the calling lane's group of G
template <int G> __device__ __forceinline__ unsigned dag_group_mask() {
    if constexpr (G == 32) return 0xffffffffu;
    else return ((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1));
}

// One group of G lanes (`lane` in [0, G), `gmask` the group's lanes), row g whose off-diagonal
// entries are acol / aval[a0, a0 + alen).  A: the off-diagonal entries (CSR aptr / acol / aval,
// columns ascending); C: the closure rows, crow(r) -> (offset, length) into ccol / cval, columns
// ascending; local(col): the column's index inside its matrix.  bm: the group's bitmap (words
// 32-bit words, one bit per column of the matrix, at most DAG_MAX_N / 32 of them, 16-byte
// aligned), cleared here.  am / fm / prods accumulate the largest product MSB, the
// largest first-value MSB and the number of products.
template <int G, typename CRow, typename Local>
__device__ __forceinline__ void dag_row_stats(unsigned *bm, int words, int kind, int64_t g, int64_t a0, int alen,
                                              const int64_t *__restrict__ aptr, const int32_t *__restrict__ acol,
                                              const int32_t *__restrict__ aval, CRow crow,
                                              const int32_t *__restrict__ ccol, const int32_t *__restrict__ cval,
                                              Local local, int lane, unsigned gmask, int &am, int &fm,
                                              unsigned long long &prods) {
    words = min(words, DAG_MAX_N / 32);              // a column past the bitmap: inconsistent
    for (int q = lane; q < (words + 3) >> 2; q += G) reinterpret_cast<uint4 *>(bm)[q] = make_uint4(0, 0, 0, 0);
    __syncwarp(gmask);
    const unsigned ncols = (unsigned)words * 32u;
    for (int p = lane; p < alen; p += G) {           // the row's own values are written first
        const int j = local(acol[a0 + p]);
        if ((unsigned)j < ncols) atomicOr(&bm[j >> 5], 1u << (j & 31));
        fm = max(fm, dag_row_msb(aval[a0 + p]));
    }
    __syncwarp(gmask);
    // products (mk (x) the entries [e0, e0 + elen) of a row), in order: marks each column's
    // first value
    auto fold = [&](int mk, int64_t e0, int elen, const int32_t *__restrict__ ecol,
                    const int32_t *__restrict__ evals, bool first) {
        for (int q = lane; q < elen; q += G) {
            const int pm = mk + dag_row_msb(evals[e0 + q]);
            am = max(am, pm);
            if (first) {
                const int j = local(ecol[e0 + q]);
                const unsigned bit = 1u << (j & 31);
                if ((unsigned)j >= ncols) {
                    am = 99;                         // inconsistent: the matrix leaves the DAG path
                } else if (!(bm[j >> 5] & bit)) {
                    fm = max(fm, pm);
                    atomicOr(&bm[j >> 5], bit);
                }
            }
        }
        if (lane == 0) prods += first ? (unsigned long long)elen : 0ull;
        __syncwarp(gmask);
    };
    // below: steps k over the parents, ascending, each adding A(i, k) (x) C(k, .).  Above: the
    // same products are the recurrence's candidates (their MSB bounds the closure's values).
    // The group loads G parents' closure rows at a time, one per lane, and steps through them.
    for (int pb = 0; pb < alen; pb += G) {
        int mk_l = 0, clen_l = 0;
        int64_t c0_l = 0;
        if (pb + lane < alen) {
            mk_l = dag_row_msb(aval[a0 + pb + lane]);
            crow(acol[a0 + pb + lane], c0_l, clen_l);
        }
        const int np = min(G, alen - pb);
        for (int t = 0; t < np; ++t) {
            const int mk = __shfl_sync(gmask, mk_l, t, G);
            const int64_t c0 = __shfl_sync(gmask, c0_l, t, G);
            const int clen = __shfl_sync(gmask, clen_l, t, G);
            fold(mk, c0, clen, ccol, cval, kind == DAG_KIND_BELOW);
        }
    }
    if (kind == DAG_KIND_ABOVE) {
        // steps k over C(i), ascending, each adding C(i, k) (x) A(k, .); the group loads G steps'
        // rows of A at a time
        int64_t c0;
        int clen;
        crow(g, c0, clen);
        for (int qb = 0; qb < clen; qb += G) {
            int mk_l = 0, klen_l = 0;
            int64_t k0_l = 0;
            if (qb + lane < clen) {
                const int32_t kg = ccol[c0 + qb + lane];
                mk_l = dag_row_msb(cval[c0 + qb + lane]);
                k0_l = aptr[kg];
                klen_l = (int)(aptr[kg + 1] - k0_l);
            }
            const int nq = min(G, clen - qb);
            for (int t = 0; t < nq; ++t) {
                const int mk = __shfl_sync(gmask, mk_l, t, G);
                const int64_t k0 = __shfl_sync(gmask, k0_l, t, G);
                const int klen = __shfl_sync(gmask, klen_l, t, G);
                fold(mk, k0, klen, acol, aval, true);
            }
        }
    }
}

}  // namespace rbg
