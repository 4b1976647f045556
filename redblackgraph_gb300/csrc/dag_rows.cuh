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
#pragma once
#include "rbg_internal.cuh"

namespace rbg {

constexpr int DAG_KIND_NONE = 0, DAG_KIND_BELOW = 1, DAG_KIND_ABOVE = 2;
constexpr int DAG_KIND_GENERAL = 3;   // entries on both sides of the diagonal (any numbering)
constexpr int DAG_TOP_MSB = 31;   // lbits - 1 for 32-bit values
constexpr int DAG_MAX_N = 8192;   // columns of a matrix the per-warp bitmap covers

// MSB of an off-diagonal value; a value no clean product yields (zero, or negative after a
// wrap) counts as reaching the top bit
__device__ __forceinline__ int dag_row_msb(int32_t v) { return v > 0 ? msb_u32((uint32_t)v) : 99; }

// One warp, row g.  A: the off-diagonal entries (CSR aptr / acol / aval, columns ascending);
// C: the closure rows, crow(r) -> (offset, length) into ccol / cval, columns ascending;
// local(col): the column's index inside its matrix.  bm: the warp's bitmap (words 32-bit
// words, one bit per column of the matrix), cleared here.  am / fm / prods accumulate the
// largest product MSB, the largest first-value MSB and the number of products.
template <typename CRow, typename Local>
__device__ __forceinline__ void dag_row_stats(unsigned *bm, int words, int kind, int64_t g,
                                              const int64_t *__restrict__ aptr, const int32_t *__restrict__ acol,
                                              const int32_t *__restrict__ aval, CRow crow,
                                              const int32_t *__restrict__ ccol, const int32_t *__restrict__ cval,
                                              Local local, int lane, int &am, int &fm,
                                              unsigned long long &prods) {
    for (int q = lane; q < words; q += 32) bm[q] = 0;
    __syncwarp();
    const int64_t a0 = aptr[g];
    const int alen = (int)(aptr[g + 1] - a0);
    const unsigned ncols = (unsigned)words * 32u;
    for (int p = lane; p < alen; p += 32) {          // the row's own values are written first
        const int j = local(acol[a0 + p]);
        if ((unsigned)j < ncols) atomicOr(&bm[j >> 5], 1u << (j & 31));
        fm = max(fm, dag_row_msb(aval[a0 + p]));
    }
    __syncwarp();
    // below: steps k over the parents, ascending, each adding A(i, k) (x) C(k, .).  Above: the
    // same products are the recurrence's candidates (their MSB bounds the closure's values)
    for (int p = 0; p < alen; ++p) {
        const int32_t kg = acol[a0 + p];
        const int mk = dag_row_msb(aval[a0 + p]);
        int64_t c0;
        int clen;
        crow(kg, c0, clen);
        for (int q = lane; q < clen; q += 32) {
            const int pm = mk + dag_row_msb(cval[c0 + q]);
            am = max(am, pm);
            if (kind == DAG_KIND_BELOW) {
                const int j = local(ccol[c0 + q]);
                const unsigned bit = 1u << (j & 31);
                if ((unsigned)j >= ncols) {
                    am = 99;                         // inconsistent: the matrix leaves the DAG path
                } else if (!(bm[j >> 5] & bit)) {
                    fm = max(fm, pm);
                    atomicOr(&bm[j >> 5], bit);
                }
            }
        }
        if (kind == DAG_KIND_BELOW && lane == 0) prods += (unsigned long long)clen;
        __syncwarp();
    }
    if (kind == DAG_KIND_ABOVE) {
        // steps k over C(i), ascending, each adding C(i, k) (x) A(k, .)
        int64_t c0;
        int clen;
        crow(g, c0, clen);
        for (int q = 0; q < clen; ++q) {
            const int32_t kg = ccol[c0 + q];
            const int mk = dag_row_msb(cval[c0 + q]);
            const int64_t k0 = aptr[kg];
            const int klen = (int)(aptr[kg + 1] - k0);
            for (int r = lane; r < klen; r += 32) {
                const int j = local(acol[k0 + r]);
                const int pm = mk + dag_row_msb(aval[k0 + r]);
                am = max(am, pm);
                const unsigned bit = 1u << (j & 31);
                if ((unsigned)j >= ncols) {
                    am = 99;                         // inconsistent: the matrix leaves the DAG path
                } else if (!(bm[j >> 5] & bit)) {
                    fm = max(fm, pm);
                    atomicOr(&bm[j >> 5], bit);
                }
            }
            if (lane == 0) prods += (unsigned long long)klen;
            __syncwarp();
        }
    }
    __syncwarp();                                    // the next row clears the bitmap
}

}  // namespace rbg
