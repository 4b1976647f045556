/*
 * avos_oracle.c -- CPU restatement of redblackgraph's AVOS closure path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA implementation is
 * checked against; nothing on the product path links or calls it.  It restates, in plain
 * sequential C, the reference algorithms for:
 *
 *   - the AVOS scalar algebra (avos_sum, MSB, avos_product) with the C core's error
 *     signalling            -- redblackgraph/core/src/redblackgraph/rbg_math.c.in:30-121
 *   - the dense Floyd-Warshall gufunc, C core semantics
 *                            -- redblackgraph/core/src/redblackgraph/warshall.c.in:51-107
 *   - the Cython Floyd-Warshall (int32, signed compare, silent wrap, CycleError)
 *                            -- redblackgraph/sparse/csgraph/_shortest_path.pyx:340-389
 *                               redblackgraph/sparse/csgraph/_rbg_math.pxi:1-87
 *   - the dense AVOS matrix product behind rb.array @ (einsum 'ij,jk')
 *                            -- redblackgraph/core/src/redblackgraph/redblack.c.src:554-594
 *   - the sparse SpGEMM pass 1 / pass 2 behind rb_matrix @
 *                            -- redblackgraph/sparse/sparsetools/rbm_math.h:14-222
 *   - vertex and edge relational composition, C core and Cython
 *                            -- redblackgraph/core/src/redblackgraph/relational_composition.c.in:47-262
 *                               redblackgraph/sparse/csgraph/_relational_composition.pyx:10-113
 *
 * Error events.  The C core reports errors through PyErr_Format and keeps looping, so the
 * exception Python finally raises is the LAST one set.  The oracle records, in loop order,
 * the kind of the last event.  Where the reference would loop forever (its MSB shifts a
 * negative signed value, rbg_math.c.in:38-46), the oracle stops and reports an overflow with
 * the RBG_EV_HANG flag: the GPU implementation raises OverflowError there instead of hanging.
 *
 * Build: gcc -O2 -fPIC -shared -o liboracle.so avos_oracle.c   (see oracle/Makefile)
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* status codes, shared with include/rbg_gb300.h */
#define RBG_OK 0
#define RBG_ERR_OVERFLOW 1
#define RBG_ERR_CYCLE 2
#define RBG_ERR_INVALID 6

/* per-product event bits */
#define RBG_EV_OVF_SIZE 1u  /* msb(x)+msb(y) >= bits          rbg_math.c.in:103-111 */
#define RBG_EV_OVF_ONES 2u  /* result collides with RED_ONE   rbg_math.c.in:113-118 */
#define RBG_EV_HANG 4u      /* reference MSB would not return rbg_math.c.in:38-46  */

/* ------------------------------------------------------------------------------------
 * Scalar algebra, C core semantics, one instance per integer width.
 * T is the storage type, U its unsigned counterpart, SIGNED says whether T is signed.
 * ------------------------------------------------------------------------------------ */
#define DEFINE_ALGEBRA(NAME, T, U, SIGNED)                                                   \
    static inline T NAME##_sum(T a, T b) {                                                   \
        /* rbg_math.c.in:30-36: non-zero minimum, RED_ONE (all ones) absorbs */              \
        if (a == 0 || (U)(~b) == 0) return b;                                                \
        if (b == 0 || (U)(~a) == 0) return a;                                                \
        if ((U)a < (U)b) return a;                                                           \
        return b;                                                                            \
    }                                                                                        \
    /* rbg_math.c.in:38-46; *hang set where the reference's shift loop never ends */         \
    static inline int NAME##_msb(T x, unsigned *ev) {                                        \
        if ((U)(~x) == 0) return 0;                                                          \
        if (SIGNED && x < 0) { *ev |= RBG_EV_HANG; return 0; }                               \
        int level = 0;                                                                       \
        U ux = (U)x;                                                                         \
        while (ux >>= 1) level++;                                                            \
        return level;                                                                        \
    }                                                                                        \
    /* rbg_math.c.in:48-121 */                                                               \
    static inline U NAME##_product(T lhs, T rhs, unsigned *ev) {                             \
        U x = (U)lhs, y = (U)rhs;                                                            \
        if (x == 0 || y == 0) return 0;                                                      \
        if (lhs == (T)-1 && rhs == (T)-1) return x;                                          \
        if (lhs == 1 && rhs == 1) return 1;                                                  \
        if (lhs == (T)-1 && rhs == 1) return 0;                                              \
        if (lhs == 1 && rhs == (T)-1) return 0;                                              \
        if (lhs == (T)-1) x = 1;                                                             \
        if (rhs == (T)-1) return (lhs & 1) ? 0 : x;                                          \
        if (rhs == 1) return (lhs & 1) ? x : 0;                                              \
        unsigned e = 0;                                                                      \
        int bp = NAME##_msb((T)y, &e);                                                       \
        if (e) { *ev |= e; return 0; }                                                       \
        int rs = NAME##_msb((T)x, &e) + bp;                                                  \
        if (e) { *ev |= e; return 0; }                                                       \
        if (rs >= (int)(sizeof(U) * 8)) *ev |= RBG_EV_OVF_SIZE;                              \
        U result = (U)((y & (U)(((U)1 << bp) - 1)) | (U)(x << bp));                          \
        if (result == (U)-1) *ev |= RBG_EV_OVF_ONES;                                         \
        return result;                                                                       \
    }                                                                                        \
    T orc_avos_sum_##NAME(T a, T b) { return NAME##_sum(a, b); }                             \
    int orc_avos_product_##NAME(T a, T b, U *out) {                                          \
        unsigned ev = 0;                                                                     \
        *out = NAME##_product(a, b, &ev);                                                    \
        return (int)ev;                                                                      \
    }                                                                                        \
    int orc_msb_##NAME(T x) { unsigned ev = 0; int m = NAME##_msb(x, &ev); return ev ? -1 : m; }

DEFINE_ALGEBRA(i8, int8_t, uint8_t, 1)
DEFINE_ALGEBRA(u8, uint8_t, uint8_t, 0)
DEFINE_ALGEBRA(i16, int16_t, uint16_t, 1)
DEFINE_ALGEBRA(u16, uint16_t, uint16_t, 0)
DEFINE_ALGEBRA(i32, int32_t, uint32_t, 1)
DEFINE_ALGEBRA(u32, uint32_t, uint32_t, 0)
DEFINE_ALGEBRA(i64, int64_t, uint64_t, 1)
DEFINE_ALGEBRA(u64, uint64_t, uint64_t, 0)

/* ------------------------------------------------------------------------------------
 * Dense Floyd-Warshall, C core semantics (warshall.c.in:51-107), in place on `w`.
 *
 * info[0] = last event kind (0 none, 1 overflow, 2 cycle)
 * info[1] = flags (RBG_EV_* ORed over the run)
 * info[2..4] = (k, i, j) of the last event
 * diameter   = MSB of the largest value ever written (signed compare for signed T,
 *              all-ones excluded), warshall.c.in:89,106
 * triangular = 1 restricts the loops to i <= k <= j (the Cython upper-triangular loop,
 *              _shortest_path.pyx:365-378); 0 is the full loop.
 * Returns the status the Python layer raises (0, RBG_ERR_OVERFLOW or RBG_ERR_CYCLE).
 * ------------------------------------------------------------------------------------ */
#define DEFINE_WARSHALL(NAME, T, U, SIGNED)                                                  \
    int orc_warshall_##NAME(int64_t n, T *w, int triangular, int64_t *diameter,             \
                            int64_t *info) {                                                 \
        T diam = 0;                                                                          \
        int last = 0;                                                                        \
        unsigned flags = 0;                                                                  \
        int64_t lk = -1, li = -1, lj = -1;                                                   \
        for (int64_t k = 0; k < n; k++) {                                                    \
            int64_t i_end = triangular ? k + 1 : n;                                          \
            for (int64_t i = 0; i < i_end; i++) {                                            \
                for (int64_t j = triangular ? k : 0; j < n; j++) {                           \
                    unsigned ev = 0;                                                         \
                    T p = (T)NAME##_product(w[i * n + k], w[k * n + j], &ev);                \
                    if (ev & RBG_EV_HANG) {                                                  \
                        flags |= ev;                                                         \
                        info[0] = RBG_ERR_OVERFLOW; info[1] = flags;                         \
                        info[2] = k; info[3] = i; info[4] = j;                               \
                        *diameter = 0;                                                       \
                        return RBG_ERR_OVERFLOW;                                             \
                    }                                                                        \
                    if (ev) { flags |= ev; last = RBG_ERR_OVERFLOW; lk = k; li = i; lj = j; } \
                    if (i == j && !(p == (T)-1 || p == 0 || p == 1)) {                       \
                        last = RBG_ERR_CYCLE; lk = k; li = i; lj = j;                        \
                    }                                                                        \
                    T v = NAME##_sum(w[i * n + j], p);                                       \
                    w[i * n + j] = v;                                                        \
                    if ((U)(~v) != 0 && v > diam) diam = v;                                  \
                }                                                                            \
            }                                                                                \
        }                                                                                    \
        unsigned ev = 0;                                                                     \
        *diameter = NAME##_msb(diam, &ev);                                                   \
        info[0] = last; info[1] = flags; info[2] = lk; info[3] = li; info[4] = lj;           \
        return last;                                                                         \
    }

DEFINE_WARSHALL(i8, int8_t, uint8_t, 1)
DEFINE_WARSHALL(u8, uint8_t, uint8_t, 0)
DEFINE_WARSHALL(i16, int16_t, uint16_t, 1)
DEFINE_WARSHALL(u16, uint16_t, uint16_t, 0)
DEFINE_WARSHALL(i32, int32_t, uint32_t, 1)
DEFINE_WARSHALL(u32, uint32_t, uint32_t, 0)
DEFINE_WARSHALL(i64, int64_t, uint64_t, 1)
DEFINE_WARSHALL(u64, uint64_t, uint64_t, 0)

/* ------------------------------------------------------------------------------------
 * Cython Floyd-Warshall (_shortest_path.pyx:340-389 with _rbg_math.pxi), int32 only.
 * Signed non-zero minimum, MSB by `while x > 1`, no overflow check (products wrap),
 * CycleError raised at the FIRST cycle in loop order.  info[0..3] = (2, k, i, j) on a
 * cycle.  Returns 0 or RBG_ERR_CYCLE.
 * ------------------------------------------------------------------------------------ */
static inline int cy_msb(int32_t x) {
    int b = 0;
    while (x > 1) { x >>= 1; b++; }
    return b;
}
static inline int32_t cy_sum(int32_t x, int32_t y) {
    if (x == 0) return y;
    if (y == 0) return x;
    return x < y ? x : y;
}
static inline int32_t cy_product(int32_t lhs, int32_t rhs) {
    uint32_t x = (uint32_t)lhs, y = (uint32_t)rhs;
    if (x == 0 || y == 0) return 0;
    if (lhs == -1 && rhs == -1) return -1;
    if (lhs == 1 && rhs == 1) return 1;
    if (lhs == -1 && rhs == 1) return 0;
    if (lhs == 1 && rhs == -1) return 0;
    if (lhs == -1) x = 1;
    if (rhs == -1) return (lhs & 1) ? 0 : (int32_t)x;
    if (rhs == 1) return (lhs & 1) ? (int32_t)x : 0;
    int bp = cy_msb((int32_t)y);
    uint64_t mask = (((uint64_t)1) << bp) - 1;
    return (int32_t)(uint32_t)(((uint64_t)y & mask) | (uint64_t)(uint32_t)(x << bp));
}
int32_t orc_cy_product(int32_t a, int32_t b) { return cy_product(a, b); }
int32_t orc_cy_sum(int32_t a, int32_t b) { return cy_sum(a, b); }

int orc_fw_cython_i32(int64_t n, int32_t *w, int triangular, int64_t *diameter,
                      int64_t *info) {
    int32_t diam = 0;
    for (int64_t k = 0; k < n; k++) {
        int64_t i_end = triangular ? k + 1 : n;
        for (int64_t i = 0; i < i_end; i++) {
            for (int64_t j = triangular ? k : 0; j < n; j++) {
                int32_t p = cy_product(w[i * n + k], w[k * n + j]);
                if (i == j && !(p == -1 || p == 0 || p == 1)) {
                    info[0] = RBG_ERR_CYCLE; info[1] = k; info[2] = i; info[3] = j;
                    *diameter = 0;
                    return RBG_ERR_CYCLE;
                }
                int32_t v = cy_sum(w[i * n + j], p);
                w[i * n + j] = v;
                if (v > diam) diam = v;
            }
        }
    }
    *diameter = cy_msb(diam);
    info[0] = 0;
    return RBG_OK;
}

/* ------------------------------------------------------------------------------------
 * Dense AVOS matrix product C[m,p] = A[m,q] (x) B[q,p] under (sum, product), C core
 * semantics (redblack.c.src:554-594: accum = sum(accum, a (x) b), then sum with out=0).
 * Returns RBG_ERR_OVERFLOW when any product signalled an overflow or would hang.
 * ------------------------------------------------------------------------------------ */
#define DEFINE_MATMUL(NAME, T, U)                                                            \
    int orc_matmul_##NAME(int64_t m, int64_t q, int64_t p, const T *a, const T *b, T *c,    \
                          int64_t *flags_out) {                                              \
        unsigned flags = 0;                                                                  \
        for (int64_t i = 0; i < m; i++)                                                      \
            for (int64_t k = 0; k < p; k++) {                                                \
                T acc = 0;                                                                   \
                for (int64_t j = 0; j < q; j++) {                                            \
                    unsigned ev = 0;                                                         \
                    T prod = (T)NAME##_product(a[i * q + j], b[j * p + k], &ev);             \
                    flags |= ev;                                                             \
                    acc = NAME##_sum(acc, prod);                                             \
                }                                                                            \
                c[i * p + k] = acc;                                                          \
            }                                                                                \
        *flags_out = flags;                                                                  \
        return flags ? RBG_ERR_OVERFLOW : RBG_OK;                                            \
    }

DEFINE_MATMUL(i8, int8_t, uint8_t)
DEFINE_MATMUL(u8, uint8_t, uint8_t)
DEFINE_MATMUL(i16, int16_t, uint16_t)
DEFINE_MATMUL(u16, uint16_t, uint16_t)
DEFINE_MATMUL(i32, int32_t, uint32_t)
DEFINE_MATMUL(u32, uint32_t, uint32_t)
DEFINE_MATMUL(i64, int64_t, uint64_t)
DEFINE_MATMUL(u64, uint64_t, uint64_t)

/* ------------------------------------------------------------------------------------
 * Sparse SpGEMM (rbm_math.h:117-222), 64-bit values (rb_matrix upcasts, rbm.py:83-105),
 * int64 indices.  Pass 1 sizes each output row; pass 2 accumulates with the linked-list
 * accumulator, drops zero sums and emits each row's columns in the accumulator's order
 * (most recently first-touched column first).  `flags_out` ORs the product events.
 * ------------------------------------------------------------------------------------ */
int64_t orc_spgemm_pass1(int64_t n_row, int64_t n_col, const int64_t *ap, const int64_t *aj,
                         const int64_t *bp, const int64_t *bj, int64_t *cp) {
    int64_t *mask = (int64_t *)malloc(sizeof(int64_t) * (n_col > 0 ? n_col : 1));
    for (int64_t c = 0; c < n_col; c++) mask[c] = -1;
    int64_t nnz = 0;
    cp[0] = 0;
    for (int64_t i = 0; i < n_row; i++) {
        for (int64_t jj = ap[i]; jj < ap[i + 1]; jj++) {
            int64_t j = aj[jj];
            for (int64_t kk = bp[j]; kk < bp[j + 1]; kk++) {
                int64_t k = bj[kk];
                if (mask[k] != i) { mask[k] = i; nnz++; }
            }
        }
        cp[i + 1] = nnz;
    }
    free(mask);
    return nnz;
}

#define DEFINE_SPGEMM2(NAME, T, U)                                                            \
    int64_t orc_spgemm_pass2_##NAME(int64_t n_row, int64_t n_col, const int64_t *ap,          \
                                    const int64_t *aj, const T *ax, const int64_t *bp,        \
                                    const int64_t *bj, const T *bx, int64_t *cp, int64_t *cj, \
                                    T *cx, int64_t *flags_out) {                              \
        int64_t *next = (int64_t *)malloc(sizeof(int64_t) * (n_col > 0 ? n_col : 1));        \
        T *sums = (T *)calloc((size_t)(n_col > 0 ? n_col : 1), sizeof(T));                   \
        for (int64_t c = 0; c < n_col; c++) next[c] = -1;                                    \
        unsigned flags = 0;                                                                   \
        int64_t nnz = 0;                                                                      \
        cp[0] = 0;                                                                            \
        for (int64_t i = 0; i < n_row; i++) {                                                 \
            int64_t head = -2, length = 0;                                                    \
            for (int64_t jj = ap[i]; jj < ap[i + 1]; jj++) {                                  \
                int64_t j = aj[jj];                                                           \
                T v = ax[jj];                                                                 \
                for (int64_t kk = bp[j]; kk < bp[j + 1]; kk++) {                              \
                    int64_t k = bj[kk];                                                       \
                    unsigned ev = 0;                                                          \
                    T prod = (T)NAME##_product(v, bx[kk], &ev);                               \
                    flags |= ev;                                                              \
                    sums[k] = NAME##_sum(sums[k], prod);                                      \
                    if (next[k] == -1) { next[k] = head; head = k; length++; }                \
                }                                                                             \
            }                                                                                 \
            for (int64_t jj = 0; jj < length; jj++) {                                         \
                if (sums[head] != 0) { cj[nnz] = head; cx[nnz] = sums[head]; nnz++; }         \
                int64_t temp = head;                                                          \
                head = next[head];                                                            \
                next[temp] = -1;                                                              \
                sums[temp] = 0;                                                               \
            }                                                                                 \
            cp[i + 1] = nnz;                                                                  \
        }                                                                                     \
        free(next);                                                                           \
        free(sums);                                                                           \
        *flags_out = flags;                                                                   \
        return nnz;                                                                           \
    }

DEFINE_SPGEMM2(i64, int64_t, uint64_t)
DEFINE_SPGEMM2(u64, uint64_t, uint64_t)

/* ------------------------------------------------------------------------------------
 * Relational composition, C core semantics (relational_composition.c.in:47-262), in the
 * reference's loop order.  info[0] = status (0, RBG_ERR_OVERFLOW, RBG_ERR_CYCLE), info[1] =
 * flags over every product, info[2] = step of the deciding event (1, 2, 3 = cycle check, 4),
 * info[3], info[4] = its row and column (cycle: the index k), info[5], info[6] = its operands
 * (cycle: u_k, v_k), info[7] = its event bits.  A product on which the reference's MSB would
 * never return stops the run there (RBG_EV_HANG), as in orc_warshall.
 * ------------------------------------------------------------------------------------ */
#define COMP_EVENT(STEP, I, J, A, B, EV)                                                     \
    do {                                                                                     \
        flags |= (EV);                                                                       \
        if ((EV) & RBG_EV_HANG) {                                                            \
            info[0] = RBG_ERR_OVERFLOW; info[1] = flags; info[2] = (STEP); info[3] = (I);    \
            info[4] = (J); info[5] = (int64_t)(A); info[6] = (int64_t)(B); info[7] = (EV);   \
            return RBG_ERR_OVERFLOW;                                                         \
        }                                                                                    \
        last = RBG_ERR_OVERFLOW; ls = (STEP); li = (I); lj = (J);                            \
        la = (int64_t)(A); lb = (int64_t)(B); lev = (EV);                                    \
    } while (0)

#define DEFINE_COMPOSE(NAME, T, U)                                                           \
    int orc_vertex_comp_##NAME(int64_t n, const T *R, const T *u, const T *v, T color, T *out, \
                               int64_t *info) {                                              \
        int last = 0; unsigned flags = 0, lev = 0;                                           \
        int64_t ls = -1, li = -1, lj = -1, la = 0, lb = 0;                                   \
        const int64_t m1 = n + 1;                                                            \
        for (int64_t p = 0; p < n; p++) {          /* step 1: out[n][p] = u (x) R[:, p] */   \
            T r = 0;                                                                         \
            for (int64_t i = 0; i < n; i++) {                                                \
                unsigned ev = 0;                                                             \
                T pr = (T)NAME##_product(u[i], R[i * n + p], &ev);                           \
                if (ev) COMP_EVENT(1, i, p, u[i], R[i * n + p], ev);                         \
                r = NAME##_sum(r, pr);                                                       \
            }                                                                                \
            out[n * m1 + p] = r;                                                             \
        }                                                                                    \
        out[n * m1 + n] = color;                                                             \
        for (int64_t m = 0; m < n; m++) {          /* step 2: out[m][n] = R[m, :] (x) v */   \
            T r = 0;                                                                         \
            for (int64_t j = 0; j < n; j++) {                                                \
                unsigned ev = 0;                                                             \
                T pr = (T)NAME##_product(R[m * n + j], v[j], &ev);                           \
                if (ev) COMP_EVENT(2, m, j, R[m * n + j], v[j], ev);                         \
                r = NAME##_sum(r, pr);                                                       \
            }                                                                                \
            out[m * m1 + n] = r;                                                             \
        }                                                                                    \
        for (int64_t k = 0; k < n; k++)           /* step 3: the cycle check */              \
            if (out[k * m1 + n] != 0 && out[n * m1 + k] != 0) {                              \
                info[0] = RBG_ERR_CYCLE; info[1] = flags; info[2] = 3; info[3] = k;          \
                info[4] = n; info[5] = (int64_t)out[n * m1 + k];                             \
                info[6] = (int64_t)out[k * m1 + n]; info[7] = 0;                             \
                return RBG_ERR_CYCLE;                                                        \
            }                                                                                \
        for (int64_t m = 0; m < n; m++)            /* step 4: R (+) vc (x) uc */             \
            for (int64_t p = 0; p < n; p++) {                                                \
                unsigned ev = 0;                                                             \
                T a = out[m * m1 + n], b = out[n * m1 + p];                                  \
                T pr = (T)NAME##_product(a, b, &ev);                                         \
                if (ev) COMP_EVENT(4, m, p, a, b, ev);                                       \
                out[m * m1 + p] = NAME##_sum(R[m * n + p], pr);                              \
            }                                                                                \
        info[0] = last; info[1] = flags; info[2] = ls; info[3] = li; info[4] = lj;           \
        info[5] = la; info[6] = lb; info[7] = lev;                                           \
        return last;                                                                         \
    }                                                                                        \
    /* edge: loop indices compared in the storage type, as the C core does */               \
    int orc_edge_comp_##NAME(int64_t n, const T *R, int64_t alpha, int64_t beta, T np, T *out,  \
                             int64_t *info) {                                                \
        int last = 0; unsigned flags = 0, lev = 0;                                           \
        int64_t ls = -1, li = -1, lj = -1, la = 0, lb = 0;                                   \
        memcpy(out, R, (size_t)(n * n) * sizeof(T));                                         \
        for (int64_t p = 0; p < n; p++) {          /* step 1: row alpha */                   \
            T r = 0;                                                                         \
            for (int64_t i = 0; i < n; i++) {                                                \
                T lhs = R[alpha * n + i];                                                    \
                if (np != 0 && (T)i == (T)beta) lhs = np;                                    \
                unsigned ev = 0;                                                             \
                T pr = (T)NAME##_product(lhs, R[i * n + p], &ev);                            \
                if (ev) COMP_EVENT(1, i, p, lhs, R[i * n + p], ev);                          \
                r = NAME##_sum(r, pr);                                                       \
            }                                                                                \
            out[alpha * n + p] = r;                                                          \
        }                                                                                    \
        for (int64_t m = 0; m < n; m++) {          /* step 2: the other rows */              \
            if ((T)m == (T)alpha) continue;                                                  \
            T lhs = R[m * n + alpha];                                                        \
            for (int64_t p = 0; p < n; p++) {                                                \
                T a = out[alpha * n + p];                                                    \
                if (a != 0) {                                                                \
                    unsigned ev = 0;                                                         \
                    T pr = (T)NAME##_product(lhs, a, &ev);                                   \
                    if (ev) COMP_EVENT(2, m, p, lhs, a, ev);                                 \
                    out[m * n + p] = NAME##_sum(R[m * n + p], pr);                           \
                } else {                                                                     \
                    out[m * n + p] = R[m * n + p];                                           \
                }                                                                            \
            }                                                                                \
        }                                                                                    \
        info[0] = last; info[1] = flags; info[2] = ls; info[3] = li; info[4] = lj;           \
        info[5] = la; info[6] = lb; info[7] = lev;                                           \
        return last;                                                                         \
    }

DEFINE_COMPOSE(i8, int8_t, uint8_t)
DEFINE_COMPOSE(u8, uint8_t, uint8_t)
DEFINE_COMPOSE(i16, int16_t, uint16_t)
DEFINE_COMPOSE(u16, uint16_t, uint16_t)
DEFINE_COMPOSE(i32, int32_t, uint32_t)
DEFINE_COMPOSE(u32, uint32_t, uint32_t)
DEFINE_COMPOSE(i64, int64_t, uint64_t)
DEFINE_COMPOSE(u64, uint64_t, uint64_t)

/* Cython relational composition (_relational_composition.pyx:10-113), int32, no events. */
void orc_vertex_comp_cy(int64_t n, const int32_t *A, const int32_t *u, const int32_t *v, int32_t color,
                        int32_t *out) {
    const int64_t m1 = n + 1;
    int32_t *ul = (int32_t *)calloc((size_t)(n > 0 ? n : 1), sizeof(int32_t));
    int32_t *vl = (int32_t *)calloc((size_t)(n > 0 ? n : 1), sizeof(int32_t));
    for (int64_t i = 0; i < n; i++)
        for (int64_t j = 0; j < n; j++) {
            ul[i] = cy_sum(ul[i], cy_product(u[j], A[j * n + i]));
            vl[i] = cy_sum(vl[i], cy_product(A[i * n + j], v[j]));
        }
    for (int64_t i = 0; i < n; i++)
        for (int64_t j = 0; j < n; j++)
            out[i * m1 + j] = ul[j] != 0 ? cy_sum(cy_product(vl[i], ul[j]), A[i * n + j]) : A[i * n + j];
    for (int64_t i = 0; i < n; i++) {
        out[i * m1 + n] = vl[i];
        out[n * m1 + i] = ul[i];
    }
    out[n * m1 + n] = color;
    free(ul);
    free(vl);
}

void orc_edge_comp_cy(int64_t n, const int32_t *R, int64_t alpha, int64_t beta, int32_t rel, int32_t *out) {
    int32_t *A = (int32_t *)malloc((size_t)(n * n) * sizeof(int32_t));
    int32_t *ul = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    memcpy(A, R, (size_t)(n * n) * sizeof(int32_t));
    A[alpha * n + beta] = rel;                     /* the Cython code edits R in place */
    for (int64_t i = 0; i < n; i++)
        for (int64_t j = 0; j < n; j++)
            ul[i] = cy_sum(ul[i], cy_product(A[alpha * n + j], A[j * n + i]));
    for (int64_t i = 0; i < n; i++)
        for (int64_t j = 0; j < n; j++) {
            if (i == alpha) out[i * n + j] = ul[j];
            else if (ul[j] != 0) out[i * n + j] = cy_sum(cy_product(A[i * n + alpha], ul[j]), A[i * n + j]);
            else out[i * n + j] = A[i * n + j];
        }
    free(A);
    free(ul);
}
