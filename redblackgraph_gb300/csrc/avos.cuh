// avos.cuh -- AVOS semiring scalar algebra for host and device (sm_103a).
//
// Two families of operations live here.
//
// 1. Reference-exact scalar ops, templated on the storage type T.  They follow the C core
//    (redblackgraph/core/src/redblackgraph/rbg_math.c.in:30-121, identical to
//    redblackgraph/sparse/sparsetools/rbm_math.h:14-110) including its overflow signalling,
//    and the Cython variant (redblackgraph/sparse/csgraph/_rbg_math.pxi:1-87: signed
//    non-zero minimum, `while x > 1` MSB, silent wrap).  MSB uses count-leading-zeros
//    instead of the reference's shift loop.  Where the reference's loop would never end (a
//    negative signed operand, rbg_math.c.in:38-46) the op reports RBG_EV_HANG instead.
//
// 2. "Lane" ops for the clean regime used by the blocked kernels.  A lane is an unsigned
//    32- or 64-bit word.  Valid values are in [2, 2^(L-1)); a zero ("no path") is encoded as
//    any word with the top bit set (canonically all ones).  In that regime
//        x (x) y = x * 2^msb(y) + (y - 2^msb(y))          (one integer multiply-add)
//        a (+) b = min(a, b)                                (one unsigned min)
//    and an encoded zero on either side yields a word with the top bit set.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define RBG_HD __host__ __device__ __forceinline__
#else
#define RBG_HD inline
#endif

#include "../../include/rbg_gb300.h"  // status codes and event bits

namespace rbg {

template <typename T> struct utype;
template <> struct utype<int8_t> { typedef uint8_t type; static const bool is_signed = true; };
template <> struct utype<uint8_t> { typedef uint8_t type; static const bool is_signed = false; };
template <> struct utype<int16_t> { typedef uint16_t type; static const bool is_signed = true; };
template <> struct utype<uint16_t> { typedef uint16_t type; static const bool is_signed = false; };
template <> struct utype<int32_t> { typedef uint32_t type; static const bool is_signed = true; };
template <> struct utype<uint32_t> { typedef uint32_t type; static const bool is_signed = false; };
template <> struct utype<int64_t> { typedef uint64_t type; static const bool is_signed = true; };
template <> struct utype<uint64_t> { typedef uint64_t type; static const bool is_signed = false; };

// index of the most significant set bit of a non-zero unsigned word
RBG_HD int msb_u32(uint32_t x) {
#if defined(__CUDA_ARCH__)
    return 31 - __clz((int)x);
#else
    return 31 - __builtin_clz(x);
#endif
}
RBG_HD int msb_u64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return 63 - __clzll((long long)x);
#else
    return 63 - __builtin_clzll(x);
#endif
}
template <typename U> RBG_HD int msb_nz(U x) {
    return sizeof(U) == 8 ? msb_u64((uint64_t)x) : msb_u32((uint32_t)x);
}

// ------------------------------------------------------------------ reference-exact ops
// avos_sum: rbg_math.c.in:30-36 (non-zero minimum in unsigned order; all ones absorbs)
template <typename T> RBG_HD T avos_sum(T a, T b) {
    typedef typename utype<T>::type U;
    if (a == 0 || (U)(~b) == 0) return b;
    if (b == 0 || (U)(~a) == 0) return a;
    return ((U)a < (U)b) ? a : b;
}

// MSB: rbg_math.c.in:38-46.  Sets RBG_EV_HANG for a negative signed value other than -1.
template <typename T> RBG_HD int avos_msb(T x, unsigned &ev) {
    typedef typename utype<T>::type U;
    if ((U)(~x) == 0) return 0;
    if (utype<T>::is_signed && x < 0) { ev |= RBG_EV_HANG; return 0; }
    if (x == 0) return 0;
    return msb_nz<U>((U)x);
}

// avos_product: rbg_math.c.in:48-121 (returns the unsigned result, events in ev)
template <typename T> RBG_HD typename utype<T>::type avos_product(T lhs, T rhs, unsigned &ev) {
    typedef typename utype<T>::type U;
    const int bits = (int)sizeof(U) * 8;
    U x = (U)lhs, y = (U)rhs;
    if (x == 0 || y == 0) return 0;
    const bool lr = (lhs == (T)-1), rr = (rhs == (T)-1);
    if (lr && rr) return x;
    if (lhs == 1 && rhs == 1) return 1;
    if (lr && rhs == 1) return 0;
    if (lhs == 1 && rr) return 0;
    if (lr) x = 1;
    if (rr) return (lhs & 1) ? (U)0 : x;
    if (rhs == 1) return (lhs & 1) ? x : (U)0;
    unsigned e = 0;
    int bp = avos_msb<T>((T)y, e);
    int mx = avos_msb<T>((T)x, e);
    if (e) { ev |= e; return 0; }
    if (mx + bp >= bits) ev |= RBG_EV_OVF_SIZE;
    U low = (bp == 0) ? (U)0 : (U)(y & (U)((((U)1) << bp) - 1));
    U result = (U)(low | (U)(x << bp));
    if (result == (U)~(U)0) ev |= RBG_EV_OVF_ONES;
    return result;
}

// Cython variants (_rbg_math.pxi): int32 storage only
RBG_HD int cy_msb(int32_t x) { return x > 1 ? msb_u32((uint32_t)x) : 0; }
RBG_HD int32_t cy_sum(int32_t x, int32_t y) {
    if (x == 0) return y;
    if (y == 0) return x;
    return x < y ? x : y;
}
RBG_HD int32_t cy_product(int32_t lhs, int32_t rhs) {
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
    uint32_t low = bp == 0 ? 0u : (y & ((1u << bp) - 1u));
    return (int32_t)(low | (x << bp));
}

// ------------------------------------------------------------------ clean-lane ops
template <typename U> struct lane {
    static constexpr int bits = (int)sizeof(U) * 8;
    static constexpr U top = ((U)1) << (bits - 1);
    static constexpr U inf = (U)~(U)0;
    RBG_HD static bool valid(U v) { return (v & top) == 0; }
    // right-operand decomposition: m = 2^msb(y), low = y - m; zero -> (0, inf)
    RBG_HD static void split(U y, U &m, U &low) {
        if (valid(y)) {
            m = ((U)1) << msb_nz<U>(y);
            low = y ^ m;
        } else {
            m = 0;
            low = inf;
        }
    }
    RBG_HD static U mul(U x, U m, U low) { return x * m + low; }
    // full clean product with the top-bit risk test (result_size >= lbits - 1)
    RBG_HD static U product(U x, U y, int lbits, bool &risk) {
        if (!valid(x) || !valid(y)) return inf;
        int s = msb_nz<U>(y);
        if (msb_nz<U>(x) + s >= lbits - 1) risk = true;
        return (x << s) | (y ^ (((U)1) << s));
    }
};

}  // namespace rbg
