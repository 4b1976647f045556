// relationship.cu -- bulk relationship lookups on resident closures.
//
// Reference: calculate_relationship, redblackgraph/reference/calc_relationship.py:54-71.  For
// two rows a, b of a transitive closure the common ancestor is the first index j (in increasing
// order) minimising a[j] + b[j] over the j where both are non-zero; the host turns the two
// values found there into the relationship name (lookup_relationship, :23-51).
//
// One warp per query: the lanes stride the two rows with coalesced loads, keep their best
// (sum, j) pair, and a shuffle reduction picks the smallest sum, ties to the smallest j.  The
// sum wraps in the matrix's own type, as numpy scalar arithmetic does on the reference's rows
// (for unsigned types the red one, the type's maximum, plus y gives y - 1); the reduction
// carries it widened to 128 bits, which keeps the type's order.
#include <cuda_runtime.h>
#include <type_traits>
#include "rbg_internal.cuh"

namespace rbg {

constexpr int RL_WARPS = 8;

template <class T>
__device__ __forceinline__ void rl_scan(const T *a, const T *b, int64_t n, int lane, __int128 &best,
                                        int64_t &bj, int64_t &bx, int64_t &by) {
    using UT = typename std::make_unsigned<T>::type;
    for (int64_t j = lane; j < n; j += 32) {
        const T x = a[j], y = b[j];
        if (x != 0 && y != 0) {
            const __int128 s = (__int128)(T)(UT)((UT)x + (UT)y);
            if (bj < 0 || s < best) {   // lanes visit j in increasing order: first minimum kept
                best = s;
                bj = j;
                bx = (int64_t)x;
                by = (int64_t)y;
            }
        }
    }
}

__device__ __forceinline__ __int128 shfl128(__int128 v, int src) {
    const unsigned long long lo = (unsigned long long)v, hi = (unsigned long long)(v >> 64);
    const unsigned long long l2 = __shfl_sync(0xffffffffu, lo, src);
    const unsigned long long h2 = __shfl_sync(0xffffffffu, hi, src);
    return (__int128)(((unsigned __int128)h2 << 64) | l2);
}

__global__ void rl_kernel(int64_t count, const rbg_lookup_t *q, int64_t *out) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * RL_WARPS;
    for (int64_t i = (int64_t)blockIdx.x * RL_WARPS + (threadIdx.x >> 5); i < count; i += warps) {
        const rbg_lookup_t Q = q[i];
        __int128 best = 0;
        int64_t bj = -1, bx = 0, by = 0;
        const bool ok = Q.n > 0 && Q.u >= 0 && Q.u < Q.rows && Q.v >= 0 && Q.v < Q.rows && Q.ld >= Q.n;
        if (ok) {
            switch (Q.dtype) {
#define RL_CASE(code, T)                                                                           \
    case code: {                                                                                   \
        const T *W = reinterpret_cast<const T *>(Q.W);                                             \
        rl_scan<T>(W + Q.u * Q.ld, W + Q.v * Q.ld, Q.n, lane, best, bj, bx, by);                   \
    } break;
                RL_CASE(RBG_DTYPE_INT8, int8_t)
                RL_CASE(RBG_DTYPE_UINT8, uint8_t)
                RL_CASE(RBG_DTYPE_INT16, int16_t)
                RL_CASE(RBG_DTYPE_UINT16, uint16_t)
                RL_CASE(RBG_DTYPE_INT32, int32_t)
                RL_CASE(RBG_DTYPE_UINT32, uint32_t)
                RL_CASE(RBG_DTYPE_INT64, int64_t)
                RL_CASE(RBG_DTYPE_UINT64, uint64_t)
#undef RL_CASE
                default: break;
            }
        }
        // reduce (best, j): smallest sum, then smallest j; lanes without a candidate have j < 0
        for (int o = 16; o > 0; o >>= 1) {
            const __int128 ob = shfl128(best, lane ^ o);
            const int64_t oj = __shfl_xor_sync(0xffffffffu, bj, o);
            const int64_t ox = __shfl_xor_sync(0xffffffffu, bx, o);
            const int64_t oy = __shfl_xor_sync(0xffffffffu, by, o);
            const bool take = oj >= 0 && (bj < 0 || ob < best || (ob == best && oj < bj));
            if (take) { best = ob; bj = oj; bx = ox; by = oy; }
        }
        if (lane == 0) {
            out[3 * i] = ok ? bj : -2;
            out[3 * i + 1] = bx;
            out[3 * i + 2] = by;
        }
    }
}

}  // namespace rbg

using namespace rbg;

extern "C" int32_t rbg_relationship_lookup(int64_t count, const rbg_lookup_t *queries, int64_t *out,
                                           rbg_stream_t stream) {
    if (count < 0 || (count > 0 && (!queries || !out))) return RBG_ERR_INVALID;
    if (count == 0) return RBG_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    note_launches(1);
    rl_kernel<<<grid_for(count * 32, RL_WARPS * 32), RL_WARPS * 32, 0, s>>>(count, queries, out);
    RBG_CUDA_TRY(cudaGetLastError());
    return RBG_OK;
}
