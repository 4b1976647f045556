// avos_gemm.cu -- dense AVOS matrix product C = A (x) B for rb.array @ (sm_103a).
//
// Reference: the AVOS einsum 'ij,jk' (redblackgraph/core/src/redblackgraph/redblack.c.src:554-594,
// reached from redblackgraph/core/redblack.py:14-38):  C[i,k] = (+)_j A[i,j] (x) B[j,k] with the
// C core scalar semantics (rbg_math.c.in:30-121).  (+) is associative and commutative, so the
// accumulation order does not change C; an OverflowError is raised when any product signals one.
//
// One tiled kernel with the full scalar semantics per term (identities, parity filters, wrap,
// overflow events), 64 x 64 outputs per CTA staged through shared memory.
#include <cuda_runtime.h>
#include <string.h>
#include <algorithm>
#include "rbg_internal.cuh"

namespace rbg {

constexpr int MM_T = 64;        // output tile edge
constexpr int MM_K = 32;        // reduction chunk
constexpr int MM_THREADS = 256; // 16 x 16 threads, 4 x 4 outputs each

__device__ __forceinline__ void mm_flush_flags(unsigned *dflags, unsigned f) {
    for (int o = 16; o > 0; o >>= 1) f |= __shfl_xor_sync(0xffffffffu, f, o);
    if ((threadIdx.x & 31) == 0 && f) atomicOr(dflags, f);
}

// Exact kernel: any storage type, full scalar semantics.
template <typename T>
__global__ void __launch_bounds__(MM_THREADS)
mm_exact_kernel(int64_t m, int64_t q, int64_t p, const T *__restrict__ A, int64_t lda,
                const T *__restrict__ B, int64_t ldb, T *__restrict__ C, int64_t ldc,
                unsigned *dflags) {
    __shared__ T As[MM_T][MM_K + 1];
    __shared__ T Bs[MM_K][MM_T + 1];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int64_t i0 = (int64_t)blockIdx.y * MM_T, k0 = (int64_t)blockIdx.x * MM_T;
    T acc[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = 0;
    unsigned ev = 0;
    for (int64_t j0 = 0; j0 < q; j0 += MM_K) {
        for (int e = threadIdx.x; e < MM_T * MM_K; e += MM_THREADS) {
            int r = e / MM_K, c = e % MM_K;
            int64_t gi = i0 + r, gj = j0 + c;
            As[r][c] = (gi < m && gj < q) ? A[gi * lda + gj] : (T)0;
            int rr = e / MM_T, cc = e % MM_T;
            int64_t bj = j0 + rr, bk = k0 + cc;
            Bs[rr][cc] = (bj < q && bk < p) ? B[bj * ldb + bk] : (T)0;
        }
        __syncthreads();
        for (int jj = 0; jj < MM_K; ++jj) {
            T a[4], b[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) a[r] = As[ty + 16 * r][jj];
#pragma unroll
            for (int c = 0; c < 4; ++c) b[c] = Bs[jj][tx + 16 * c];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    acc[r][c] = avos_sum<T>(acc[r][c], (T)avos_product<T>(a[r], b[c], ev));
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            int64_t gi = i0 + ty + 16 * r, gk = k0 + tx + 16 * c;
            if (gi < m && gk < p) C[gi * ldc + gk] = acc[r][c];
        }
    mm_flush_flags(dflags, ev);
}

template <typename T>
static int matmul_t(int64_t m, int64_t q, int64_t p, const T *A, int64_t lda, const T *B,
                    int64_t ldb, T *C, int64_t ldc, unsigned *dflags, cudaStream_t s) {
    if (m == 0 || p == 0) return RBG_OK;
    if (q == 0) {
        RBG_CUDA_TRY(cudaMemset2DAsync(C, ldc * sizeof(T), 0, p * sizeof(T), m, s));
        return RBG_OK;
    }
    dim3 grid((unsigned)((p + MM_T - 1) / MM_T), (unsigned)((m + MM_T - 1) / MM_T));
    note_launches(1);
    mm_exact_kernel<T><<<grid, MM_THREADS, 0, s>>>(m, q, p, A, lda, B, ldb, C, ldc, dflags);
    RBG_CUDA_TRY(cudaGetLastError());
    return RBG_OK;
}

}  // namespace rbg

using namespace rbg;

extern "C" int32_t rbg_avos_matmul_workspace_bytes(int32_t dtype, int64_t m, int64_t q, int64_t p,
                                                   int64_t *bytes) {
    if (!bytes || dtype_bytes(dtype) == 0 || m < 0 || q < 0 || p < 0) return RBG_ERR_INVALID;
    *bytes = 256;
    return RBG_OK;
}

extern "C" int32_t rbg_avos_matmul(int32_t dtype, int64_t m, int64_t q, int64_t p, const void *A,
                                   int64_t lda, const void *B, int64_t ldb, void *C, int64_t ldc,
                                   void *workspace, int64_t workspace_bytes, uint32_t *flags,
                                   rbg_stream_t stream) {
    if (m < 0 || q < 0 || p < 0 || !flags || lda < q || ldb < p || ldc < p) return RBG_ERR_INVALID;
    if (dtype_bytes(dtype) == 0) return RBG_ERR_INVALID;
    if (workspace_bytes < 256 || !workspace) return RBG_ERR_NOMEM;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    unsigned *dflags = reinterpret_cast<unsigned *>(workspace);
    RBG_CUDA_TRY(cudaMemsetAsync(dflags, 0, sizeof(unsigned), s));
    int rc = RBG_ERR_INVALID;
    RBG_DISPATCH_DTYPE(dtype, T,
        rc = matmul_t<T>(m, q, p, reinterpret_cast<const T *>(A), lda,
                         reinterpret_cast<const T *>(B), ldb, reinterpret_cast<T *>(C), ldc, dflags, s));
    if (rc) return rc;
    unsigned hf = 0;
    RBG_CUDA_TRY(cudaMemcpyAsync(&hf, dflags, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    *flags = hf;
    return (hf & (RBG_EV_OVF_SIZE | RBG_EV_OVF_ONES | RBG_EV_HANG)) ? RBG_ERR_OVERFLOW : RBG_OK;
}
