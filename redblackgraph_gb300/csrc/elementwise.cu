// elementwise.cu -- element-wise AVOS sum / product over device arrays (sm_103a).
//
// Reference: the scalar algebra redblackgraph/core/src/redblackgraph/rbg_math.c.in:30-121
// (exposed as c_avos_sum / c_avos_product, redblackgraphmodule.c:491-533) and the GPU
// element-wise kernels avos_sum_kernel / avos_product_kernel (redblackgraph/gpu/
// avos_kernels.py:150-176).  The product is written in the unsigned type, as the C core returns.
#include <cuda_runtime.h>
#include "rbg_internal.cuh"

namespace rbg {

template <typename T>
__global__ void ew_kernel(int op, int64_t n, const T *__restrict__ x, const T *__restrict__ y,
                          T *__restrict__ z, unsigned *dflags) {
    unsigned ev = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        z[i] = op == 0 ? avos_sum<T>(x[i], y[i]) : (T)avos_product<T>(x[i], y[i], ev);
    }
    for (int o = 16; o > 0; o >>= 1) ev |= __shfl_xor_sync(0xffffffffu, ev, o);
    if ((threadIdx.x & 31) == 0 && ev) atomicOr(dflags, ev);
}

}  // namespace rbg

using namespace rbg;

// op: 0 = avos_sum, 1 = avos_product.  `workspace` >= 256 bytes.  Synchronises `stream`.
extern "C" int32_t rbg_avos_elementwise(int32_t op, int32_t dtype, int64_t n, const void *x,
                                        const void *y, void *z, void *workspace,
                                        int64_t workspace_bytes, uint32_t *flags,
                                        rbg_stream_t stream) {
    if ((op != 0 && op != 1) || n < 0 || !flags || dtype_bytes(dtype) == 0) return RBG_ERR_INVALID;
    if (!workspace || workspace_bytes < 256) return RBG_ERR_NOMEM;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    unsigned *dflags = reinterpret_cast<unsigned *>(workspace);
    RBG_CUDA_TRY(cudaMemsetAsync(dflags, 0, sizeof(unsigned), s));
    if (n > 0) {
        const int g = grid_for(n, 256);
        note_launches(1);
        RBG_DISPATCH_DTYPE(dtype, T,
            ew_kernel<T><<<g, 256, 0, s>>>(op, n, reinterpret_cast<const T *>(x),
                                           reinterpret_cast<const T *>(y), reinterpret_cast<T *>(z),
                                           dflags));
        RBG_CUDA_TRY(cudaGetLastError());
    }
    unsigned hf = 0;
    RBG_CUDA_TRY(cudaMemcpyAsync(&hf, dflags, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    RBG_CUDA_TRY(cudaStreamSynchronize(s));
    *flags = hf;
    return (hf & (RBG_EV_OVF_SIZE | RBG_EV_OVF_ONES | RBG_EV_HANG)) ? RBG_ERR_OVERFLOW : RBG_OK;
}
