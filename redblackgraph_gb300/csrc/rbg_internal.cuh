// rbg_internal.cuh -- shared host/device plumbing for the rbg_gb300 kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <limits.h>
#include "avos.cuh"
#include "../../include/rbg_gb300.h"

namespace rbg {

// Device-side status block, zeroed (then the "first"/"last" slots initialised) per call.
struct DevStatus {
    unsigned int flags;            // RBG_EV_* ORed by every kernel
    unsigned int pad0;
    unsigned long long mx;         // clean path: max over time of valid lane values
    long long mx_signed;           // exact path: max written value, signed order
    unsigned long long mx_unsigned;// exact path: max written value, unsigned order
    long long last_ovf;            // exact path: sequential index of the last overflow event
    long long last_cycle;          // exact path: sequential index of the last cycle event
    long long first_hang;          // exact path: first index where the reference would hang
    long long first_cycle;         // exact path: first cycle index (Cython raises here)
    long long first_ovf;           // exact path: first overflow index
    unsigned long long executed;   // relaxations the blocked kernels executed (not skipped)
    long long pad1[6];
};
static_assert(sizeof(DevStatus) == 128, "status block is 128 bytes");

__global__ void status_init_kernel(DevStatus *st, int count);

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

#define RBG_CUDA_TRY(expr)                                   \
    do {                                                     \
        cudaError_t _e = (expr);                             \
        if (_e != cudaSuccess) return RBG_ERR_CUDA;          \
    } while (0)

// grid size for grid-stride loops: a multiple of the SM count
int grid_for(int64_t work, int threads);

// running count of kernel launches issued by this library (rbg_launch_count)
void note_launches(int64_t k);

template <typename T> struct dtype_of;
template <> struct dtype_of<int8_t> { static const int value = RBG_DTYPE_INT8; };
template <> struct dtype_of<uint8_t> { static const int value = RBG_DTYPE_UINT8; };
template <> struct dtype_of<int16_t> { static const int value = RBG_DTYPE_INT16; };
template <> struct dtype_of<uint16_t> { static const int value = RBG_DTYPE_UINT16; };
template <> struct dtype_of<int32_t> { static const int value = RBG_DTYPE_INT32; };
template <> struct dtype_of<uint32_t> { static const int value = RBG_DTYPE_UINT32; };
template <> struct dtype_of<int64_t> { static const int value = RBG_DTYPE_INT64; };
template <> struct dtype_of<uint64_t> { static const int value = RBG_DTYPE_UINT64; };

inline int dtype_bytes(int dtype) {
    switch (dtype) {
        case RBG_DTYPE_INT8: case RBG_DTYPE_UINT8: return 1;
        case RBG_DTYPE_INT16: case RBG_DTYPE_UINT16: return 2;
        case RBG_DTYPE_INT32: case RBG_DTYPE_UINT32: return 4;
        case RBG_DTYPE_INT64: case RBG_DTYPE_UINT64: return 8;
        default: return 0;
    }
}

}  // namespace rbg

// Dispatch a templated call over the eight storage types.
#define RBG_DISPATCH_DTYPE(dtype, T, ...)                                  \
    switch (dtype) {                                                       \
        case RBG_DTYPE_INT8: { typedef int8_t T; __VA_ARGS__; } break;     \
        case RBG_DTYPE_UINT8: { typedef uint8_t T; __VA_ARGS__; } break;   \
        case RBG_DTYPE_INT16: { typedef int16_t T; __VA_ARGS__; } break;   \
        case RBG_DTYPE_UINT16: { typedef uint16_t T; __VA_ARGS__; } break; \
        case RBG_DTYPE_INT32: { typedef int32_t T; __VA_ARGS__; } break;   \
        case RBG_DTYPE_UINT32: { typedef uint32_t T; __VA_ARGS__; } break; \
        case RBG_DTYPE_INT64: { typedef int64_t T; __VA_ARGS__; } break;   \
        case RBG_DTYPE_UINT64: { typedef uint64_t T; __VA_ARGS__; } break; \
        default: return RBG_ERR_INVALID;                                   \
    }
