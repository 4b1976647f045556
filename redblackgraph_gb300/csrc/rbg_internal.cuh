// rbg_internal.cuh -- shared host/device plumbing for the rbg_gb300 kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <limits.h>
#include <mutex>
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

// SM count of the current device
int sm_count();

// Kernel attributes set with cudaFuncSetAttribute (dynamic shared memory above 48 KB) belong to
// the context of the device that was current, so a process driving several GPUs sets them once
// per device: run() calls `configure` the first time it sees the current device and returns that
// status on every later call on the device.
class PerDeviceOnce {
public:
    template <typename F> int run(F &&configure) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) return RBG_ERR_CUDA;
        if (dev < 0 || dev >= kMaxDevices) return RBG_ERR_INVALID;
        std::lock_guard<std::mutex> lk(mu_);
        if (!done_[dev]) {
            rc_[dev] = configure();
            done_[dev] = true;
        }
        return rc_[dev];
    }
    static constexpr int kMaxDevices = 64;

private:
    std::mutex mu_;
    bool done_[kMaxDevices] = {};
    int rc_[kMaxDevices] = {};
};

// Host <-> device copies of a call's small tables and results through page-locked memory.  A
// copy from or to pageable memory goes through the driver's staging buffers: a read waits there
// for its stream and holds up other host threads' pageable copies meanwhile, which serialises
// calls on different streams.  Each host thread keeps one grow-only page-locked arena instead.
// up() stages and enqueues an upload; down() enqueues a download whose bytes land in `host` at
// finish(), which synchronises the stream.  The arena is reused only after finish(), so no staged
// upload is overwritten while it may still be pending; a request that does not fit, and every
// request while a NoHostAlloc guard is alive (rbg_fw_dense_noalloc), copies pageable memory.
class HostStaging {
public:
    HostStaging(cudaStream_t s, size_t hint);
    int up(void *dev, const void *host, size_t bytes);
    int down(void *host, const void *dev, size_t bytes);
    int finish();

private:
    struct Pending { void *host; const void *staged; size_t bytes; };
    cudaStream_t s_;
    Pending pend_[8];
    int npend_ = 0;
};
struct NoHostAlloc {
    NoHostAlloc();
    ~NoHostAlloc();
};

// running count of kernel launches issued by this library (rbg_launch_count); while a graph is
// being recorded (launch_recording(true)) launches are counted when the graph runs instead
void note_launches(int64_t k);
void launch_recording(bool on);

// Benchmark timer (rbg_profile_begin / rbg_profile_end_slots): CUDA events around the kernels
// of each slot, recorded on the launching stream while the timer is on.  Slots: 0 phase-3
// tiles, 1 panels, 2 diagonal tiles, 3 convert + finalize, 4 DAG path scan, 5 DAG path
// closure by levels (with its CSR), 6 DAG path statistics, 7 DAG path write, 8 DAG path replay
// of matrices in any numbering (pattern, triples, replay).
constexpr int TIMER_SLOTS = 9;
cudaEvent_t timer_begin(int slot, cudaStream_t s);
void timer_end(int slot, cudaEvent_t start, cudaStream_t s);
bool timer_on();

// Row statistics the closure can record while it writes the result (rbg_fw_batch_rows,
// storage int32): the nonzero count of every output row, which 32-column chunks of it hold a
// nonzero, and each component's largest value.  Component c's row i is output row
// row_id[row_base[c] + i] (row_base[c] + i when row_id is null); the chunk masks follow the
// layout of the compaction (ceil(n / 2048) words per row, component c's rows from word
// ceil(offset_c / 2048) + row_base[c] + c).  row_count null: nothing is recorded.
struct RowStats {
    const int64_t *row_base = nullptr;
    const int32_t *row_id = nullptr;
    int64_t *row_count = nullptr;
    unsigned long long *chunk_mask = nullptr;
    int32_t *comp_max = nullptr;
    bool operator==(const RowStats &o) const {
        return row_base == o.row_base && row_id == o.row_id && row_count == o.row_count &&
               chunk_mask == o.chunk_mask && comp_max == o.comp_max;
    }
};

// dag.cu: the closure by levels as an enqueue-only sequence for callers inside this library.
// The workspace is laid out for at most `nnz_bound` stored entries of A, so nothing is read back
// before the levels.  With `captured` the stream is being captured into a CUDA graph and the
// level loop becomes a while node that the device ends when a level comes out empty (no host
// synchronisation at all); otherwise the host looks at the frontier once per chunk of levels.
// The device counters (DagCounters) are left in the workspace for the caller to read later.
struct DagCounters {
    int placed, nwide, flags, nlevels;       // flags: 1 pool too small, 2 row past the block table
    unsigned long long reserved, max_abs, total;
    long long level;                         // the graph loop's level counter
};
size_t dag_workspace_for(int64_t n, int64_t nnz_bound);
int dag_enqueue(const rbg_csr_t *A, int64_t nnz_bound, void *workspace, int32_t *pool_cols, int32_t *pool_vals,
                int64_t pool_capacity, int64_t *row_off, int32_t *row_len, cudaStream_t s, bool captured,
                DagCounters **counters, int64_t *launches);
constexpr int DAG_GRAPH_CHUNK = 4;           // levels per iteration of the graph's while node

// fw_tri.cu: the components of an int32 or int64 batch that are acyclic and in the clean regime
// (at most 16 off-diagonal entries per row, at most 8192 rows), closed through the DAG closure by
// levels (in any numbering: off the topological order the loop is replayed on the closure's
// pattern for the diameter and the overflow decision); sets closed[i] = TRI_CLOSED and results[i] for each
// of them and leaves every other component untouched.  closed[i] = TRI_TOP_BIT marks a component
// the closure went through completely whose loop computes a product reaching bit 31: 32-bit
// lanes would only report that risk, so the caller goes on with 64-bit lanes (int64) or the
// exact kernel (int32).  Scratch comes from the caller's workspace (`ws`,
// `ws_bytes`); a workspace too small for a closure leaves its components to the other paths.
// ld_in / ld_out are the row strides of every block (0: each block's own n).  With
// RBG_MODE_GRAPH in `mode` the whole sequence is replayed from a cached CUDA graph.
constexpr char TRI_OPEN = 0, TRI_CLOSED = 1, TRI_TOP_BIT = 2;
template <typename T>
int tri_batch(int64_t count, const int64_t *sizes, const int64_t *in_off, const int64_t *out_off, int64_t ld_in,
              int64_t ld_out, const T *in, T *out, rbg_result_t *results, char *closed, unsigned char *ws,
              size_t ws_bytes, uint32_t mode, cudaStream_t stream, const RowStats &rs);

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
