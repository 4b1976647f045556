// fw_dense.cu -- dense AVOS transitive closure (Floyd-Warshall) for GB300 (sm_103a).
//
// Reference: redblackgraph/core/src/redblackgraph/warshall.c.in:51-107 (C core gufunc) and
// redblackgraph/sparse/csgraph/_shortest_path.pyx:340-389 (Cython).  Both run the in-place
// sequential triple loop k, i, j; the closure value of every cell AND the diameter (MSB of the
// largest value ever written, including values later replaced, warshall.c.in:89) depend on that
// order.  This file reproduces it exactly with two paths:
//
// 1. Blocked path ("snapshot-exact" blocked Floyd-Warshall), for inputs in the clean regime
//    (off-diagonal values 0 or in [2, 2^(bits-1)), diagonal in {-1, 0, 1}).  There row k and
//    column k are invariant during round k, so a round block K = [K0, K0+64) factors into
//      phase 1  the 64x64 diagonal tile, sequential in k, which also records the row and column
//               snapshots d_{k-1}(k, .) and d_{k-1}(., k) inside the tile;
//      phase 2  the row panel (K, J) and column panel (I, K): forward substitution with those
//               snapshots gives d_{k-1}(k, j) and d_{k-1}(i, k) for every k in K (kept in two
//               panel buffers) and the end-of-round panel values;
//      phase 3  every other cell: W(i,j) <- W(i,j) (+) sum_k CP(i,k) (x) RP(k,j), where CP/RP are
//               exactly the operands the sequential loop uses at step k.
//    Because the operands are the sequential ones, the set of products -- hence overflow and
//    cycle detection -- is identical to the reference, and the result needs no distributivity.
//    The running maximum is recovered per cell from its first valid product in k order (bit
//    masks over the round), which is the value the sequential loop writes first.
//    Arithmetic runs in 32-bit lanes (64-bit lanes when values need them): x (x) y is a single
//    multiply-add x * 2^msb(y) + (y - 2^msb(y)); (+) is an unsigned min with "zero" encoded as
//    any word with the top bit set.
//
// 2. Exact path: one k per step, all (i, j) in parallel, with the reference's full scalar
//    semantics (identities, parity filters, wrap, overflow/cycle signalling).  It replays the
//    in-place order (rows above k see the old row k, rows below see the new one; W(i,k) changes
//    at j = k) and tracks the sequential index of every error event so the exception raised is
//    the reference's (the C core keeps the LAST error set; Cython raises at the FIRST cycle).
//    Used for unclean inputs, and re-run whenever the blocked path saw a cycle or a product
//    reaching the top bit.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>
#include <algorithm>
#include <vector>
#include <atomic>
#include <mutex>
#include <type_traits>
#include "rbg_internal.cuh"

namespace rbg {

constexpr int FW_B = 64;         // round width (k block) and diagonal tile edge
constexpr int FW_P = 128;        // panel tile length / phase-3 tile rows
constexpr int FW_THREADS = 256;

__global__ void status_init_kernel(DevStatus *st, int count) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < count) {
        DevStatus s;
        memset(&s, 0, sizeof(s));
        s.mx_signed = 0;
        s.mx_unsigned = 0;
        s.last_ovf = -1;
        s.last_cycle = -1;
        s.first_hang = LLONG_MAX;
        s.first_cycle = LLONG_MAX;
        s.first_ovf = LLONG_MAX;
        st[t] = s;
    }
}

static std::atomic<long long> g_launches(0);
static thread_local int t_recording = 0;   // launches recorded into a graph are counted when it runs
void note_launches(int64_t k) {
    if (!t_recording) g_launches.fetch_add(k, std::memory_order_relaxed);
}
void launch_recording(bool on) { t_recording = on ? 1 : 0; }

// the calling thread's page-locked staging arena (see HostStaging)
struct StageArena {
    unsigned char *p = nullptr;
    size_t cap = 0, used = 0;
    bool pending = false;                    // staged uploads may still be in flight
    int no_alloc = 0;                        // NoHostAlloc guards alive
    ~StageArena() {
        if (p) cudaFreeHost(p);
    }
    void *take(size_t bytes) {
        if (no_alloc || !p) return nullptr;
        const size_t at = align_up(used, 64);
        if (at + bytes > cap) return nullptr;
        used = at + bytes;
        return p + at;
    }
};
static thread_local StageArena t_stage;

NoHostAlloc::NoHostAlloc() { ++t_stage.no_alloc; }
NoHostAlloc::~NoHostAlloc() { --t_stage.no_alloc; }

HostStaging::HostStaging(cudaStream_t s, size_t hint) : s_(s) {
    StageArena &a = t_stage;
    if (a.no_alloc || a.pending || hint <= a.cap) return;
    if (a.used == 0) {                       // nothing staged: grow (with slack)
        if (a.p) cudaFreeHost(a.p);
        a.p = nullptr;
        a.cap = 0;
        const size_t want = std::max<size_t>(align_up(hint + hint / 4, 4096), 64 << 10);
        if (cudaHostAlloc(reinterpret_cast<void **>(&a.p), want, cudaHostAllocDefault) == cudaSuccess) a.cap = want;
        else a.p = nullptr;
    }
}

int HostStaging::up(void *dev, const void *host, size_t bytes) {
    if (bytes == 0) return RBG_OK;
    void *st = t_stage.take(bytes);
    if (!st) {
        RBG_CUDA_TRY(cudaMemcpyAsync(dev, host, bytes, cudaMemcpyHostToDevice, s_));
        return RBG_OK;
    }
    memcpy(st, host, bytes);
    t_stage.pending = true;
    RBG_CUDA_TRY(cudaMemcpyAsync(dev, st, bytes, cudaMemcpyHostToDevice, s_));
    return RBG_OK;
}

int HostStaging::down(void *host, const void *dev, size_t bytes) {
    if (bytes == 0) return RBG_OK;
    void *st = npend_ < 8 ? t_stage.take(bytes) : nullptr;
    if (!st) {
        RBG_CUDA_TRY(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, s_));
        return RBG_OK;
    }
    RBG_CUDA_TRY(cudaMemcpyAsync(st, dev, bytes, cudaMemcpyDeviceToHost, s_));
    pend_[npend_++] = Pending{host, st, bytes};
    return RBG_OK;
}

int HostStaging::finish() {
    RBG_CUDA_TRY(cudaStreamSynchronize(s_));
    for (int k = 0; k < npend_; ++k) memcpy(pend_[k].host, pend_[k].staged, pend_[k].bytes);
    npend_ = 0;
    t_stage.used = 0;
    t_stage.pending = false;
    return RBG_OK;
}

// Opt-in per-kernel timing: CUDA events recorded on the launching stream around each launch of
// the blocked kernels (0 = tile, 1 = panel, 2 = diagonal, 3 = convert + finalize).
struct KernelTimer {
    bool on = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending[TIMER_SLOTS];
    std::vector<cudaEvent_t> pool;
    cudaEvent_t get() {
        if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    }
};
static KernelTimer g_timer;

cudaEvent_t timer_begin(int kid, cudaStream_t s) {
    (void)kid;
    if (!g_timer.on) return nullptr;
    cudaEvent_t e = g_timer.get();
    cudaEventRecord(e, s);
    return e;
}
void timer_end(int kid, cudaEvent_t start, cudaStream_t s) {
    if (!g_timer.on || !start) return;
    cudaEvent_t e = g_timer.get();
    cudaEventRecord(e, s);
    g_timer.pending[kid].push_back({start, e});
}
bool timer_on() { return g_timer.on; }

int grid_for(int64_t work, int threads) {
    const int sms = sm_count();
    int64_t blocks = (work + threads - 1) / threads;
    int64_t cap = (int64_t)sms * 16;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return (int)blocks;
}

// ------------------------------------------------------------------------------------------
// device helpers
// ------------------------------------------------------------------------------------------
template <typename U> struct signed_of;
template <> struct signed_of<uint32_t> { typedef int32_t type; };
template <> struct signed_of<uint64_t> { typedef int64_t type; };

template <typename U> __device__ __forceinline__ U umin(U a, U b) { return a < b ? a : b; }

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// Reduce a per-thread running max and OR of flags into the status block.
__device__ __forceinline__ void flush_status(DevStatus *st, unsigned long long mx, unsigned flags) {
    mx = warp_max_u64(mx);
    for (int o = 16; o > 0; o >>= 1) flags |= __shfl_xor_sync(0xffffffffu, flags, o);
    if ((threadIdx.x & 31) == 0) {
        if (mx) atomicMax(&st->mx, mx);
        if (flags) atomicOr(&st->flags, flags);
    }
}

// ------------------------------------------------------------------------------------------
// components: every kernel below works on a table of independent matrices (a batch; a single
// closure is a batch of one).  Components are sorted by size, descending, so the components
// still active in round r (n > 64 r) are a prefix of the table; each launch covers that prefix
// and a CTA finds its component by binary search in the launch's CTA prefix sums.
// ------------------------------------------------------------------------------------------
struct FwComp {
    int64_t n, np;            // size, padded size (a multiple of FW_P)
    int64_t in_off, out_off;  // element offsets of the input / output matrices
    int64_t ld_in, ld_out;    // their leading dimensions
    int64_t work_off;         // lane offset of the np x np work matrix
    int64_t cp_off, rp_off;   // lane offsets of the snapshot panels (FW_B x np each, t-major)
    int64_t any_off;          // offset (64-bit words) of the panel masks: per 64-line group,
                              // column panel then row panel (np / 64 each, 0 = all lines
                              // zero), then per line, column panel then row panel (np each)
    int64_t rb_index;         // round-buffer index
    int64_t occ_off;          // byte offset of the (np/64)^2 block-occupancy map (1 = nonzero)
    int32_t triangular, status_index;
    int32_t orig, pad_;       // index in the caller's batch (row statistics)
};

__device__ __forceinline__ int fw_find(const int64_t *__restrict__ prefix, int count, int64_t cta) {
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(prefix + mid) <= cta) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// ------------------------------------------------------------------------------------------
// convert: storage T -> lane work matrix U (clean-regime check, d_0 contribution)
// ------------------------------------------------------------------------------------------
// Work encoding: valid off-diagonal values as is; zeros, the diagonal, the padding and (in
// triangular mode) the ignored lower triangle as all ones.  `lbits` is the effective width
// min(storage bits, lane bits).  The running maximum must include d_0(i, j), the value the
// reference writes at k = 0 (warshall.c.in:88-89); later rounds add each cell's first value.
constexpr int CONV_ROWS = 8;   // rows of the padded matrix per CTA in convert / finalize

template <typename T, typename U>
__global__ void __launch_bounds__(FW_THREADS)
fw_convert_kernel(const T *__restrict__ in_base, U *__restrict__ work_base,
                  unsigned char *__restrict__ occ_base, const FwComp *__restrict__ comps,
                  const int64_t *__restrict__ prefix, int count, int lbits, int sbits,
                  DevStatus *st_base) {
    typedef typename utype<T>::type TU;
    typedef lane<U> L;
    const int ci = fw_find(prefix, count, blockIdx.x);
    const FwComp c = comps[ci];
    const T *in = in_base + c.in_off;
    U *work = work_base + c.work_off;
    const int64_t n = c.n, np = c.np, ld = c.ld_in;
    const int triangular = c.triangular;
    DevStatus *st = st_base + c.status_index;
    unsigned char *occ = occ_base + c.occ_off;
    const int nb = (int)(np / FW_B);
    const TU tmax = (TU)~(TU)0;
    const unsigned long long slimit = 1ull << (sbits - 1);   // storage top bit
    const unsigned long long llimit = 1ull << (lbits - 1);   // effective lane top bit
    unsigned flags = 0;
    unsigned long long mx = 0;
    // one warp per row (CONV_ROWS = 8 warps): small components keep every lane busy
    static_assert(CONV_ROWS * 32 == FW_THREADS, "one warp per converted row");
    const int64_t r0 = ((int64_t)blockIdx.x - prefix[ci]) * CONV_ROWS;
    const int64_t i = r0 + (threadIdx.x >> 5);
    const int lane_id = threadIdx.x & 31;
    if (i < np) {
        // W(i, 0) for the k = 0 product of d_0 (row 0 / column 0 products are identities)
        const bool rowlive = i < n;
        const TU wi0 = (rowlive && i > 0 && !triangular) ? (TU)in[i * ld] : (TU)0;
        const bool xi = wi0 != 0 && wi0 != 1 && wi0 != tmax && (unsigned long long)wi0 < llimit;
        U *wrow = work + i * np;
        for (int64_t j0 = (int64_t)lane_id * 4; j0 < np; j0 += 32 * 4) {
            U w4[4];
            bool live = false;
            if (rowlive && !xi && j0 + 4 <= n && (i < j0 || i >= j0 + 4)) {
                // fast path: four off-diagonal zeros (the common case) encode as zeros and add
                // nothing to the running maximum (no W(i, 0) (x) W(0, j) term on this row)
                const TU a = (TU)in[i * ld + j0], b = (TU)in[i * ld + j0 + 1];
                const TU c2 = (TU)in[i * ld + j0 + 2], d = (TU)in[i * ld + j0 + 3];
                if ((a | b | c2 | d) == 0) {
                    const U inf = L::inf;
                    w4[0] = w4[1] = w4[2] = w4[3] = inf;
                    *reinterpret_cast<uint4 *>(wrow + j0) = *reinterpret_cast<const uint4 *>(w4);
                    if (sizeof(U) == 8)
                        *reinterpret_cast<uint4 *>(wrow + j0 + 2) = *reinterpret_cast<const uint4 *>(w4 + 2);
                    continue;
                }
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int64_t j = j0 + k;
                U w = L::inf;
                if (rowlive && j < n) {
                    const TU v = (TU)in[i * ld + j];
                    if (i == j) {
                        if (!(v == 0 || v == 1 || v == tmax)) flags |= RBG_EV_UNCLEAN;
                    } else if (!(triangular && i > j) && v != 0) {
                        const unsigned long long uv = (unsigned long long)v;
                        if (v == 1 || v == tmax || uv >= slimit) flags |= RBG_EV_UNCLEAN;
                        else if (uv >= llimit) flags |= RBG_EV_WIDE;
                        else w = (U)uv;
                    }
                    if (i != j && !(triangular && i > j)) {
                        // d_0 = W(i,j) (+) W(i,0) (x) W(0,j): the value the reference writes at k = 0
                        U d0 = w;
                        if (xi && j > 0) {
                            const TU b = (TU)in[j];
                            if (b != 0 && b != 1 && b != tmax && (unsigned long long)b < llimit) {
                                bool risk = false;
                                const U p = L::product((U)wi0, (U)b, lbits, risk);
                                if (!risk) d0 = umin(d0, p);
                            }
                        }
                        if (L::valid(d0) && (unsigned long long)d0 > mx) mx = (unsigned long long)d0;
                    }
                }
                w4[k] = w;
                live |= L::valid(w);
            }
            *reinterpret_cast<uint4 *>(wrow + j0) = *reinterpret_cast<const uint4 *>(w4);
            if (sizeof(U) == 8)
                *reinterpret_cast<uint4 *>(wrow + j0 + 2) = *reinterpret_cast<const uint4 *>(w4 + 2);
            if (live) occ[(i / FW_B) * nb + j0 / FW_B] = 1;
        }
    }
    flush_status(st, mx, flags);
}

// ------------------------------------------------------------------------------------------
// phases 1 and 2 (diagonal tile, then the row and column panels)
// ------------------------------------------------------------------------------------------
#include "fw_panels.cuh"

// ------------------------------------------------------------------------------------------
// kernel B: phase 3 over BM x BN tiles, register micro-tiles TM x TN, 256 threads
// ------------------------------------------------------------------------------------------
// ---- bulk asynchronous copies global -> shared (the TMA unit), completing on an mbarrier
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint32_t bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
}
// every wait is bounded: false when the phase did not complete within the tries
constexpr int MBAR_TRIES = 1 << 20;
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (int it = 0; it < MBAR_TRIES; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// orders this thread's earlier generic accesses to shared memory before later async-proxy ones
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// `bytes` (a multiple of 16) from global `src` to shared `dst` (both 16-byte aligned)
__device__ __forceinline__ void bulk_to_smem(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(dst), "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

template <typename U, int BN> struct TileSmem {
    U CPt[FW_B][FW_P];       // CPt[q][i] = d_{t-1}(i, t) for the q-th active step t
    U RPm[FW_B][BN];         // 2^msb(d_{t-1}(t, j)) (0 for zero), q-th active step
    U RPl[FW_B][BN];         // d_{t-1}(t, j) - 2^msb   (inf for zero), q-th active step
    unsigned long long maskC[FW_P];   // bit t: CP(i, t) valid
    unsigned long long maskR[BN];     // bit t: RP(t, j) valid
    int active[FW_B];                 // active[q] = t
    int qof[FW_B];                    // qof[t] = q (or -1)
    unsigned long long colAny, rowAny;
};

// Line masks and group masks of the panels (written by the panel kernel of this round):
//   gm[0 .. nb)          column panel, per 64-row group: OR of its rows' masks (0 = no snapshots)
//   gm[nb .. 2 nb)       row panel, per 64-column group
//   gm[2 nb .. 2 nb + np)        column panel, per row i: bit t = CP(i, t) valid
//   gm[2 nb + np .. 2 nb + 2 np) row panel, per column j: bit t = RP(t, j) valid
// A line mask is meaningful only when its group mask is nonzero (groups with no nonzero line
// skip the panel pass and leave their line masks and snapshots from an earlier round), and a
// group's snapshot row t is written only when bit t of its group mask is set.
// Returns false when the snapshot copies did not complete within the bounded wait (the item's
// component is then marked RBG_EV_TIMEOUT and the CTA stops taking items).
template <typename U, int BN, int TM, int TN>
__device__ __forceinline__ bool tile_item(TileSmem<U, BN> &S, int ci, int64_t local, U *__restrict__ work_base,
                                          const unsigned long long *__restrict__ mask_base,
                                          unsigned char *__restrict__ occ_base,
                                          const FwComp *__restrict__ comps, int64_t K0, int lbits,
                                          DevStatus *st_base, uint32_t bar, uint32_t &parity) {
    typedef lane<U> L;
    constexpr int BM = FW_P;
    constexpr int TX = BN / TN;           // threads along columns
    constexpr int TY = BM / TM;           // threads along rows
    static_assert(TX * TY == FW_THREADS, "micro-tile layout must use 256 threads");
    static_assert(BM % 32 == 0 && BN % 32 == 0, "mask reduction works on whole warps");
    constexpr int HN = TN / 2;            // each thread owns two column groups of HN
    constexpr int PER = 16 / sizeof(U);
    const FwComp cmp = comps[ci];
    const int64_t np = cmp.np;
    U *work = work_base + cmp.work_off;
    const U *cpbuf = work_base + cmp.cp_off;
    const U *rpbuf = work_base + cmp.rp_off;
    const int nb = (int)(np / FW_B);
    const unsigned long long *gmC = mask_base + cmp.any_off;
    const unsigned long long *gmR = gmC + nb;
    const unsigned long long *lmC = gmC + 2 * nb;
    const unsigned long long *lmR = lmC + np;
    unsigned char *occ = occ_base + cmp.occ_off;
    DevStatus *st = st_base + cmp.status_index;
    const int tJn = (int)(np / BN);
    const int tI = (int)(local / tJn), tJ = (int)(local % tJn);
    const int64_t I0 = (int64_t)tI * BM, J0 = (int64_t)tJ * BN;
    const int tid = threadIdx.x, lane_id = tid & 31;
    if (tid == 0) { S.colAny = 0; S.rowAny = 0; }
    __syncthreads();

    // ---- line masks of this tile's rows and columns; their ORs give the active steps
    for (int e = tid; e < BM + BN; e += FW_THREADS) {
        // the line mask and its group mask are loaded together; a line of a group without
        // snapshots this round counts as zero
        unsigned long long m;
        if (e < BM) {
            const int64_t i = I0 + e;
            const unsigned long long lm = lmC[i], gm = gmC[i / FW_B];
            m = gm ? lm : 0ull;
            S.maskC[e] = m;
        } else {
            const int64_t j = J0 + (e - BM);
            const unsigned long long lm = lmR[j], gm = gmR[j / FW_B];
            m = gm ? lm : 0ull;
            S.maskR[e - BM] = m;
        }
        const unsigned lo = __reduce_or_sync(0xffffffffu, (unsigned)m);
        const unsigned hi = __reduce_or_sync(0xffffffffu, (unsigned)(m >> 32));
        if (lane_id == 0 && (lo | hi))
            atomicOr(e < BM ? &S.colAny : &S.rowAny, ((unsigned long long)hi << 32) | lo);
    }
    __syncthreads();
    const unsigned long long act = S.colAny & S.rowAny;
    if (act == 0) return true;   // uniform across the block
    const int na = __popcll(act);
    if (tid < FW_B) {
        const bool on = (act >> tid) & 1ull;
        const int q = __popcll(act & ((1ull << tid) - 1ull));
        if (on) S.active[q] = tid;
        S.qof[tid] = on ? q : -1;
    }
    __syncthreads();

    // ---- accumulators (loaded first, so that they are in flight with the staging loads)
    const int ty = tid / TX, tx = tid % TX;
    const int r0 = ty * TM;
    int cidx[TN];
#pragma unroll
    for (int c = 0; c < TN; ++c) cidx[c] = (c < HN) ? tx * HN + c : BN / 2 + tx * HN + (c - HN);
    U acc[TM][TN];
    unsigned long long wasInf = 0;
    unsigned rowWork = 0;   // bit r: row r0 + r has a nonzero operand at some active step
#pragma unroll
    for (int r = 0; r < TM; ++r) rowWork |= (unsigned)((S.maskC[r0 + r] & act) != 0) << r;
    static_assert(HN * sizeof(U) == 16, "each column group is one 16-byte vector");
#pragma unroll
    for (int r = 0; r < TM; ++r) {
        if (!((rowWork >> r) & 1u)) continue;       // cannot change: neither read nor written
        const U *row = work + (I0 + r0 + r) * np + J0;
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            uint4 v4 = *reinterpret_cast<const uint4 *>(row + cidx[half * HN]);
            const U *w = reinterpret_cast<const U *>(&v4);
#pragma unroll
            for (int k = 0; k < HN; ++k) {
                const int c = half * HN + k;
                acc[r][c] = w[k];
                wasInf |= (unsigned long long)(!L::valid(w[k])) << (r * TN + c);
            }
        }
    }

    // ---- stage the active steps' panel snapshots: every live 64-line piece (the column panel's
    // two row halves, the row panel's BN / 64 column groups of step t) is one bulk asynchronous
    // copy into the shared tables, issued by the first warp and completing on the CTA's mbarrier
    // while the accumulator loads above are in flight; a dead piece (a group without a snapshot
    // at step t) reads as the encoded zero.  The panel kernel stores snapshots already encoded
    // (an invalid operand as the encoded zero), so the rows are copied as they are; the row
    // panel's rows are split into (2^msb, low) pairs in shared memory afterwards.
    {
        constexpr int PC = BM / FW_B, PR = BN / FW_B, PP = PC + PR;   // pieces per active step
        constexpr uint32_t PIECE = FW_B * sizeof(U);                   // bytes per piece
        static_assert(PC == 2, "a tile is two 64-row groups high");
        const unsigned long long cg0 = gmC[I0 / FW_B], cg1 = gmC[I0 / FW_B + 1];
        auto live = [&](int p, int t) -> bool {
            const unsigned long long g = p == 0 ? cg0 : p == 1 ? cg1 : gmR[J0 / FW_B + (p - PC)];
            return (g >> t) & 1ull;
        };
        if (tid < 32) {
            fence_proxy_async_smem();          // the previous item's reads of the tables come first
            uint32_t bytes = 0;
            for (int e = tid; e < na * PP; e += 32) {
                const int q = e / PP, p = e % PP, t = S.active[q];
                if (!live(p, t)) continue;
                const U *src = p < PC ? cpbuf + (int64_t)t * np + I0 + p * FW_B
                                      : rpbuf + (int64_t)t * np + J0 + (p - PC) * FW_B;
                U *dst = p < PC ? &S.CPt[q][p * FW_B] : &S.RPm[q][(p - PC) * FW_B];
                bulk_to_smem(smem_u32(dst), src, PIECE, bar);
                bytes += PIECE;
            }
            bytes = __reduce_add_sync(0xffffffffu, bytes);
            if (tid == 0) mbar_arrive_expect_tx(bar, bytes);
        }
        const uint4 inf4 = make_uint4(0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu);
        constexpr int VP = FW_B / PER;                                 // 16-byte vectors per piece
        for (int e = tid; e < na * PP * VP; e += FW_THREADS) {
            const int piece = e / VP, v = e % VP, q = piece / PP, p = piece % PP;
            if (live(p, S.active[q])) continue;
            U *dst = p < PC ? &S.CPt[q][p * FW_B + v * PER] : &S.RPm[q][(p - PC) * FW_B + v * PER];
            *reinterpret_cast<uint4 *>(dst) = inf4;
        }
        const bool landed = mbar_wait(bar, parity);
        if (__syncthreads_or(!landed)) {
            // give copies still in flight a bounded time to land before the CTA leaves
            mbar_wait(bar, parity);
            if (tid == 0) atomicOr(&st->flags, RBG_EV_TIMEOUT);
            return false;
        }
        parity ^= 1u;
        for (int e = tid; e < na * (BN / PER); e += FW_THREADS) {
            const int q = e / (BN / PER), c = (e % (BN / PER)) * PER;
            const uint4 v = *reinterpret_cast<const uint4 *>(&S.RPm[q][c]);
            const U *w = reinterpret_cast<const U *>(&v);
            U m[PER], low[PER];
#pragma unroll
            for (int k = 0; k < PER; ++k) L::split(w[k], m[k], low[k]);
            *reinterpret_cast<uint4 *>(&S.RPm[q][c]) = *reinterpret_cast<const uint4 *>(m);
            *reinterpret_cast<uint4 *>(&S.RPl[q][c]) = *reinterpret_cast<const uint4 *>(low);
        }
    }
    __syncthreads();
    // risk: some computed product x (x) y with msb(x) + msb(y) >= lbits - 1, i.e. for some
    // active step the largest column-panel MSB plus the largest row-panel MSB reaches it
    bool risk = false;
    for (int q = tid >> 5; q < na; q += FW_THREADS / 32) {
        int mc = -1000, mr = -1000;
        for (int r = lane_id; r < BM; r += 32) {
            const U x = S.CPt[q][r];
            if (L::valid(x)) mc = max(mc, msb_nz<U>(x));
        }
        for (int c = lane_id; c < BN; c += 32) {
            const U m = S.RPm[q][c];
            if (m) mr = max(mr, msb_nz<U>(m));
        }
        mc = __reduce_max_sync(0xffffffffu, mc);
        mr = __reduce_max_sync(0xffffffffu, mr);
        if (mc >= 0 && mr >= 0 && mc + mr >= lbits - 1) risk = true;
    }

    unsigned steps_done = 0;
    for (int q = 0; q < na; ++q) {
        U x[TM], m[TN], l[TN];
        bool anyx = false;
#pragma unroll
        for (int r = 0; r < TM; ++r) {
            x[r] = S.CPt[q][r0 + r];
            anyx |= L::valid(x[r]);
        }
        // the warp's rows all zero at this step: every product is zero
        if (!__any_sync(0xffffffffu, anyx)) continue;
        ++steps_done;
#pragma unroll
        for (int c = 0; c < TN; ++c) { m[c] = S.RPm[q][cidx[c]]; l[c] = S.RPl[q][cidx[c]]; }
#pragma unroll
        for (int r = 0; r < TM; ++r)
#pragma unroll
            for (int c = 0; c < TN; ++c) acc[r][c] = umin(acc[r][c], x[r] * m[c] + l[c]);
    }
    if (lane_id == 0 && steps_done)
        atomicAdd(&st->executed, (unsigned long long)steps_done * 32 * TM * TN);

    // ---- write back, cycle test on the global diagonal, first values for the running max
    unsigned flags = risk ? RBG_EV_RISK : 0u;
    unsigned long long mx = 0;
    // Cells of the row/column panel (in K) saw only encoded-zero products, so their
    // accumulators still hold what the panel launch stored: writing them back is a no-op.
#pragma unroll
    for (int r = 0; r < TM; ++r) {
        if (!((rowWork >> r) & 1u)) continue;
        const int64_t gi = I0 + r0 + r;
        U *row = work + gi * np + J0;
        bool anyw = false;
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            uint4 v4;
            U *w = reinterpret_cast<U *>(&v4);
#pragma unroll
            for (int k = 0; k < HN; ++k) {
                const int c = half * HN + k;
                const int64_t gj = J0 + cidx[c];
                U v = acc[r][c];
                const bool valid = L::valid(v);
                if (gi == gj) {
                    if (valid) flags |= RBG_EV_CYCLE;
                    v = L::inf;   // the diagonal stays encoded zero
                } else if (valid && ((wasInf >> (r * TN + c)) & 1ull)) {
                    const unsigned long long both = S.maskC[r0 + r] & S.maskR[cidx[c]];
                    const int qf = S.qof[__ffsll((long long)both) - 1];
                    const U first = S.CPt[qf][r0 + r] * S.RPm[qf][cidx[c]] + S.RPl[qf][cidx[c]];
                    if ((unsigned long long)first > mx) mx = (unsigned long long)first;
                }
                w[k] = L::valid(v) ? v : L::inf;
                anyw |= L::valid(v);
            }
            *reinterpret_cast<uint4 *>(row + cidx[half * HN]) = v4;
            if (anyw) occ[(gi / FW_B) * nb + (J0 + cidx[half * HN]) / FW_B] = 1;
            anyw = false;
        }
    }
    flush_status(st, mx, flags);
    return true;
}

// Tile worklist: candidate tile (I, J) of this round is an item when some step t has a nonzero
// column-panel snapshot in one of its rows and a nonzero row-panel snapshot in one of its
// columns (the OR of the 64-line group masks of both sides intersect).
template <int BN>
__global__ void fw_tile_list_kernel(const FwComp *__restrict__ comps, const int64_t *__restrict__ prefix,
                                    int count, const unsigned long long *__restrict__ mask_base,
                                    int2 *__restrict__ list, int *__restrict__ counters) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= prefix[count]) return;
    const int ci = fw_find(prefix, count, c);
    const FwComp cmp = comps[ci];
    const int64_t local = c - prefix[ci];
    const int tJn = (int)(cmp.np / BN);
    const int tI = (int)(local / tJn), tJ = (int)(local % tJn);
    const int nb = (int)(cmp.np / FW_B);
    const unsigned long long *gmC = mask_base + cmp.any_off;
    const unsigned long long *gmR = gmC + nb;
    constexpr int GC = BN / FW_B;
    unsigned long long r = 0;
#pragma unroll
    for (int gq = 0; gq < GC; ++gq) r |= gmR[tJ * GC + gq];
    if ((r & (gmC[2 * tI] | gmC[2 * tI + 1])) == 0) return;
    const int slot = atomicAdd(&counters[CNT_TILE], 1);
    list[slot] = make_int2(ci, (int)local);
}

template <typename U, int BN, int TM, int TN>
__global__ void __launch_bounds__(FW_THREADS, (TM * TN * sizeof(U) <= 128) ? 3 : 2)
fw_tile_kernel(U *__restrict__ work_base, const unsigned long long *__restrict__ any_base,
               unsigned char *__restrict__ occ_base,
               const FwComp *__restrict__ comps, const int2 *__restrict__ list, int *__restrict__ counters,
               int64_t K0, int lbits, DevStatus *st_base) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TileSmem<U, BN> &S = *reinterpret_cast<TileSmem<U, BN> *>(smem_raw);
    __shared__ int s_item;
    __shared__ __align__(8) unsigned long long s_bar;   // completion of the snapshot copies
    const uint32_t bar = smem_u32(&s_bar);
    uint32_t parity = 0;
    const int total = counters[CNT_TILE];
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        s_item = atomicAdd(&counters[CUR_TILE], 1);
    }
    __syncthreads();
    int i = s_item;
    while (i < total) {
        // the next item is claimed now and published after this one: the claim's round trip
        // overlaps the item.  tile_item's first barrier comes before its first shared-memory
        // write, so one barrier per item keeps the items apart.
        int nxt = 0;
        if (threadIdx.x == 0) nxt = atomicAdd(&counters[CUR_TILE], 1);
        const int2 e = list[i];
        const bool ok = tile_item<U, BN, TM, TN>(S, e.x, e.y, work_base, any_base, occ_base, comps, K0, lbits,
                                                 st_base, bar, parity);
        if (!ok) {   // uniform: the CTA stops; the item it had claimed next is marked as well
            if (threadIdx.x == 0 && nxt < total)
                atomicOr(&st_base[comps[list[nxt].x].status_index].flags, RBG_EV_TIMEOUT);
            return;
        }
        if (threadIdx.x == 0) s_item = nxt;
        __syncthreads();
        i = s_item;
    }
}

// ------------------------------------------------------------------------------------------
// finalize: lane work matrix -> storage T (restores the diagonal and, in triangular mode, the
// untouched lower triangle from the input)
// ------------------------------------------------------------------------------------------
template <typename T, typename U>
__global__ void __launch_bounds__(FW_THREADS)
fw_finalize_kernel(const T *__restrict__ in_base, const U *__restrict__ work_base,
                   T *__restrict__ out_base, const FwComp *__restrict__ comps,
                   const int64_t *__restrict__ prefix, int count, const DevStatus *st_base,
                   const unsigned char *__restrict__ occ_base, RowStats rs) {
    const int ci = fw_find(prefix, count, blockIdx.x);
    const FwComp c = comps[ci];
    // a component that needs another path keeps its input untouched (it may be in place), and
    // so does one whose closure stopped at a bounded wait
    if (st_base[c.status_index].flags & (RBG_EV_UNCLEAN | RBG_EV_WIDE | RBG_EV_RISK | RBG_EV_CYCLE | RBG_EV_TIMEOUT))
        return;
    const T *in = in_base + c.in_off;
    const U *work = work_base + c.work_off;
    T *out = out_base + c.out_off;
    const int64_t n = c.n, np = c.np;
    const int64_t r0 = ((int64_t)blockIdx.x - prefix[ci]) * CONV_ROWS;
    // a 64 x 64 block that never held a valid value is all zero: its lanes are not read
    const unsigned char *occ = occ_base + c.occ_off;
    const int64_t nb = np / FW_B;
    const int64_t i = r0 + (threadIdx.x >> 5);   // one warp per row (warp-uniform)
    const int lane_id = threadIdx.x & 31;
    if (i < n) {
        const U *wrow = work + i * np;
        const unsigned char *orow = occ + (i / FW_B) * nb;
        const bool stats = rs.row_count != nullptr;
        unsigned long long *mrow = nullptr;
        if (stats && rs.chunk_mask)
            mrow = rs.chunk_mask + (c.in_off + 2047) / 2048 + rs.row_base[c.orig] + c.orig +
                   i * ((n + 2047) / 2048);
        int nnz = 0;
        long long mx = 0;
        unsigned long long word = 0;
        // four consecutive columns per lane (one 16-byte lane vector, one 64-column block):
        // 128 columns per warp and step
        constexpr int PER = 16 / sizeof(U);
        for (int64_t b = 0; b < n; b += 128) {
            const int64_t j0 = b + lane_id * 4;
            T v[4];
            U w[4];
            const bool occupied = j0 < n && orow[j0 / FW_B] != 0;
            if (occupied) {
#pragma unroll
                for (int k = 0; k < 4; k += PER)
                    *reinterpret_cast<uint4 *>(w + k) = *reinterpret_cast<const uint4 *>(wrow + j0 + k);
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int64_t j = j0 + k;
                v[k] = (T)0;
                if (j >= n) continue;
                if (i == j || (c.triangular && i > j)) v[k] = in[i * c.ld_in + j];
                else if (occupied) v[k] = lane<U>::valid(w[k]) ? (T)w[k] : (T)0;
            }
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (j0 + k < n) out[i * c.ld_out + j0 + k] = v[k];
            if (stats) {
                int here = 0;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    here += v[k] != (T)0;
                    mx = max(mx, (long long)v[k]);
                }
                nnz += here;
                // chunk 4s + q (s = b / 128) is columns held by lanes 8q .. 8q + 7
                const unsigned bal = __ballot_sync(0xffffffffu, here != 0);
                unsigned q4 = 0;
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if ((bal >> (8 * q)) & 0xffu) q4 |= 1u << q;
                const int64_t s = b >> 7;
                word |= (unsigned long long)q4 << (4 * (s & 15));
                if ((s & 15) == 15 || b + 128 >= n) {
                    if (mrow && lane_id == 0) mrow[s >> 4] = word;
                    word = 0;
                }
            }
        }
        if (stats) {
            nnz = __reduce_add_sync(0xffffffffu, nnz);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            if (lane_id == 0) {
                const int64_t at = rs.row_base[c.orig] + i;
                rs.row_count[rs.row_id ? (int64_t)rs.row_id[at] : at] = nnz;
                if (rs.comp_max && mx > 0) atomicMax(rs.comp_max + c.orig, (int)mx);
            }
        }
    }
}

// ------------------------------------------------------------------------------------------
// exact path: sequential order, full reference semantics
// ------------------------------------------------------------------------------------------
// SEM = 0: C core (any T).  SEM = 1: Cython (int32).
template <typename T, int SEM>
__device__ __forceinline__ T ex_product(T x, T y, unsigned &ev) {
    if (SEM == 1) return (T)cy_product((int32_t)x, (int32_t)y);
    return (T)avos_product<T>(x, y, ev);
}
template <typename T, int SEM> __device__ __forceinline__ T ex_sum(T a, T b) {
    if (SEM == 1) return (T)cy_sum((int32_t)a, (int32_t)b);
    return avos_sum<T>(a, b);
}

template <typename T, int SEM>
__device__ __forceinline__ void ex_event(DevStatus *st, unsigned ev, bool diag, T p,
                                         long long seq, unsigned &flags) {
    if (SEM == 0 && ev) {
        flags |= ev;
        if (ev & RBG_EV_HANG) atomicMin(&st->first_hang, seq);
        if (ev & (RBG_EV_OVF_SIZE | RBG_EV_OVF_ONES)) {
            atomicMax(&st->last_ovf, seq);
            atomicMin(&st->first_ovf, seq);
        }
    }
    if (diag && !(p == (T)-1 || p == 0 || p == 1)) {
        flags |= RBG_EV_CYCLE;
        atomicMax(&st->last_cycle, seq);
        atomicMin(&st->first_cycle, seq);
    }
}

template <typename T, int SEM>
__device__ __forceinline__ void ex_track(T v, long long &smax, unsigned long long &umax) {
    typedef typename utype<T>::type TU;
    if (SEM == 0 && (TU)(~v) == 0) return;   // warshall.c.in:89 skips all ones
    if (utype<T>::is_signed) {
        long long s = (long long)v;
        if (s > smax) smax = s;
    } else {
        unsigned long long u = (unsigned long long)(TU)v;
        if (u > umax) umax = u;
    }
}

__device__ __forceinline__ void flush_exact(DevStatus *st, long long smax, unsigned long long umax,
                                            unsigned flags) {
    for (int o = 16; o > 0; o >>= 1) {
        long long s2 = __shfl_xor_sync(0xffffffffu, smax, o);
        unsigned long long u2 = __shfl_xor_sync(0xffffffffu, umax, o);
        unsigned f2 = __shfl_xor_sync(0xffffffffu, flags, o);
        smax = s2 > smax ? s2 : smax;
        umax = u2 > umax ? u2 : umax;
        flags |= f2;
    }
    if ((threadIdx.x & 31) == 0) {
        if (smax > 0) atomicMax(&st->mx_signed, smax);
        if (umax > 0) atomicMax(&st->mx_unsigned, umax);
        if (flags) atomicOr(&st->flags, flags);
    }
}

// Row k of round k (i == k in the reference loop), plus the old row / column copies.
template <typename T, int SEM>
__global__ void __launch_bounds__(FW_THREADS)
fw_exact_row_kernel(T *__restrict__ w, int64_t ld, int64_t n, int64_t k, int triangular,
                    T *__restrict__ oldrow, T *__restrict__ oldcol, T *__restrict__ newrow,
                    DevStatus *st) {
    unsigned flags = 0;
    long long smax = 0;
    unsigned long long umax = 0;
    const T old_kk = w[k * ld + k];
    unsigned ev0 = 0;
    const T new_kk = ex_sum<T, SEM>(old_kk, ex_product<T, SEM>(old_kk, old_kk, ev0));
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n;
         j += (int64_t)gridDim.x * blockDim.x) {
        const T oj = w[k * ld + j];
        oldrow[j] = oj;
        oldcol[j] = w[j * ld + k];
        T nv = oj;
        if (!triangular || j >= k) {
            unsigned ev = 0;
            T x = (j <= k) ? old_kk : new_kk;
            T p = ex_product<T, SEM>(x, oj, ev);
            long long seq = ((long long)k * n + k) * n + j;
            ex_event<T, SEM>(st, ev, j == k, p, seq, flags);
            nv = ex_sum<T, SEM>(oj, p);
            ex_track<T, SEM>(nv, smax, umax);
        }
        newrow[j] = nv;
    }
    flush_exact(st, smax, umax, flags);
}

template <typename T, int SEM>
__global__ void __launch_bounds__(FW_THREADS)
fw_exact_cells_kernel(T *__restrict__ w, int64_t ld, int64_t n, int64_t k, int triangular,
                      const T *__restrict__ oldrow, const T *__restrict__ oldcol,
                      const T *__restrict__ newrow, DevStatus *st) {
    unsigned flags = 0;
    long long smax = 0;
    unsigned long long umax = 0;
    const int64_t total = n * n;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx / n, j = idx - i * n;
        if (i == k) {
            w[k * ld + j] = newrow[j];
            continue;
        }
        if (triangular && !(i < k && j >= k)) continue;
        const T* rowk = (i < k) ? oldrow : newrow;   // rows above k run before row k
        const T old_a = oldcol[i];
        unsigned ev = 0;
        T x = old_a;
        if (j > k) {
            unsigned ev2 = 0;   // W(i,k) was updated at j == k (its events counted there)
            x = ex_sum<T, SEM>(old_a, ex_product<T, SEM>(old_a, rowk[k], ev2));
        }
        T p = ex_product<T, SEM>(x, rowk[j], ev);
        long long seq = ((long long)k * n + i) * n + j;
        ex_event<T, SEM>(st, ev, i == j, p, seq, flags);
        T nv = ex_sum<T, SEM>(w[i * ld + j], p);
        w[i * ld + j] = nv;
        ex_track<T, SEM>(nv, smax, umax);
    }
    flush_exact(st, smax, umax, flags);
}

template <typename T, int SEM>
static int run_exact(const T *in, int64_t ld_in, T *out, int64_t ld_out, int64_t n, int triangular,
                     unsigned char *ws, DevStatus *st, cudaStream_t stream) {
    if (in != out)
        RBG_CUDA_TRY(cudaMemcpy2DAsync(out, ld_out * sizeof(T), in, ld_in * sizeof(T),
                                       n * sizeof(T), n, cudaMemcpyDeviceToDevice, stream));
    T *oldrow = reinterpret_cast<T *>(ws);
    T *oldcol = oldrow + align_up(n, 32);
    T *newrow = oldcol + align_up(n, 32);
    const int gr = grid_for(n, FW_THREADS);
    const int gc = grid_for(n * n, FW_THREADS);
    note_launches(2 * n);
    for (int64_t k = 0; k < n; ++k) {
        fw_exact_row_kernel<T, SEM><<<gr, FW_THREADS, 0, stream>>>(out, ld_out, n, k, triangular,
                                                                   oldrow, oldcol, newrow, st);
        fw_exact_cells_kernel<T, SEM><<<gc, FW_THREADS, 0, stream>>>(out, ld_out, n, k, triangular,
                                                                     oldrow, oldcol, newrow, st);
    }
    RBG_CUDA_TRY(cudaGetLastError());
    return RBG_OK;
}

// ------------------------------------------------------------------------------------------
// host driver
// ------------------------------------------------------------------------------------------
// Phase-3 tile shapes: BM = 128 rows always; 32-bit lanes have a wide (128 columns, 8 x 8 cells
// per thread) and a narrow (64 columns, 4 x 8 cells) shape, chosen per round (RBG_MODE_TILE_NARROW
// or the autotuner); 64-bit lanes use 64 columns, 8 x 4 cells.
template <typename U> struct TileCfg;
template <> struct TileCfg<uint32_t> { static const int BN = 128, TM = 8, TN = 8; };
template <> struct TileCfg<uint64_t> { static const int BN = 64, TM = 8, TN = 4; };
template <typename U> struct TileNarrow;
template <> struct TileNarrow<uint32_t> { static const int BN = 64, TM = 4, TN = 8; };
template <> struct TileNarrow<uint64_t> { static const int BN = 64, TM = 8, TN = 4; };


// Everything a (batched) blocked run needs on the host: the component table (sorted by size,
// descending), the per-kernel CTA prefix sums, the per-round active counts and the workspace
// layout.  A single matrix is a plan of one.
struct FwPlan {
    int count = 0;
    std::vector<FwComp> comps;
    std::vector<int64_t> pre_conv, pre_panel, pre_tile, pre_tile_n;   // _n: narrow tiles
    std::vector<int> active;                // active[r] = components with n > 64 r
    size_t off_status = 0, off_comps = 0, off_pconv = 0, off_ppanel = 0, off_ptile = 0, off_ptile_n = 0;
    size_t off_rb = 0, off_any = 0, off_lanes = 0, off_exact = 0, total = 0;
    size_t off_occ = 0, occ_bytes = 0, off_plist = 0, off_tlist = 0, off_counters = 0;
};

// sizes[i], in_off[i], out_off[i] of component i (input order); lane = bytes per lane word
static void build_plan(FwPlan &P, int64_t count, const int64_t *sizes, const int64_t *in_off,
                       const int64_t *out_off, size_t lane, int triangular, int tile_bn,
                       int elem_bytes, int tile_bn_narrow = 64, const int64_t *orig = nullptr) {
    P.count = (int)count;
    std::vector<int> order((size_t)count);
    for (int64_t i = 0; i < count; ++i) order[(size_t)i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return sizes[x] > sizes[y]; });
    P.comps.assign((size_t)count, FwComp());
    P.pre_conv.assign((size_t)count + 1, 0);
    P.pre_panel.assign((size_t)count + 1, 0);
    P.pre_tile.assign((size_t)count + 1, 0);
    P.pre_tile_n.assign((size_t)count + 1, 0);
    int64_t lanes = 0, anys = 0, maxn = 0, occs = 0;
    for (int64_t k = 0; k < count; ++k) {
        const int i = order[(size_t)k];
        FwComp &c = P.comps[(size_t)k];
        c.n = sizes[i];
        c.np = (int64_t)align_up((size_t)std::max<int64_t>(c.n, 1), FW_P);
        c.in_off = in_off[i];
        c.out_off = out_off[i];
        c.ld_in = c.ld_out = c.n;
        c.work_off = lanes; lanes += c.np * c.np;
        c.cp_off = lanes; lanes += (int64_t)FW_B * c.np;
        c.rp_off = lanes; lanes += (int64_t)FW_B * c.np;
        lanes = (int64_t)align_up((size_t)lanes, 64);
        c.any_off = anys; anys += 2 * (c.np / FW_B) + 2 * c.np;
        c.rb_index = k;
        c.occ_off = occs; occs += (c.np / FW_B) * (c.np / FW_B);
        c.triangular = triangular;
        c.status_index = i;
        c.orig = orig ? (int32_t)orig[i] : i;
        P.pre_conv[(size_t)k + 1] = P.pre_conv[(size_t)k] + (c.np + CONV_ROWS - 1) / CONV_ROWS;
        const bool big = c.n > FW_B;   // n <= 64: the diagonal tile is the whole matrix
        P.pre_panel[(size_t)k + 1] = P.pre_panel[(size_t)k] + (big ? 2 * (c.np / PN_LINES) : 0);
        P.pre_tile[(size_t)k + 1] = P.pre_tile[(size_t)k] + (big ? (c.np / tile_bn) * (c.np / FW_P) : 0);
        P.pre_tile_n[(size_t)k + 1] =
            P.pre_tile_n[(size_t)k] + (big ? (c.np / tile_bn_narrow) * (c.np / FW_P) : 0);
        maxn = std::max(maxn, c.n);
    }
    const int rounds = (int)((maxn + FW_B - 1) / FW_B);
    P.active.assign((size_t)rounds, 0);
    for (int r = 0; r < rounds; ++r) {
        int a = 0;
        while (a < count && P.comps[(size_t)a].n > (int64_t)r * FW_B) ++a;
        P.active[(size_t)r] = a;
    }
    size_t o = 0;
    P.off_status = o; o = align_up(o + (size_t)count * sizeof(DevStatus), 256);
    P.off_comps = o; o = align_up(o + (size_t)count * sizeof(FwComp), 256);
    P.off_pconv = o; o = align_up(o + ((size_t)count + 1) * 8, 256);
    P.off_ppanel = o; o = align_up(o + ((size_t)count + 1) * 8, 256);
    P.off_ptile = o; o = align_up(o + ((size_t)count + 1) * 8, 256);
    P.off_ptile_n = o; o = align_up(o + ((size_t)count + 1) * 8, 256);
    P.off_rb = o; o = align_up(o + (size_t)count * (lane == 8 ? sizeof(RoundBuf<uint64_t>) : sizeof(RoundBuf<uint32_t>)), 256);
    P.off_any = o; o = align_up(o + (size_t)anys * 8, 256);
    P.off_occ = o; P.occ_bytes = (size_t)occs; o = align_up(o + (size_t)occs, 256);
    const int a0 = rounds > 0 ? P.active[0] : 0;
    P.off_plist = o; o = align_up(o + (size_t)std::max<int64_t>(P.pre_panel[(size_t)a0], 1) * 8, 256);
    P.off_tlist = o;
    o = align_up(o + (size_t)std::max<int64_t>(std::max(P.pre_tile[(size_t)a0], P.pre_tile_n[(size_t)a0]), 1) * 8,
                 256);
    P.off_counters = o; o = align_up(o + 64, 256);
    P.off_lanes = o; o = align_up(o + (size_t)lanes * lane, 256);
    P.off_exact = o; o = align_up(o + 3 * align_up((size_t)maxn, 32) * elem_bytes + 256, 256);
    P.total = o;
}

static int read_status(DevStatus *d, DevStatus *h, int count, cudaStream_t stream) {
    HostStaging hs(stream, (size_t)count * sizeof(DevStatus));
    const int rc = hs.down(h, d, (size_t)count * sizeof(DevStatus));
    if (rc) return rc;
    return hs.finish();
}

template <typename U>
static int configure_kernels() {
    static PerDeviceOnce once;   // one per lane type, for every device
    return once.run([] {
    typedef TileCfg<U> C;
    RBG_CUDA_TRY(cudaFuncSetAttribute(fw_panel_kernel<U>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sizeof(PanelSmem<U>)));
    RBG_CUDA_TRY(cudaFuncSetAttribute(fw_diag_kernel<U>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sizeof(DiagSmem<U>)));
    RBG_CUDA_TRY(cudaFuncSetAttribute(fw_tile_kernel<U, C::BN, C::TM, C::TN>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sizeof(TileSmem<U, C::BN>)));
    typedef TileNarrow<U> N;
    RBG_CUDA_TRY(cudaFuncSetAttribute(fw_tile_kernel<U, N::BN, N::TM, N::TN>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sizeof(TileSmem<U, N::BN>)));
    return (int)RBG_OK;
    });
}

// Upload the plan's tables into the workspace.
static int upload_plan(const FwPlan &P, unsigned char *ws, cudaStream_t stream) {
    const size_t b0 = P.comps.size() * sizeof(FwComp), b1 = P.pre_conv.size() * 8, b2 = P.pre_panel.size() * 8,
                 b3 = P.pre_tile.size() * 8, b4 = P.pre_tile_n.size() * 8;
    HostStaging hs(stream, b0 + b1 + b2 + b3 + b4 + 5 * 64);
    int rc = hs.up(ws + P.off_comps, P.comps.data(), b0);
    if (!rc) rc = hs.up(ws + P.off_pconv, P.pre_conv.data(), b1);
    if (!rc) rc = hs.up(ws + P.off_ppanel, P.pre_panel.data(), b2);
    if (!rc) rc = hs.up(ws + P.off_ptile, P.pre_tile.data(), b3);
    if (!rc) rc = hs.up(ws + P.off_ptile_n, P.pre_tile_n.data(), b4);
    return rc;
}

// Launch the whole blocked closure of a plan (conversion, every round, finalization) on
// `stream`, without synchronising.  Components whose status asks for another path are left
// untouched in `out` by the finalization.
template <typename T, typename U>
static int launch_blocked(const FwPlan &P, const T *in, T *out, unsigned char *ws, cudaStream_t stream,
                          bool stop_after_convert, DevStatus *h_status, const unsigned char *shapes = nullptr,
                          cudaEvent_t *round_events = nullptr, const RowStats &rs = RowStats()) {
    typedef TileCfg<U> C;
    const int configured = configure_kernels<U>();   // once per device
    if (configured) return configured;
    const int cnt = P.count;
    DevStatus *st = reinterpret_cast<DevStatus *>(ws + P.off_status);
    const FwComp *comps = reinterpret_cast<const FwComp *>(ws + P.off_comps);
    const int64_t *pconv = reinterpret_cast<const int64_t *>(ws + P.off_pconv);
    const int64_t *ppanel = reinterpret_cast<const int64_t *>(ws + P.off_ppanel);
    const int64_t *ptile = reinterpret_cast<const int64_t *>(ws + P.off_ptile);
    const int64_t *ptile_n = reinterpret_cast<const int64_t *>(ws + P.off_ptile_n);
    typedef TileNarrow<U> N;
    RoundBuf<U> *rbs = reinterpret_cast<RoundBuf<U> *>(ws + P.off_rb);
    unsigned long long *any = reinterpret_cast<unsigned long long *>(ws + P.off_any);
    U *lanes = reinterpret_cast<U *>(ws + P.off_lanes);
    const int sbits = (int)sizeof(T) * 8;
    const int lbits = std::min<int>(sbits, (int)sizeof(U) * 8);

    note_launches(2);
    unsigned char *occ = ws + P.off_occ;
    int2 *plist = reinterpret_cast<int2 *>(ws + P.off_plist);
    int2 *tlist = reinterpret_cast<int2 *>(ws + P.off_tlist);
    int *counters = reinterpret_cast<int *>(ws + P.off_counters);
    const int sms = sm_count();
    const int64_t persist = 2 * (int64_t)sms;   // two CTAs per SM for both persistent kernels

    RBG_CUDA_TRY(cudaMemsetAsync(occ, 0, std::max<size_t>(P.occ_bytes, 1), stream));
    status_init_kernel<<<(cnt + 127) / 128, 128, 0, stream>>>(st, cnt);
    {
        cudaEvent_t tc = timer_begin(3, stream);
        fw_convert_kernel<T, U><<<(unsigned)P.pre_conv[cnt], FW_THREADS, 0, stream>>>(
            in, lanes, occ, comps, pconv, cnt, lbits, sbits, st);
        timer_end(3, tc, stream);
    }
    RBG_CUDA_TRY(cudaGetLastError());
    if (stop_after_convert) {
        int rc = read_status(st, h_status, cnt, stream);
        if (rc) return rc;
        if (h_status[0].flags & (RBG_EV_UNCLEAN | RBG_EV_WIDE)) return RBG_OK;
    }
    for (size_t r = 0; r < P.active.size(); ++r) {
        const int a = P.active[r];
        const int64_t K0 = (int64_t)r * FW_B;
        const bool narrow = shapes && shapes[r];
        const int64_t np_ = P.pre_panel[(size_t)a], nt_ = narrow ? P.pre_tile_n[(size_t)a] : P.pre_tile[(size_t)a];
        note_launches(1 + (np_ > 0 ? 2 : 0) + (nt_ > 0 ? 2 : 0));
        cudaEvent_t td = timer_begin(2, stream);
        fw_diag_kernel<U><<<a, DG_THREADS, sizeof(DiagSmem<U>), stream>>>(lanes, any, rbs, comps, counters,
                                                                           K0, lbits, st);
        timer_end(2, td, stream);
        if (np_ > 0) {
            cudaEvent_t t0 = timer_begin(1, stream);
            fw_panel_list_kernel<<<(unsigned)((np_ + 255) / 256), 256, 0, stream>>>(comps, ppanel, a, K0, occ,
                                                                                    plist, counters);
            fw_panel_kernel<U><<<(unsigned)std::min<int64_t>(np_, persist), PN_THREADS, sizeof(PanelSmem<U>),
                                 stream>>>(lanes, any, occ, rbs, comps, plist, counters, K0, lbits, st);
            timer_end(1, t0, stream);
        }
        if (round_events) RBG_CUDA_TRY(cudaEventRecord(round_events[2 * r], stream));
        if (nt_ > 0) {
            cudaEvent_t t0 = timer_begin(0, stream);
            const unsigned tl = (unsigned)((nt_ + 255) / 256);
            // persistent grids: as many CTAs as fit on the SMs (3 per SM for the narrow 32-bit shape)
            const int per_sm = (N::TM * N::TN * (int)sizeof(U) <= 128) ? 3 : 2;
            const unsigned tg = (unsigned)std::min<int64_t>(nt_, narrow ? (int64_t)per_sm * sms : persist);
            if (narrow) {
                fw_tile_list_kernel<N::BN><<<tl, 256, 0, stream>>>(comps, ptile_n, a, any, tlist, counters);
                fw_tile_kernel<U, N::BN, N::TM, N::TN><<<tg, FW_THREADS, sizeof(TileSmem<U, N::BN>), stream>>>(
                    lanes, any, occ, comps, tlist, counters, K0, lbits, st);
            } else {
                fw_tile_list_kernel<C::BN><<<tl, 256, 0, stream>>>(comps, ptile, a, any, tlist, counters);
                fw_tile_kernel<U, C::BN, C::TM, C::TN><<<tg, FW_THREADS, sizeof(TileSmem<U, C::BN>), stream>>>(
                    lanes, any, occ, comps, tlist, counters, K0, lbits, st);
            }
            timer_end(0, t0, stream);
        }
        if (round_events) RBG_CUDA_TRY(cudaEventRecord(round_events[2 * r + 1], stream));
    }
    RBG_CUDA_TRY(cudaGetLastError());
    note_launches(1);
    {
        cudaEvent_t tf = timer_begin(3, stream);
        fw_finalize_kernel<T, U><<<(unsigned)P.pre_conv[cnt], FW_THREADS, 0, stream>>>(
            in, lanes, out, comps, pconv, cnt, st, occ, rs);
        timer_end(3, tf, stream);
    }
    RBG_CUDA_TRY(cudaGetLastError());
    return RBG_OK;
}

static void decode_seq(long long seq, int64_t n, rbg_result_t *r) {
    if (seq < 0 || seq == LLONG_MAX) { r->k = r->i = r->j = -1; return; }
    r->j = seq % n;
    r->i = (seq / n) % n;
    r->k = seq / n / n;
}

template <typename U>
static void single_plan(FwPlan &P, int64_t n, int64_t ld_in, int64_t ld_out, int triangular, int elem_bytes) {
    const int64_t zero = 0;
    build_plan(P, 1, &n, &zero, &zero, sizeof(U), triangular, TileCfg<U>::BN, elem_bytes);
    P.comps[0].ld_in = ld_in;
    P.comps[0].ld_out = ld_out;
}

static size_t single_workspace(int64_t n, int dtype) {
    FwPlan P32, P64;
    single_plan<uint32_t>(P32, n, n, n, 0, dtype_bytes(dtype));
    size_t t = P32.total;
    if (dtype_bytes(dtype) == 8) {
        single_plan<uint64_t>(P64, n, n, n, 0, 8);
        t = std::max(t, P64.total);
    }
    return t;
}

// Exact sequential-order run; fills `res` from the reference's error conventions.
template <typename T>
static int exact_dense(int64_t n, const T *in, int64_t ld_in, T *out, int64_t ld_out, bool cython,
                       int triangular, unsigned char *ws, size_t off_status, size_t off_exact,
                       rbg_result_t *res, cudaStream_t stream) {
    DevStatus h;
    DevStatus *st = reinterpret_cast<DevStatus *>(ws + off_status);
    note_launches(1);
    status_init_kernel<<<1, 32, 0, stream>>>(st, 1);
    int rc = cython ? run_exact<T, 1>(in, ld_in, out, ld_out, n, triangular, ws + off_exact, st, stream)
                    : run_exact<T, 0>(in, ld_in, out, ld_out, n, triangular, ws + off_exact, st, stream);
    if (rc) return rc;
    rc = read_status(st, &h, 1, stream);
    if (rc) return rc;
    res->path = RBG_PATH_EXACT;
    res->flags = h.flags;
    if (cython) {
        if (h.first_cycle != LLONG_MAX) {
            res->status = RBG_ERR_CYCLE;
            decode_seq(h.first_cycle, n, res);
            res->diameter = 0;
        } else {
            res->status = RBG_OK;
            res->diameter = h.mx_signed > 1 ? msb_u64((unsigned long long)h.mx_signed) : 0;
        }
        return RBG_OK;
    }
    if (h.first_hang != LLONG_MAX) {
        res->status = RBG_ERR_OVERFLOW;   // the reference would loop forever here
        decode_seq(h.first_hang, n, res);
        res->diameter = 0;
        return RBG_OK;
    }
    if (h.last_ovf >= 0 || h.last_cycle >= 0) {
        const bool ovf_last = h.last_ovf > h.last_cycle;
        res->status = ovf_last ? RBG_ERR_OVERFLOW : RBG_ERR_CYCLE;
        decode_seq(ovf_last ? h.last_ovf : h.last_cycle, n, res);
    } else {
        res->status = RBG_OK;
    }
    const unsigned long long mxv = utype<T>::is_signed
        ? (unsigned long long)std::max<long long>(h.mx_signed, 0) : h.mx_unsigned;
    res->diameter = mxv ? msb_u64(mxv) : 0;
    return RBG_OK;
}

static void result_from_blocked(const DevStatus &h, int path, rbg_result_t *res) {
    res->executed = (int64_t)h.executed;
    res->status = (h.flags & RBG_EV_TIMEOUT) ? RBG_ERR_TIMEOUT : RBG_OK;
    res->flags = h.flags;
    res->diameter = h.mx ? msb_u64(h.mx) : 0;
    res->path = path;
}

// Modes under which a matrix numbered in a topological order may take the DAG path.
static bool dag_path_allowed(uint32_t mode) {
    return !(mode & (RBG_MODE_NO_DAG | RBG_MODE_TRIANGULAR | RBG_MODE_FORCE_EXACT | RBG_MODE_FORCE_WIDE));
}

// Single matrix: the DAG path for int32 / int64 matrices numbered in a topological order, else
// 32-bit lanes, then 64-bit lanes when 64-bit values need them, then the exact sequential-order
// kernel for anything outside the clean regime, cycles and top-bit products.  A matrix whose
// loop the DAG path found to compute a product reaching bit 31 (`top_bit`, from the DAG path of
// this call or of the batch that hands it over) skips the 32-bit lanes, which could only report
// that risk: int64 goes on with 64-bit lanes, int32 with the exact kernel.
template <typename T>
static int fw_dense_t(int64_t n, const T *in, int64_t ld_in, T *out, int64_t ld_out, uint32_t mode,
                      unsigned char *ws, size_t ws_bytes, bool try_dag, rbg_result_t *res, cudaStream_t stream,
                      bool top_bit = false) {
    const bool cython = (mode & RBG_MODE_CYTHON) != 0;
    const int triangular = (mode & RBG_MODE_TRIANGULAR) ? 1 : 0;
    memset(res, 0, sizeof(*res));
    res->k = res->i = res->j = -1;
    if constexpr (std::is_same<T, int32_t>::value || std::is_same<T, int64_t>::value) {
        if (try_dag && dag_path_allowed(mode)) {
            const int64_t zero = 0;
            char closed = TRI_OPEN;
            const int rc = tri_batch<T>(1, &n, &zero, &zero, ld_in, ld_out, in, out, res, &closed, ws, ws_bytes, mode,
                                        stream, RowStats());
            if (rc) return rc;
            if (closed == TRI_CLOSED) return RBG_OK;
            top_bit = closed == TRI_TOP_BIT;
        }
    }
    DevStatus h;
    FwPlan P;
    single_plan<uint32_t>(P, n, ld_in, ld_out, triangular, (int)sizeof(T));
    if (!(mode & RBG_MODE_FORCE_EXACT) && !(top_bit && sizeof(T) == 4)) {
        bool wide = sizeof(T) == 8 && ((mode & RBG_MODE_FORCE_WIDE) || top_bit);
        if (!wide) {
            int rc = upload_plan(P, ws, stream);
            if (rc) return rc;
            rc = launch_blocked<T, uint32_t>(P, in, out, ws, stream, true, &h);
            if (rc) return rc;
            if (!(h.flags & (RBG_EV_UNCLEAN | RBG_EV_WIDE))) {
                rc = read_status(reinterpret_cast<DevStatus *>(ws + P.off_status), &h, 1, stream);
                if (rc) return rc;
            }
            const unsigned f = h.flags;
            if (!(f & (RBG_EV_UNCLEAN | RBG_EV_CYCLE | RBG_EV_WIDE | RBG_EV_RISK))) {
                result_from_blocked(h, RBG_PATH_BLOCKED32, res);
                return RBG_OK;
            }
            wide = sizeof(T) == 8 && !(f & (RBG_EV_UNCLEAN | RBG_EV_CYCLE));
        }
        if (wide) {
            FwPlan P64;
            single_plan<uint64_t>(P64, n, ld_in, ld_out, triangular, (int)sizeof(T));
            int rc = upload_plan(P64, ws, stream);
            if (rc) return rc;
            rc = launch_blocked<T, uint64_t>(P64, in, out, ws, stream, true, &h);
            if (rc) return rc;
            if (!(h.flags & (RBG_EV_UNCLEAN | RBG_EV_WIDE))) {
                rc = read_status(reinterpret_cast<DevStatus *>(ws + P64.off_status), &h, 1, stream);
                if (rc) return rc;
            }
            if (!(h.flags & (RBG_EV_UNCLEAN | RBG_EV_CYCLE | RBG_EV_WIDE | RBG_EV_RISK))) {
                result_from_blocked(h, RBG_PATH_BLOCKED64, res);
                return RBG_OK;
            }
        }
    }
    return exact_dense<T>(n, in, ld_in, out, ld_out, cython, triangular, ws, P.off_status, P.off_exact,
                          res, stream);
}

// Batch: every component in one blocked run with 32-bit lanes; components that need another
// path (64-bit lanes, exact order) are then closed one by one with the single-matrix path,
// reusing the workspace.
// ------------------------------------------------------------------------------------------
// CUDA-graph replay of a batch's launch sequence (RBG_MODE_GRAPH)
// ------------------------------------------------------------------------------------------
// The blocked pass of a batch is a fixed sequence of ~5 launches per round whose grids depend
// only on the plan.  With RBG_MODE_GRAPH the sequence is captured once into a CUDA graph,
// keyed by everything it bakes in (types, sizes, offsets, buffers, workspace), and replayed by
// later calls with the same key.  A small LRU cache holds the instantiated graphs.
struct GraphKey {
    int tbytes, ubytes, triangular;
    const void *in;
    void *out;
    void *ws;
    std::vector<int64_t> sizes, offsets;
    std::vector<unsigned char> shapes;
    RowStats rs;
    bool operator==(const GraphKey &o) const {
        return tbytes == o.tbytes && ubytes == o.ubytes && triangular == o.triangular && in == o.in &&
               out == o.out && ws == o.ws && sizes == o.sizes && offsets == o.offsets && shapes == o.shapes &&
               rs == o.rs;
    }
};
struct GraphEntry {
    GraphKey key;
    cudaGraphExec_t exec;
    long long launches;
    unsigned long long stamp;
};
static std::mutex g_graph_mu;
static std::vector<GraphEntry> g_graphs;
static unsigned long long g_graph_clock = 0;
constexpr size_t GRAPH_CACHE = 8;

// launches of one blocked pass (as launch_blocked counts them)
static long long blocked_launches(const FwPlan &P) {
    long long n = 3;
    for (size_t r = 0; r < P.active.size(); ++r) {
        const int a = P.active[r];
        n += 1 + (P.pre_panel[(size_t)a] > 0 ? 2 : 0) + (P.pre_tile[(size_t)a] > 0 ? 2 : 0);
    }
    return n;
}

template <typename T, typename U>
static int launch_blocked_graph(const FwPlan &P, int64_t count, const int64_t *sizes, const int64_t *offsets,
                                const T *in, T *out, unsigned char *ws, cudaStream_t stream, int triangular,
                                const std::vector<unsigned char> &shapes, const RowStats &rs) {
    if (g_timer.on)   // timed per kernel: launched directly
        return launch_blocked<T, U>(P, in, out, ws, stream, false, nullptr, shapes.data(), nullptr, rs);
    GraphKey key{(int)sizeof(T), (int)sizeof(U), triangular, in, out, ws,
                 std::vector<int64_t>(sizes, sizes + count), std::vector<int64_t>(offsets, offsets + count),
                 shapes, rs};
    {
        std::lock_guard<std::mutex> lk(g_graph_mu);
        for (auto &e : g_graphs) {
            if (e.key == key) {
                e.stamp = ++g_graph_clock;
                RBG_CUDA_TRY(cudaGraphLaunch(e.exec, stream));
                note_launches(e.launches);
                return RBG_OK;
            }
        }
    }
    // record on a private stream (the caller's may be the legacy default stream, which cannot be
    // captured); nothing runs while recording, and the graph is launched on the caller's stream
    static thread_local cudaStream_t cap = nullptr;
    if (!cap) RBG_CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    RBG_CUDA_TRY(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    t_recording = 1;
    const int rc = launch_blocked<T, U>(P, in, out, ws, cap, false, nullptr, shapes.data(), nullptr, rs);
    t_recording = 0;
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(cap, &graph);
    if (rc || ec != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return rc ? rc : RBG_ERR_CUDA;
    }
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) return RBG_ERR_CUDA;
    RBG_CUDA_TRY(cudaGraphLaunch(exec, stream));
    const long long nl = blocked_launches(P);
    note_launches(nl);
    std::lock_guard<std::mutex> lk(g_graph_mu);
    if (g_graphs.size() >= GRAPH_CACHE) {
        size_t old = 0;
        for (size_t k = 1; k < g_graphs.size(); ++k)
            if (g_graphs[k].stamp < g_graphs[old].stamp) old = k;
        cudaDeviceSynchronize();   // the evicted graph may still run on another stream
        cudaGraphExecDestroy(g_graphs[old].exec);
        g_graphs.erase(g_graphs.begin() + (long)old);
    }
    g_graphs.push_back(GraphEntry{std::move(key), exec, nl, ++g_graph_clock});
    return RBG_OK;
}

// ------------------------------------------------------------------------------------------
// autotuner (RBG_MODE_AUTOTUNE): the phase-3 tile shape of every round
// ------------------------------------------------------------------------------------------
// Round r of a batch runs the components larger than 64 r, so rounds stand for size classes.
// The first call for a batch layout (keyed by the number of components active in each round)
// closes the batch twice, with wide and with narrow tiles in every round, timing each round's
// phase 3 with events; each round then keeps the faster shape, for every later call with that
// key (in-process cache).  Both passes compute the full closure, so the call's results are those
// of the second pass; a call whose input and output are the same buffer is not tuned.
struct TuneEntry {
    int tbytes, triangular;
    std::vector<int> active;
    std::vector<unsigned char> shapes;
};
static std::mutex g_tune_mu;
static std::vector<TuneEntry> g_tune;

static bool tune_lookup(int tbytes, int triangular, const std::vector<int> &active, std::vector<unsigned char> &shapes) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (const auto &e : g_tune)
        if (e.tbytes == tbytes && e.triangular == triangular && e.active == active) {
            shapes = e.shapes;
            return true;
        }
    return false;
}

template <typename T>
static int tune_blocked(const FwPlan &P, const T *in, T *out, unsigned char *ws, cudaStream_t stream, int triangular,
                        std::vector<unsigned char> &shapes, const RowStats &rs) {
    const size_t R = P.active.size();
    std::vector<cudaEvent_t> ev(4 * R, nullptr);
    for (auto &e : ev) RBG_CUDA_TRY(cudaEventCreate(&e));
    std::vector<float> ms[2];
    int rc = RBG_OK;
    for (int shape = 0; shape < 2 && rc == RBG_OK; ++shape) {
        std::vector<unsigned char> all(R, (unsigned char)shape);
        rc = launch_blocked<T, uint32_t>(P, in, out, ws, stream, false, nullptr, all.data(), ev.data() + 2 * R * shape,
                                         rs);
    }
    if (rc == RBG_OK && cudaStreamSynchronize(stream) != cudaSuccess) rc = RBG_ERR_CUDA;
    if (rc == RBG_OK) {
        shapes.assign(R, 0);
        for (size_t r = 0; r < R; ++r) {
            float w = 0.f, n = 0.f;
            cudaEventElapsedTime(&w, ev[2 * r], ev[2 * r + 1]);
            cudaEventElapsedTime(&n, ev[2 * R + 2 * r], ev[2 * R + 2 * r + 1]);
            shapes[r] = n < 0.97f * w ? 1 : 0;   // narrow only when clearly faster
        }
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune.push_back(TuneEntry{(int)sizeof(T), triangular, P.active, shapes});
    }
    for (auto &e : ev) cudaEventDestroy(e);
    return rc;
}

template <typename T>
static int fw_batch_t(int64_t count, const int64_t *sizes, const int64_t *offsets, const T *in, T *out,
                      uint32_t mode, unsigned char *ws, size_t ws_bytes, rbg_result_t *results, cudaStream_t stream,
                      const RowStats &rs = RowStats()) {
    const int triangular = (mode & RBG_MODE_TRIANGULAR) ? 1 : 0;
    for (int64_t i = 0; i < count; ++i) {
        memset(&results[i], 0, sizeof(rbg_result_t));
        results[i].k = results[i].i = results[i].j = -1;
    }
    // matrices numbered in a topological order take the DAG path; the rest form a sub-batch
    std::vector<char> closed((size_t)count, 0);
    if constexpr (std::is_same<T, int32_t>::value || std::is_same<T, int64_t>::value) {
        if (dag_path_allowed(mode)) {
            const int rc = tri_batch<T>(count, sizes, offsets, offsets, 0, 0, in, out, results, closed.data(), ws,
                                        ws_bytes, mode, stream, rs);
            if (rc) return rc;
        }
    }
    // components the DAG path found to reach bit 31 skip the batched 32-bit pass
    std::vector<int64_t> idx, top;
    for (int64_t i = 0; i < count; ++i) {
        if (closed[(size_t)i] == TRI_OPEN) idx.push_back(i);
        else if (closed[(size_t)i] == TRI_TOP_BIT) top.push_back(i);
    }
    for (int64_t i : top) {
        const int rc = fw_dense_t<T>(sizes[i], in + offsets[i], sizes[i], out + offsets[i], sizes[i], mode, ws,
                                     ws_bytes, false, &results[i], stream, true);
        if (rc) return rc;
    }
    if (idx.empty()) return RBG_OK;
    const bool whole = (int64_t)idx.size() == count;
    std::vector<int64_t> sub_sizes, sub_offsets;
    if (!whole) {
        for (int64_t i : idx) {
            sub_sizes.push_back(sizes[i]);
            sub_offsets.push_back(offsets[i]);
        }
    }
    const int64_t cnt = (int64_t)idx.size();
    const int64_t *sz = whole ? sizes : sub_sizes.data();
    const int64_t *of = whole ? offsets : sub_offsets.data();
    std::vector<char> redo((size_t)cnt, 1);
    if (!(mode & (RBG_MODE_FORCE_EXACT | RBG_MODE_FORCE_WIDE))) {
        FwPlan P;
        build_plan(P, cnt, sz, of, of, 4, triangular, TileCfg<uint32_t>::BN, (int)sizeof(T), 64,
                   whole ? nullptr : idx.data());
        int rc = upload_plan(P, ws, stream);
        if (rc) return rc;
        std::vector<unsigned char> shapes(P.active.size(), (mode & RBG_MODE_TILE_NARROW) ? 1 : 0);
        bool done = false;
        if ((mode & RBG_MODE_AUTOTUNE) && !tune_lookup((int)sizeof(T), triangular, P.active, shapes) &&
            (const void *)in != (const void *)out) {
            rc = tune_blocked<T>(P, in, out, ws, stream, triangular, shapes, rs);
            if (rc) return rc;
            done = true;
        }
        if (!done)
            rc = (mode & RBG_MODE_GRAPH)
                     ? launch_blocked_graph<T, uint32_t>(P, cnt, sz, of, in, out, ws, stream, triangular, shapes, rs)
                     : launch_blocked<T, uint32_t>(P, in, out, ws, stream, false, nullptr, shapes.data(), nullptr,
                                                   rs);
        if (rc) return rc;
        std::vector<DevStatus> h((size_t)cnt);
        rc = read_status(reinterpret_cast<DevStatus *>(ws + P.off_status), h.data(), (int)cnt, stream);
        if (rc) return rc;
        for (int64_t k = 0; k < cnt; ++k) {
            if (!(h[(size_t)k].flags & (RBG_EV_UNCLEAN | RBG_EV_CYCLE | RBG_EV_WIDE | RBG_EV_RISK))) {
                result_from_blocked(h[(size_t)k], RBG_PATH_BLOCKED32, &results[idx[(size_t)k]]);
                redo[(size_t)k] = 0;
            }
        }
    }
    for (int64_t k = 0; k < cnt; ++k) {
        const int64_t i = idx[(size_t)k];
        if (!redo[(size_t)k] || sizes[i] == 0) continue;
        int rc = fw_dense_t<T>(sizes[i], in + offsets[i], sizes[i], out + offsets[i], sizes[i], mode, ws,
                               ws_bytes, false, &results[i], stream);
        if (rc) return rc;
    }
    return RBG_OK;
}

}  // namespace rbg

using namespace rbg;

extern "C" int32_t rbg_version(void) { return 100; }

extern "C" int64_t rbg_launch_count(void) { return (int64_t)g_launches.load(); }

extern "C" int32_t rbg_profile_begin(void) {
    for (auto &v : g_timer.pending) {
        for (auto &pr : v) { g_timer.pool.push_back(pr.first); g_timer.pool.push_back(pr.second); }
        v.clear();
    }
    g_timer.on = true;
    return RBG_OK;
}

extern "C" int32_t rbg_profile_end(double *ms, int64_t *launches) {
    return rbg_profile_end_slots(ms, launches, 4);
}

extern "C" int32_t rbg_profile_end_slots(double *ms, int64_t *launches, int32_t slots) {
    if (!ms || !launches || slots < 1 || slots > TIMER_SLOTS) return RBG_ERR_INVALID;
    g_timer.on = false;
    for (int k = slots; k < TIMER_SLOTS; ++k) {   // slots not asked for are dropped
        for (auto &pr : g_timer.pending[k]) { g_timer.pool.push_back(pr.first); g_timer.pool.push_back(pr.second); }
        g_timer.pending[k].clear();
    }
    for (int k = 0; k < slots; ++k) {
        double tot = 0.0;
        for (auto &pr : g_timer.pending[k]) {
            float t = 0.f;
            RBG_CUDA_TRY(cudaEventSynchronize(pr.second));
            RBG_CUDA_TRY(cudaEventElapsedTime(&t, pr.first, pr.second));
            tot += t;
            g_timer.pool.push_back(pr.first);
            g_timer.pool.push_back(pr.second);
        }
        ms[k] = tot;
        launches[k] = (int64_t)g_timer.pending[k].size();
        g_timer.pending[k].clear();
    }
    return RBG_OK;
}

extern "C" int32_t rbg_fw_dense_workspace_bytes(int32_t dtype, int64_t n, uint32_t mode, int64_t *bytes) {
    if (!bytes || n < 0 || dtype_bytes(dtype) == 0) return RBG_ERR_INVALID;
    (void)mode;
    *bytes = (int64_t)single_workspace(n, dtype);
    return RBG_OK;
}

extern "C" int32_t rbg_fw_dense(int32_t dtype, int64_t n, const void *in, int64_t ld_in, void *out,
                                int64_t ld_out, uint32_t mode, void *workspace, int64_t workspace_bytes,
                                rbg_result_t *result, rbg_stream_t stream) {
    if (!result || n < 0 || (n > 0 && (!in || !out || !workspace)) || ld_in < n || ld_out < n)
        return RBG_ERR_INVALID;
    const int bytes = dtype_bytes(dtype);
    if (bytes == 0) return RBG_ERR_INVALID;
    if ((mode & RBG_MODE_CYTHON) && dtype != RBG_DTYPE_INT32) return RBG_ERR_INVALID;
    memset(result, 0, sizeof(*result));
    result->k = result->i = result->j = -1;
    if (n == 0) return RBG_OK;
    if (workspace_bytes < (int64_t)single_workspace(n, dtype)) return RBG_ERR_NOMEM;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    unsigned char *ws = reinterpret_cast<unsigned char *>(workspace);
    int rc = RBG_ERR_INVALID;
    RBG_DISPATCH_DTYPE(dtype, T,
        rc = fw_dense_t<T>(n, reinterpret_cast<const T *>(in), ld_in, reinterpret_cast<T *>(out),
                           ld_out, mode, ws, (size_t)workspace_bytes, true, result, s));
    return rc;
}

// ------------------------------------------------------------------------------------------
// Closure without any device allocation by the caller.
//
// Some callers cannot call cudaMalloc at all: code running where allocation is forbidden or
// would deadlock (inside a foreign allocator's callback, under an allocation-free real-time
// policy), or a host program that only owns the input and output buffers and must not grow the
// device heap.  rbg_fw_dense_noalloc takes its scratch from this file-scope device array
// instead of a workspace argument.  Every GPU that loads the library holds the array until the
// process exits.  All calls share it: each call clears or fully rewrites the scratch state it
// reads, but two calls whose work overlaps on the GPU (different streams, or different host
// threads on the same device) race on it and must be serialised by the caller.
// ------------------------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_noalloc_scratch[RBG_NOALLOC_SCRATCH_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[NOALLOC_MAX_DEVICES];   // the array's device address, per device

// Device address of the scratch array on the current device.  In host code the array's name is
// only a host-side stand-in, so the address is asked of the runtime once per device (with that
// device current) and cached; this first call must come before any stream capture.  Outside a
// capture every call asks again and replaces a cached address that changed (the module is
// loaded afresh after cudaDeviceReset), so a reset never leaves a dangling address behind.
static int noalloc_scratch(cudaStream_t s, void **ptr) {
    int dev = 0;
    RBG_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return RBG_ERR_INVALID;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    RBG_CUDA_TRY(cudaStreamIsCapturing(s, &cs));
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (cs == cudaStreamCaptureStatusNone || !g_noalloc_ptr[dev]) {
        if (cs != cudaStreamCaptureStatusNone) return RBG_ERR_INVALID;   // set-up inside a capture
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) return RBG_ERR_CUDA;
        g_noalloc_ptr[dev] = p;
    }
    *ptr = g_noalloc_ptr[dev];
    return RBG_OK;
}

extern "C" int32_t rbg_fw_dense_noalloc(int32_t dtype, int64_t n, const void *in, int64_t ld_in, void *out,
                                        int64_t ld_out, uint32_t mode, rbg_result_t *result,
                                        rbg_stream_t stream) {
    if (!result || n < 0 || (n > 0 && (!in || !out)) || ld_in < n || ld_out < n) return RBG_ERR_INVALID;
    if (dtype_bytes(dtype) == 0) return RBG_ERR_INVALID;
    if ((mode & RBG_MODE_CYTHON) && dtype != RBG_DTYPE_INT32) return RBG_ERR_INVALID;
    memset(result, 0, sizeof(*result));
    result->k = result->i = result->j = -1;
    if (n > RBG_NOALLOC_MAX_N || single_workspace(n, dtype) > (size_t)RBG_NOALLOC_SCRATCH_BYTES)
        return RBG_ERR_CAPACITY;   // beyond what the fixed scratch array holds
    if (n == 0) return RBG_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    void *ws = nullptr;
    int rc = noalloc_scratch(s, &ws);
    if (rc) return rc;
    mode &= ~RBG_MODE_GRAPH;   // instantiating a graph may take driver memory
    NoHostAlloc pageable;      // and no page-locked staging: pageable copies only
    rc = RBG_ERR_INVALID;
    RBG_DISPATCH_DTYPE(dtype, T,
        rc = fw_dense_t<T>(n, reinterpret_cast<const T *>(in), ld_in, reinterpret_cast<T *>(out), ld_out,
                           mode, reinterpret_cast<unsigned char *>(ws), (size_t)RBG_NOALLOC_SCRATCH_BYTES, true,
                           result, s));
    return rc;
}

// Workspace sizes of recent batch layouts: a batch closed again (every step of a benchmark, a
// serving arena) skips building its plan twice per call just to size the workspace.
struct WsEntry {
    int32_t dtype;
    int triangular;
    std::vector<int64_t> sizes;
    size_t bytes;
};
static std::mutex g_ws_mu;
static std::vector<WsEntry> g_ws_cache;

static size_t batch_workspace_uncached(int32_t dtype, int64_t count, const int64_t *sizes, uint32_t mode);

static size_t batch_workspace(int32_t dtype, int64_t count, const int64_t *sizes, uint32_t mode) {
    const int tri = (mode & RBG_MODE_TRIANGULAR) ? 1 : 0;
    {
        std::lock_guard<std::mutex> lk(g_ws_mu);
        for (const auto &e : g_ws_cache)
            if (e.dtype == dtype && e.triangular == tri && (int64_t)e.sizes.size() == count &&
                (count == 0 || memcmp(e.sizes.data(), sizes, (size_t)count * 8) == 0))
                return e.bytes;
    }
    const size_t b = batch_workspace_uncached(dtype, count, sizes, mode);
    std::lock_guard<std::mutex> lk(g_ws_mu);
    if (g_ws_cache.size() >= 4) g_ws_cache.erase(g_ws_cache.begin());
    g_ws_cache.push_back(WsEntry{dtype, tri, std::vector<int64_t>(sizes, sizes + count), b});
    return b;
}

static size_t batch_workspace_uncached(int32_t dtype, int64_t count, const int64_t *sizes, uint32_t mode) {
    std::vector<int64_t> off((size_t)count, 0);
    FwPlan P;
    build_plan(P, count, sizes, off.data(), off.data(), 4, (mode & RBG_MODE_TRIANGULAR) ? 1 : 0,
               TileCfg<uint32_t>::BN, dtype_bytes(dtype));
    int64_t maxn = 0;
    for (int64_t i = 0; i < count; ++i) maxn = std::max(maxn, sizes[i]);
    return std::max(P.total, single_workspace(maxn, dtype));
}

extern "C" int32_t rbg_fw_batch_workspace_bytes(int32_t dtype, int64_t count, const int64_t *sizes,
                                                uint32_t mode, int64_t *bytes) {
    if (!bytes || count < 0 || (count > 0 && !sizes) || dtype_bytes(dtype) == 0) return RBG_ERR_INVALID;
    for (int64_t i = 0; i < count; ++i)
        if (sizes[i] < 0) return RBG_ERR_INVALID;
    *bytes = (int64_t)batch_workspace(dtype, count, sizes, mode);
    return RBG_OK;
}

static int32_t fw_batch_entry(int32_t dtype, int64_t count, const int64_t *sizes, const int64_t *offsets,
                              const void *in, void *out, uint32_t mode, void *workspace, int64_t workspace_bytes,
                              rbg_result_t *results, rbg_stream_t stream, const RowStats &rs) {
    if (count < 0 || (count > 0 && (!sizes || !offsets || !in || !out || !workspace || !results)))
        return RBG_ERR_INVALID;
    if (dtype_bytes(dtype) == 0) return RBG_ERR_INVALID;
    if ((mode & RBG_MODE_CYTHON) && dtype != RBG_DTYPE_INT32) return RBG_ERR_INVALID;
    if (count == 0) return RBG_OK;
    for (int64_t i = 0; i < count; ++i)
        if (sizes[i] < 0 || offsets[i] < 0) return RBG_ERR_INVALID;
    if (workspace_bytes < (int64_t)batch_workspace(dtype, count, sizes, mode)) return RBG_ERR_NOMEM;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    unsigned char *ws = reinterpret_cast<unsigned char *>(workspace);
    int rc = RBG_ERR_INVALID;
    RBG_DISPATCH_DTYPE(dtype, T,
        rc = fw_batch_t<T>(count, sizes, offsets, reinterpret_cast<const T *>(in), reinterpret_cast<T *>(out),
                           mode, ws, (size_t)workspace_bytes, results, s, rs));
    return rc;
}

extern "C" int32_t rbg_fw_batch(int32_t dtype, int64_t count, const int64_t *sizes, const int64_t *offsets,
                                const void *in, void *out, uint32_t mode, void *workspace,
                                int64_t workspace_bytes, rbg_result_t *results, rbg_stream_t stream) {
    return fw_batch_entry(dtype, count, sizes, offsets, in, out, mode, workspace, workspace_bytes, results, stream,
                          RowStats());
}

extern "C" int32_t rbg_fw_batch_rows(int32_t dtype, int64_t count, const int64_t *sizes, const int64_t *offsets,
                                     const void *in, void *out, uint32_t mode, void *workspace,
                                     int64_t workspace_bytes, const rbg_row_stats_t *stats, rbg_result_t *results,
                                     rbg_stream_t stream) {
    if (!stats || !stats->row_base || !stats->row_count || dtype != RBG_DTYPE_INT32) return RBG_ERR_INVALID;
    RowStats rs;
    rs.row_base = stats->row_base;
    rs.row_id = stats->row_id;
    rs.row_count = stats->row_count;
    rs.chunk_mask = reinterpret_cast<unsigned long long *>(stats->chunk_mask);
    rs.comp_max = stats->comp_max;
    return fw_batch_entry(dtype, count, sizes, offsets, in, out, mode, workspace, workspace_bytes, results, stream,
                          rs);
}
