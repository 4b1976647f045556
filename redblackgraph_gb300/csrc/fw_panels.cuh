// fw_panels.cuh -- phases 1 and 2 of the snapshot-exact blocked Floyd-Warshall round.
// Included by fw_dense.cu (which defines FW_B, FW_P, lane<>, umin, flush_status, DevStatus).
//
// Phase 1 (fw_diag_kernel, one CTA per round): the 64 x 64 diagonal tile in sequential k order.
//   It writes the tile's end-of-round values and, into a round buffer, the snapshots
//       cs[t][a] = d_{t-1}(a, t)   (column t as step t reads it)
//       rs(t, b) = d_{t-1}(t, b)   (row t as step t reads it), stored split as (2^msb, low)
//   with per-step maxima of msb (for the exact top-bit test) and validity masks.
// Phase 2 (fw_panel_kernel, 64 panel columns or rows per CTA): each panel column (row panel) or
//   row (column panel) is held in registers by PN_LANES lanes and runs its forward substitution
//       P(a, j) <- P(a, j) (+) cs[t][a] (x) P(t, j)      (row panel, t = K0..K0+63)
//       P(i, b) <- P(i, b) (+) P(i, t) (x) rs(t, b)      (column panel)
//   storing the step-t operands P(t, j) / P(i, t) (the phase-3 snapshots) t-major.
#pragma once

constexpr int DG_THREADS = 256;   // phase 1: 4 threads per column, 16 rows each
constexpr int DG_ROWS = 16;

// Round buffer (global memory, written by phase 1, read by phase 2).
template <typename U> struct RoundBuf {
    U cs[FW_B][FW_B];                 // cs[t][a]
    U rsm[FW_B][FW_B];                // rsm[t][b] = 2^msb(rs(t,b)), 0 for zero
    U rsl[FW_B][FW_B];                // rsl[t][b] = rs(t,b) - 2^msb, inf for zero
    unsigned long long maskCS[FW_B];  // maskCS[a] bit t: cs[t][a] valid
    unsigned long long maskRS[FW_B];  // maskRS[b] bit t: rs(t,b) valid
    int msbCS[FW_B];                  // max msb over valid cs[t][.]
    int msbRS[FW_B];                  // max msb over valid rs(t, .)
};

template <typename U> __device__ __forceinline__ int msb_or_neg(U v) {
    return lane<U>::valid(v) ? msb_nz<U>(v) : -100000;
}

// Shared tables are read by four lane groups at element offsets 0, 16, 32, 48.  Padding each
// 16-element group by one 16-byte vector puts the four groups' vectors in distinct banks.
template <typename U> struct Pad {
    static constexpr int P = 16 / (int)sizeof(U);
    static constexpr int LD = FW_B + 4 * P;
    __device__ __forceinline__ static int at(int c) { return c + P * (c >> 4); }
};

// 16 consecutive lane words from 16-byte aligned shared memory
template <typename U> __device__ __forceinline__ void load16(const U *p, U (&x)[DG_ROWS]) {
    const uint4 *q = reinterpret_cast<const uint4 *>(p);
    constexpr int PER = 16 / sizeof(U);
#pragma unroll
    for (int i = 0; i < DG_ROWS / PER; ++i) {
        uint4 v = q[i];
        const U *w = reinterpret_cast<const U *>(&v);
#pragma unroll
        for (int k = 0; k < PER; ++k) x[i * PER + k] = w[k];
    }
}

// ------------------------------------------------------------------------------ phase 1
template <typename U> struct DiagSmem {
    U CS[FW_B][Pad<U>::LD];           // CS[t][Pad::at(a)]
    U Y[FW_B][FW_B];                  // Y[t][b] = rs(t, b)
    typename signed_of<U>::type colmax[FW_B][DG_THREADS / FW_B];
};

// Thread (b = tid % 64, h = tid / 64) holds rows a = 16 h + l (l = 0..15) of column b.  Steps
// run in blocks of 16, fully unrolled, so the row of step t is the static register R[t % 16]
// of the threads with h = t / 16.  One barrier per step: step t's writes go to slot t only.
template <typename U>
__global__ void __launch_bounds__(DG_THREADS)
fw_diag_kernel(U *__restrict__ work_base, unsigned long long *__restrict__ any_base, RoundBuf<U> *__restrict__ rbs,
               const FwComp *__restrict__ comps, int *__restrict__ counters, int64_t K0, int lbits,
               DevStatus *st_base) {
    typedef lane<U> L;
    typedef typename signed_of<U>::type SU;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    DiagSmem<U> &S = *reinterpret_cast<DiagSmem<U> *>(smem_raw);
    const int tid = threadIdx.x;
    const FwComp cmp = comps[blockIdx.x];             // one CTA per active component
    U *work = work_base + cmp.work_off;
    const int64_t np = cmp.np;
    RoundBuf<U> *rb = rbs + cmp.rb_index;
    DevStatus *st = st_base + cmp.status_index;
    if (tid == 0) atomicAdd(&st->executed, (unsigned long long)FW_B * FW_B * FW_B);
    for (int e = tid; e < 2 * (int)(np / FW_B); e += DG_THREADS) any_base[cmp.any_off + e] = 0;
    if (blockIdx.x == 0 && tid < 4) counters[tid] = 0;   // this round's worklists start empty
    const int b = tid % FW_B, h = tid / FW_B;
    U R[DG_ROWS];
#pragma unroll
    for (int l = 0; l < DG_ROWS; ++l) R[l] = work[(K0 + h * DG_ROWS + l) * np + K0 + b];
    bool risk = false;
    SU pm[4] = {0, 0, 0, 0};
    for (int T = 0; T < FW_B / DG_ROWS; ++T) {
#pragma unroll
        for (int l = 0; l < DG_ROWS; ++l) {
            const int t = T * DG_ROWS + l;
            if (b == t) {   // publish column t (invariant during step t)
                SU cm = -1;
#pragma unroll
                for (int r = 0; r < DG_ROWS; ++r) {
                    S.CS[t][Pad<U>::at(h * DG_ROWS) + r] = R[r];
                    cm = max(cm, (SU)R[r]);
                }
                S.colmax[t][h] = cm;
            }
            if (h == T) S.Y[t][b] = R[l];   // row t (invariant during step t)
            __syncthreads();
            const U y = S.Y[t][b];
            U m, low;
            L::split(y, m, low);
            SU cm = max(max(S.colmax[t][0], S.colmax[t][1]), max(S.colmax[t][2], S.colmax[t][3]));
            if (L::valid(y) && cm > 0 && msb_nz<U>((U)cm) + msb_nz<U>(y) >= lbits - 1) risk = true;
            U x[DG_ROWS];
            load16<U>(&S.CS[t][Pad<U>::at(h * DG_ROWS)], x);
#pragma unroll
            for (int r = 0; r < DG_ROWS; ++r) {
                const U v = umin(R[r], x[r] * m + low);
                R[r] = v;
                pm[r & 3] = max(pm[r & 3], (SU)v);
            }
        }
    }
    // end-of-round tile; a valid diagonal cell means a cycle
    bool cyc = false;
#pragma unroll
    for (int r = 0; r < DG_ROWS; ++r) {
        const int a = h * DG_ROWS + r;
        U v = R[r];
        if (a == b) {
            cyc |= L::valid(v);
            v = L::inf;
        }
        work[(K0 + a) * np + K0 + b] = L::valid(v) ? v : L::inf;
    }
    __syncthreads();
    // round buffer: snapshots, splits, masks and per-step maxima
    for (int e = tid; e < FW_B * FW_B; e += DG_THREADS) {
        const int t = e / FW_B, c = e % FW_B;
        const U x = S.CS[t][Pad<U>::at(c)];
        rb->cs[t][c] = L::valid(x) ? x : L::inf;
        U m, low;
        L::split(S.Y[t][c], m, low);
        rb->rsm[t][c] = m;
        rb->rsl[t][c] = low;
    }
    if (tid < FW_B) {
        unsigned long long mc = 0, mr = 0;
        int bc = -100000, br = -100000;
        for (int t = 0; t < FW_B; ++t) {
            const U x = S.CS[t][Pad<U>::at(tid)], y = S.Y[t][tid];
            mc |= (unsigned long long)L::valid(x) << t;
            mr |= (unsigned long long)L::valid(y) << t;
            bc = max(bc, msb_or_neg<U>(S.CS[tid][Pad<U>::at(t)]));   // step tid's maximum
            br = max(br, msb_or_neg<U>(S.Y[tid][t]));
        }
        rb->maskCS[tid] = mc;
        rb->maskRS[tid] = mr;
        rb->msbCS[tid] = bc;
        rb->msbRS[tid] = br;
    }
    SU smx = max(max(pm[0], pm[1]), max(pm[2], pm[3]));
    unsigned flags = (risk ? RBG_EV_RISK : 0u) | (cyc ? RBG_EV_CYCLE : 0u);
    flush_status(st, smx > 0 ? (unsigned long long)smx : 0ull, flags);
}

// ------------------------------------------------------------------------------ phase 2
// PN_LANES lanes of a warp share one panel column (row panel) or row (column panel),
// PN_CELLS cells each.  The step-t operand P(t, j) / P(i, t) lives in lane h = t / PN_CELLS of
// the group and is broadcast with a shuffle, so the 64 steps need no barrier.  Steps run in
// fully unrolled blocks of PN_CELLS, keeping every register index static.
constexpr int PN_LINES = 64;                      // panel columns / rows per CTA
constexpr int PN_CELLS = 16;                      // cells of a line held by one lane
constexpr int PN_LANES = FW_B / PN_CELLS;         // lanes per line
constexpr int PN_THREADS = PN_LINES * PN_LANES;

// N consecutive lane words from 16-byte aligned memory
template <typename U, int N> __device__ __forceinline__ void loadN(const U *p, U (&x)[N]) {
    const uint4 *q = reinterpret_cast<const uint4 *>(p);
    constexpr int PER = 16 / sizeof(U);
#pragma unroll
    for (int i = 0; i < N / PER; ++i) {
        uint4 v = q[i];
        const U *w = reinterpret_cast<const U *>(&v);
#pragma unroll
        for (int k = 0; k < PER; ++k) x[i * PER + k] = w[k];
    }
}

template <typename U> struct PanelSmem {
    U TA[FW_B][Pad<U>::LD];           // row panel: cs[t][a]; column panel: rsm[t][b] (padded)
    U RSl[FW_B][Pad<U>::LD];          //               rsl[t][b]   (padded)
    unsigned long long maskCS[FW_B];
    unsigned long long maskRS[FW_B];
    int msbCS[FW_B];
    int msbRS[FW_B];
    U Z[FW_B][PN_LINES];              // Z[t][line]: the line's step-t operand (its snapshot)
    unsigned long long any;           // OR of the item's line masks
};

template <typename U> __device__ __forceinline__ U shfl_lane(U v, int src) {
    if (sizeof(U) == 8) {
        unsigned long long x = (unsigned long long)v;
        return (U)__shfl_sync(0xffffffffu, x, src);
    }
    return (U)__shfl_sync(0xffffffffu, (unsigned)v, src);
}

// One panel item: 64 lines (a 64 x 64 block) of component ci's row panel (local < np / 64)
// or column panel.
template <typename U>
__device__ __forceinline__ void panel_item(PanelSmem<U> &S, int ci, int local, U *__restrict__ work_base,
                                           unsigned long long *__restrict__ any_base,
                                           unsigned char *__restrict__ occ_base,
                                           const RoundBuf<U> *__restrict__ rbs,
                                           const FwComp *__restrict__ comps, int64_t K0, int lbits,
                                           DevStatus *st_base) {
    typedef lane<U> L;
    typedef typename signed_of<U>::type SU;
    const int tid = threadIdx.x;
    const FwComp cmp = comps[ci];
    const int64_t np = cmp.np;
    U *work = work_base + cmp.work_off;
    U *cpbuf = work_base + cmp.cp_off;
    U *rpbuf = work_base + cmp.rp_off;
    unsigned long long *anyCP = any_base + cmp.any_off;   // group masks, per 64-line group
    unsigned long long *anyRP = anyCP + np / FW_B;
    unsigned long long *lineCP = anyRP + np / FW_B;        // line masks (bit t: snapshot valid)
    unsigned long long *lineRP = lineCP + np;
    unsigned char *occ = occ_base + cmp.occ_off;     // (np/64)^2 block occupancy
    const int nb = (int)(np / FW_B);
    const RoundBuf<U> *rb = rbs + cmp.rb_index;
    DevStatus *st = st_base + cmp.status_index;
    const int nct = (int)(np / PN_LINES);             // items per panel
    const bool rowPanel = local < nct;
    const int cta = rowPanel ? local : local - nct;

    const int lanei = tid & 31;
    const int h = lanei & (PN_LANES - 1);             // cells h*PN_CELLS .. of the line
    const int grp = lanei & ~(PN_LANES - 1);          // first lane of this line's group
    const int line = tid / PN_LANES;
    const int64_t g = (int64_t)cta * PN_LINES + line; // global column / row
    const bool inK = g >= K0 && g < K0 + FW_B;        // the diagonal tile's own cells
    const int c0 = h * PN_CELLS;
    constexpr unsigned ALL_INF = (1u << PN_CELLS) - 1u;
    bool risk = false;
    unsigned steps_done = 0;                          // steps this warp did not skip
    unsigned long long seen = 0;                      // bit t: the step-t operand is valid
    unsigned startInf = 0;                            // bit r: cell r was zero at round start
    U R[PN_CELLS];
    U *rowp = work + g * np + K0 + c0;                // column panel: this thread's cells
    if (inK) {
#pragma unroll
        for (int r = 0; r < PN_CELLS; ++r) R[r] = L::inf;
    } else if (rowPanel) {
#pragma unroll
        for (int r = 0; r < PN_CELLS; ++r) R[r] = work[(K0 + c0 + r) * np + g];
    } else {
        loadN<U, PN_CELLS>(rowp, R);   // 16-byte aligned: K0 and c0 are multiples of 8 words
    }
#pragma unroll
    for (int r = 0; r < PN_CELLS; ++r) startInf |= (unsigned)(!L::valid(R[r])) << r;
    // the pivot tables are loaded before the all-zero test so that both loads are in flight
    // together (batched 16-byte loads; the shared-memory stores follow the test)
    constexpr int PER = 16 / sizeof(U);
    constexpr int NV = FW_B * FW_B / PER / PN_THREADS;   // vectors per table per thread
    uint4 va[NV], vb[NV];
    unsigned long long mcs = 0, mrs = 0;
    int bcs = 0, brs = 0;
    if (tid < FW_B) {
        mcs = rb->maskCS[tid];
        mrs = rb->maskRS[tid];
        bcs = rb->msbCS[tid];
        brs = rb->msbRS[tid];
    }
    {
        const uint4 *ta = reinterpret_cast<const uint4 *>(rowPanel ? &rb->cs[0][0] : &rb->rsm[0][0]);
        const uint4 *tb = reinterpret_cast<const uint4 *>(&rb->rsl[0][0]);
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            va[i] = ta[tid + i * PN_THREADS];
            if (!rowPanel) vb[i] = tb[tid + i * PN_THREADS];
        }
    }
    // 64 lines that are all zero stay zero this round: no snapshots, no write-back, and the
    // group flag stays 0 so the tile kernel reads none of them
    if (!__syncthreads_or(startInf != ALL_INF)) return;

    if (tid == 0) S.any = 0;
    {
        U *da = &S.TA[0][0];
        U *db = &S.RSl[0][0];
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            const int e = (tid + i * PN_THREADS) * PER, t = e / FW_B, c = e % FW_B;
            const int o = t * Pad<U>::LD + Pad<U>::at(c);
            *reinterpret_cast<uint4 *>(da + o) = va[i];
            if (!rowPanel) *reinterpret_cast<uint4 *>(db + o) = vb[i];
        }
    }
    if (tid < FW_B) {
        S.maskCS[tid] = mcs;
        S.maskRS[tid] = mrs;
        S.msbCS[tid] = bcs;
        S.msbRS[tid] = brs;
    }
    __syncthreads();

    const int pc0 = Pad<U>::at(c0);
    const U *tabA = &S.TA[0][pc0];
    const U *tabB = &S.RSl[0][pc0];
    bool changed = false;                             // some cell of this thread decreased
    if (__all_sync(0xffffffffu, startInf == ALL_INF)) {
        // the warp's lines are all zero: they stay zero (a line only meets its own cells as
        // step operands), so only their snapshots are written, as zeros
#pragma unroll
        for (int l = 0; l < PN_CELLS; ++l) S.Z[h * PN_CELLS + l][line] = L::inf;
    } else {
        for (int T = 0; T < PN_LANES; ++T) {
            // the step operands of block T are lane T's cells; if they are all zero for every
            // line of the warp at the block's start, no step of the block updates anything (an
            // update needs a valid step operand), so they stay zero: skip the block
            bool mine = false;
            if (h == T) {
#pragma unroll
                for (int r = 0; r < PN_CELLS; ++r) mine |= L::valid(R[r]);
            }
            if (!__any_sync(0xffffffffu, mine)) {
                if (h == T) {
#pragma unroll
                    for (int l = 0; l < PN_CELLS; ++l) S.Z[T * PN_CELLS + l][line] = R[l];
                }
                continue;
            }
#pragma unroll
            for (int l = 0; l < PN_CELLS; ++l) {
                const int t = T * PN_CELLS + l;
                const U z = shfl_lane<U>(R[l], grp | T);  // P(t, j) or P(i, t): invariant at step t
                const bool zv = L::valid(z);
                seen |= (unsigned long long)zv << t;
                if (h == 0) S.Z[t][line] = z;
                // a zero step operand makes every product of the step a zero: skip the step when
                // it is zero for the whole warp (closures of family trees are sparse); operands
                // are read only for the steps that run
                if (!__any_sync(0xffffffffu, zv)) continue;
                ++steps_done;
                U xa[PN_CELLS];
                loadN<U, PN_CELLS>(tabA + t * Pad<U>::LD, xa);
                if (rowPanel) {
                    U m, low;
                    L::split(z, m, low);
                    if (zv && S.msbCS[t] + msb_nz<U>(z) >= lbits - 1) risk = true;
#pragma unroll
                    for (int r = 0; r < PN_CELLS; ++r) {
                        const U v = umin(R[r], xa[r] * m + low);
                        changed |= v != R[r];
                        R[r] = v;
                    }
                } else {
                    U xb[PN_CELLS];
                    loadN<U, PN_CELLS>(tabB + t * Pad<U>::LD, xb);
                    if (zv && msb_nz<U>(z) + S.msbRS[t] >= lbits - 1) risk = true;
#pragma unroll
                    for (int r = 0; r < PN_CELLS; ++r) {
                        const U v = umin(R[r], z * xa[r] + xb[r]);
                        changed |= v != R[r];
                        R[r] = v;
                    }
                }
            }
        }
    }
    if (seen && h == 0) atomicOr(&S.any, seen);
    __syncthreads();   // the snapshots (written by lane h == 0 of each group) and S.any are visible
    const unsigned long long anyMask = S.any;
    {
        // t-major, coalesced over the CTA's lines; only the steps some line of this group has
        // valid are written (the tile kernel reads a snapshot row only under its mask bit), and
        // an invalid operand is written as the encoded zero, so that the tile kernel can copy the
        // rows into shared memory as they are
        U *dst = rowPanel ? rpbuf : cpbuf;
        const int64_t base = (int64_t)cta * PN_LINES;
        for (int e = tid; e < FW_B * PN_LINES; e += PN_THREADS) {
            const int t = e / PN_LINES;
            if ((anyMask >> t) & 1ull) {
                const U z = S.Z[t][e % PN_LINES];
                dst[(int64_t)t * np + base + e % PN_LINES] = L::valid(z) ? z : L::inf;
            }
        }
    }
    // write back the cells that changed; the running maximum needs each newly valid cell's
    // first valid product
    SU smx = 0;
    bool wrote = false;
#pragma unroll
    for (int r = 0; r < PN_CELLS; ++r) {
        const U v = R[r];
        const bool vv = L::valid(v);
        const int c = c0 + r;
        if (!inK && changed) {
            if (rowPanel) work[(K0 + c) * np + g] = vv ? v : L::inf;
            else rowp[r] = vv ? v : L::inf;
            wrote |= vv;
        }
        if (vv && ((startInf >> r) & 1u)) {
            const unsigned long long both = seen & (rowPanel ? S.maskCS[c] : S.maskRS[c]);
            const int tf = __ffsll((long long)both) - 1;
            U first;
            const U zf = S.Z[tf][line];
            if (rowPanel) {
                U m, low;
                L::split(zf, m, low);
                first = S.TA[tf][Pad<U>::at(c)] * m + low;
            } else {
                first = zf * S.TA[tf][Pad<U>::at(c)] + S.RSl[tf][Pad<U>::at(c)];
            }
            smx = max(smx, (SU)first);
        }
    }
    if ((tid & 31) == 0 && steps_done)
        atomicAdd(&st->executed, (unsigned long long)steps_done * 32 * PN_CELLS);
    if (h == 0) (rowPanel ? lineRP : lineCP)[g] = seen;
    if (tid == 0) (rowPanel ? anyRP : anyCP)[cta] = anyMask;
    if (wrote) {
        const int kb = (int)(K0 / FW_B);
        occ[rowPanel ? (int64_t)kb * nb + cta : (int64_t)cta * nb + kb] = 1;
    }
    flush_status(st, smx > 0 ? (unsigned long long)smx : 0ull, risk ? RBG_EV_RISK : 0u);
}

// Work counters of a round: [0] panel items, [1] panel cursor, [2] tile items, [3] tile cursor.
// Reset by the diagonal kernel at the start of every round.
constexpr int CNT_PANEL = 0, CUR_PANEL = 1, CNT_TILE = 2, CUR_TILE = 3;

// Panel worklist: candidate c of this round's panel prefix -> item if its 64 x 64 block of the
// work matrix holds a nonzero (a zero block stays zero and needs no forward substitution).
__global__ void fw_panel_list_kernel(const FwComp *__restrict__ comps, const int64_t *__restrict__ prefix,
                                     int count, int64_t K0, const unsigned char *__restrict__ occ_base,
                                     int2 *__restrict__ list, int *__restrict__ counters) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= prefix[count]) return;
    const int ci = fw_find(prefix, count, c);
    const FwComp cmp = comps[ci];
    const int local = (int)(c - prefix[ci]);
    const int nb = (int)(cmp.np / FW_B);
    const bool rowPanel = local < nb;
    const int grp = rowPanel ? local : local - nb;
    const int kb = (int)(K0 / FW_B);
    if (grp == kb) return;                           // the diagonal block itself
    const unsigned char *occ = occ_base + cmp.occ_off;
    if (!occ[rowPanel ? (int64_t)kb * nb + grp : (int64_t)grp * nb + kb]) return;
    const int slot = atomicAdd(&counters[CNT_PANEL], 1);
    list[slot] = make_int2(ci, local);
}

// Persistent panel kernel: CTAs pull items from the worklist until it is exhausted.
template <typename U>
__global__ void __launch_bounds__(PN_THREADS, 2)
fw_panel_kernel(U *__restrict__ work_base, unsigned long long *__restrict__ any_base,
                unsigned char *__restrict__ occ_base,
                const RoundBuf<U> *__restrict__ rbs, const FwComp *__restrict__ comps,
                const int2 *__restrict__ list, int *__restrict__ counters, int64_t K0, int lbits,
                DevStatus *st_base) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    PanelSmem<U> &S = *reinterpret_cast<PanelSmem<U> *>(smem_raw);
    __shared__ int s_item;
    const int total = counters[CNT_PANEL];
    if (threadIdx.x == 0) s_item = atomicAdd(&counters[CUR_PANEL], 1);
    __syncthreads();
    int i = s_item;
    while (i < total) {
        // the next item is claimed now and published after this one (its round trip overlaps
        // the item); panel_item's first barrier precedes its first shared-memory write
        int nxt = 0;
        if (threadIdx.x == 0) nxt = atomicAdd(&counters[CUR_PANEL], 1);
        const int2 e = list[i];
        panel_item<U>(S, e.x, e.y, work_base, any_base, occ_base, rbs, comps, K0, lbits, st_base);
        if (threadIdx.x == 0) s_item = nxt;
        __syncthreads();
        i = s_item;
    }
}
