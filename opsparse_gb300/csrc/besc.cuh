// besc.cuh — CTA-per-row expand / bitonic sort / compress for the numeric phase of rows
// of up to 4,096 products (E1 rows with many outputs, E2 rows of the mid shape).  Replaces OpSparse's shared-hash
// kernels of its middle and large bins (kernels/symbolic.cuh:74-261,
// kernels/numeric.cuh:109-302) for those rows.
//
// Per row:
//   1. scan the lengths of the B rows selected by A's row (shared memory);
//   2. expand every product p into a key: numeric (column << kIdBits) | p, symbolic the
//      bare column; numeric also records the product's A entry (own[p]);
//   3. sort the keys with a bitonic network over the whole CTA: each thread holds PER
//      consecutive keys in registers; partners within a thread are exchanged in
//      registers, within a warp by shuffles, across warps through shared memory.
//      Packed product indices make equal columns sort in ascending product order
//      (= ascending j), so no stable sort is needed;
//   4. symbolic: count the distinct columns;  numeric: number the runs of equal columns
//      (block scan of run heads) and fold each run in order with one FMA per product —
//      the oracle's sequence, bit for bit — writing C in column order.
// PER is chosen per row (the smallest power-of-two network that holds it), so a row pays
// for a network of at most twice its size.  All loops run to block-uniform bounds.
//
// Shapes with kRank replace steps 3-4 of the numeric phase, for rows whose columns span
// fewer than kRankWinBits columns, by a column-window rank (besc_rank_fold): no sort at
// all.  Each product sets its column's bit in a window bitmap with a shared-memory OR; the
// OR's old value tells a product whose column an earlier OR already set ("late").  The
// prefix popcounts of the window's words give every column its position in C's row.  The
// column's first product (the one whose OR set the bit) folds itself and stores the entry
// at that position; a late product stores its operands in a list keyed (position,
// product).  The listed keys are sorted in one warp and each column with late products is
// re-folded in ascending product order with its first product merged in, so every entry
// is still the oracle's fold, bit for bit.  A row with more late products than the list
// holds takes the sort.
#pragma once

#include <type_traits>

#include "esc.cuh"

namespace opsg {

constexpr int kRankWinBits = 65536;              // columns a rank-path row may span
constexpr int kRankWords = kRankWinBits / 32;     // window bitmap words
constexpr int kRankChunk = 128;                   // bitmap words per warp step of the prefix sweep
constexpr int kRankLateMax = 128;                 // late products listed for the re-fold
static_assert(kRankWords % kRankChunk == 0, "whole chunks");

template <int NT, int PMAX, int ACAP, int MINB, bool RANK = false>
struct BescShape {
    static constexpr int kThreads = NT;
    static constexpr int kMinBlocks = MINB;             // CTAs per SM the registers must allow
    static constexpr int kWarps = NT / 32;
    static constexpr int kPMax = PMAX;
    static constexpr int kCap = NT * PMAX;              // products per row, at most
    static constexpr int kAEntries = ACAP;              // A entries per row, at most
    static constexpr int kIdBits = ceil_log2_c(kCap);   // bits of a product index
    static constexpr int kPadSlots = kCap + kCap / 32;  // keys with one pad slot per 32
    static constexpr bool kRank = RANK;                 // numeric rows may take the rank path
    static_assert(!RANK || (PMAX % kUnroll == 0 && PMAX <= 32 && 2 * kIdBits <= 32), "rank-path layout");

    static constexpr size_t up16(size_t x) { return (x + 15) / 16 * 16; }
    static constexpr size_t cmax(size_t a, size_t b) { return a > b ? a : b; }
    // [keys (sort exchange) | product ids + run heads (fold) | rank path: entry by
    //  position, aliased] [own] [rank path: first product by position, window bitmap, word
    //  prefixes, late list and its operands] [scan]
    template <bool kNum, typename KT, typename T>
    static constexpr size_t region0()
    {
        return cmax(cmax(up16(sizeof(KT) * kPadSlots), kNum ? up16(2 * (size_t)kCap + 4 * ((size_t)kCap + 1)) : 0),
                    kNum && RANK ? up16(sizeof(T) * (size_t)kCap) + up16(4 * (size_t)kCap) : 0);
    }
    template <typename T>
    static constexpr size_t rank_region()
    {
        return up16(2 * (size_t)kCap) + 4 * (size_t)kRankWords + 2 * (size_t)kRankWords +
               (4 + 2 * sizeof(T)) * (size_t)kRankLateMax;
    }
    template <bool kNum, typename KT, typename T>
    static constexpr size_t smem()
    {
        return region0<kNum, KT, T>() + (kNum ? up16(2 * (size_t)kCap) : 0) +
               (kNum && RANK ? rank_region<T>() : 0) + 8 * (size_t)ACAP;
    }
};

using BescE1 = BescShape<128, 8, 1024, 6, true>;        // E1 rows of more than kSplitNnz outputs
using BescE1Sort = BescShape<128, 8, 1024, 6>;          // the same rows where B is wider than the window
using BescE1Batch = BescShape<128, 8, 480, 7, true>;    // the batch's rows of 513 to 1,024 products
using BescMid = BescShape<256, 16, 1280, 4>;            // E2 rows of at most 4,096 products
using BescMidRank = BescShape<256, 16, 1280, 3, true>;  // the batch's rows of 1,025 to 4,096 products

// Block-shared scratch of the besc routine.  reset() by one thread before the first row;
// besc_row leaves it reset on return.
struct BescScratch {
    unsigned bad;   // a B column outside [0, N) was seen
    unsigned cmin;  // the row's column window (rank path): the smallest first column and the
    unsigned cmax;  // largest last column of its B rows
    int late;       // late products of the row
    int listed;     // late products listed so far (rank path)
    int n;          // the row's products (rank path's scan)
    unsigned wbad;  // a product outside the window (unsorted B row): the row takes the sort
    __device__ __forceinline__ void reset()
    {
        bad = 0u;
        cmin = 0xffffffffu;
        cmax = 0u;
        late = 0;
        listed = 0;
        n = 0;
        wbad = 0u;
    }
};

__device__ __forceinline__ int bpad(int e) { return e + (e >> 5); }

// Ascending bitonic sort of NT*PER keys, thread t holding elements t*PER .. t*PER+PER-1.
// `buf` (NT*PER padded slots) carries the exchanges between warps.
template <int NT, int PER, typename KT>
__device__ __forceinline__ void block_bitonic(KT (&x)[PER], KT *buf)
{
    const int tid = threadIdx.x;
    constexpr int n = NT * PER;
    constexpr int kWarpSpan = 32 * PER;
#pragma unroll
    for (int k = 2; k <= PER; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
#pragma unroll
            for (int i = 0; i < PER; ++i) {
                if ((i & j) == 0) {
                    const bool asc = ((tid * PER + i) & k) == 0;
                    const KT a = x[i], b = x[i | j];
                    const bool sw = asc ? (b < a) : (a < b);
                    x[i] = sw ? b : a;
                    x[i | j] = sw ? a : b;
                }
            }
        }
    }
#pragma unroll 1
    for (int k = 2 * PER; k <= n; k <<= 1) {
        const bool asc = ((tid * PER) & k) == 0;
#pragma unroll 1
        for (int j = k >> 1; j >= PER; j >>= 1) {
            const bool take_min = (((tid * PER) & j) == 0) == asc;
            if (j >= kWarpSpan) {  // partner thread in another warp
#pragma unroll
                for (int i = 0; i < PER; ++i) buf[bpad(tid * PER + i)] = x[i];
                __syncthreads();
                const int pt = tid ^ (j / PER);
#pragma unroll
                for (int i = 0; i < PER; ++i) {
                    const KT y = buf[bpad(pt * PER + i)];
                    x[i] = take_min ? (x[i] < y ? x[i] : y) : (x[i] < y ? y : x[i]);
                }
                __syncthreads();
            } else {
#pragma unroll
                for (int i = 0; i < PER; ++i) {
                    const KT y = __shfl_xor_sync(kFull, x[i], j / PER);
                    x[i] = take_min ? (x[i] < y ? x[i] : y) : (x[i] < y ? y : x[i]);
                }
            }
        }
#pragma unroll
        for (int j = PER / 2; j > 0; j >>= 1) {
#pragma unroll
            for (int i = 0; i < PER; ++i) {
                if ((i & j) == 0) {
                    const KT a = x[i], b = x[i | j];
                    const bool sw = asc ? (b < a) : (a < b);
                    x[i] = sw ? b : a;
                    x[i | j] = sw ? a : b;
                }
            }
        }
    }
}

// Sort the row's n keys (in skeys, padded) and count (symbolic) or fold and write
// (numeric).  Returns the number of distinct columns (block-uniform).
template <typename Shape, int PER, int kIdBits, bool kNum, typename T, typename KT>
__device__ __forceinline__ int besc_sort_fold(const SpgemmArgs<T> &g, int n, int a0, KT *skeys, unsigned short *spid,
                                              int *hidx, const unsigned short *own, const int *s_incl,
                                              const int *s_b0, int off, int n_expect, int *s_warp_sums, KT *s_last)
{
    using AccT = Acc<T>;
    using S = typename AccT::S;
    constexpr int NT = Shape::kThreads;
    const int tid = threadIdx.x;
    const int lane = lane_id();
    const int warp = tid >> 5;
    KT x[PER];
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid * PER + i;
        x[i] = e < n ? skeys[bpad(e)] : ~KT(0);
    }
    __syncthreads();  // skeys is the exchange buffer from here on
    block_bitonic<NT, PER, KT>(x, skeys);
    // run heads: element e starts a run if its column differs from element e-1's
    KT before = __shfl_up_sync(kFull, x[PER - 1], 1);
    if (lane == 31) s_last[warp] = x[PER - 1];
    __syncthreads();
    if (lane == 0) before = warp ? s_last[warp - 1] : KT(0);
    unsigned hm = 0;
    int h = 0;
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid * PER + i;
        const KT prev = i ? x[i - 1] : before;
        const bool head = e < n && (e == 0 || (x[i] >> kIdBits) != (prev >> kIdBits));
        hm |= head ? (1u << i) : 0u;
        h += head ? 1 : 0;
    }
    int total = 0;
    const int incl = block_inclusive_scan(h, s_warp_sums, &total);
    if constexpr (kNum) {
        // product ids in sorted order and the element index of every run head, written
        // over the (now free) key buffer
        constexpr KT kIdMask = (KT(1) << kIdBits) - 1;
        int pos = incl - h;
#pragma unroll
        for (int i = 0; i < PER; ++i) {
            const int e = tid * PER + i;
            if (e < n) spid[e] = (unsigned short)(x[i] & kIdMask);
            if ((hm >> i) & 1u) hidx[pos++] = e;
        }
        if (tid == 0) hidx[total] = n;
        __syncthreads();
        if (tid == 0 && !g.soff && total != n_expect) atomicOr(&g.info->flags, kErrCountMismatch);
        // runs in head order (thread tid takes runs tid, tid + NT, ...: consecutive threads
        // write consecutive entries of C), each thread walking its runs one product per
        // step with the operands of kFoldUnroll steps loaded together: a warp issues about
        // as many FP64 FMAs as its busiest lane has products, where a fixed kUnroll-wide
        // fold per run issued kUnroll FMAs for a run of one product
        const int K = tid < total ? (total - tid + NT - 1) / NT : 0;
        fold_own_runs<T>(
            0, K, INT_MAX, [&](int k) { return hidx[tid + k * NT]; }, [&](int k) { return hidx[tid + k * NT + 1]; },
            [&](int t, T &a, T &b, int &kb) {
                const int q = spid[t];
                const int o = own[q];
                kb = s_b0[o] + q - (o ? s_incl[o - 1] : 0);
                a = __ldg(g.aval + a0 + o);
                b = __ldg(g.bval + kb);
            },
            [&](int k, int, int kb, S s) {
                const int hh = tid + k * NT;
                if (hh < n_expect) {
                    g.c_col[off + hh] = __ldg(g.bcol + kb);
                    g.c_val[off + hh] = AccT::fin(s);
                }
            });
    }
    return total;
}

// Shared memory of one CTA of the besc routine: [keys | ids + heads | entry by position]
// [own] [rank path: first product by position, window bitmap, word prefixes,
// late list and its operands] [scan].
template <typename Shape, bool kNum, typename KT, typename T>
struct BescSmem {
    KT *skeys;
    unsigned short *spid;
    int *hidx;
    T *rval;                 // rank path, by position: the entry's value and column
    int *rcol;
    unsigned short *own;
    unsigned short *rfirst;  // rank path, by position: the first product
    unsigned *bm;            // rank path: window bitmap, all zero between rows
    unsigned short *wpre;    // rank path: set bits before each bitmap word
    unsigned *late_list;     // rank path: late products, (position, product, slot) keys
    T *la;                   // rank path: late products' operands by slot
    T *lb;
    int *s_incl;
    int *s_b0;
    __device__ __forceinline__ explicit BescSmem(unsigned char *p)
    {
        skeys = reinterpret_cast<KT *>(p);
        spid = reinterpret_cast<unsigned short *>(p);
        hidx = reinterpret_cast<int *>(p + Shape::up16(2 * (size_t)Shape::kCap));
        rval = reinterpret_cast<T *>(p);
        rcol = reinterpret_cast<int *>(p + Shape::up16(sizeof(T) * (size_t)Shape::kCap));
        p += Shape::template region0<kNum, KT, T>();
        own = nullptr;
        rfirst = nullptr;
        bm = nullptr;
        wpre = nullptr;
        late_list = nullptr;
        la = lb = nullptr;
        if constexpr (kNum) {
            own = reinterpret_cast<unsigned short *>(p);
            p += Shape::up16(2 * (size_t)Shape::kCap);
            if constexpr (Shape::kRank) {
                rfirst = reinterpret_cast<unsigned short *>(p);
                p += Shape::up16(2 * (size_t)Shape::kCap);
                bm = reinterpret_cast<unsigned *>(p);
                p += 4 * (size_t)kRankWords;
                wpre = reinterpret_cast<unsigned short *>(p);
                p += 2 * (size_t)kRankWords;
                la = reinterpret_cast<T *>(p);
                p += sizeof(T) * (size_t)kRankLateMax;
                lb = reinterpret_cast<T *>(p);
                p += sizeof(T) * (size_t)kRankLateMax;
                late_list = reinterpret_cast<unsigned *>(p);
                p += 4 * (size_t)kRankLateMax;
            }
        }
        s_incl = reinterpret_cast<int *>(p);
        s_b0 = s_incl + Shape::kAEntries;
    }
    // Clears the window bitmap; every thread calls it before the first row, and a barrier
    // separates it from the row.
    __device__ __forceinline__ void init() const
    {
        if constexpr (kNum && Shape::kRank) {
            uint4 *bm4 = reinterpret_cast<uint4 *>(bm);
            for (int i = threadIdx.x; i < kRankWords / 4; i += Shape::kThreads) bm4[i] = make_uint4(0u, 0u, 0u, 0u);
        }
    }
};

// Key of a late product in the rank path's list: position, product, list slot (the slot
// rides below the product index; it only locates the operands).
constexpr int kRankSlotBits = 7;
static_assert((1 << kRankSlotBits) >= kRankLateMax, "slot field");

// Operands of product q of a row (A entry own[q], B position from the row's scan).
template <typename T, typename SM>
__device__ __forceinline__ void besc_operands(const SpgemmArgs<T> &g, int a0, const SM &sm, int q, T &a, T &b)
{
    const int o = sm.own[q];
    const int kb = sm.s_b0[o] + q - (o ? sm.s_incl[o - 1] : 0);
    a = __ldg(g.aval + a0 + o);
    b = __ldg(g.bval + kb);
}

// Re-fold of the columns with late products (n_late listed, at most kRankLateMax).  Warp 0
// sorts the list; then thread e takes listed key e, and where it heads its position's run
// folds the run merged with the column's first product (its operands reloaded), in
// ascending product order, the late products' operands read from shared memory.
// Block-uniform; every thread calls it.
template <int kIdBits, typename T, typename SM>
__device__ __forceinline__ void besc_rank_refold(const SpgemmArgs<T> &g, int a0, const SM &sm, int n_late)
{
    using AccT = Acc<T>;
    using S = typename AccT::S;
    constexpr int kPosShift = kIdBits + kRankSlotBits;
    constexpr unsigned kSlotMask = (1u << kRankSlotBits) - 1u;
    const int tid = threadIdx.x;
    const int lane = lane_id();
    if (tid < 32) {
        auto sort_list = [&](auto per_tag) {
            constexpr int PER = decltype(per_tag)::value;
            unsigned x[PER];
#pragma unroll
            for (int i = 0; i < PER; ++i) {
                const int e = lane * PER + i;
                x[i] = e < n_late ? sm.late_list[e] : 0xffffffffu;
            }
            warp_bitonic_blocked<PER, unsigned>(x);
            __syncwarp();
#pragma unroll
            for (int i = 0; i < PER; ++i) {
                const int e = lane * PER + i;
                if (e < n_late) sm.late_list[e] = x[i];
            }
        };
        if (n_late <= 32) sort_list(std::integral_constant<int, 1>{});
        else if (n_late <= 64) sort_list(std::integral_constant<int, 2>{});
        else sort_list(std::integral_constant<int, 4>{});
    }
    __syncthreads();
    for (int e = tid; e < n_late; e += blockDim.x) {
        const unsigned key = sm.late_list[e];
        const unsigned pos = key >> kPosShift;
        if (e > 0 && (sm.late_list[e - 1] >> kPosShift) == pos) continue;  // not the run's head
        const unsigned q1 = sm.rfirst[pos];
        T a1, b1;
        besc_operands<T>(g, a0, sm, (int)q1, a1, b1);
        S s = AccT::zero();
        bool first_done = false;
        for (int t = e; t < n_late; ++t) {
            const unsigned kt = sm.late_list[t];
            if ((kt >> kPosShift) != pos) break;
            if (!first_done && q1 < ((kt >> kRankSlotBits) & ((1u << kIdBits) - 1u))) {
                s = AccT::step(s, a1, b1);
                first_done = true;
            }
            s = AccT::step(s, sm.la[kt & kSlotMask], sm.lb[kt & kSlotMask]);
        }
        if (!first_done) s = AccT::step(s, a1, b1);
        sm.rval[pos] = AccT::fin(s);
    }
    __syncthreads();
}

// 128-word chunks of the window bitmap a rank-path row uses.
__device__ __forceinline__ int besc_rank_chunks(const BescScratch *sc)
{
    return (int)(((sc->cmax - sc->cmin) >> 5) / kRankChunk) + 1;
}

// Clears the first nchunks chunks of the window bitmap (all threads of the CTA).
__device__ __forceinline__ void besc_rank_clear(unsigned *bm, int nchunks)
{
    uint4 *bm4 = reinterpret_cast<uint4 *>(bm);
    for (int i = threadIdx.x; i < nchunks * (kRankChunk / 4); i += blockDim.x) bm4[i] = make_uint4(0u, 0u, 0u, 0u);
}

// Rank path of one numeric row, after the expansion marked the window bitmap (n products,
// keys in skeys; sc->cmin/cmax the row's column window, spanning fewer than kRankWinBits
// columns; `late` = this thread's late products, bit k for product tid + k * NT; n_late
// the row's count, at most kRankLateMax).  Returns the row's entry count and leaves the
// bitmap all zero.  Block-uniform; every thread calls it.
template <typename Shape, int kIdBits, typename T, typename KT>
__device__ __forceinline__ int besc_rank_fold(const SpgemmArgs<T> &g, int n, int a0,
                                              const BescSmem<Shape, true, KT, T> &sm, BescScratch *sc,
                                              int *s_warp_sums, int off, int n_expect, unsigned late, int n_late)
{
    using AccT = Acc<T>;
    constexpr int NT = Shape::kThreads;
    constexpr int NW = Shape::kWarps;
    constexpr int PER = Shape::kPMax;  // products per thread: q = tid + k * NT
    static_assert(2 * kIdBits + kRankSlotBits <= 32, "late-list key");
    const int tid = threadIdx.x;
    const int lane = lane_id();
    const int warp = tid >> 5;
    const unsigned cmin = sc->cmin;
    const int nchunks = besc_rank_chunks(sc);
    uint4 *bm4 = reinterpret_cast<uint4 *>(sm.bm);
    unsigned col[PER];
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int q = tid + k * NT;
        col[k] = q < n ? (unsigned)(sm.skeys[bpad(q)] >> kIdBits) : 0u;
    }
    // 2. prefix popcounts: each warp sweeps a contiguous run of 128-word chunks, a lane
    //    four words at a time (counts, barrier, then prefixes)
    const int cpw = (nchunks + NW - 1) / NW;
    const int c0 = min(nchunks, warp * cpw);
    const int c1 = min(nchunks, c0 + cpw);
    int cnt = 0;
    for (int c = c0; c < c1; ++c) {
        const uint4 v = bm4[c * 32 + lane];
        cnt += __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
    }
    cnt = (int)__reduce_add_sync(kFull, (unsigned)cnt);
    if (lane == 0) s_warp_sums[warp] = cnt;
    __syncthreads();
    int base = 0;
    for (int w = 0; w < warp; ++w) base += s_warp_sums[w];
    uint2 *wpre2 = reinterpret_cast<uint2 *>(sm.wpre);
    for (int c = c0; c < c1; ++c) {
        const uint4 v = bm4[c * 32 + lane];
        const int p0 = __popc(v.x), p1 = __popc(v.y), p2 = __popc(v.z);
        const int sum = p0 + p1 + p2 + __popc(v.w);
        int incl = sum;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int t = __shfl_up_sync(kFull, incl, d);
            if (lane >= d) incl += t;
        }
        const unsigned e0 = (unsigned)(base + incl - sum);
        wpre2[c * 32 + lane] = make_uint2(e0 | ((e0 + p0) << 16), (e0 + p0 + p1) | ((e0 + p0 + p1 + p2) << 16));
        base += __shfl_sync(kFull, incl, 31);
    }
    __syncthreads();
    // 3. positions: a column's first product folds itself and stores the entry and its own
    //    index at the column's position, a late product its operands and key in the list
    //    (the operand loads of up to 8 products in flight together)
    constexpr int G = PER < 8 ? PER : 8;
    static_assert(PER % G == 0, "whole groups");
#pragma unroll
    for (int k0 = 0; k0 < PER; k0 += G) {
        int pos[G], o[G], kb[G];
#pragma unroll
        for (int u = 0; u < G; ++u) {
            const int k = k0 + u;
            const int q = tid + k * NT;
            pos[u] = 0;
            o[u] = 0;
            kb[u] = 0;
            if (q < n) {
                const unsigned d = col[k] - cmin;
                const int w = (int)(d >> 5);
                pos[u] = (int)sm.wpre[w] + __popc(sm.bm[w] & ((1u << (d & 31u)) - 1u));
                o[u] = sm.own[q];
                kb[u] = sm.s_b0[o[u]] + q - (o[u] ? sm.s_incl[o[u] - 1] : 0);
            }
        }
        T av[G], bv[G];
#pragma unroll
        for (int u = 0; u < G; ++u) {
            const bool valid = tid + (k0 + u) * NT < n;
            av[u] = valid ? __ldg(g.aval + a0 + o[u]) : T(0);
            bv[u] = valid ? __ldg(g.bval + kb[u]) : T(0);
        }
#pragma unroll
        for (int u = 0; u < G; ++u) {
            const int k = k0 + u;
            const int q = tid + k * NT;
            if (q < n) {
                if ((late >> k) & 1u) {
                    const int slot = atomicAdd(&sc->listed, 1);
                    sm.la[slot] = av[u];
                    sm.lb[slot] = bv[u];
                    sm.late_list[slot] = ((unsigned)pos[u] << (kIdBits + kRankSlotBits)) |
                                         ((unsigned)q << kRankSlotBits) | (unsigned)slot;
                } else {
                    sm.rval[pos[u]] = AccT::fin(AccT::step(AccT::zero(), av[u], bv[u]));
                    sm.rcol[pos[u]] = (int)col[k];
                    sm.rfirst[pos[u]] = (unsigned short)q;
                }
            }
        }
    }
    __syncthreads();
    // 4. columns with late products, re-folded in order
    if (n_late > 0) besc_rank_refold<kIdBits, T>(g, a0, sm, n_late);
    // 5. the row's entries in column order; the bitmap is cleared for the next row
    const int total = n - n_late;
    if (tid == 0 && !g.soff && total != n_expect) atomicOr(&g.info->flags, kErrCountMismatch);
    for (int i = tid; i < total; i += NT) {
        if (i < n_expect) {
            g.c_col[off + i] = sm.rcol[i];
            g.c_val[off + i] = sm.rval[i];
        }
    }
    besc_rank_clear(sm.bm, nchunks);
    return total;
}

// Scan of A's row for the rank shapes: the B-row lengths into s_incl / s_b0 (as
// esc_scan_row) and the row's column window from the B rows' first and last columns
// (B rows are sorted) into sc->cmin / cmax.  Rows of at most 128 A entries are scanned by
// warp 0 alone, four entries a lane with their loads in flight together; longer rows by
// the CTA.  Returns the product count on every thread; ends with a barrier.
template <int NT, typename T>
__device__ __forceinline__ int besc_rank_scan_row(const SpgemmArgs<T> &g, int a0, int lenA, int *s_incl,
                                                  int *s_b0, int *s_warp_sums, BescScratch *sc)
{
    const int tid = threadIdx.x;
    const int lane = lane_id();
    if (lenA > 128) {
        unsigned lo = 0xffffffffu, hi = 0u;
        for (int q = tid; q < lenA; q += NT) {
            const int j = __ldg(g.acol + a0 + q);
            const int b0 = __ldg(g.brpt + j), b1 = __ldg(g.brpt + j + 1);
            if (b1 > b0) {
                lo = min(lo, (unsigned)__ldg(g.bcol + b0));
                hi = max(hi, (unsigned)__ldg(g.bcol + b1 - 1));
            }
        }
        lo = __reduce_min_sync(kFull, lo);
        hi = __reduce_max_sync(kFull, hi);
        if (lane == 0 && lo <= hi) {
            atomicMin(&sc->cmin, lo);
            atomicMax(&sc->cmax, hi);
        }
        return esc_scan_row<NT, T>(g, a0, lenA, s_incl, s_b0, s_warp_sums);  // ends with a barrier
    }
    if (tid < 32) {
        int b0[4], b1[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int q = u * 32 + lane;
            b0[u] = q < lenA ? __ldg(g.acol + a0 + q) : -1;  // A's column, then B's row start
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int j = b0[u];
            b0[u] = j >= 0 ? __ldg(g.brpt + j) : 0;
            b1[u] = j >= 0 ? __ldg(g.brpt + j + 1) : 0;
        }
        unsigned lo = 0xffffffffu, hi = 0u;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (b1[u] > b0[u]) {
                lo = min(lo, (unsigned)__ldg(g.bcol + b0[u]));
                hi = max(hi, (unsigned)__ldg(g.bcol + b1[u] - 1));
            }
        }
        int running = 0;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int q = u * 32 + lane;
            int incl = b1[u] - b0[u];
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int t = __shfl_up_sync(kFull, incl, d);
                if (lane >= d) incl += t;
            }
            if (q < lenA) {
                s_incl[q] = running + incl;
                s_b0[q] = b0[u];
            }
            running += __shfl_sync(kFull, incl, 31);
        }
        lo = __reduce_min_sync(kFull, lo);
        hi = __reduce_max_sync(kFull, hi);
        if (lane == 0) {
            sc->n = running;
            if (lo <= hi) {
                sc->cmin = lo;
                sc->cmax = hi;
            }
        }
    }
    __syncthreads();
    return sc->n;
}

// One row r (at most Shape::kCap products, Shape::kAEntries A entries) by the whole CTA:
// expand, sort (or rank), then count (symbolic) or fold and write (numeric).  Symbolic and
// one-pass calls write the row's count to c_rpt[r]; the count is also added to nnz_acc
// (thread 0).  s_warp_sums (32 ints), s_last (32 keys) and sc are block-shared scratch;
// sc must be reset on entry and is reset again on return.  Every thread of the CTA calls
// it; it ends with a barrier.  Rank shapes: when the row's column window (known from the
// scan) spans fewer than kRankWinBits columns, the expansion also marks each product's
// column in the window bitmap, so the rank path starts at its prefix sweep.
template <typename Shape, bool kNum, typename T, typename KT>
__device__ __forceinline__ void besc_row(const SpgemmArgs<T> &g, int r, const BescSmem<Shape, kNum, KT, T> &sm,
                                         int *s_warp_sums, KT *s_last, BescScratch *sc,
                                         unsigned long long &nnz_acc)
{
    constexpr int NT = Shape::kThreads;
    constexpr int kIdBits = kNum ? Shape::kIdBits : 0;
    constexpr bool kRank = kNum && Shape::kRank;
    const int tid = threadIdx.x;
    const int lane = lane_id();
    const int warp = tid >> 5;
    const int a0 = __ldg(g.arpt + r);
    const int lenA = __ldg(g.arpt + r + 1) - a0;
    int n;
    bool rank_ok = false;
    unsigned cmin = 0u, span = 0u;
    if constexpr (kRank) {
        n = besc_rank_scan_row<NT, T>(g, a0, lenA, sm.s_incl, sm.s_b0, s_warp_sums, sc);
        cmin = sc->cmin;
        span = sc->cmax - cmin;
        rank_ok = n > 0 && n <= Shape::kCap && sc->cmin <= sc->cmax && span < (unsigned)kRankWinBits;
    } else {
        n = esc_scan_row<NT, T>(g, a0, lenA, sm.s_incl, sm.s_b0, s_warp_sums);
    }
    int off = 0, n_expect = 0;
    if constexpr (kNum) {
        if (g.soff) {  // one-pass: the row's staging slot, count unknown
            off = __ldg(g.soff + r);
            n_expect = INT_MAX;
        } else {
            off = __ldg(g.c_rpt + r);
            n_expect = __ldg(g.c_rpt + r + 1) - off;
        }
    }
    // expansion: kUnroll chunks of 32 products per warp, loads in flight together; product
    // q = tid + k * NT is this thread's k-th (k = step * kUnroll + u)
    bool bad = false, wbad = false;
    unsigned late = 0u;
    for (int c0 = warp * 32, kb = 0; c0 < n; c0 += kUnroll * NT, kb += kUnroll) {
        int oo[kUnroll], kk[kUnroll];
        bool v[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            const int c = c0 + u * NT;
            oo[u] = 0;
            kk[u] = 0;
            v[u] = c < n ? esc_expand_chunk(sm.s_incl, sm.s_b0, lenA, n, c, &oo[u], &kk[u]) : false;
        }
        int col[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) col[u] = v[u] ? __ldg(g.bcol + kk[u]) : 0;
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            const int q = c0 + u * NT + lane;
            if (!v[u] || q >= Shape::kCap) continue;  // listed rows have at most kCap products
            bad |= (unsigned)col[u] >= (unsigned)g.N;
            sm.skeys[bpad(q)] = ((KT)(unsigned)col[u] << kIdBits) | (KT)(kNum ? q : 0);
            if constexpr (kNum) sm.own[q] = (unsigned short)oo[u];
            if constexpr (kRank) {
                if (rank_ok) {
                    const unsigned d = (unsigned)col[u] - cmin;
                    if (d <= span) {
                        const unsigned bit = 1u << (d & 31u);
                        if (atomicOr(&sm.bm[d >> 5], bit) & bit) late |= 1u << (kb + u);
                    } else {
                        wbad = true;
                    }
                }
            }
        }
    }
    if constexpr (kRank) {
        if (rank_ok) {
            const int nl = (int)__reduce_add_sync(kFull, (unsigned)__popc(late));
            if (lane == 0 && nl) atomicAdd(&sc->late, nl);
            if (wbad) sc->wbad = 1u;
        }
    }
    if (bad) sc->bad = 1u;
    __syncthreads();
    if (tid == 0 && sc->bad) atomicOr(&g.info->flags, kErrBadColumn);
    const int m = min(n, Shape::kCap);
    constexpr int P = Shape::kPMax;
    int total = -1;
    if constexpr (kRank) {
        if (rank_ok) {
            const int n_late = sc->late;
            if (n_late > kRankLateMax || sc->wbad) {
                besc_rank_clear(sm.bm, besc_rank_chunks(sc));  // the sort takes the row
            } else {
                total = besc_rank_fold<Shape, kIdBits, T, KT>(g, n, a0, sm, sc, s_warp_sums, off, n_expect, late,
                                                              n_late);
            }
            if (tid == 0) atomicAdd(&g.info->rank_rows[total < 0 ? 2 : (n_late ? 1 : 0)], 1);
        }
    }
    if (total >= 0) {
    } else if (m <= NT * (P / 4)) {
        total = besc_sort_fold<Shape, P / 4, kIdBits, kNum, T, KT>(g, m, a0, sm.skeys, sm.spid, sm.hidx, sm.own,
                                                                   sm.s_incl, sm.s_b0, off, n_expect, s_warp_sums,
                                                                   s_last);
    } else if (m <= NT * (P / 2)) {
        total = besc_sort_fold<Shape, P / 2, kIdBits, kNum, T, KT>(g, m, a0, sm.skeys, sm.spid, sm.hidx, sm.own,
                                                                   sm.s_incl, sm.s_b0, off, n_expect, s_warp_sums,
                                                                   s_last);
    } else {
        total = besc_sort_fold<Shape, P, kIdBits, kNum, T, KT>(g, m, a0, sm.skeys, sm.spid, sm.hidx, sm.own,
                                                               sm.s_incl, sm.s_b0, off, n_expect, s_warp_sums,
                                                               s_last);
    }
    if (!kNum || g.soff) {
        if (tid == 0) {
            g.c_rpt[r] = total;
            nnz_acc += (unsigned long long)total;
        }
    }
    __syncthreads();
    if (tid == 0) sc->reset();  // read by every thread before the barrier above
}

template <typename Shape, bool kNum, typename T, typename KT>
__global__ void __launch_bounds__(Shape::kThreads, Shape::kMinBlocks) k_besc_rows(SpgemmArgs<T> g, const int *__restrict__ list,
                                                               const int *count_ptr, int *cursor)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int tid = threadIdx.x;
    __shared__ int s_warp_sums[32];
    __shared__ KT s_last[32];
    __shared__ int s_row;
    __shared__ BescScratch s_sc;
    const BescSmem<Shape, kNum, KT, T> sm(smem_raw);

    const int count = *count_ptr;
    unsigned long long nnz_acc = 0;
    if (tid == 0) s_sc.reset();
    sm.init();
    // rows are drawn one at a time when the CTA is free (lists are longest first, and a CTA
    // takes only a few rows of a single call: drawing ahead would fix the schedule early)
    for (;;) {
        if (tid == 0) s_row = atomicAdd(cursor, 1);
        __syncthreads();
        const int it = s_row;
        __syncthreads();
        if (it >= count) break;
        besc_row<Shape, kNum, T, KT>(g, __ldg(list + it), sm, s_warp_sums, s_last, &s_sc, nnz_acc);
    }
    if (tid == 0 && nnz_acc) atomicAdd(&g.info->total_nnz, nnz_acc);
}

}  // namespace opsg
