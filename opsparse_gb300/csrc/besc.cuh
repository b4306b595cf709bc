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
#pragma once

#include "esc.cuh"

namespace opsg {

template <int NT, int PMAX, int ACAP, int MINB>
struct BescShape {
    static constexpr int kThreads = NT;
    static constexpr int kMinBlocks = MINB;             // CTAs per SM the registers must allow
    static constexpr int kWarps = NT / 32;
    static constexpr int kPMax = PMAX;
    static constexpr int kCap = NT * PMAX;              // products per row, at most
    static constexpr int kAEntries = ACAP;              // A entries per row, at most
    static constexpr int kIdBits = ceil_log2_c(kCap);   // bits of a product index
    static constexpr int kPadSlots = kCap + kCap / 32;  // keys with one pad slot per 32

    static constexpr size_t up16(size_t x) { return (x + 15) / 16 * 16; }
    // [keys (sort exchange) | product ids + run heads (fold), aliased] [own] [scan]
    template <bool kNum, typename KT>
    static constexpr size_t region0()
    {
        return up16(sizeof(KT) * kPadSlots) > (kNum ? up16(2 * (size_t)kCap + 4 * ((size_t)kCap + 1)) : 0)
                   ? up16(sizeof(KT) * kPadSlots)
                   : up16(2 * (size_t)kCap + 4 * ((size_t)kCap + 1));
    }
    template <bool kNum, typename KT>
    static constexpr size_t smem()
    {
        return region0<kNum, KT>() + (kNum ? up16(2 * (size_t)kCap) : 0) + 8 * (size_t)ACAP;
    }
};

using BescE1 = BescShape<128, 8, 1024, 4>;    // E1 rows of more than kSplitNnz outputs
using BescMid = BescShape<256, 16, 1280, 4>;  // E2 rows of at most 4,096 products

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

// Shared memory of one CTA of the besc routine: [keys | ids + heads] [own] [scan].
template <typename Shape, bool kNum, typename KT>
struct BescSmem {
    KT *skeys;
    unsigned short *spid;
    int *hidx;
    unsigned short *own;
    int *s_incl;
    int *s_b0;
    __device__ __forceinline__ explicit BescSmem(unsigned char *p)
    {
        skeys = reinterpret_cast<KT *>(p);
        spid = reinterpret_cast<unsigned short *>(p);
        hidx = reinterpret_cast<int *>(p + Shape::up16(2 * (size_t)Shape::kCap));
        p += Shape::template region0<kNum, KT>();
        own = nullptr;
        if constexpr (kNum) {
            own = reinterpret_cast<unsigned short *>(p);
            p += Shape::up16(2 * (size_t)Shape::kCap);
        }
        s_incl = reinterpret_cast<int *>(p);
        s_b0 = s_incl + Shape::kAEntries;
    }
};

// One row r (at most Shape::kCap products, Shape::kAEntries A entries) by the whole CTA:
// expand, sort, then count (symbolic) or fold and write (numeric).  Symbolic and one-pass
// calls write the row's count to c_rpt[r]; the count is also added to nnz_acc (thread 0).
// s_warp_sums (32 ints), s_last (32 keys) and s_bad are block-shared scratch; *s_bad must
// be 0 on entry and is 0 again on return.  Every thread of the CTA calls it; it ends with
// a barrier.
template <typename Shape, bool kNum, typename T, typename KT>
__device__ __forceinline__ void besc_row(const SpgemmArgs<T> &g, int r, const BescSmem<Shape, kNum, KT> &sm,
                                         int *s_warp_sums, KT *s_last, unsigned *s_bad,
                                         unsigned long long &nnz_acc)
{
    constexpr int NT = Shape::kThreads;
    constexpr int kIdBits = kNum ? Shape::kIdBits : 0;
    const int tid = threadIdx.x;
    const int lane = lane_id();
    const int warp = tid >> 5;
    const int a0 = __ldg(g.arpt + r);
    const int lenA = __ldg(g.arpt + r + 1) - a0;
    const int n = esc_scan_row<NT, T>(g, a0, lenA, sm.s_incl, sm.s_b0, s_warp_sums);
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
    // expansion: kUnroll chunks of 32 products per warp, loads in flight together
    bool bad = false;
    for (int c0 = warp * 32; c0 < n; c0 += kUnroll * NT) {
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
        }
    }
    if (bad) *s_bad = 1u;
    __syncthreads();
    if (tid == 0 && *s_bad) atomicOr(&g.info->flags, kErrBadColumn);
    const int m = min(n, Shape::kCap);
    constexpr int P = Shape::kPMax;
    int total;
    if (m <= NT * (P / 4)) {
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
    if (tid == 0) *s_bad = 0u;  // read by every thread before the barrier above
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
    __shared__ unsigned s_bad;
    const BescSmem<Shape, kNum, KT> sm(smem_raw);

    const int count = *count_ptr;
    unsigned long long nnz_acc = 0;
    if (tid == 0) s_bad = 0u;
    for (;;) {
        if (tid == 0) s_row = atomicAdd(cursor, 1);
        __syncthreads();
        const int it = s_row;
        __syncthreads();
        if (it >= count) break;
        besc_row<Shape, kNum, T, KT>(g, __ldg(list + it), sm, s_warp_sums, s_last, &s_bad, nnz_acc);
    }
    if (tid == 0 && nnz_acc) atomicAdd(&g.info->total_nnz, nnz_acc);
}

}  // namespace opsg
