// wsort.cuh — one warp per row, no hash table: expand the row's products into shared
// memory, sort (column, product index) keys in registers with a warp bitonic network,
// fold every run of equal columns in ascending product order, and write C in column
// order.  Used for rows whose products mostly land in distinct columns (web-like rows:
// nnz(C row) close to the product count).  For them a hash table costs a probe per
// product and still needs a sort of the table afterwards; sorting the products once
// does strictly less.  Replaces, for those rows, OpSparse's shared-hash numeric and
// symbolic kernels of the small and middle bins (kernels/numeric.cuh:109-205,
// kernels/symbolic.cuh:74-130).
//
// Keys: numeric packs (column << kIdBits) | product index, so equal columns sort in
// ascending product order (= ascending j, the oracle's order) and the sort needs no
// stability.  Symbolic sorts bare columns and counts the distinct ones.
#pragma once

#include "kernels.cuh"

namespace opsg {

constexpr int kWsortFlopMax = 512;  // largest row of the 16-per-lane variant
static_assert(kE1OnePassFlopMax <= kWsortFlopMax, "one-pass E1 rows use the warp sort");

// Shared-memory index of element e with one pad word per 32: the blocked register layout
// (lane l holds elements l*PER .. l*PER+PER-1) then reads and writes without bank
// conflicts, and so does the expansion's contiguous stores.
__device__ __forceinline__ int wpad(int e) { return e + (e >> 5); }

template <int PMAX>
struct WsortShape {
    static constexpr int kMax = 32 * PMAX;                     // products per row, at most
    static constexpr int kWarps = PMAX <= 4 ? 8 : 4;           // warps per CTA
    static constexpr int kThreads = 32 * kWarps;
    // CTAs per SM the registers must allow: 4 for both the 128-key variant (8 warps per
    // CTA, 64 registers) and the 32-key symbolic variant (128 registers); 5 for the
    // 512-key variant (at most 102 registers; with no bound it took 103-127, which left 4
    // CTAs, and measured slower on both the web graph and the batch)
    static constexpr int kMinBlocks = PMAX >= 32 ? 4 : (PMAX <= 4 ? 4 : 5);
    static constexpr int kIdBits = PMAX <= 4 ? 7 : (PMAX <= 8 ? 8 : (PMAX <= 16 ? 9 : 10));
    static constexpr int kKeySlots = kMax + kMax / 32;         // padded key array
    static constexpr int kHeadSlots = kMax + 32;               // run heads + end marker

    template <bool kNum, typename T, typename KT>
    static constexpr size_t per_warp()
    {
        return (sizeof(KT) * kKeySlots + 15) / 16 * 16 + (kNum ? sizeof(int) * kHeadSlots + 2 * sizeof(T) * kMax : 0);
    }
    template <bool kNum, typename T, typename KT>
    static constexpr size_t smem()
    {
        return (size_t)kWarps * per_warp<kNum, T, KT>();
    }
};

// Sort the row's `flop` keys (already in skey at padded positions), then count (symbolic)
// or fold and write (numeric) the runs.  Returns the number of distinct columns.
template <int PER, int kIdBits, bool kNum, typename T, typename KT>
__device__ __forceinline__ int wsort_row(const SpgemmArgs<T> &g, int flop, KT *skey, int *heads, const T *sa,
                                         const T *sb, long long off, int n_expect)
{
    using AccT = Acc<T>;
    using S = typename AccT::S;
    const int lane = lane_id();
    KT x[PER];
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = lane * PER + i;
        x[i] = e < flop ? skey[wpad(e)] : ~KT(0);
    }
    warp_bitonic_blocked<PER, KT>(x);
    const KT before = __shfl_up_sync(kFull, x[PER - 1], 1);
    unsigned hm = 0;
    int h = 0;
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = lane * PER + i;
        const KT prev = i ? x[i - 1] : before;
        const bool head = e < flop && (e == 0 || (x[i] >> kIdBits) != (prev >> kIdBits));
        hm |= head ? (1u << i) : 0u;
        h += head ? 1 : 0;
    }
    int incl = h;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int t = __shfl_up_sync(kFull, incl, d);
        if (lane >= d) incl += t;
    }
    const int total = __shfl_sync(kFull, incl, 31);
    if constexpr (kNum) {
        int pos = incl - h;
#pragma unroll
        for (int i = 0; i < PER; ++i) {
            const int e = lane * PER + i;
            skey[wpad(e)] = x[i];
            if ((hm >> i) & 1u) heads[pos++] = e;
        }
        if (lane == 0) heads[total] = flop;
        __syncwarp();
        constexpr KT kIdMask = (KT(1) << kIdBits) - 1;
        // heads in lane order: consecutive lanes write consecutive entries of C
        for (int hh = lane; hh < total; hh += 32) {
            const int e0 = heads[hh], e1 = heads[hh + 1];
            const KT k0 = skey[wpad(e0)];
            S s = AccT::zero();
            for (int t = e0; t < e1; ++t) {
                const int pid = (int)(skey[wpad(t)] & kIdMask);
                s = AccT::step(s, sa[pid], sb[pid]);
            }
            if (hh < n_expect) {
                g.c_col[off + hh] = (int)(k0 >> kIdBits);
                g.c_val[off + hh] = AccT::fin(s);
            }
        }
        __syncwarp();
    }
    return total;
}

// Shared memory of one warp of the warp-sort routine: keys, then (numeric) the products'
// A and B values and the run heads.
template <int PMAX, bool kNum, typename T, typename KT>
struct WsortSmem {
    KT *skey;
    T *sa;
    T *sb;
    int *heads;
    __device__ __forceinline__ explicit WsortSmem(unsigned char *base)
    {
        using Sh = WsortShape<PMAX>;
        skey = reinterpret_cast<KT *>(base);
        base += (sizeof(KT) * Sh::kKeySlots + 15) / 16 * 16;
        sa = sb = nullptr;
        heads = nullptr;
        if constexpr (kNum) {
            sa = reinterpret_cast<T *>(base);
            sb = sa + Sh::kMax;
            heads = reinterpret_cast<int *>(sb + Sh::kMax);
        }
    }
};

// One row r (flop <= 32*PMAX products) by one warp: expand, sort, then count (symbolic) or
// fold and write (numeric).  Rows of at most 64 products sort 64 keys, at most 128 sort
// 128, and so on up to 32*PMAX.  Symbolic and one-pass calls write the count to c_rpt[r]
// and add it to nnz_acc (lane 0).  All lanes call it.
template <int PMAX, bool kNum, typename T, typename KT>
__device__ __forceinline__ void wsort_process_row(const SpgemmArgs<T> &g, int r,
                                                  const WsortSmem<PMAX, kNum, T, KT> &sm,
                                                  unsigned long long &nnz_acc)
{
    using Sh = WsortShape<PMAX>;
    constexpr int kIdBits = kNum ? Sh::kIdBits : 0;
    const int lane = lane_id();
    KT *skey = sm.skey;
    T *sa = sm.sa, *sb = sm.sb;
    int *heads = sm.heads;
    const int a0 = __ldg(g.arpt + r);
    const int a1 = __ldg(g.arpt + r + 1);
    const int flop = __ldg(g.row_flop + r);
    long long off = 0;
    int n_expect = 0;
    if constexpr (kNum) {
        if (g.soff) {  // one-pass: the row's staging slot, count unknown
            off = __ldg(g.soff + r);
            n_expect = INT_MAX;
        } else {
            off = __ldg(g.c_rpt + r);
            n_expect = __ldg(g.c_rpt + r + 1) - (int)off;
        }
    }
    // expansion: windows of 32 A entries, kUnroll chunks of 32 products in flight
    int wbase = 0;
    bool bad = false;
    for (int wa = a0; wa < a1; wa += 32) {
        const int q = wa + lane;
        int b0 = 0, bl = 0;
        T av = T(0);
        if (q < a1) {
            const int j = __ldg(g.acol + q);
            b0 = __ldg(g.brpt + j);
            bl = __ldg(g.brpt + j + 1) - b0;
            if constexpr (kNum) av = __ldg(g.aval + q);
        }
        int incl = bl;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int t = __shfl_up_sync(kFull, incl, d);
            if (lane >= d) incl += t;
        }
        const int wtot = __shfl_sync(kFull, incl, 31);
        for (int c = 0; c < wtot; c += 32 * kUnroll) {
            int kk[kUnroll];
            T oav[kUnroll];
            bool v[kUnroll];
#pragma unroll
            for (int u = 0; u < kUnroll; ++u) {
                const int p = c + u * 32 + lane;
                v[u] = p < wtot;
                int lo = 0;
#pragma unroll
                for (int step = 16; step >= 1; step >>= 1) {
                    const int vv = __shfl_sync(kFull, incl, lo + step - 1);
                    if (vv <= p) lo += step;
                }
                const int o_incl = __shfl_sync(kFull, incl, lo);
                const int o_bl = __shfl_sync(kFull, bl, lo);
                const int o_b0 = __shfl_sync(kFull, b0, lo);
                oav[u] = kNum ? shfl(av, lo) : T(0);
                kk[u] = o_b0 + (p - (o_incl - o_bl));
            }
            int col[kUnroll];
            T bv[kUnroll];
#pragma unroll
            for (int u = 0; u < kUnroll; ++u) {
                col[u] = v[u] ? __ldg(g.bcol + kk[u]) : 0;
                bv[u] = (kNum && v[u]) ? __ldg(g.bval + kk[u]) : T(0);
            }
#pragma unroll
            for (int u = 0; u < kUnroll; ++u) {
                const int idx = wbase + c + u * 32 + lane;
                if (!v[u] || idx >= Sh::kMax) continue;  // listed rows have flop <= kMax
                bad |= (unsigned)col[u] >= (unsigned)g.N;
                skey[wpad(idx)] = ((KT)(unsigned)col[u] << kIdBits) | (KT)(kNum ? idx : 0);
                if constexpr (kNum) {
                    sa[idx] = oav[u];
                    sb[idx] = bv[u];
                }
            }
        }
        wbase += wtot;
    }
    if (bad) atomicOr(&g.info->flags, kErrBadColumn);
    __syncwarp();
    // the smallest power-of-two network that holds the row
    int total = 0;
    if (flop <= 64) {
        total = wsort_row<2, kIdBits, kNum, T, KT>(g, flop, skey, heads, sa, sb, off, n_expect);
    } else if (flop <= 128) {
        total = wsort_row<4, kIdBits, kNum, T, KT>(g, flop, skey, heads, sa, sb, off, n_expect);
    } else if constexpr (PMAX >= 8) {
        if (flop <= 256) {
            total = wsort_row<8, kIdBits, kNum, T, KT>(g, flop, skey, heads, sa, sb, off, n_expect);
        } else if constexpr (PMAX >= 16) {
            if (flop <= 512) {
                total = wsort_row<16, kIdBits, kNum, T, KT>(g, flop, skey, heads, sa, sb, off, n_expect);
            } else if constexpr (PMAX >= 32) {
                total = wsort_row<32, kIdBits, kNum, T, KT>(g, flop, skey, heads, sa, sb, off, n_expect);
            }
        }
    }
    if (!kNum || g.soff) {
        if (lane == 0) {
            g.c_rpt[r] = total;
            nnz_acc += (unsigned long long)total;
        }
    } else {
        if (lane == 0 && total != n_expect) atomicOr(&g.info->flags, kErrCountMismatch);
    }
    __syncwarp();
}

// One warp per listed row (flop <= 32*PMAX).  PMAX = 32 is used for the symbolic count of
// rows of up to 1024 products.  The row count is read from device memory, so lists split
// on the device need no host round trip.
template <int PMAX, bool kNum, typename T, typename KT>
__global__ void __launch_bounds__(WsortShape<PMAX>::kThreads, WsortShape<PMAX>::kMinBlocks) k_wsort_rows(SpgemmArgs<T> g, const int *__restrict__ list,
                                                                         const int *count_ptr)
{
    using Sh = WsortShape<PMAX>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5;
    const WsortSmem<PMAX, kNum, T, KT> sm(smem_raw + (size_t)warp * Sh::template per_warp<kNum, T, KT>());
    const int count = *count_ptr;
    const long long warp0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    unsigned long long nnz_acc = 0;
    for (long long it = warp0; it < count; it += nwarps)
        wsort_process_row<PMAX, kNum, T, KT>(g, __ldg(list + it), sm, nnz_acc);
    if (!kNum || g.soff) warp_add_u64(nnz_acc, &g.info->total_nnz);
}

}  // namespace opsg
