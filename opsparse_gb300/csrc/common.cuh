// common.cuh — device building blocks shared by every SpGEMM kernel.
//
// Everything here is written for sm_103a: 32-wide warps, warp-synchronous shuffles,
// __match_any_sync for in-chunk de-duplication, shared-memory CAS for hash slots.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace opsg {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kEmpty = -1;  // empty hash slot / invalid column

// Row classes.  Each row of C is assigned one class by the setup kernel from its
// intermediate-product count ("flop") and its A-row length; the symbolic and numeric
// phases both use this classification, so numeric re-walks exactly what symbolic did.
enum RowClass : int {
    kClsR8 = 0,   // flop <= 8,  lenA <= 8  : 8 lanes per row, registers only
    kClsR16 = 1,  // flop <= 16, lenA <= 16 : 16 lanes per row
    kClsR32 = 2,  // flop <= 32, lenA <= 32 : one warp per row
    kClsW = 3,    // flop <= 128            : one warp per row, register sort
    kClsE1 = 4,   // flop <= 1024, lenA <= 1024   : warp sort, warp hash or CTA bitonic sort
    kClsE2 = 5,   // flop <= 13312, lenA <= 2560  : CTA bitonic sort (<= 4096) or CTA radix sort
    kClsD = 6,    // larger                 : whole-GPU stable radix sort (dense accumulator fallback)
    kNumClasses = 7
};

// Extra device lists after the kNumClasses class lists: the numeric re-binning of the E1
// rows and the size split of the E2 rows.
// The last three split the E1 rows of a one-pass call into those computed in the
// counting phase (by warp sort, or expand/sort/compress above kE1OnePassFlopMax products)
// and those left to two passes.
enum : int {
    kXlE1Sort = 0,
    kXlE1Hash = 1,
    kXlE1Esc = 2,
    kXlE2Mid = 3,
    kXlE2Large = 4,
    kXlE1One = 5,
    kXlE1Two = 6,
    kXlE1OneLarge = 7,
    kNumExtraLists = 8
};
constexpr int kNumLists = kNumClasses + kNumExtraLists;

constexpr int kSmallFlopMax = 8;   // R8 rows: symbolic inside k_setup, numeric k_small_rows
constexpr int kWarpFlopMax = 128;  // W rows: warp register sort of at most 128 products
constexpr int kEsc1FlopMax = 1024;
constexpr int kEsc1AMax = 1024;
constexpr int kEsc2FlopMax = 13312;
constexpr int kEsc2AMax = 2560;
// Entries of more than kBlockFoldMin products fold in kFoldBlocks consecutive blocks of
// ceil(m / kFoldBlocks) products each (each block the plain ascending-j fold from zero),
// the block states merged in block order (Acc::merge).  An entry has at most as many
// products as A's row has entries (a B row holds a column once), so only D rows, whose A
// rows may exceed every other class's limit, can have such entries.
constexpr int kBlockFoldMin = 2560;
constexpr int kFoldBlocks = 32;
static_assert(kBlockFoldMin >= kEsc2AMax && kBlockFoldMin >= kEsc1AMax && kBlockFoldMin >= 128,
              "entries of more than kBlockFoldMin products occur only in D rows");
// E1 rows computed in the counting phase of a one-pass call: by warp sort up to this many
// products, by CTA expand/sort/compress above; column-window rows (below) keep two passes
constexpr int kE1OnePassFlopMax = 512;
// Column-window rows: rows whose B rows are long (at least 16 products per A entry) and
// whose products all fall within kWinBits consecutive columns (banded and stencil
// matrices).  They fold many products per output: counted over a window bitmap, computed
// through a hash table, never sorted product by product.
constexpr int kWinBits = 32768;

// Runtime row-class thresholds (the autotuner's search space).  Each bound is capped by
// the compiled capacity of its kernel; a bound of 0 switches the class off.
struct Thresholds {
    int r8;   // <= kSmallFlopMax
    int r16;  // <= 16
    int r32;  // <= 32
    int w;    // <= kWarpFlopMax
    int e1;   // <= kEsc1FlopMax
    int e2;   // <= kEsc2FlopMax
};

__host__ __device__ inline Thresholds default_thresholds() { return Thresholds{8, 16, 32, 128, 1024, 13312}; }

// Error bits written by kernels into DevInfo::flags (read back by the host).
enum : int {
    kErrRowFlopOverflow = 1,  // a row has more than INT_MAX intermediate products
    kErrProbeLimit = 2,       // a hash probe sequence exceeded its table (cannot happen if sizes are right)
    kErrCountMismatch = 4,    // numeric found a different nnz than symbolic
    kErrBadColumn = 8,        // an input column index is outside [0, cols)
};

// Device-side counters of one SpGEMM call.  Lives in the handle's workspace.
struct DevInfo {
    int counts[kNumClasses];      // rows listed in each class
    int flags;                    // kErr* bits
    int max_flop;                 // clamped to INT_MAX
    unsigned long long total_flop;
    unsigned long long total_nnz;
    int next[2][kNumClasses];     // dynamic row cursors of the [symbolic, numeric] kernels
    int split[3];                 // E1 rows re-binned for the numeric phase: [warp sort, hash, expand/sort]
    int split2[2];                // E2 rows by size, fixed at the symbolic phase: [mid shape, large shape]
    int next_mid[2];              // row cursor of the mid-shape E2 kernel [symbolic, numeric]
    int split1[3];                // E1 rows of a one-pass call: [warp sort, two passes, expand/sort/compress]
    unsigned long long staged_flop;  // products of the rows a one-pass call may stage
    int e1_one;                   // E1 rows a one-pass call may stage
    unsigned long long d_len_a;   // A entries of the D rows
    unsigned long long d_flop;    // products of the D rows
    int d_cursor;                 // long runs listed by the D-row short-run fold
    int rank_rows[3];             // CTA expand rows by the column-window rank path: [no late
                                  // products, late products re-folded, too many late: sorted]
};

// Arguments shared by every SpGEMM kernel.
template <typename T>
struct SpgemmArgs {
    const int *__restrict__ arpt;
    const int *__restrict__ acol;
    const T *__restrict__ aval;
    const int *__restrict__ brpt;
    const int *__restrict__ bcol;
    const T *__restrict__ bval;
    int M;             // rows of A and C
    int K;             // cols of A == rows of B
    int N;             // cols of B and C
    const int *__restrict__ row_flop;
    int *c_rpt;        // symbolic: per-row nnz written at [r]; numeric: row offsets
    int *c_col;
    T *c_val;
    DevInfo *info;
    // One-pass numeric (run inside the counting phase, values known): when set, row r
    // writes its entries to c_col/c_val + soff[r] (a staging area holding every staged
    // row's products at the exclusive prefix of their counts), its count to c_rpt[r] and
    // the count to info->total_nnz, as the counting kernels do; k_place_staged moves the
    // entries into C after the scan.
    const int *soff;
    // Slots per output entry of the warp-hash numeric table (2 or 4; 0 means 4), capped by
    // the kernel's table capacity: a tuning knob of the E1 rows with few outputs.
    int hash_slots;
};

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// 64-bit warp sum.
__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v)
{
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) v += __shfl_xor_sync(kFull, v, d);
    return v;
}

// Fibonacci hashing: the top log2(TS) bits of key * 2^32/phi.
__device__ __forceinline__ uint32_t hash_slot(int key, int log_ts)
{
    return ((uint32_t)key * 2654435761u) >> (32 - log_ts);
}

constexpr int ceil_log2_c(int x)
{
    int l = 0;
    while ((1 << l) < x) ++l;
    return l;
}

__host__ __device__ __forceinline__ int ceil_log2(int x)
{
    int l = 0;
    while ((1 << l) < x) ++l;
    return l;
}

// ----------------------------------------------------------------------------------
// Value accumulation policies.  S is the per-slot accumulator state (8 bytes in both
// cases).  FP64: one correctly rounded FMA per product, folded in ascending j — the same
// sequence the oracle evaluates, so results are bit-identical.  FP32: compensated dot
// product (Ogita, Rump, Oishi 2005, "Dot2"), rounded to float once at the end.
template <typename T>
struct Acc;

template <>
struct Acc<double> {
    using S = double;
    __device__ __forceinline__ static S zero() { return 0.0; }
    __device__ __forceinline__ static S step(S s, double a, double b) { return __fma_rn(a, b, s); }
    __device__ __forceinline__ static double fin(S s) { return s; }
    // states of two consecutive blocks of an entry's products
    __device__ __forceinline__ static S merge(S u, S v) { return __dadd_rn(u, v); }
    __device__ __forceinline__ static S shfl(S v, int src) { return __shfl_sync(0xffffffffu, v, src); }
};

template <>
struct Acc<float> {
    using S = float2;  // x: running sum, y: running compensation
    __device__ __forceinline__ static S zero() { return make_float2(0.f, 0.f); }
    __device__ __forceinline__ static S step(S st, float a, float b)
    {
        const float h = __fmul_rn(a, b);        // TwoProduct: h + r == a*b
        const float r = __fmaf_rn(a, b, -h);
        const float s = __fadd_rn(st.x, h);     // TwoSum: s + q == st.x + h
        const float z = __fsub_rn(s, st.x);
        const float q = __fadd_rn(__fsub_rn(st.x, __fsub_rn(s, z)), __fsub_rn(h, z));
        return make_float2(s, __fadd_rn(st.y, __fadd_rn(q, r)));
    }
    __device__ __forceinline__ static float fin(S st) { return __fadd_rn(st.x, st.y); }
    // states of two consecutive blocks: TwoSum of the sums, the compensations added, then
    // the TwoSum error
    __device__ __forceinline__ static S merge(S u, S v)
    {
        const float s = __fadd_rn(u.x, v.x);
        const float z = __fsub_rn(s, u.x);
        const float q = __fadd_rn(__fsub_rn(u.x, __fsub_rn(s, z)), __fsub_rn(v.x, z));
        return make_float2(s, __fadd_rn(__fadd_rn(u.y, v.y), q));
    }
    __device__ __forceinline__ static S shfl(S v, int src)
    {
        return make_float2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
    }
};

template <typename T>
__device__ __forceinline__ T shfl(T v, int src, int width = 32)
{
    return __shfl_sync(kFull, v, src, width);
}

// Fold the products of one match group into s, in ascending lane order.  Every lane
// of the warp must call this (it shuffles).  `members` is the group's lane mask for
// the group leader and 0 for everyone else; a[] and b[] are the lanes' operands.
template <typename T>
__device__ __forceinline__ typename Acc<T>::S fold_group(typename Acc<T>::S s, unsigned members, T a, T b)
{
    const int lane = lane_id();
    while (__any_sync(kFull, members != 0u)) {
        const int src = members ? (__ffs(members) - 1) : lane;
        const T am = shfl(a, src);
        const T bm = shfl(b, src);
        if (members) {
            s = Acc<T>::step(s, am, bm);
            members &= members - 1u;
        }
    }
    return s;
}

// fold_group for an entry folded in blocks (c = products per block, 0 for a plain entry):
// cur is the current block's state, tot the merge of the finished blocks, pos the number of
// the entry's products folded so far.
template <typename T>
__device__ __forceinline__ void fold_group_blocked(typename Acc<T>::S &cur, typename Acc<T>::S &tot, int &pos, int c,
                                                   unsigned members, T a, T b)
{
    const int lane = lane_id();
    while (__any_sync(kFull, members != 0u)) {
        const int src = members ? (__ffs(members) - 1) : lane;
        const T am = shfl(a, src);
        const T bm = shfl(b, src);
        if (members) {
            if (c && pos && pos % c == 0) {  // the first product of a new block
                tot = pos == c ? cur : Acc<T>::merge(tot, cur);
                cur = Acc<T>::zero();
            }
            cur = Acc<T>::step(cur, am, bm);
            ++pos;
            members &= members - 1u;
        }
    }
}

// ----------------------------------------------------------------------------------
// Warp-cooperative enumeration of a row's intermediate products in j-major order.
//
// The A entries [a_begin, a_end) are visited in windows of 32 (window starts at
// a_begin, a_begin + stride, ...).  For each window the lanes load one A entry each,
// scan the lengths of the selected B rows, and then walk the window's products in
// chunks of 32: lane p of a chunk handles product c+p, whose owner A entry is found by
// a 5-step binary search over the scanned lengths.  f(valid, k, a, p) is called once per
// chunk with all 32 lanes converged; k indexes B.col/B.val, a is the owner's A value and
// p the owner's index into A.col/A.val.
template <bool kNeedVal, typename T, typename F>
__device__ __forceinline__ void warp_products(int a_begin, int a_end, int stride, const int *__restrict__ acol,
                                              const T *__restrict__ aval, const int *__restrict__ brpt, F &&f)
{
    const int lane = lane_id();
    for (int wa = a_begin; wa < a_end; wa += stride) {
        const int q = wa + lane;
        int b0 = 0, bl = 0;
        T av = T(0);
        if (q < a_end) {
            const int j = __ldg(acol + q);
            b0 = __ldg(brpt + j);
            bl = __ldg(brpt + j + 1) - b0;
            if (kNeedVal) av = __ldg(aval + q);
        }
        int incl = bl;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int t = __shfl_up_sync(kFull, incl, d);
            if (lane >= d) incl += t;
        }
        const unsigned total = (unsigned)__shfl_sync(kFull, incl, 31);
        for (unsigned c = 0; c < total; c += 32) {
            const int p = (int)(c + lane);
            const bool valid = (unsigned)p < total;
            int lo = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1) {
                const int v = __shfl_sync(kFull, incl, lo + step - 1);
                if (v <= p) lo += step;
            }
            const int o_incl = __shfl_sync(kFull, incl, lo);
            const int o_bl = __shfl_sync(kFull, bl, lo);
            const int o_b0 = __shfl_sync(kFull, b0, lo);
            const T o_av = kNeedVal ? shfl(av, lo) : T(0);
            const int k = o_b0 + (p - (o_incl - o_bl));
            f(valid, k, o_av, wa + lo);
        }
    }
}

// Ascending bitonic sort of the 32*PER keys held blocked across the warp.  Partner
// distances of PER and above are exchanged with shuffles, smaller ones in registers.
// The merge size k and the shuffle distances run as loops, not unrolled: only the
// per-register work is unrolled, which keeps the code small enough for the instruction
// cache (a fully unrolled 512-key network stalls on instruction fetch).
template <int PER, typename KT>
__device__ __forceinline__ void warp_bitonic_blocked(KT (&x)[PER])
{
    const int lane = lane_id();
    constexpr int n = 32 * PER;
    // merges of size <= PER are entirely in registers
#pragma unroll
    for (int k = 2; k <= PER; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
#pragma unroll
            for (int i = 0; i < PER; ++i) {
                if ((i & j) == 0) {
                    const bool asc = ((lane * PER + i) & k) == 0;
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
        // direction is uniform over a lane's registers: k > PER
        const bool asc = ((lane * PER) & k) == 0;
#pragma unroll 1
        for (int j = k >> 1; j >= PER; j >>= 1) {
            const bool take_min = (((lane * PER) & j) == 0) == asc;
#pragma unroll
            for (int i = 0; i < PER; ++i) {
                const KT y = __shfl_xor_sync(kFull, x[i], j / PER);
                x[i] = take_min ? (x[i] < y ? x[i] : y) : (x[i] < y ? y : x[i]);
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

// Row-aligned enumeration with the operands loaded ahead: the first 32 entries of kU
// consecutive B rows are loaded together, then handed to f in order (B rows longer than
// 32 continue chunk by chunk before the next row starts).  f(valid, col, b, a) is called
// with all lanes converged, in ascending j and, within a B row, ascending position.
template <int kU, bool kNeedVal, typename T, typename F>
__device__ __forceinline__ void warp_rowwise_products_pf(int a_begin, int a_end, const int *__restrict__ acol,
                                                         const T *__restrict__ aval, const int *__restrict__ brpt,
                                                         const int *__restrict__ bcol, const T *__restrict__ bval,
                                                         F &&f)
{
    const int lane = lane_id();
    for (int wa = a_begin; wa < a_end; wa += 32) {
        const int q = wa + lane;
        int b0 = 0, b1 = 0;
        T av = T(0);
        if (q < a_end) {
            const int j = __ldg(acol + q);
            b0 = __ldg(brpt + j);
            b1 = __ldg(brpt + j + 1);
            if (kNeedVal) av = __ldg(aval + q);
        }
        const int m = min(32, a_end - wa);
        for (int t0 = 0; t0 < m; t0 += kU) {
            int col[kU], s0[kU], s1[kU];
            T bv[kU], a[kU];
            bool v[kU];
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const int t = min(t0 + u, 31);
                s0[u] = __shfl_sync(kFull, b0, t);
                s1[u] = __shfl_sync(kFull, b1, t);
                a[u] = kNeedVal ? shfl(av, t) : T(0);
                v[u] = t0 + u < m && s0[u] + lane < s1[u];
                col[u] = v[u] ? __ldg(bcol + s0[u] + lane) : 0;
                bv[u] = (kNeedVal && v[u]) ? __ldg(bval + s0[u] + lane) : T(0);
            }
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                if (t0 + u >= m) break;  // warp-uniform
                f(v[u], col[u], bv[u], a[u]);
                for (int c = s0[u] + 32; c < s1[u]; c += 32) {
                    const bool vv = c + lane < s1[u];
                    const int cc = vv ? __ldg(bcol + c + lane) : 0;
                    const T bb = (kNeedVal && vv) ? __ldg(bval + c + lane) : T(0);
                    f(vv, cc, bb, a[u]);
                }
            }
        }
    }
}

// Claim (or find) the slot of `key` in an open-addressing table of ts = 2^log_ts
// slots.  Linear probing, bounded by the table size; returns -1 (and raises
// kErrProbeLimit) only if the table is full, which the sizing rules exclude.
// *is_new is set when this call inserted the key.
__device__ __forceinline__ int table_claim(int *keys, int key, int log_ts, bool *is_new, int *flags)
{
    const uint32_t mask = (1u << log_ts) - 1u;
    uint32_t h = hash_slot(key, log_ts);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const int old = atomicCAS(keys + h, kEmpty, key);
        if (old == kEmpty) {
            *is_new = true;
            return (int)h;
        }
        if (old == key) {
            *is_new = false;
            return (int)h;
        }
        h = (h + 1u) & mask;
    }
    atomicOr(flags, kErrProbeLimit);
    *is_new = false;
    return -1;
}

// Block-wide inclusive scan of one int per thread (blockDim.x a multiple of 32, at
// most 1024).  `warp_sums` is shared scratch of 32 ints.  Returns the inclusive
// prefix; *total receives the block total.  Contains two __syncthreads().
__device__ __forceinline__ int block_inclusive_scan(int v, int *warp_sums, int *total)
{
    const int lane = lane_id();
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int t = __shfl_up_sync(kFull, v, d);
        if (lane >= d) v += t;
    }
    if (lane == 31) warp_sums[warp] = v;
    __syncthreads();
    if (warp == 0) {
        int w = lane < nwarps ? warp_sums[lane] : 0;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int t = __shfl_up_sync(kFull, w, d);
            if (lane >= d) w += t;
        }
        if (lane < nwarps) warp_sums[lane] = w;
    }
    __syncthreads();
    const int before = warp ? warp_sums[warp - 1] : 0;
    *total = warp_sums[nwarps - 1];
    return v + before;
}

}  // namespace opsg
