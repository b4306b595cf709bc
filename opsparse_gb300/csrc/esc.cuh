// esc.cuh — expand / sort / compress rows, one CTA per row: the symbolic count of the E2
// rows (hash table) and the numeric phase of the E2 rows above 4,096 products (radix
// sort); also the device-side re-binning and ordering of class lists.  Replaces OpSparse's
// per-bin shared-hash kernels for its large bins (kernels/symbolic.cuh:74-261,
// kernels/numeric.cuh:109-302).
//
// Every thread of the CTA takes part in every step, so a row costs a few load-latency
// levels instead of one dependent chain per warp:
//   1. scan the lengths of the B rows selected by A's row into shared memory;
//   2. expand: product p (thread-strided) finds its A entry by binary search over that
//      scan and loads its column key;
//   symbolic: 3. insert the keys into a shared-memory hash table (order-free) and count;
//   numeric:  3. stable LSD radix sort of (key, product index), 8-bit digits; each warp
//                owns a contiguous slice and scatters it in order, so products of equal
//                key stay in ascending product order (= ascending j);
//             4. the first element of each key run computes the run's output position
//                (block scan of run heads) and folds the run's products in order with
//                one FMA each — the oracle's sequence, bit for bit — then writes C.
// Loops run to block-uniform bounds; all __syncthreads are reached by every thread.
#pragma once

#include <climits>

#include "kernels.cuh"

namespace opsg {

constexpr int pow2_at_least(int x)
{
    int p = 1;
    while (p < x) p <<= 1;
    return p;
}

template <int NT, int PCAP, int ACAP>
struct EscShape {
    static constexpr int kThreads = NT;
    static constexpr int kWarps = NT / 32;
    static constexpr int kProducts = PCAP;     // products per row, at most
    static constexpr int kAEntries = ACAP;     // A entries per row, at most
    static constexpr int kTable = pow2_at_least(2 * PCAP);  // symbolic hash slots
    static constexpr int kDigits = 256;
    // numeric: keys x2 (u32), ids x2 (u16), owner per product (u16), per-warp digit
    // counters, A-entry scan + B row starts
    // radix histograms: 16-bit counters (a warp's slice and every offset are < 2^16)
    static constexpr size_t kNumericSmem = (size_t)PCAP * (4 + 4 + 2 + 2 + 2) + (size_t)kWarps * kDigits * 2 +
                                           (size_t)ACAP * 8 + 32 * 4 + 64;
    static_assert(PCAP < 65536, "16-bit radix offsets");
    static_assert(PCAP / 16 < NT / 32 * 128, "long-run list fits the histogram space");
    static constexpr size_t kSymbolicSmem = (size_t)kTable * 4 + (size_t)ACAP * 8 + 32 * 4 + 64;
};

using EscMid = EscShape<256, 4096, 1280>;     // 75,968 B numeric: three CTAs per SM
using EscLarge = EscShape<1024, 13312, 2560>;  // 223,424 B numeric: one 1024-thread CTA per SM

constexpr int kUnroll = 4;  // chunks (expansion) or products (fold) with loads in flight together
constexpr int kLongRun = 16;  // numeric: runs of this many products or more are folded by a warp

// Smallest t in [0, n) with incl[t] > p (incl non-decreasing, incl[n-1] > p).
__device__ __forceinline__ int esc_owner(const int *incl, int n, int p)
{
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (incl[mid] <= p) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Smallest t in [0, n) with incl[t] > p, found by the whole warp (p warp-uniform) with a
// 32-ary search: each round the lanes probe 32 evenly spaced entries and a ballot
// narrows the range 32-fold, so n <= 1024 takes two shared-memory round trips.
__device__ __forceinline__ int warp_owner(const int *incl, int n, int p)
{
    const int lane = lane_id();
    int lo = 0, hi = n;
    for (;;) {
        const int step = (hi - lo + 31) >> 5;
        const int q = lo + (lane + 1) * step - 1;
        const bool le = q < hi && incl[q] <= p;
        const int nb = __popc(__ballot_sync(kFull, le));
        if (step <= 1) return lo + nb;
        lo += nb * step;
        hi = min(hi, lo + step);
    }
}

// Warp-cooperative expansion of products [c, c+32) of a row (all 32 lanes call it).
// A 32-ary warp search finds the owner A entry o0 of product c; each lane then loads the
// scan value of entry o0+lane and finds its own owner with a 5-step shuffle search.
// If the product lies beyond those 32 entries (possible only when B rows are empty)
// the lane falls back to its own binary search.  Sets *k to the product's index into
// B.col/B.val and *o to its A entry; returns whether the lane has a product.
__device__ __forceinline__ bool esc_expand_chunk(const int *s_incl, const int *s_b0, int lenA, int flop, int c,
                                                 int *o, int *k)
{
    const int lane = lane_id();
    const int p = c + lane;
    const bool valid = p < flop;
    const int o0 = warp_owner(s_incl, lenA, c);
    const int t = o0 + lane;
    const int it = t < lenA ? s_incl[t] : INT_MAX;
    int lo = 0;
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1) {
        const int v = __shfl_sync(kFull, it, lo + step - 1);
        if (v <= p) lo += step;
    }
    const int it31 = __shfl_sync(kFull, it, 31);
    int own = o0 + lo;
    if (valid && it31 <= p) own = esc_owner(s_incl, lenA, p);
    *o = own;
    *k = valid ? s_b0[own] + p - (own ? s_incl[own - 1] : 0) : 0;
    return valid;
}

// Block-wide scan of the B-row lengths of A's row into s_incl/s_b0; returns the row's
// product count.  Caller guarantees lenA <= ACAP.
template <int NT, typename T>
__device__ __forceinline__ int esc_scan_row(const SpgemmArgs<T> &g, int a0, int lenA, int *s_incl, int *s_b0,
                                            int *warp_sums)
{
    int running = 0;
    for (int base = 0; base < lenA; base += NT) {
        const int q = base + (int)threadIdx.x;
        int b0 = 0, bl = 0;
        if (q < lenA) {
            const int j = __ldg(g.acol + a0 + q);
            b0 = __ldg(g.brpt + j);
            bl = __ldg(g.brpt + j + 1) - b0;
        }
        int wtot = 0;
        const int incl = block_inclusive_scan(bl, warp_sums, &wtot);
        if (q < lenA) {
            s_incl[q] = running + incl;
            s_b0[q] = b0;
        }
        running += wtot;
        __syncthreads();
    }
    return running;
}

// Distinct columns of one row (lenA A entries already scanned into s_incl / s_b0, flop
// products) by the whole CTA in a shared-memory hash table of at least 2 slots per product
// (order-free claims; kUnroll chunks of column loads in flight before the first claim).
// Returns the count on every thread; s_count is block-shared scratch.  Every thread of the
// CTA calls it.
template <typename Shape, typename T>
__device__ __forceinline__ int esc_count_row(const SpgemmArgs<T> &g, int lenA, int flop, int *table,
                                             const int *s_incl, const int *s_b0, int *s_count)
{
    constexpr int NT = Shape::kThreads;
    const int tid = threadIdx.x;
    const int lane = lane_id();
    const int warp = tid >> 5;
    const int log_ts = max(6, ceil_log2(2 * max(flop, 1)));
    const int ts = 1 << log_ts;
    for (int i = tid; i < ts; i += NT) table[i] = kEmpty;
    if (tid == 0) *s_count = 0;
    __syncthreads();
    int cnt = 0;
    for (int c0 = warp * 32; c0 < flop; c0 += kUnroll * NT) {
        int kk[kUnroll];
        bool v[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            const int c = c0 + u * NT;
            int o = 0;
            kk[u] = 0;
            v[u] = c < flop ? esc_expand_chunk(s_incl, s_b0, lenA, flop, c, &o, &kk[u]) : false;
        }
        int col[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) col[u] = v[u] ? __ldg(g.bcol + kk[u]) : 0;
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            if (!v[u]) continue;
            if ((unsigned)col[u] >= (unsigned)g.N) {
                atomicOr(&g.info->flags, kErrBadColumn);
                continue;
            }
            bool is_new = false;
            table_claim(table, col[u], log_ts, &is_new, &g.info->flags);
            cnt += is_new ? 1 : 0;
        }
    }
    cnt = (int)__reduce_add_sync(kFull, (unsigned)cnt);
    if (lane == 0 && cnt) atomicAdd(s_count, cnt);
    __syncthreads();
    return *s_count;
}

template <typename Shape, bool kNum, typename T>
__global__ void __launch_bounds__(Shape::kThreads, 1) k_esc_rows(SpgemmArgs<T> g, const int *__restrict__ list,
                                                              const int *count_ptr, int *cursor)
{
    using AccT = Acc<T>;
    using S = typename AccT::S;
    constexpr int NT = Shape::kThreads;
    constexpr int NW = Shape::kWarps;
    constexpr int PCAP = Shape::kProducts;
    constexpr int ACAP = Shape::kAEntries;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int tid = threadIdx.x;
    const int lane = lane_id();
    const int warp = tid >> 5;
    __shared__ int s_warp_sums[32];
    __shared__ int s_count;
    unsigned long long nnz_acc = 0;

    // shared memory carve-up
    unsigned char *p = smem_raw;
    unsigned *key0 = nullptr, *key1 = nullptr;
    unsigned short *id0 = nullptr, *id1 = nullptr, *own = nullptr;
    unsigned short *hist = nullptr;
    int *table = nullptr;
    if constexpr (kNum) {
        key0 = reinterpret_cast<unsigned *>(p);
        p += sizeof(unsigned) * PCAP;
        key1 = reinterpret_cast<unsigned *>(p);
        p += sizeof(unsigned) * PCAP;
        hist = reinterpret_cast<unsigned short *>(p);
        p += sizeof(unsigned short) * NW * Shape::kDigits;
    } else {
        table = reinterpret_cast<int *>(p);
        p += sizeof(int) * Shape::kTable;
    }
    int *s_incl = reinterpret_cast<int *>(p);
    p += sizeof(int) * ACAP;
    int *s_b0 = reinterpret_cast<int *>(p);
    p += sizeof(int) * ACAP;
    if constexpr (kNum) {
        id0 = reinterpret_cast<unsigned short *>(p);
        p += sizeof(unsigned short) * PCAP;
        id1 = reinterpret_cast<unsigned short *>(p);
        p += sizeof(unsigned short) * PCAP;
        own = reinterpret_cast<unsigned short *>(p);
    }
    const int count = *count_ptr;
    const int key_bits = max(1, ceil_log2(max(g.N, 2)));
    const int passes = (key_bits + 7) / 8;

    __shared__ int s_row;
    // rows are taken from a shared cursor, so a CTA that drew heavy rows does not hold
    // up the kernel while others sit idle
    for (;;) {
        if (tid == 0) s_row = atomicAdd(cursor, 1);
        __syncthreads();
        const int it = s_row;
        __syncthreads();
        if (it >= count) break;
        const int r = __ldg(list + it);
        const int a0 = __ldg(g.arpt + r);
        const int lenA = __ldg(g.arpt + r + 1) - a0;
        const int flop = esc_scan_row<NT, T>(g, a0, lenA, s_incl, s_b0, s_warp_sums);

        if constexpr (!kNum) {
            // ---------------------------------------------------------- symbolic --
            const int tot = esc_count_row<Shape, T>(g, lenA, flop, table, s_incl, s_b0, &s_count);
            if (tid == 0) {
                g.c_rpt[r] = tot;
                nnz_acc += (unsigned long long)tot;
            }
            __syncthreads();
        } else {
            // ----------------------------------------------------------- numeric --
            // one-pass: the row's staging slot, count unknown until the runs are found
            const int off = g.soff ? __ldg(g.soff + r) : __ldg(g.c_rpt + r);
            const int n_expect = g.soff ? INT_MAX : __ldg(g.c_rpt + r + 1) - off;
            const int n = flop;
            for (int c0 = warp * 32; c0 < n; c0 += kUnroll * NT) {
                int oo[kUnroll], kk[kUnroll];
                bool v[kUnroll];
#pragma unroll
                for (int u = 0; u < kUnroll; ++u) {
                    const int c = c0 + u * NT;
                    oo[u] = 0;
                    kk[u] = 0;
                    v[u] = c < n ? esc_expand_chunk(s_incl, s_b0, lenA, n, c, &oo[u], &kk[u]) : false;
                }
                unsigned key[kUnroll];
#pragma unroll
                for (int u = 0; u < kUnroll; ++u) key[u] = v[u] ? (unsigned)__ldg(g.bcol + kk[u]) : 0u;
                bool bad = false;
#pragma unroll
                for (int u = 0; u < kUnroll; ++u) {
                    const int i = c0 + u * NT + lane;
                    if (v[u]) {
                        bad |= key[u] >= (unsigned)g.N;
                        key0[i] = key[u];
                        id0[i] = (unsigned short)i;
                        own[i] = (unsigned short)oo[u];
                    }
                }
                if (bad) atomicOr(&g.info->flags, kErrBadColumn);  // B column outside [0, N)
            }
            __syncthreads();
            unsigned *kin = key0, *kout = key1;
            unsigned short *iin = id0, *iout = id1;
            const int per = (n + NW - 1) / NW;
            const int rb = min(n, warp * per);
            const int re = min(n, rb + per);
            unsigned short *wh = hist + warp * Shape::kDigits;
            for (int pass = 0; pass < passes; ++pass) {
                const int shift = 8 * pass;
                const int nbits = min(8, key_bits - shift);
                // the warp's 16-bit counters, two to a word, counted with shared-memory
                // atomics (order-free; a slice holds fewer than 2^16 elements)
                unsigned *wh32 = reinterpret_cast<unsigned *>(wh);
                for (int d = lane; d < Shape::kDigits / 2; d += 32) wh32[d] = 0u;
                __syncwarp();
                for (int i = rb + lane; i < re; i += 32) {
                    const unsigned d = (kin[i] >> shift) & 255u;
                    atomicAdd(&wh32[d >> 1], 1u << ((d & 1u) * 16));
                }
                __syncthreads();
                // exclusive offsets in (digit, warp) order: element i of the scan is
                // hist[i % NW][i / NW]
                constexpr int kPer = NW * Shape::kDigits / NT;
                int v[kPer];
                int sum = 0;
#pragma unroll
                for (int e = 0; e < kPer; ++e) {
                    const int i = tid * kPer + e;
                    v[e] = hist[(i % NW) * Shape::kDigits + i / NW];
                    sum += v[e];
                }
                int tot = 0;
                const int incl = block_inclusive_scan(sum, s_warp_sums, &tot);
                int run = incl - sum;
#pragma unroll
                for (int e = 0; e < kPer; ++e) {
                    const int i = tid * kPer + e;
                    hist[(i % NW) * Shape::kDigits + i / NW] = (unsigned short)run;
                    run += v[e];
                }
                __syncthreads();
                // stable scatter of this warp's slice, 32 elements at a time, in order
                for (int c = rb; c < re; c += 32) {
                    const int i = c + lane;
                    const bool valid = i < re;
                    const unsigned key = valid ? kin[i] : 0u;
                    const unsigned short id = valid ? iin[i] : (unsigned short)0;
                    const int d = (int)((key >> shift) & 255u);
                    // lanes holding the same digit: one ballot per digit bit
                    unsigned peers = c + 32 <= re ? kFull : __ballot_sync(kFull, valid);
#pragma unroll
                    for (int b = 0; b < 8; ++b) {
                        if (b < nbits) {
                            const bool bit = (d >> b) & 1;
                            const unsigned m = __ballot_sync(kFull, bit);
                            peers &= bit ? m : ~m;
                        }
                    }
                    const int leader = __ffs(peers) - 1;
                    int base = 0;
                    if (lane == leader && valid) base = wh[d];
                    base = __shfl_sync(kFull, base, leader);
                    const int pos = base + __popc(peers & lanemask_lt());
                    __syncwarp();
                    if (lane == leader && valid) wh[d] = (unsigned short)(base + __popc(peers));
                    if (valid) {
                        kout[pos] = key;
                        iout[pos] = id;
                    }
                    __syncwarp();
                }
                __syncthreads();
                unsigned *tk = kin;
                kin = kout;
                kout = tk;
                unsigned short *ti = iin;
                iin = iout;
                iout = ti;
            }
            // run heads: thread tid owns positions [ib, ie) and the runs whose head lies
            // there; hidx[h] = position of head h, which is also C entry h of the row
            // (kept in the free ping-pong key buffer)
            const int E = (n + NT - 1) / NT;
            const int ib = min(n, tid * E);
            const int ie = min(n, ib + E);
            int heads = 0;
            for (int i = ib; i < ie; ++i) heads += (i == 0 || kin[i] != kin[i - 1]) ? 1 : 0;
            if (tid == 0) s_count = 0;
            int total = 0;
            const int hincl = block_inclusive_scan(heads, s_warp_sums, &total);
            if (tid == 0 && !g.soff && total != n_expect) atomicOr(&g.info->flags, kErrCountMismatch);
            if (tid == 0 && g.soff) {
                g.c_rpt[r] = total;
                nnz_acc += (unsigned long long)total;
            }
            int *hidx = reinterpret_cast<int *>(kout);
            const int hs = hincl - heads, he = hincl;
            for (int i = ib, h = hs; i < ie; ++i)
                if (i == 0 || kin[i] != kin[i - 1]) hidx[h++] = i;
            __syncthreads();
            auto run_end = [&](int h) { return h + 1 < total ? hidx[h + 1] : n; };
            // runs of kLongRun or more products are listed (in the histogram space, free
            // after the sort) for the warp-per-run fold
            int *long_runs = reinterpret_cast<int *>(hist);
            for (int h = hs; h < he; ++h)
                if (run_end(h) - hidx[h] >= kLongRun) long_runs[atomicAdd(&s_count, 1)] = h;
            __syncthreads();
            // product t's operands (t a sorted position)
            auto operands = [&](int t, T &a, T &b) {
                const int q = iin[t];
                const int o = own[q];
                const int k = s_b0[o] + q - (o ? s_incl[o - 1] : 0);
                a = __ldg(g.aval + a0 + o);
                b = __ldg(g.bval + k);
            };
            auto write_c = [&](int h, int t, S s) {
                if (h < n_expect) {
                    g.c_col[off + h] = (int)kin[t];
                    g.c_val[off + h] = AccT::fin(s);
                }
            };
            // long runs: one warp each.  The lanes load the operands of the next 32
            // products while the fold of the current 32 runs; lane 0 folds them in order
            // from shuffles, so the run costs about one FMA latency per product.
            const int n_long = s_count;
            for (int w = warp; w < n_long; w += NW) {
                const int h = long_runs[w];
                const int i0 = hidx[h], i1 = run_end(h);
                T a = T(0), b = T(0);
                if (i0 + lane < i1) operands(i0 + lane, a, b);
                S s = AccT::zero();
                for (int t = i0; t < i1; t += 32) {
                    T na = T(0), nb = T(0);
                    if (t + 32 + lane < i1) operands(t + 32 + lane, na, nb);
                    const int m = min(32, i1 - t);
#pragma unroll
                    for (int u = 0; u < 32; ++u) {
                        const T au = shfl(a, u), bu = shfl(b, u);
                        if (lane == 0 && u < m) s = AccT::step(s, au, bu);
                    }
                    a = na;
                    b = nb;
                }
                if (lane == 0) write_c(h, i0, s);
            }
            // short runs: this thread's own runs, packed steps (long ones skipped)
            fold_own_runs<T>(
                hs, he, kLongRun, [&](int h) { return hidx[h]; }, run_end,
                [&](int t, T &a, T &b, int &) { operands(t, a, b); },
                [&](int h, int t, int, S s) { write_c(h, t, s); });
            __syncthreads();
        }
    }
    if (!kNum || g.soff) block_add_u64(nnz_acc, &g.info->total_nnz);
}

// Device-side re-binning of a class list into kWays sub-lists (out + w*stride), with
// the row counts added to out_counts[w].  Row order inside a sub-list follows the
// warp-aggregated atomics, which is fine: every sub-list kernel schedules rows itself.
template <int kWays, typename Pick>
__global__ void k_split_list(const int *__restrict__ list, const int *count_ptr, Pick pick, int *out, int stride,
                             int *out_counts)
{
    const int count = *count_ptr;
    const int lane = lane_id();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i - lane < count; i += gridDim.x * blockDim.x) {
        const bool in = i < count;
        int r = 0, w = -1;
        if (in) {
            r = list[i];
            w = pick(r);
        }
#pragma unroll
        for (int c = 0; c < kWays; ++c) {
            const unsigned m = __ballot_sync(kFull, w == c);
            if (!m) continue;
            int b = 0;
            if (lane == 0) b = atomicAdd(&out_counts[c], __popc(m));
            b = __shfl_sync(kFull, b, 0);
            if (w == c) out[(size_t)c * stride + b + __popc(m & lanemask_lt())] = r;
        }
    }
}

// Numeric re-binning of the E1 rows by their output size (known after the symbolic
// phase): 0 = warp sort (at most kWsortFlopMax products, fewer than two products per
// output), 1 = warp hash (at most kSplitNnz outputs: hashing folds the many products
// per output cheaply), 2 = expand/sort/compress.
constexpr int kSplitNnz = 256;

struct PickE1 {
    const int *c_rpt;
    const int *row_flop;
    int sort_flop_max;
    __device__ int operator()(int r) const
    {
        const int nnz = c_rpt[r + 1] - c_rpt[r];
        const int f = row_flop[r];
        if (f <= sort_flop_max && f < 2 * nnz) return 0;
        return nnz <= kSplitNnz ? 1 : 2;
    }
};

// E1 rows of a one-pass call: 0 = staged (a staging slot of one or more products) with at
// most kE1OnePassFlopMax products, 1 = not staged, 2 = staged with more products.
struct PickStaged {
    const int *soff;
    const int *row_flop;
    __device__ int operator()(int r) const
    {
        if (soff[r + 1] <= soff[r]) return 1;
        return row_flop[r] <= kE1OnePassFlopMax ? 0 : 2;
    }
};

// E2 rows by size: 0 = mid shape (EscMid), 1 = large shape (EscLarge).
struct PickE2 {
    const int *arpt;
    const int *row_flop;
    __device__ int operator()(int r) const
    {
        const bool mid = row_flop[r] <= EscMid::kProducts && arpt[r + 1] - arpt[r] <= EscMid::kAEntries;
        return mid ? 0 : 1;
    }
};

// Orders a class list by product count, largest first, so that with dynamic row
// scheduling the longest rows start first (longest-processing-time order).  One CTA;
// lists longer than kLptMax stay as they are.
constexpr int kLptMax = 4096;

static __global__ void __launch_bounds__(1024) k_sort_heavy_first(int *list, const int *count_ptr,
                                                           const int *__restrict__ row_flop)
{
    // Rows are grouped by product count in quarter-octave buckets, largest first: one
    // histogram, one scan, one scatter.  Scheduling only needs the heavy rows early; the
    // order inside a bucket is free (every row's result is independent of it).
    constexpr int kBuckets = 128;
    __shared__ int s_rows[kLptMax];
    __shared__ unsigned char s_bucket[kLptMax];
    __shared__ int s_next[kBuckets];
    const int n = *count_ptr;
    if (n <= 1 || n > kLptMax) return;
    for (int i = threadIdx.x; i < kBuckets; i += blockDim.x) s_next[i] = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int r = list[i];
        const unsigned f = (unsigned)max(row_flop[r], 1);
        const int lz = 31 - __clz(f);  // floor(log2 f)
        const int frac = lz >= 2 ? (int)((f >> (lz - 2)) & 3u) : 0;
        const int b = kBuckets - 1 - min(kBuckets - 1, 4 * lz + frac);
        s_rows[i] = r;
        s_bucket[i] = (unsigned char)b;
        atomicAdd(&s_next[b], 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int b = 0; b < kBuckets; ++b) {
            const int c = s_next[b];
            s_next[b] = run;
            run += c;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) list[atomicAdd(&s_next[s_bucket[i]], 1)] = s_rows[i];
}

}  // namespace opsg
