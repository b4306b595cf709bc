// batch_rows.cuh — the persistent kernels of the batched SpGEMM (batch.cu).
//
// A batch's problems are laid out as block-diagonal segments (see batch.cu).  Instead of
// classifying each segment on its own and launching each class's kernels per segment, one
// setup kernel walks the rows of every segment of every problem and pushes each row into one
// of four global queues by its product count:
//   kQ128:  at most 128 products;
//   kQWarp: 129 .. warp_max (<= 512) products;
//   kQE1:   warp_max+1 .. 1,024 products (and at most 1,024 A entries);
//   kQMid:  1,025 .. 4,096 products (and at most 1,280 A entries).
// Rows beyond all four are only counted; a batch that has any runs the per-segment pipeline
// instead.  Each queue is then drained by ONE persistent kernel per phase that spans every
// problem: its warps (or CTAs) take rows through the queue's atomic cursor until it is
// empty, with the shape and occupancy of its row size:
//   symbolic  kQ128, kQWarp, kQE1: a warp per row, distinct columns counted in a shared-memory
//             hash table of 2 slots per product (256, 1,024, 2,048 slots);
//             kQMid: a 256-thread CTA per row, hash table of 2 slots per product (esc.cuh);
//   numeric   kQ128: a warp per row, register bitonic network of up to 128 keys, 8 warps per
//             CTA (wsort.cuh); kQWarp: the same with networks of up to 512 keys, 4 warps per
//             CTA; kQE1: a 128-thread CTA per row (besc.cuh, 1,024 keys); kQMid: a 256-thread
//             CTA per row (4,096 keys).
// The four kernels of a phase run concurrently on their own streams.  The numeric routines
// are the single-product kernels' (the same bits); every output entry is folded in
// ascending j.
//
// Replaces, for a batch, OpSparse's per-bin dispatch (src/opsparse/core_algo/spgemm/
// spgemm_phases.cu:52-121, 148-206), which launches each bin's kernel on its own stream for
// one matrix at a time.
#pragma once

#include "besc.cuh"
#include "wsort.cuh"

namespace opsg {

constexpr int kBatchQ128 = 128;       // rows of the kQ128 queue, at most (WsortShape<4>::kMax)
constexpr int kBatchWarpMax = 512;    // rows of the kQWarp queue, at most (WsortShape<16>::kMax)
constexpr int kBatchChunk = 8;        // warp-queue rows a warp takes per cursor step
constexpr int kBatchMaxSegs = 16;     // segments one persistent launch covers (their arguments sit in shared memory)
constexpr int kBatchCountThreads = 256;
static_assert(WsortShape<4>::kMax == kBatchQ128 && WsortShape<16>::kMax == kBatchWarpMax, "warp-queue capacities");
static_assert(EscMid::kProducts >= BescMidRank::kCap && EscMid::kAEntries >= BescMidRank::kAEntries, "kQMid rows fit both shapes");

enum BatchQueue : int { kQ128 = 0, kQWarp = 1, kQE1 = 2, kQMid = 3, kQBeyond = 4, kNumBatchQueues = 4 };

// Device-side state of a batch's queues.
struct BatchQueues {
    int count[kNumBatchQueues + 1];     // rows in each queue, and beyond them
    int cursor[2][kNumBatchQueues];     // [symbolic, numeric][queue]
    int flags;                          // kErr* bits of the setup kernel (a bad A column)
};

// Segment of global row gr: the last s with seg_row_base[s] <= gr.
__device__ __forceinline__ int batch_segment(const int *seg_row_base, int nseg, int gr)
{
    int lo = 0, hi = nseg;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (seg_row_base[mid] <= gr) lo = mid;
        else hi = mid;
    }
    return lo;
}

// One thread per global row (grid-stride): the row's products (into its segment's
// row_flop), empty rows' counts, and the queue each row joins (queue c holds its rows at
// queues[c * total_rows ..]).  Segment arguments come from segs (structure only).  Queue
// entries are global row numbers.
static __global__ void __launch_bounds__(256) k_batch_setup(const SpgemmArgs<double> *__restrict__ segs,
                                                            const int *__restrict__ seg_row_base, int nseg,
                                                            int total_rows, int warp_max, int *__restrict__ queues,
                                                            BatchQueues *q)
{
    const int lane = lane_id();
    for (long long g0 = (long long)blockIdx.x * blockDim.x; g0 < total_rows; g0 += (long long)gridDim.x * blockDim.x) {
        const int gr = (int)(g0 + threadIdx.x);
        int cls = -1;  // a BatchQueue
        if (gr < total_rows) {
            const int s = batch_segment(seg_row_base, nseg, gr);
            const SpgemmArgs<double> &g = segs[s];
            const int r = gr - seg_row_base[s];
            const int a0 = __ldg(g.arpt + r), a1 = __ldg(g.arpt + r + 1);
            long long flop = 0;
            bool bad = false;
            for (int p = a0; p < a1; p += 4) {
                int j[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) j[u] = p + u < a1 ? __ldg(g.acol + p + u) : -1;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (p + u >= a1) break;
                    if ((unsigned)j[u] < (unsigned)g.K) flop += __ldg(g.brpt + j[u] + 1) - __ldg(g.brpt + j[u]);
                    else bad = true;
                }
            }
            if (bad) atomicOr(&q->flags, kErrBadColumn);
            const int lenA = a1 - a0;
            const_cast<int *>(g.row_flop)[r] = flop > INT_MAX ? INT_MAX : (int)flop;
            if (flop == 0) g.c_rpt[r] = 0;
            else if (flop <= kBatchQ128) cls = kQ128;
            else if (flop <= warp_max) cls = kQWarp;
            else if (flop <= BescE1Batch::kCap && lenA <= BescE1Batch::kAEntries) cls = kQE1;
            else if (flop <= BescMidRank::kCap && lenA <= BescMidRank::kAEntries) cls = kQMid;
            else cls = kQBeyond;
        }
#pragma unroll
        for (int c = 0; c <= kQBeyond; ++c) {
            const unsigned mk = __ballot_sync(kFull, cls == c);
            if (!mk) continue;
            const int leader = __ffs(mk) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(&q->count[c], __popc(mk));
            base = __shfl_sync(kFull, base, leader);
            if (cls == c && c < kNumBatchQueues)
                queues[(size_t)c * total_rows + base + __popc(mk & lanemask_lt())] = gr;
        }
    }
}

// Copies the segment arguments and first rows into shared memory.
template <typename T>
__device__ __forceinline__ void batch_load_segs(const SpgemmArgs<T> *segs, const int *seg_row_base, int nseg,
                                                SpgemmArgs<T> *s_segs, int *s_base)
{
    for (int i = threadIdx.x; i < nseg; i += blockDim.x) s_segs[i] = segs[i];
    for (int i = threadIdx.x; i <= nseg; i += blockDim.x) s_base[i] = seg_row_base[i];
    __syncthreads();
}

// Distinct columns of a row (A entries [a0, a1)) by one warp in a hash table of 2^log_ts
// slots (at least 2 per product): windows of 32 A entries, kCountUnroll chunks of 32
// products with their column loads in flight together.  Returns the count on every lane.
__device__ __forceinline__ int warp_hash_count(const SpgemmArgs<double> &g, int a0, int a1, int *keys, int log_ts)
{
    const int lane = lane_id();
    for (int i = lane; i < (1 << log_ts); i += 32) keys[i] = kEmpty;
    __syncwarp();
    int cnt = 0;
    bool bad = false;
    for (int wa = a0; wa < a1; wa += 32) {
        const int q = wa + lane;
        int b0 = 0, bl = 0;
        if (q < a1) {
            const int j = __ldg(g.acol + q);
            b0 = __ldg(g.brpt + j);
            bl = __ldg(g.brpt + j + 1) - b0;
        }
        int incl = bl;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int t = __shfl_up_sync(kFull, incl, d);
            if (lane >= d) incl += t;
        }
        const int wtot = __shfl_sync(kFull, incl, 31);
        for (int c = 0; c < wtot; c += 32 * kCountUnroll) {
            int col[kCountUnroll];
#pragma unroll
            for (int u = 0; u < kCountUnroll; ++u) {
                const int p = c + u * 32 + lane;
                int lo = 0;
#pragma unroll
                for (int step = 16; step >= 1; step >>= 1) {
                    const int vv = __shfl_sync(kFull, incl, lo + step - 1);
                    if (vv <= p) lo += step;
                }
                const int o_incl = __shfl_sync(kFull, incl, lo);
                const int o_bl = __shfl_sync(kFull, bl, lo);
                const int o_b0 = __shfl_sync(kFull, b0, lo);
                col[u] = p < wtot ? __ldg(g.bcol + o_b0 + (p - (o_incl - o_bl))) : kEmpty;
            }
#pragma unroll
            for (int u = 0; u < kCountUnroll; ++u) {
                if (col[u] == kEmpty) continue;
                if ((unsigned)col[u] >= (unsigned)g.N) {
                    bad = true;
                    continue;
                }
                bool is_new = false;
                table_claim(keys, col[u], log_ts, &is_new, &g.info->flags);
                cnt += is_new ? 1 : 0;
            }
        }
    }
    if (__any_sync(kFull, bad) && lane == 0) atomicOr(&g.info->flags, kErrBadColumn);
    __syncwarp();
    return (int)__reduce_add_sync(kFull, (unsigned)cnt);
}

// Symbolic persistent kernel of a warp queue (rows of at most TMAX/2 products): every warp
// counts kBatchChunk rows per cursor step in its own table of at most TMAX slots.  Rows of
// at most 32 A entries whose B rows are long (16 or more products per A entry) and whose
// products fall within one window of consecutive columns are counted over a window bitmap
// in the same space instead (window_row_short, kernels.cuh), when it is large enough: a
// window of kWinBits columns, or twice that where the table space is 2 * kWinWords words
// (one marking OR per product and a sweep of the window's words, no hash probes).
template <int TMAX>
__global__ void __launch_bounds__(kBatchCountThreads) k_batch_count_rows(const SpgemmArgs<double> *__restrict__ segs,
                                                                         const int *__restrict__ seg_row_base,
                                                                         int nseg, const int *__restrict__ queue,
                                                                         const int *count, int *cursor)
{
    constexpr bool kWindow = TMAX >= kWinWords;  // the table's space holds the window bitmap
    constexpr int kWB = TMAX >= 2 * kWinWords ? 2 * kWinBits : kWinBits;  // window columns
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ SpgemmArgs<double> s_segs[kBatchMaxSegs];
    __shared__ int s_base[kBatchMaxSegs + 1];
    batch_load_segs<double>(segs, seg_row_base, nseg, s_segs, s_base);
    const int lane = lane_id();
    int *keys = reinterpret_cast<int *>(smem_raw) + (threadIdx.x >> 5) * TMAX;
    bool win_clean = false;  // the window bitmap is all-zero
    unsigned long long nnz_unused = 0;
    const int n = *count;
    for (;;) {
        int u0 = 0;
        if (lane == 0) u0 = atomicAdd(cursor, kBatchChunk);
        u0 = __shfl_sync(kFull, u0, 0);
        if (u0 >= n) break;
        const int u1 = min(n, u0 + kBatchChunk);
        for (int u = u0; u < u1; ++u) {
            const int gr = __ldg(queue + u);
            const int s = batch_segment(s_base, nseg, gr);
            const SpgemmArgs<double> &g = s_segs[s];
            const int r = gr - s_base[s];
            const int a0 = __ldg(g.arpt + r), a1 = __ldg(g.arpt + r + 1);
            const int flop = __ldg(g.row_flop + r);
            if (kWindow && flop >= 16 * (a1 - a0) && a1 - a0 <= 32) {
                const int nnz_b = __ldg(g.brpt + g.K);
                const bool bcol16 = ((size_t)g.bcol & 15) == 0;
                if (window_row_short<double, kWB>(g, r, a0, a1, nnz_b, bcol16, reinterpret_cast<unsigned *>(keys),
                                                  win_clean, nnz_unused))
                    continue;
            }
            win_clean = false;  // the hash table reuses the space
            const int log_ts = min(ceil_log2_c(TMAX), max(5, ceil_log2(2 * max(flop, 1))));
            const int tot = warp_hash_count(g, a0, a1, keys, log_ts);
            if (lane == 0) g.c_rpt[r] = tot;
            __syncwarp();
        }
    }
}

// Numeric persistent kernel of a warp queue (rows of at most 32*PMAX products): every warp
// takes kBatchChunk rows per step through the queue's cursor until it is empty.
template <int PMAX, typename T, typename KT>
__global__ void __launch_bounds__(WsortShape<PMAX>::kThreads, WsortShape<PMAX>::kMinBlocks)
    k_batch_warp_rows(const SpgemmArgs<T> *__restrict__ segs, const int *__restrict__ seg_row_base, int nseg,
                      const int *__restrict__ queue, const int *count, int *cursor)
{
    using Sh = WsortShape<PMAX>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ SpgemmArgs<T> s_segs[kBatchMaxSegs];
    __shared__ int s_base[kBatchMaxSegs + 1];
    batch_load_segs<T>(segs, seg_row_base, nseg, s_segs, s_base);
    const int lane = lane_id();
    const int warp = threadIdx.x >> 5;
    const WsortSmem<PMAX, true, T, KT> sm(smem_raw + (size_t)warp * Sh::template per_warp<true, T, KT>());
    const int n = *count;
    unsigned long long nnz_unused = 0;  // the counts were made by the symbolic phase
    for (;;) {
        int u0 = 0;
        if (lane == 0) u0 = atomicAdd(cursor, kBatchChunk);
        u0 = __shfl_sync(kFull, u0, 0);
        if (u0 >= n) break;
        const int u1 = min(n, u0 + kBatchChunk);
        for (int u = u0; u < u1; ++u) {
            const int gr = __ldg(queue + u);
            const int s = batch_segment(s_base, nseg, gr);
            wsort_process_row<PMAX, true, T, KT>(s_segs[s], gr - s_base[s], sm, nnz_unused);
        }
    }
}

// Persistent kernel of a CTA queue (rows of at most Shape::kCap products), one phase:
// every CTA takes one row per step through the queue's cursor until it is empty.  The
// symbolic phase writes each row's count to c_rpt.
template <typename Shape, bool kNum, typename T, typename KT>
__global__ void __launch_bounds__(Shape::kThreads, Shape::kMinBlocks)
    k_batch_cta_rows(const SpgemmArgs<T> *__restrict__ segs, const int *__restrict__ seg_row_base, int nseg,
                     const int *__restrict__ queue, const int *count, int *cursor)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ SpgemmArgs<T> s_segs[kBatchMaxSegs];
    __shared__ int s_base[kBatchMaxSegs + 1];
    __shared__ int s_warp_sums[32];
    __shared__ KT s_last[32];
    __shared__ int s_unit;
    __shared__ BescScratch s_sc;
    if (threadIdx.x == 0) s_sc.reset();
    batch_load_segs<T>(segs, seg_row_base, nseg, s_segs, s_base);
    const BescSmem<Shape, kNum, KT, T> sm(smem_raw);
    sm.init();
    const int n = *count;
    unsigned long long nnz_unused = 0;
    for (;;) {
        if (threadIdx.x == 0) s_unit = atomicAdd(cursor, 1);
        __syncthreads();
        const int u = s_unit;
        __syncthreads();
        if (u >= n) break;
        const int gr = __ldg(queue + u);
        const int s = batch_segment(s_base, nseg, gr);
        besc_row<Shape, kNum, T, KT>(s_segs[s], gr - s_base[s], sm, s_warp_sums, s_last, &s_sc, nnz_unused);
    }
}

// Symbolic persistent kernel of the kQMid queue: every CTA counts one row per cursor step
// in a shared-memory hash table (EscMid's symbolic shape).
static __global__ void __launch_bounds__(EscMid::kThreads, 1) k_batch_cta_count(const SpgemmArgs<double> *__restrict__ segs,
                                                                        const int *__restrict__ seg_row_base,
                                                                        int nseg, const int *__restrict__ queue,
                                                                        const int *count, int *cursor)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ SpgemmArgs<double> s_segs[kBatchMaxSegs];
    __shared__ int s_base[kBatchMaxSegs + 1];
    __shared__ int s_warp_sums[32];
    __shared__ int s_unit;
    __shared__ int s_count;
    batch_load_segs<double>(segs, seg_row_base, nseg, s_segs, s_base);
    int *table = reinterpret_cast<int *>(smem_raw);
    int *s_incl = table + EscMid::kTable;
    int *s_b0 = s_incl + EscMid::kAEntries;
    const int n = *count;
    for (;;) {
        if (threadIdx.x == 0) s_unit = atomicAdd(cursor, 1);
        __syncthreads();
        const int u = s_unit;
        __syncthreads();
        if (u >= n) break;
        const int gr = __ldg(queue + u);
        const int s = batch_segment(s_base, nseg, gr);
        const SpgemmArgs<double> &g = s_segs[s];
        const int r = gr - s_base[s];
        const int a0 = __ldg(g.arpt + r);
        const int lenA = __ldg(g.arpt + r + 1) - a0;
        const int flop = esc_scan_row<EscMid::kThreads, double>(g, a0, lenA, s_incl, s_b0, s_warp_sums);
        const int tot = esc_count_row<EscMid, double>(g, lenA, flop, table, s_incl, s_b0, &s_count);
        if (threadIdx.x == 0) g.c_rpt[r] = tot;
        __syncthreads();
    }
}

// Totals of each segment's scanned row pointers: out[s] = c_rpt_s[M_s].
template <typename T>
__global__ void k_batch_totals(const SpgemmArgs<T> *__restrict__ segs, int nseg, long long *out)
{
    for (int s = threadIdx.x; s < nseg; s += blockDim.x) out[s] = segs[s].c_rpt[segs[s].M];
}

}  // namespace opsg
