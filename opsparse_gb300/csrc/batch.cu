// batch.cu — many independent SpGEMMs C_b = A_b * B_b in one pass (no counterpart in
// OpSparse).
//
// Problems are grouped into segments whose total intermediate products (an upper bound on
// nnz(C)) fit int32.  Each segment is laid out on the device as one block-diagonal
// product: A_seg stacks the A_b with their columns shifted to select the B_b rows, and
// B_seg stacks the B_b with their own (local) columns.  A row of A_seg only reaches its
// own problem's rows of B_seg, so C_seg is the stack of the C_b, with local columns.  One
// row classification then covers every row of every problem in the segment (a global bin
// queue per row class), and the single-matrix kernels run unchanged on it.
//
// ops_batch_create runs the flop count, segmentation, gather, classification, symbolic
// phase and scan of every segment, and allocates all outputs.  ops_batch_execute runs the
// numeric phase of all segments (re-gathering A's and B's values, which may change between
// calls): the first call records it on the stream as a CUDA graph, later calls replay that
// graph with one cudaGraphLaunch.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <new>
#include <vector>

#include <cub/cub.cuh>

#include "batch_rows.cuh"
#include "common.cuh"
#include "internal.hpp"

using namespace opsg;
using namespace opsg_internal;

namespace {

struct Item {  // device copy of an ops_batch_item plus its placement in its segment
    int rows, cols_a, cols_b;
    long long a_nnz, b_nnz;
    const int *a_rpt, *a_col;
    const void *a_val;
    const int *b_rpt, *b_col;
    const void *b_val;
    int row_base;       // first row of the problem in its segment's A_seg / C_seg
    int k_base;         // first row of the problem's B block in B_seg
    long long a_base;   // first entry of the problem in A_seg
    long long b_base;   // first entry of the problem in B_seg
    long long c_rpt_base;  // first entry of the problem's rebased row_ptr in the result arena
};

struct Segment {
    int first, count;   // problems [first, first + count)
    int M, K, N;        // A_seg is M x K, B_seg is K x N
    long long a_nnz, b_nnz, flop;
    int *a_rpt = nullptr, *a_col = nullptr, *b_rpt = nullptr, *b_col = nullptr;
    void *a_val = nullptr, *b_val = nullptr;
    int *c_rpt = nullptr, *c_col = nullptr;
    void *c_val = nullptr;
    long long c_nnz = 0;
    ops_handle_s *h = nullptr;  // per-segment plan (classes, workspace); the per-segment path only
    int *row_flop = nullptr;    // persistent path: per-row products
    DevInfo *info = nullptr;    // persistent path: error flags of the segment's rows
};

// The batch helpers walk flattened element spaces: a segment's A entries (or rows, or
// B entries, or B rows) are the concatenation of its problems', and each problem's share
// starts at its base offset.  A CTA takes a fixed chunk of the space, finds the problem
// holding the chunk's first element by binary search over the bases, and walks forward,
// so a 65,536-row problem is spread over many CTAs instead of one.
enum Field : int { kFARpt, kFACol, kFBRpt, kFBCol };
constexpr int kFlatChunk = 4096;

template <int F>
__device__ __forceinline__ long long field_base(const Item &it)
{
    if constexpr (F == kFARpt) return it.row_base;
    if constexpr (F == kFACol) return it.a_base;
    if constexpr (F == kFBRpt) return it.k_base;
    return it.b_base;
}

// Last problem in [0, count) whose base is <= e (bases non-decreasing, base(0) == 0).
template <int F>
__device__ __forceinline__ int flat_problem(const Item *__restrict__ items, int count, long long e)
{
    int lo = 0, hi = count;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (field_base<F>(items[mid]) <= e) lo = mid;
        else hi = mid;
    }
    return lo;
}

// per-problem intermediate products, over all A entries of all problems (a_base holds the
// problems' offsets in that concatenation while this runs); flop[] must start at zero
__global__ void k_batch_flop(const Item *__restrict__ items, int n, long long total, unsigned long long *flop)
{
    __shared__ int s_b;
    const int lane = lane_id();
    for (long long c0 = (long long)blockIdx.x * kFlatChunk; c0 < total; c0 += (long long)gridDim.x * kFlatChunk) {
        if (threadIdx.x == 0) s_b = flat_problem<kFACol>(items, n, c0);
        __syncthreads();
        int b = s_b;
        const long long c1 = min(total, c0 + kFlatChunk);
        for (long long e0 = c0; e0 < c1; e0 += blockDim.x) {
            const long long e = e0 + threadIdx.x;
            unsigned long long f = 0;
            if (e < c1) {
                while (b + 1 < n && items[b + 1].a_base <= e) ++b;
                const Item &it = items[b];
                const int j = it.a_col[e - it.a_base];
                if ((unsigned)j < (unsigned)it.cols_a) f = (unsigned long long)(it.b_rpt[j + 1] - it.b_rpt[j]);
            }
            // a warp's entries almost always belong to one problem: one atomic then
            const int bb = e < c1 ? b : -1;
            const int b0 = __shfl_sync(kFull, bb, 0);
            if (__all_sync(kFull, bb == b0)) {
                unsigned long long sum = f;
#pragma unroll
                for (int d = 16; d >= 1; d >>= 1) sum += __shfl_xor_sync(kFull, sum, d);
                if (lane == 0 && b0 >= 0 && sum) atomicAdd(&flop[b0], sum);
            } else if (bb >= 0 && f) {
                atomicAdd(&flop[bb], f);
            }
        }
        __syncthreads();
    }
}

// Builds one segment's block-diagonal structure field F: A's row pointers (shifted to the
// problem's first A entry), A's columns (shifted to the problem's first B row), B's row
// pointers (shifted to its first B entry), or B's columns (local).
template <int F>
__global__ void k_batch_gather_field(const Item *__restrict__ items, int count, long long total, int *__restrict__ dst)
{
    __shared__ int s_b;
    for (long long c0 = (long long)blockIdx.x * kFlatChunk; c0 < total; c0 += (long long)gridDim.x * kFlatChunk) {
        if (threadIdx.x == 0) s_b = flat_problem<F>(items, count, c0);
        __syncthreads();
        int b = s_b;
        const long long c1 = min(total, c0 + kFlatChunk);
        for (long long e = c0 + threadIdx.x; e < c1; e += blockDim.x) {
            while (b + 1 < count && field_base<F>(items[b + 1]) <= e) ++b;
            const Item &it = items[b];
            const long long i = e - field_base<F>(it);
            if constexpr (F == kFARpt) dst[e] = (int)(it.a_base + it.a_rpt[i]);
            if constexpr (F == kFACol) dst[e] = it.a_col[i] + it.k_base;
            if constexpr (F == kFBRpt) dst[e] = (int)(it.b_base + it.b_rpt[i]);
            if constexpr (F == kFBCol) dst[e] = it.b_col[i];
        }
        __syncthreads();
    }
}

// Values of one segment's A (F = kFACol) or B (F = kFBCol) entries.
template <int F, typename T>
__global__ void k_batch_gather_vals(const Item *__restrict__ items, int count, long long total, T *__restrict__ dst)
{
    __shared__ int s_b;
    for (long long c0 = (long long)blockIdx.x * kFlatChunk; c0 < total; c0 += (long long)gridDim.x * kFlatChunk) {
        if (threadIdx.x == 0) s_b = flat_problem<F>(items, count, c0);
        __syncthreads();
        int b = s_b;
        const long long c1 = min(total, c0 + kFlatChunk);
        for (long long e = c0 + threadIdx.x; e < c1; e += blockDim.x) {
            while (b + 1 < count && field_base<F>(items[b + 1]) <= e) ++b;
            const Item &it = items[b];
            const T *src = static_cast<const T *>(F == kFACol ? it.a_val : it.b_val);
            dst[e] = src[e - field_base<F>(it)];
        }
        __syncthreads();
    }
}

// Last row pointers of a segment's A and B (their entry counts).
__global__ void k_batch_last(int *a_last, int a_nnz, int *b_last, int b_nnz)
{
    if (threadIdx.x == 0) {
        *a_last = a_nnz;
        *b_last = b_nnz;
    }
}

int flat_grid(long long total, int sms) { return (int)std::max<long long>(1, std::min<long long>((total + kFlatChunk - 1) / kFlatChunk, (long long)sms * 16)); }

// Per-problem row_ptr rebased to start at 0, written to the result arena.
__global__ void k_batch_rebase(const Item *__restrict__ items, int first, int count, const int *__restrict__ c_rpt,
                               int *out)
{
    for (int b = blockIdx.x; b < count; b += gridDim.x) {
        const Item it = items[first + b];
        const int base = c_rpt[it.row_base];
        for (int r = threadIdx.x; r <= it.rows; r += blockDim.x) out[it.c_rpt_base + r] = c_rpt[it.row_base + r] - base;
    }
}

}  // namespace

struct ops_batch_s {
    ops_handle_s *owner = nullptr;
    int dtype = OPS_F64;
    int n = 0;
    std::vector<Item> items;     // host copy
    Item *d_items = nullptr;
    std::vector<Segment> segs;
    int *c_rpt_arena = nullptr;  // all rebased per-problem row pointers
    void *mem = nullptr;         // one allocation for every segment's inputs and row pointers
    long long flop = 0, nnz = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t graph_stream = nullptr;
    // persistent path (batch_rows.cuh): one setup kernel, and one kernel per row-size queue
    // and phase, over every segment
    bool persistent = false;
    bool key64 = false;            // numeric sort keys need 64 bits (a segment has > 2^20 columns)
    void *pmem = nullptr;          // queues, per-row products, segment arguments, scan scratch
    opsg::BatchQueues *q = nullptr;
    int *queues = nullptr;         // [kNumBatchQueues][total_rows] global row numbers
    long long total_rows = 0;      // rows of every segment
    int queue_rows[kNumBatchQueues] = {};  // rows in each queue
    int grid[2][kNumBatchQueues] = {};     // [symbolic, numeric][queue] persistent grid sizes
    int *d_base = nullptr;         // [nseg + 1] first global row of each segment
    SpgemmArgs<double> *d_sym = nullptr;  // symbolic arguments per segment
    void *d_num = nullptr;         // numeric arguments per segment (SpgemmArgs<T>)
    long long *d_totals = nullptr;
    void *cub_tmp = nullptr;
    size_t cub_bytes = 0;
};

extern "C" int ops_spgemm_symbolic(ops_handle_t, int32_t, int32_t, int32_t, const int32_t *, const int32_t *, int64_t,
                                   const int32_t *, const int32_t *, int64_t, int32_t *, int64_t *, void *);
extern "C" int ops_spgemm_numeric(ops_handle_t, int, int32_t, int32_t, int32_t, const int32_t *, const int32_t *,
                                  const void *, const int32_t *, const int32_t *, const void *, const int32_t *,
                                  int32_t *, void *, void *);

namespace {

// A batch's device memory comes from its handle's stream-ordered pool, which keeps freed
// memory for the next allocation: a repeated batch of similar size (and the autotuner's
// candidate runs) maps no new memory for its outputs (tens of GB for thousands of
// problems) and creates no new segment handles.  The memory goes back to the pool here,
// after the device is idle, and the segment handles go to the handle's spares.
void batch_release(ops_batch_s *b)
{
    if (!b) return;
    cudaDeviceSynchronize();
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (Segment &s : b->segs) {
        if (s.h) b->owner->spare.push_back(s.h);
        if (s.c_col) cudaFreeAsync(s.c_col, 0);
        if (s.c_val) cudaFreeAsync(s.c_val, 0);
    }
    if (b->mem) cudaFreeAsync(b->mem, 0);
    if (b->pmem) cudaFreeAsync(b->pmem, 0);
    if (b->d_items) cudaFreeAsync(b->d_items, 0);
    cudaStreamSynchronize(0);
    (void)cudaGetLastError();
    delete b;
}

size_t seg_bytes(const Segment &s, size_t vs)
{
    return align_up(4 * ((size_t)s.M + 1), 256) + align_up(4 * (size_t)std::max(1LL, s.a_nnz), 256) +
           align_up(vs * (size_t)std::max(1LL, s.a_nnz), 256) + align_up(4 * ((size_t)s.K + 1), 256) +
           align_up(4 * (size_t)std::max(1LL, s.b_nnz), 256) + align_up(vs * (size_t)std::max(1LL, s.b_nnz), 256) +
           align_up(4 * ((size_t)s.M + 1), 256);
}


#define OPS_CHECK_B(expr)                  \
    do {                                   \
        int s_ = (expr);                   \
        if (s_ != OPS_OK) return bail(s_); \
    } while (0)

// C of one segment from the pool, its rebased per-problem row pointers.
int alloc_segment_c(ops_batch_s *b, ops_handle_s *h, Segment &s, size_t vs, cudaStream_t st)
{
    void *cc = nullptr, *cv = nullptr;
    cudaError_t e = cudaMallocFromPoolAsync(&cc, 4 * (size_t)std::max<long long>(s.c_nnz, 1), h->pool, st);
    if (e == cudaSuccess) e = cudaMallocFromPoolAsync(&cv, vs * (size_t)std::max<long long>(s.c_nnz, 1), h->pool, st);
    if (e != cudaSuccess) {
        if (cc) cudaFreeAsync(cc, st);
        return fail(h, status_of(e), "allocating a segment's C");
    }
    s.c_col = static_cast<int *>(cc);
    s.c_val = cv;
    if (s.count > 0) {
        k_batch_rebase<<<std::min(s.count, 65535), 256, 0, st>>>(b->d_items, s.first, s.count, s.c_rpt,
                                                                b->c_rpt_arena);
        OPS_CUDA(h, cudaGetLastError());
    }
    return OPS_OK;
}

// Per-segment path: every segment classified, counted and scanned by the single-product
// pipeline on a handle of its own.
int plan_segments(ops_batch_s *b, ops_handle_s *h, size_t vs, cudaStream_t st)
{
    for (Segment &s : b->segs) {
        int stt = OPS_OK;
        if (!h->spare.empty()) {
            s.h = h->spare.back();
            h->spare.pop_back();
        } else {
            stt = ops_handle_create(&s.h);
        }
        if (stt != OPS_OK) return fail(h, stt, "creating a segment handle");
        s.h->th = h->th;
        s.h->hash_slots = h->hash_slots;
        int64_t nnz = 0;
        stt = ops_spgemm_symbolic(s.h, s.M, s.K, s.N, s.a_rpt, s.a_col, s.a_nnz, s.b_rpt, s.b_col, s.b_nnz, s.c_rpt,
                                  &nnz, st);
        if (stt != OPS_OK) return fail(h, stt, std::string("segment symbolic: ") + s.h->last_error);
        s.c_nnz = nnz;
        b->nnz += nnz;
        OPS_CHECK(alloc_segment_c(b, h, s, vs, st));
    }
    return OPS_OK;
}

template <typename KernelT>
int occupancy_grid(ops_handle_s *h, KernelT kernel, int threads, size_t smem)
{
    int per_sm = 0;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess) {
        (void)cudaGetLastError();
        per_sm = 1;
    }
    return std::max(1, per_sm) * h->num_sms;
}

// Arguments of one segment's product.
template <typename T>
SpgemmArgs<T> seg_args(const Segment &s)
{
    SpgemmArgs<T> g{};
    g.arpt = s.a_rpt;
    g.acol = s.a_col;
    g.aval = static_cast<const T *>(s.a_val);
    g.brpt = s.b_rpt;
    g.bcol = s.b_col;
    g.bval = static_cast<const T *>(s.b_val);
    g.M = s.M;
    g.K = s.K;
    g.N = s.N;
    g.row_flop = s.row_flop;
    g.c_rpt = s.c_rpt;
    g.c_col = s.c_col;
    g.c_val = static_cast<T *>(s.c_val);
    g.info = s.info;
    g.soff = nullptr;
    return g;
}

// The persistent kernel of queue c for one phase, on stream s.  Grid sizes are the
// kernel's occupancy on every SM, computed on first use.
template <typename KernelT, typename T>
int launch_queue(ops_batch_s *b, int phase, int c, KernelT kernel, int threads, size_t smem, const SpgemmArgs<T> *args,
                 cudaStream_t s)
{
    ops_handle_s *h = b->owner;
    int &grid = b->grid[phase][c];
    if (!grid) grid = occupancy_grid(h, kernel, threads, smem);
    kernel<<<grid, threads, smem, s>>>(args, b->d_base, (int)b->segs.size(), b->queues + (size_t)c * b->total_rows,
                                       &b->q->count[c], &b->q->cursor[phase][c]);
    OPS_CUDA(h, cudaGetLastError());
    return OPS_OK;
}

// One phase of the persistent path: the kernel of every non-empty queue, each on a stream
// of its own forked from st and joined back into it, so the queues share the GPU and none
// waits for the tail of another.
template <typename LaunchOne>
int fork_queues(ops_batch_s *b, cudaStream_t st, LaunchOne launch_one)
{
    ops_handle_s *h = b->owner;
    static_assert(kNumBatchQueues <= kNumClasses, "one handle stream per queue");
    OPS_CUDA(h, cudaEventRecord(h->ev_fork, st));
    for (int c = 0; c < kNumBatchQueues; ++c) {
        if (b->queue_rows[c] <= 0) continue;
        cudaStream_t s = h->side[c];
        OPS_CUDA(h, cudaStreamWaitEvent(s, h->ev_fork, 0));
        OPS_CHECK(launch_one(c, s));
        OPS_CUDA(h, cudaEventRecord(h->ev_join[c], s));
        OPS_CUDA(h, cudaStreamWaitEvent(st, h->ev_join[c], 0));
    }
    return OPS_OK;
}

int launch_batch_symbolic(ops_batch_s *b, cudaStream_t st)
{
    const SpgemmArgs<double> *a = b->d_sym;
    constexpr int W = kBatchCountThreads / 32;
    return fork_queues(b, st, [&](int c, cudaStream_t s) {
        switch (c) {
            case kQ128:
                return launch_queue(b, 0, c, k_batch_count_rows<2 * kBatchQ128>, kBatchCountThreads,
                                    (size_t)W * 2 * kBatchQ128 * sizeof(int), a, s);
            case kQWarp:  // twice the table a row needs: room for the wide column window
                return launch_queue(b, 0, c, k_batch_count_rows<4 * kBatchWarpMax>, kBatchCountThreads,
                                    (size_t)W * 4 * kBatchWarpMax * sizeof(int), a, s);
            case kQE1:
                return launch_queue(b, 0, c, k_batch_count_rows<2 * BescE1Batch::kCap>, kBatchCountThreads,
                                    (size_t)W * 2 * BescE1Batch::kCap * sizeof(int), a, s);
            default:  // the table and the A-entry scan of EscMid's symbolic shape
                return launch_queue(b, 0, c, k_batch_cta_count, EscMid::kThreads,
                                    (size_t)EscMid::kTable * 4 + (size_t)EscMid::kAEntries * 8, a, s);
        }
    });
}

template <typename T, typename KT>
int launch_batch_numeric(ops_batch_s *b, cudaStream_t st)
{
    static_assert(sizeof(SpgemmArgs<T>) == sizeof(SpgemmArgs<double>), "argument layout is the value type's");
    const SpgemmArgs<T> *a = static_cast<const SpgemmArgs<T> *>(b->d_num);
    return fork_queues(b, st, [&](int c, cudaStream_t s) {
        switch (c) {
            case kQ128:
                return launch_queue(b, 1, c, k_batch_warp_rows<4, T, KT>, WsortShape<4>::kThreads,
                                    WsortShape<4>::smem<true, T, KT>(), a, s);
            case kQWarp:
                return launch_queue(b, 1, c, k_batch_warp_rows<16, T, KT>, WsortShape<16>::kThreads,
                                    WsortShape<16>::smem<true, T, KT>(), a, s);
            case kQE1:
                return launch_queue(b, 1, c, k_batch_cta_rows<BescE1Batch, true, T, KT>, BescE1Batch::kThreads,
                                    BescE1Batch::smem<true, KT, T>(), a, s);
            default:
                return launch_queue(b, 1, c, k_batch_cta_rows<BescMidRank, true, T, KT>, BescMidRank::kThreads,
                                    BescMidRank::smem<true, KT, T>(), a, s);
        }
    });
}

// Persistent path: when the batch has at most kBatchMaxSegs segments and every row fits one
// of the queues (batch_rows.cuh), classifies every row of every segment with one kernel,
// counts them with one persistent kernel per queue, scans each segment's row pointers and
// allocates C.  Leaves `used` false, having changed nothing a per-segment plan needs, when
// the batch does not qualify.
int plan_persistent(ops_batch_s *b, ops_handle_s *h, size_t vs, cudaStream_t st, bool &used)
{
    used = false;
    const int nseg = (int)b->segs.size();
    if (!h->batch_persistent || nseg == 0 || nseg > kBatchMaxSegs) return OPS_OK;
    long long total_rows = 0;
    int max_m = 0, max_n = 0;
    for (const Segment &s : b->segs) {
        total_rows += s.M;
        max_m = std::max(max_m, s.M);
        max_n = std::max(max_n, s.N);
    }
    if (total_rows == 0 || total_rows > INT_MAX) return OPS_OK;
    size_t cub_bytes = 0;
    OPS_CUDA(h, cub::DeviceScan::ExclusiveSum(nullptr, cub_bytes, (int *)nullptr, (int *)nullptr, max_m + 1));
    const size_t A = 256;
    size_t bytes = align_up(sizeof(BatchQueues), A) + align_up(4 * (size_t)kNumBatchQueues * total_rows, A) +
                   align_up(4 * (size_t)(nseg + 1), A) + 2 * align_up(sizeof(SpgemmArgs<double>) * nseg, A) +
                   align_up(8 * (size_t)nseg, A) + align_up(cub_bytes, A) + align_up(sizeof(DevInfo) * nseg, A);
    for (const Segment &s : b->segs) bytes += align_up(4 * (size_t)std::max(1, s.M), A);
    void *pm = nullptr;
    OPS_CUDA(h, cudaMallocFromPoolAsync(&pm, bytes, h->pool, st));
    b->pmem = pm;
    unsigned char *m = static_cast<unsigned char *>(pm);
    auto carve = [&](size_t n) {
        unsigned char *p = m;
        m += align_up(n, A);
        return p;
    };
    b->total_rows = total_rows;
    b->q = reinterpret_cast<BatchQueues *>(carve(sizeof(BatchQueues)));
    b->queues = reinterpret_cast<int *>(carve(4 * (size_t)kNumBatchQueues * total_rows));
    b->d_base = reinterpret_cast<int *>(carve(4 * (size_t)(nseg + 1)));
    b->d_sym = reinterpret_cast<SpgemmArgs<double> *>(carve(sizeof(SpgemmArgs<double>) * nseg));
    b->d_num = carve(sizeof(SpgemmArgs<double>) * nseg);
    b->d_totals = reinterpret_cast<long long *>(carve(8 * (size_t)nseg));
    b->cub_tmp = carve(cub_bytes);
    b->cub_bytes = cub_bytes;
    DevInfo *infos = reinterpret_cast<DevInfo *>(carve(sizeof(DevInfo) * nseg));
    std::vector<int> base(nseg + 1, 0);
    std::vector<SpgemmArgs<double>> sym(nseg);
    for (int i = 0; i < nseg; ++i) {
        Segment &s = b->segs[i];
        s.row_flop = reinterpret_cast<int *>(carve(4 * (size_t)std::max(1, s.M)));
        s.info = infos + i;
        base[i + 1] = base[i] + s.M;
        sym[i] = seg_args<double>(s);
    }
    // pageable copies: the source is staged before the call returns
    OPS_CUDA(h, cudaMemcpyAsync(b->d_base, base.data(), 4 * (size_t)(nseg + 1), cudaMemcpyHostToDevice, st));
    OPS_CUDA(h, cudaMemcpyAsync(b->d_sym, sym.data(), sizeof(SpgemmArgs<double>) * nseg, cudaMemcpyHostToDevice, st));
    OPS_CUDA(h, cudaMemsetAsync(b->q, 0, sizeof(BatchQueues), st));
    OPS_CUDA(h, cudaMemsetAsync(infos, 0, sizeof(DevInfo) * nseg, st));
    for (const Segment &s : b->segs) OPS_CUDA(h, cudaMemsetAsync(s.c_rpt + s.M, 0, sizeof(int), st));
    const int warp_max = std::max(kBatchQ128, std::min(kBatchWarpMax, h->batch_warp_max));
    k_batch_setup<<<(int)std::min<long long>((total_rows + 255) / 256, (long long)h->num_sms * 16), 256, 0, st>>>(
        b->d_sym, b->d_base, nseg, (int)total_rows, warp_max, b->queues, b->q);
    OPS_CUDA(h, cudaGetLastError());
    BatchQueues hq{};
    OPS_CUDA(h, cudaMemcpyAsync(&hq, b->q, sizeof(BatchQueues), cudaMemcpyDeviceToHost, st));
    OPS_CUDA(h, cudaStreamSynchronize(st));
    if (hq.flags & kErrBadColumn) return fail(h, OPS_INVALID_CSR, "A has a column index outside [0, cols)");
    for (int c = 0; c < kNumBatchQueues; ++c) b->queue_rows[c] = hq.count[c];
    if (hq.count[kQBeyond] > 0) {  // rows beyond the queues: the per-segment pipeline takes the batch
        OPS_CUDA(h, cudaFreeAsync(pm, st));
        b->pmem = nullptr;
        for (Segment &s : b->segs) {
            s.row_flop = nullptr;
            s.info = nullptr;
        }
        return OPS_OK;
    }
    // symbolic: one persistent kernel per queue, then each segment's scan
    OPS_CHECK(launch_batch_symbolic(b, st));
    for (const Segment &s : b->segs) {
        size_t cb = cub_bytes;
        OPS_CUDA(h, cub::DeviceScan::ExclusiveSum(b->cub_tmp, cb, s.c_rpt, s.c_rpt, s.M + 1, st));
    }
    k_batch_totals<double><<<1, 64, 0, st>>>(b->d_sym, nseg, b->d_totals);
    OPS_CUDA(h, cudaGetLastError());
    std::vector<long long> totals(nseg);
    std::vector<DevInfo> hinfo(nseg);
    OPS_CUDA(h, cudaMemcpyAsync(totals.data(), b->d_totals, 8 * (size_t)nseg, cudaMemcpyDeviceToHost, st));
    OPS_CUDA(h, cudaMemcpyAsync(hinfo.data(), infos, sizeof(DevInfo) * nseg, cudaMemcpyDeviceToHost, st));
    OPS_CUDA(h, cudaStreamSynchronize(st));
    for (int i = 0; i < nseg; ++i) {
        if (hinfo[i].flags & kErrBadColumn) return fail(h, OPS_INVALID_CSR, "B has a column index outside [0, cols)");
        if (hinfo[i].flags & kErrProbeLimit) return fail(h, OPS_PROBE_LIMIT, "symbolic hash table overflow");
        if (totals[i] > INT_MAX || totals[i] < 0) return fail(h, OPS_INT32_OVERFLOW, "a segment's nnz exceeds INT32_MAX");
    }
    // C of every segment; numeric arguments
    std::vector<SpgemmArgs<double>> num(nseg);
    for (int i = 0; i < nseg; ++i) {
        Segment &s = b->segs[i];
        s.c_nnz = totals[i];
        b->nnz += s.c_nnz;
        OPS_CHECK(alloc_segment_c(b, h, s, vs, st));
        num[i] = seg_args<double>(s);  // the value pointers are reinterpreted by the value type
    }
    OPS_CUDA(h, cudaMemcpyAsync(b->d_num, num.data(), sizeof(SpgemmArgs<double>) * nseg, cudaMemcpyHostToDevice, st));
    b->key64 = max_n > (1 << (32 - BescMidRank::kIdBits));  // the widest product index of the numeric keys
    b->persistent = true;
    used = true;
    return OPS_OK;
}

}  // namespace

extern "C" int ops_batch_create(ops_handle_t h, int dtype, int32_t count, const ops_batch_item *items,
                                ops_batch_t *out, void *stream)
{
    if (!h || !out || count < 0 || (count > 0 && !items)) return OPS_INVALID_ARGUMENT;
    if (dtype != OPS_F64 && dtype != OPS_F32) return fail(h, OPS_INVALID_ARGUMENT, "unknown dtype");
    *out = nullptr;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t vs = dtype == OPS_F64 ? 8 : 4;
    ops_batch_s *b = new (std::nothrow) ops_batch_s();
    if (!b) return OPS_EXCEPTION;
    b->owner = h;
    b->dtype = dtype;
    b->n = count;
    b->items.resize(count);
    for (int i = 0; i < count; ++i) {
        const ops_batch_item &s = items[i];
        if (s.rows < 0 || s.cols_a < 0 || s.cols_b < 0 || s.a_nnz < 0 || s.b_nnz < 0 || (s.rows > 0 && !s.a_rpt) ||
            (s.cols_a > 0 && !s.b_rpt) || (s.a_nnz > 0 && (!s.a_col || !s.a_val)) ||
            (s.b_nnz > 0 && (!s.b_col || !s.b_val))) {
            batch_release(b);
            return fail(h, OPS_INVALID_ARGUMENT, "bad batch item " + std::to_string(i));
        }
        Item &it = b->items[i];
        it.rows = s.rows;
        it.cols_a = s.cols_a;
        it.cols_b = s.cols_b;
        it.a_nnz = s.a_nnz;
        it.b_nnz = s.b_nnz;
        it.a_rpt = s.a_rpt;
        it.a_col = s.a_col;
        it.a_val = s.a_val;
        it.b_rpt = s.b_rpt;
        it.b_col = s.b_col;
        it.b_val = s.b_val;
    }
    auto bail = [&](int status) {
        batch_release(b);
        return status;
    };
    // 1. per-problem products (device), then segmentation on the host
    std::vector<unsigned long long> flop(std::max(count, 1), 0ull);
    long long total_a = 0;
    for (Item &it : b->items) {  // offsets of the problems' A entries in one concatenation
        it.a_base = total_a;
        total_a += it.a_nnz;
    }
    {
        void *p = nullptr;
        cudaError_t e = cudaMallocFromPoolAsync(&p, sizeof(Item) * std::max(count, 1), h->pool, st);
        if (e != cudaSuccess) return bail(fail(h, status_of(e), "allocating batch descriptors"));
        b->d_items = static_cast<Item *>(p);
        void *f = nullptr;
        e = cudaMallocFromPoolAsync(&f, sizeof(unsigned long long) * std::max(count, 1), h->pool, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_items, b->items.data(), sizeof(Item) * count, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(f, 0, sizeof(unsigned long long) * std::max(count, 1), st);
        if (e == cudaSuccess && count > 0 && total_a > 0) {
            k_batch_flop<<<flat_grid(total_a, h->num_sms), 256, 0, st>>>(b->d_items, count, total_a,
                                                                      static_cast<unsigned long long *>(f));
            e = cudaGetLastError();
        }
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(flop.data(), f, sizeof(unsigned long long) * count, cudaMemcpyDeviceToHost, st);
        if (f) cudaFreeAsync(f, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            return bail(fail(h, status_of(e), std::string("batch flop count: ") + cudaGetErrorString(e)));
        }
    }
    const long long kLimit = 0x7fff0000LL;  // products (>= nnz(C)), rows and nnz per segment stay in int32
    int first = 0;
    while (first < count) {
        Segment s{};
        s.first = first;
        long long M = 0, K = 0, an = 0, bn = 0, fl = 0;
        int N = 0, i = first;
        for (; i < count; ++i) {
            const Item &it = b->items[i];
            const long long f = (long long)flop[i];
            if (i > first && (fl + f > kLimit || M + it.rows > kLimit || K + it.cols_a > kLimit ||
                              an + it.a_nnz > kLimit || bn + it.b_nnz > kLimit))
                break;
            if (f > kLimit || it.a_nnz > kLimit || it.b_nnz > kLimit)
                return bail(fail(h, OPS_INT32_OVERFLOW, "a batch item exceeds the int32 limits of one product"));
            Item &w = b->items[i];
            w.row_base = (int)M;
            w.k_base = (int)K;
            w.a_base = an;
            w.b_base = bn;
            M += it.rows;
            K += it.cols_a;
            an += it.a_nnz;
            bn += it.b_nnz;
            fl += f;
            N = std::max(N, it.cols_b);
        }
        s.count = i - first;
        s.M = (int)M;
        s.K = (int)K;
        s.N = N;
        s.a_nnz = an;
        s.b_nnz = bn;
        s.flop = fl;
        b->flop += fl;
        b->segs.push_back(s);
        first = i;
    }
    // result row_ptr offsets
    long long rb = 0;
    for (Item &it : b->items) {
        it.c_rpt_base = rb;
        rb += it.rows + 1;
    }
    // 2. one allocation for every segment's inputs and row pointers plus the rebased arena
    size_t total = align_up(4 * (size_t)std::max(1LL, rb), 256);
    for (const Segment &s : b->segs) total += seg_bytes(s, vs);
    {
        cudaError_t e = cudaMallocFromPoolAsync(&b->mem, total, h->pool, st);
        if (e != cudaSuccess) return bail(fail(h, status_of(e), "allocating batch arena"));
        e = cudaMemcpyAsync(b->d_items, b->items.data(), sizeof(Item) * count, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return bail(fail(h, status_of(e), "copying batch descriptors"));
    }
    unsigned char *m = static_cast<unsigned char *>(b->mem);
    b->c_rpt_arena = reinterpret_cast<int *>(m);
    m += align_up(4 * (size_t)std::max(1LL, rb), 256);
    for (Segment &s : b->segs) {
        s.a_rpt = reinterpret_cast<int *>(m);
        m += align_up(4 * ((size_t)s.M + 1), 256);
        s.a_col = reinterpret_cast<int *>(m);
        m += align_up(4 * (size_t)std::max(1LL, s.a_nnz), 256);
        s.a_val = m;
        m += align_up(vs * (size_t)std::max(1LL, s.a_nnz), 256);
        s.b_rpt = reinterpret_cast<int *>(m);
        m += align_up(4 * ((size_t)s.K + 1), 256);
        s.b_col = reinterpret_cast<int *>(m);
        m += align_up(4 * (size_t)std::max(1LL, s.b_nnz), 256);
        s.b_val = m;
        m += align_up(vs * (size_t)std::max(1LL, s.b_nnz), 256);
        s.c_rpt = reinterpret_cast<int *>(m);
        m += align_up(4 * ((size_t)s.M + 1), 256);
        // 3. structure and last row pointers (no host sync)
        k_batch_last<<<1, 32, 0, st>>>(s.a_rpt + s.M, (int)s.a_nnz, s.b_rpt + s.K, (int)s.b_nnz);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess && s.count > 0) {
            const Item *its = b->d_items + s.first;
            const int sms = h->num_sms;
            if (s.M) k_batch_gather_field<kFARpt><<<flat_grid(s.M, sms), 256, 0, st>>>(its, s.count, s.M, s.a_rpt);
            if (s.a_nnz)
                k_batch_gather_field<kFACol><<<flat_grid(s.a_nnz, sms), 256, 0, st>>>(its, s.count, s.a_nnz, s.a_col);
            if (s.K) k_batch_gather_field<kFBRpt><<<flat_grid(s.K, sms), 256, 0, st>>>(its, s.count, s.K, s.b_rpt);
            if (s.b_nnz)
                k_batch_gather_field<kFBCol><<<flat_grid(s.b_nnz, sms), 256, 0, st>>>(its, s.count, s.b_nnz, s.b_col);
            e = cudaGetLastError();
        }
        if (e != cudaSuccess) return bail(fail(h, status_of(e), std::string("batch gather: ") + cudaGetErrorString(e)));
    }
    // 4. classification, symbolic phase, scan and C: one setup kernel and one persistent
    // kernel per row-size queue over every segment, or segment by segment when some row is
    // beyond the queues
    bool persistent = false;
    OPS_CHECK_B(plan_persistent(b, h, vs, st, persistent));
    if (!persistent) OPS_CHECK_B(plan_segments(b, h, vs, st));
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return bail(fail(h, status_of(e), "batch create"));
    *out = b;
    return OPS_OK;
}

namespace {

// Values of every segment's A and B gathered from the problems' arrays.
int gather_values(ops_batch_s *b, cudaStream_t st)
{
    ops_handle_s *h = b->owner;
    for (Segment &s : b->segs) {
        if (s.count == 0) continue;
        const Item *its = b->d_items + s.first;
        const int sms = h->num_sms;
        if (b->dtype == OPS_F64) {
            if (s.a_nnz)
                k_batch_gather_vals<kFACol, double><<<flat_grid(s.a_nnz, sms), 256, 0, st>>>(
                    its, s.count, s.a_nnz, static_cast<double *>(s.a_val));
            if (s.b_nnz)
                k_batch_gather_vals<kFBCol, double><<<flat_grid(s.b_nnz, sms), 256, 0, st>>>(
                    its, s.count, s.b_nnz, static_cast<double *>(s.b_val));
        } else {
            if (s.a_nnz)
                k_batch_gather_vals<kFACol, float><<<flat_grid(s.a_nnz, sms), 256, 0, st>>>(
                    its, s.count, s.a_nnz, static_cast<float *>(s.a_val));
            if (s.b_nnz)
                k_batch_gather_vals<kFBCol, float><<<flat_grid(s.b_nnz, sms), 256, 0, st>>>(
                    its, s.count, s.b_nnz, static_cast<float *>(s.b_val));
        }
        OPS_CUDA(h, cudaGetLastError());
    }
    return OPS_OK;
}

int record_numeric(ops_batch_s *b, cudaStream_t st)
{
    ops_handle_s *h = b->owner;
    OPS_CHECK(gather_values(b, st));
    if (b->persistent) {
        // cursors and flags of the numeric pass start at zero
        OPS_CUDA(h, cudaMemsetAsync(b->q->cursor[1], 0, sizeof(b->q->cursor[1]), st));
        OPS_CUDA(h, cudaMemsetAsync(b->segs[0].info, 0, sizeof(DevInfo) * b->segs.size(), st));
        if (b->dtype == OPS_F64)
            return b->key64 ? launch_batch_numeric<double, unsigned long long>(b, st)
                            : launch_batch_numeric<double, unsigned>(b, st);
        return b->key64 ? launch_batch_numeric<float, unsigned long long>(b, st)
                        : launch_batch_numeric<float, unsigned>(b, st);
    }
    for (Segment &s : b->segs) {
        if (s.count == 0) continue;
        const int stt = ops_spgemm_numeric(s.h, b->dtype, s.M, s.K, s.N, s.a_rpt, s.a_col, s.a_val, s.b_rpt, s.b_col,
                                           s.b_val, s.c_rpt, s.c_col, s.c_val, st);
        if (stt != OPS_OK) return fail(h, stt, std::string("segment numeric: ") + s.h->last_error);
    }
    return OPS_OK;
}

}  // namespace

extern "C" int ops_batch_execute(ops_batch_t b, int use_graph, void *stream)
{
    if (!b) return OPS_INVALID_ARGUMENT;
    ops_handle_s *h = b->owner;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (!use_graph) return record_numeric(b, st);
    if (b->exec && b->graph_stream == st) {
        OPS_CUDA(h, cudaGraphLaunch(b->exec, st));
        return OPS_OK;
    }
    if (!st) return fail(h, OPS_INVALID_ARGUMENT, "graph replay needs a created stream, not the legacy stream");
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    OPS_CUDA(h, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const int rec = record_numeric(b, st);
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(st, &g);
    if (rec != OPS_OK) {
        if (g) cudaGraphDestroy(g);
        return rec;
    }
    if (ec != cudaSuccess) {
        (void)cudaGetLastError();
        return fail(h, status_of(ec), std::string("capturing the batch: ") + cudaGetErrorString(ec));
    }
    b->graph = g;
    OPS_CUDA(h, cudaGraphInstantiate(&b->exec, g, 0));
    b->graph_stream = st;
    OPS_CUDA(h, cudaGraphLaunch(b->exec, st));
    return OPS_OK;
}

extern "C" int ops_batch_check(ops_batch_t b, void *stream)
{
    if (!b) return OPS_INVALID_ARGUMENT;
    if (b->persistent) {
        std::vector<DevInfo> hinfo(b->segs.size());
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        OPS_CUDA(b->owner, cudaMemcpyAsync(hinfo.data(), b->segs[0].info, sizeof(DevInfo) * hinfo.size(),
                                           cudaMemcpyDeviceToHost, st));
        OPS_CUDA(b->owner, cudaStreamSynchronize(st));
        for (const DevInfo &d : hinfo) {
            if (d.flags & kErrBadColumn) return fail(b->owner, OPS_INVALID_CSR, "B has a column index outside [0, cols)");
            if (d.flags & kErrCountMismatch)
                return fail(b->owner, OPS_COUNT_MISMATCH, "numeric found a different nnz than symbolic");
            if (d.flags & kErrProbeLimit) return fail(b->owner, OPS_PROBE_LIMIT, "hash table overflow");
        }
        return OPS_OK;
    }
    for (Segment &s : b->segs) {
        if (s.count == 0) continue;
        const int stt = ops_spgemm_check(s.h, stream);
        if (stt != OPS_OK) return fail(b->owner, stt, s.h->last_error);
    }
    return OPS_OK;
}

extern "C" int ops_batch_result(ops_batch_t b, int32_t index, int32_t **c_rpt, int32_t **c_col, void **c_val,
                                int64_t *c_nnz)
{
    if (!b || index < 0 || index >= b->n || !c_rpt || !c_col || !c_val || !c_nnz) return OPS_INVALID_ARGUMENT;
    const Item &it = b->items[index];
    const Segment *seg = nullptr;
    for (const Segment &s : b->segs)
        if (index >= s.first && index < s.first + s.count) seg = &s;
    if (!seg) return OPS_INVALID_ARGUMENT;
    int base = 0, end = 0;
    OPS_CUDA(b->owner, cudaMemcpy(&base, seg->c_rpt + it.row_base, sizeof(int), cudaMemcpyDeviceToHost));
    OPS_CUDA(b->owner, cudaMemcpy(&end, seg->c_rpt + it.row_base + it.rows, sizeof(int), cudaMemcpyDeviceToHost));
    const size_t vs = b->dtype == OPS_F64 ? 8 : 4;
    *c_rpt = b->c_rpt_arena + it.c_rpt_base;
    *c_col = seg->c_col + base;
    *c_val = static_cast<unsigned char *>(seg->c_val) + vs * (size_t)base;
    *c_nnz = end - base;
    return OPS_OK;
}

extern "C" int ops_batch_info(ops_batch_t b, int32_t *segments, int64_t *flop, int64_t *nnz)
{
    if (!b) return OPS_INVALID_ARGUMENT;
    if (segments) *segments = (int32_t)b->segs.size();
    if (flop) *flop = b->flop;
    if (nnz) *nnz = b->nnz;
    return OPS_OK;
}

extern "C" int ops_batch_queues(ops_batch_t b, int32_t *persistent, int64_t *warp_rows, int64_t *cta_rows)
{
    if (!b || !persistent || !warp_rows || !cta_rows) return OPS_INVALID_ARGUMENT;
    *persistent = b->persistent ? 1 : 0;
    *warp_rows = b->persistent ? (int64_t)b->queue_rows[kQ128] + b->queue_rows[kQWarp] : 0;
    *cta_rows = b->persistent ? (int64_t)b->queue_rows[kQE1] + b->queue_rows[kQMid] : 0;
    return OPS_OK;
}

extern "C" int ops_batch_destroy(ops_batch_t b)
{
    batch_release(b);
    return OPS_OK;
}

// ---------------------------------------------------------------------- autotuner ----
// Coordinate descent over every field of ops_tuning: the row-class thresholds {R8, R16,
// R32, W, E1, E2}, the warp-hash table's slots per output entry (hash-table size), the
// batch plan (persistent kernels over row-size queues, or per segment) and the largest row
// a warp takes in the persistent kernels (threads per row: a warp, or a 128- or 256-thread
// CTA above it).  Starting from the handle's current tuning, each parameter in turn takes
// each of its candidate values while the others stay fixed, and the fastest value is kept.
// A candidate is timed with CUDA events as the median of `reps` complete runs (plan +
// numeric) of the given batch; pass a representative sample of the real workload.  The
// best tuning is installed on the handle; its thresholds are returned.
namespace {

float time_candidate(ops_handle_s *h, int dtype, int32_t count, const ops_batch_item *items, int reps,
                     cudaStream_t st, int *status)
{
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    std::vector<float> ms;
    *status = OPS_OK;
    for (int r = 0; r < reps + 1 && *status == OPS_OK; ++r) {
        cudaEventRecord(e0, st);
        ops_batch_t b = nullptr;
        *status = ops_batch_create(h, dtype, count, items, &b, st);
        if (*status == OPS_OK) *status = ops_batch_execute(b, 0, st);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        if (r > 0) ms.push_back(t);  // the first run warms the pool and the caches
        ops_batch_destroy(b);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms.empty()) return 1e30f;
    std::sort(ms.begin(), ms.end());
    return ms[ms.size() / 2];
}

constexpr int kTuneParams = 9;  // 6 thresholds, hash_slots, batch_persistent, batch_warp_max

void tuning_to_array(const ops_tuning &t, int *v)
{
    for (int i = 0; i < 6; ++i) v[i] = t.thresholds[i];
    v[6] = t.hash_slots;
    v[7] = t.batch_persistent;
    v[8] = t.batch_warp_max;
}

ops_tuning tuning_from_array(const int *v)
{
    ops_tuning t{};
    for (int i = 0; i < 6; ++i) t.thresholds[i] = v[i];
    t.hash_slots = v[6];
    t.batch_persistent = v[7];
    t.batch_warp_max = v[8];
    return t;
}

}  // namespace

extern "C" int ops_autotune(ops_handle_t h, int dtype, int32_t count, const ops_batch_item *items, int reps,
                            int32_t *best, float *best_ms, void *stream)
{
    if (!h || !items || count <= 0 || !best || reps < 1) return OPS_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    ops_tuning saved{};
    OPS_CHECK(ops_handle_get_tuning(h, &saved));
    int cur[kTuneParams];
    tuning_to_array(saved, cur);
    const std::vector<std::vector<int>> cand = {{8, 0},          {16, 0},       {32, 0}, {128, 64, 32, 0},
                                                {1024, 512, 256, 0}, {13312, 4096}, {4, 2},  {1, 0},
                                                {512, 256, 128}};
    auto apply = [&](const int *v) {
        const ops_tuning t = tuning_from_array(v);
        return ops_handle_set_tuning(h, &t);
    };
    int status = apply(cur);
    if (status != OPS_OK) return status;
    float best_t = time_candidate(h, dtype, count, items, reps, st, &status);
    if (status != OPS_OK) {
        ops_handle_set_tuning(h, &saved);
        return status;
    }
    for (int p = 0; p < kTuneParams; ++p) {
        for (int v : cand[p]) {
            if (v == cur[p]) continue;
            int trial[kTuneParams];
            std::memcpy(trial, cur, sizeof(trial));
            trial[p] = v;
            status = apply(trial);
            if (status != OPS_OK) break;
            const float t = time_candidate(h, dtype, count, items, reps, st, &status);
            if (status != OPS_OK) break;
            if (t < best_t) {
                best_t = t;
                std::memcpy(cur, trial, sizeof(cur));
            }
        }
        if (status != OPS_OK) {
            ops_handle_set_tuning(h, &saved);
            return status;
        }
    }
    OPS_CHECK(apply(cur));
    std::memcpy(best, cur, 6 * sizeof(int32_t));
    if (best_ms) *best_ms = best_t;
    return OPS_OK;
}

// Tuning records: a JSON object {"<key>": [r8, r16, r32, w, e1, e2], ...} in one file.
namespace {

std::string read_file(const char *path)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) return std::string();
    std::string s;
    char buf[4096];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) s.append(buf, n);
    std::fclose(f);
    return s;
}

// Parses the records written by ops_tuning_store (keys without quotes or backslashes).
std::vector<std::pair<std::string, std::vector<int>>> parse_records(const std::string &s)
{
    std::vector<std::pair<std::string, std::vector<int>>> out;
    size_t i = 0;
    while ((i = s.find('"', i)) != std::string::npos) {
        const size_t j = s.find('"', i + 1);
        if (j == std::string::npos) break;
        std::string key = s.substr(i + 1, j - i - 1);
        const size_t a = s.find('[', j), b = s.find(']', j);
        if (a == std::string::npos || b == std::string::npos || b < a) break;
        std::vector<int> v;
        const char *p = s.c_str() + a + 1;
        const char *e = s.c_str() + b;
        while (p < e) {
            char *q = nullptr;
            const long x = std::strtol(p, &q, 10);
            if (q == p) {
                ++p;
                continue;
            }
            v.push_back((int)x);
            p = q;
        }
        out.emplace_back(key, v);
        i = b + 1;
    }
    return out;
}

}  // namespace

namespace {

// Writes the record `key` = values[0..n) into the JSON file at path (other records kept).
int store_values(const char *path, const char *key, const int *values, int n)
{
    if (!path || !key || !values) return OPS_INVALID_ARGUMENT;
    for (const char *c = key; *c; ++c)
        if (*c == '"' || *c == '\\') return OPS_INVALID_ARGUMENT;
    auto recs = parse_records(read_file(path));
    std::vector<int> v(values, values + n);
    bool found = false;
    for (auto &r : recs)
        if (r.first == key) {
            r.second = v;
            found = true;
        }
    if (!found) recs.emplace_back(key, v);
    FILE *f = std::fopen(path, "wb");
    if (!f) return OPS_EXCEPTION;
    std::fprintf(f, "{\n");
    for (size_t k = 0; k < recs.size(); ++k) {
        std::fprintf(f, "  \"%s\": [", recs[k].first.c_str());
        for (size_t t = 0; t < recs[k].second.size(); ++t) std::fprintf(f, t ? ", %d" : "%d", recs[k].second[t]);
        std::fprintf(f, "]%s\n", k + 1 < recs.size() ? "," : "");
    }
    std::fprintf(f, "}\n");
    std::fclose(f);
    return OPS_OK;
}

}  // namespace

extern "C" int ops_tuning_store(const char *path, const char *key, const int32_t *th)
{
    return store_values(path, key, th, 6);
}

extern "C" int ops_tuning_lookup(const char *path, const char *key, int32_t *th)
{
    if (!path || !key || !th) return OPS_INVALID_ARGUMENT;
    for (const auto &r : parse_records(read_file(path)))
        if (r.first == key && r.second.size() >= 6) {
            std::memcpy(th, r.second.data(), 6 * sizeof(int32_t));
            return OPS_OK;
        }
    return OPS_NOT_SUPPORTED;
}

extern "C" int ops_tuning_store_record(const char *path, const char *key, const ops_tuning *t)
{
    if (!t) return OPS_INVALID_ARGUMENT;
    int v[kTuneParams];
    tuning_to_array(*t, v);
    return store_values(path, key, v, kTuneParams);
}

extern "C" int ops_tuning_lookup_record(const char *path, const char *key, ops_tuning *t)
{
    if (!path || !key || !t) return OPS_INVALID_ARGUMENT;
    for (const auto &r : parse_records(read_file(path)))
        if (r.first == key && (r.second.size() == 6 || r.second.size() == (size_t)kTuneParams)) {
            int v[kTuneParams] = {0, 0, 0, 0, 0, 0, 4, 1, 512};  // fields a thresholds-only record lacks
            std::memcpy(v, r.second.data(), r.second.size() * sizeof(int));
            *t = tuning_from_array(v);
            return OPS_OK;
        }
    return OPS_NOT_SUPPORTED;
}
