// spgemm.cu — handle, pipeline and C ABI of the GB300 SpGEMM library.
//
// Pipeline of one C = A*B (compare src/opsparse/core_algo/spgemm/spgemm.cu:16-62 and
// spgemm_phases.cu:12-206 of OpSparse):
//   1. k_setup: product count per row + class lists             (one kernel, no host sync
//      between count and scatter, unlike h_symbolic_binning's D2H/H2D round trip)
//   2. read back class sizes and max products                   (host sync #1)
//   3. symbolic kernels, one stream per non-empty class, joined back onto the caller's
//      stream with events                                       (multi-stream bin dispatch)
//   4. exclusive scan of row nnz into C.row_ptr (CUB)
//   5. read back nnz(C)                                         (host sync #2)
//   6. C allocated from the handle's stream-ordered pool
//   7. numeric kernels on the same per-class streams, reusing step 1's classes
// Workspace (class lists, counters, scan scratch, dense-row scratch) lives in a
// cudaMemPool owned by the handle and is reused across calls; streams and events are
// created once per handle, never per call.
#include <cub/cub.cuh>

#include <algorithm>
#include <array>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "besc.cuh"
#include "wsort.cuh"
#include "internal.hpp"
#include "opsparse_gb300.h"

using namespace opsg;
using namespace opsg_internal;

namespace {

const char *kVersion = "opsparse_gb300 0.2 (sm_103a)";
constexpr int kBatchWarpMaxLo = 128;   // range of ops_tuning.batch_warp_max
constexpr int kBatchWarpMaxHi = 512;

struct Mat {
    int rows, cols;
    const int *rpt, *col;
    const void *val;
};

template <typename Shape, typename T>
void set_besc_attrs()
{
    cudaFuncSetAttribute(k_besc_rows<Shape, true, T, unsigned>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)Shape::template smem<true, unsigned, T>());
    cudaFuncSetAttribute(k_besc_rows<Shape, true, T, unsigned long long>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)Shape::template smem<true, unsigned long long, T>());
    cudaFuncSetAttribute(k_besc_rows<Shape, false, T, unsigned>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)Shape::template smem<false, unsigned, T>());
}

// Launch the CTA-per-row bitonic kernel of `Shape` on `s`: numeric keys pack the product
// index below the column and need 64 bits when the two do not fit in 32.
template <typename Shape, bool kNum, typename T>
void launch_besc(const SpgemmArgs<T> &g, const int *list, const int *count_ptr, int *cursor, int grid,
                 cudaStream_t s)
{
    if (!kNum) {
        k_besc_rows<Shape, false, T, unsigned>
            <<<grid, Shape::kThreads, Shape::template smem<false, unsigned, T>(), s>>>(g, list, count_ptr, cursor);
    } else if (ceil_log2(std::max(g.N, 2)) + Shape::kIdBits <= 32) {
        k_besc_rows<Shape, true, T, unsigned>
            <<<grid, Shape::kThreads, Shape::template smem<true, unsigned, T>(), s>>>(g, list, count_ptr, cursor);
    } else {
        k_besc_rows<Shape, true, T, unsigned long long>
            <<<grid, Shape::kThreads, Shape::template smem<true, unsigned long long, T>(), s>>>(g, list, count_ptr,
                                                                                             cursor);
    }
}

// The E1 expand rows' numeric kernel: the rank shape where B has at most kRankWinBits
// columns (every row fits the window), else the sort-only shape, whose smaller shared
// memory keeps one more CTA per SM for rows that could not take the rank path.
template <typename T>
void launch_besc_e1(const SpgemmArgs<T> &g, const int *list, const int *count_ptr, int *cursor, int grid,
                    cudaStream_t s)
{
    if (g.N <= kRankWinBits) launch_besc<BescE1, true, T>(g, list, count_ptr, cursor, grid, s);
    else launch_besc<BescE1Sort, true, T>(g, list, count_ptr, cursor, grid, s);
}

template <typename T>
void set_smem_attrs()
{
    cudaFuncSetAttribute(k_warp_rows<true, T, 2 * kSplitNnz>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)warp_rows_smem<true, T, 2 * kSplitNnz>());
    cudaFuncSetAttribute(k_esc_rows<EscLarge, true, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)EscLarge::kNumericSmem);
    cudaFuncSetAttribute(k_esc_rows<EscLarge, false, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)EscLarge::kSymbolicSmem);
    cudaFuncSetAttribute(k_esc_rows<EscMid, false, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)EscMid::kSymbolicSmem);
    cudaFuncSetAttribute(k_warp_rows<false, T, 2 * kEsc1FlopMax>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)warp_rows_smem<false, T, 2 * kEsc1FlopMax>());
    set_besc_attrs<BescE1, T>();
    set_besc_attrs<BescE1Sort, T>();
    set_besc_attrs<BescMid, T>();
    cudaFuncSetAttribute(k_wsort_rows<4, true, T, unsigned>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)WsortShape<4>::smem<true, T, unsigned>());
    cudaFuncSetAttribute(k_wsort_rows<4, true, T, unsigned long long>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)WsortShape<4>::smem<true, T, unsigned long long>());
    cudaFuncSetAttribute(k_wsort_rows<16, true, T, unsigned>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)WsortShape<16>::smem<true, T, unsigned>());
    cudaFuncSetAttribute(k_wsort_rows<16, true, T, unsigned long long>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)WsortShape<16>::smem<true, T, unsigned long long>());
}

int ensure_ws(ops_handle_s *h, int M, cudaStream_t st)
{
    if (h->ws && h->ws_M >= M) return OPS_OK;
    size_t cub_bytes = 0;
    OPS_CUDA(h, cub::DeviceScan::ExclusiveSum(nullptr, cub_bytes, (int *)nullptr, (int *)nullptr, M + 1, st));
    // one list per class, three for the numeric re-binning of E1 rows and two for the
    // E2 rows by size
    const size_t lists_b = align_up(sizeof(int) * (size_t)(kNumLists) * (size_t)M, 256);
    const size_t flop_b = align_up(sizeof(int) * (size_t)M, 256);
    const size_t soff_b = align_up(sizeof(int) * ((size_t)M + 1), 256);
    const size_t info_b = align_up(sizeof(DevInfo), 256);
    const size_t total = lists_b + flop_b + soff_b + info_b + align_up(cub_bytes, 256);
    if (h->ws) {
        OPS_CUDA(h, cudaFreeAsync(h->ws, st));
        h->ws = nullptr;
    }
    void *p = nullptr;
    OPS_CUDA(h, cudaMallocFromPoolAsync(&p, total, h->pool, st));
    h->ws = static_cast<unsigned char *>(p);
    h->ws_bytes = total;
    h->ws_M = M;
    h->lists = reinterpret_cast<int *>(h->ws);
    h->row_flop = reinterpret_cast<int *>(h->ws + lists_b);
    h->soff = reinterpret_cast<int *>(h->ws + lists_b + flop_b);
    h->info = reinterpret_cast<DevInfo *>(h->ws + lists_b + flop_b + soff_b);
    h->cub_tmp = h->ws + lists_b + flop_b + soff_b + info_b;
    h->cub_bytes = cub_bytes;
    h->plan_valid = false;
    return OPS_OK;
}

// Region ends of the dense-row scratch for `ctas` CTAs: [vals | bits | tot | cnt | pos],
// each region 256-byte aligned.
std::array<size_t, 5> dense_offsets(int N, int ctas)
{
    const size_t n = (size_t)N * (size_t)ctas, words = (size_t)(N + 31) / 32 * (size_t)ctas;
    std::array<size_t, 5> o{};
    o[0] = align_up(n * 8, 256);
    o[1] = o[0] + align_up(words * 4, 256);
    o[2] = o[1] + align_up(n * 8, 256);
    o[3] = o[2] + align_up(n * 4, 256);
    o[4] = o[3] + align_up(n * 4, 256);
    return o;
}

// Dense-row scratch: per CTA, N accumulator slots (8 bytes), ceil(N/32) bitmap words, and
// for entries folded in blocks N merged-block slots (8 bytes), N product counts and N
// positions (4 bytes each).
int ensure_dense(ops_handle_s *h, int N, int rows, cudaStream_t st)
{
    const size_t words = (size_t)(N + 31) / 32;
    const size_t per_cta = (size_t)N * 24 + words * 4;
    int ctas = std::min(rows, 2 * h->num_sms);
    const size_t by_budget = per_cta ? h->dense_budget / per_cta : (size_t)ctas;
    ctas = (int)std::max<size_t>(1, std::min<size_t>((size_t)ctas, by_budget));
    const size_t need = dense_offsets(N, ctas)[4] + 256;
    if (need > h->dense_bytes) {
        if (h->dense) {
            OPS_CUDA(h, cudaFreeAsync(h->dense, st));
            h->dense = nullptr;
            h->dense_bytes = 0;
        }
        void *p = nullptr;
        OPS_CUDA(h, cudaMallocFromPoolAsync(&p, need, h->pool, st));
        OPS_CUDA(h, cudaMemsetAsync(p, 0, need, st));
        h->dense = static_cast<unsigned char *>(p);
        h->dense_bytes = need;
    }
    h->dense_ctas = ctas;
    return OPS_OK;
}

template <typename T>
DenseScratch<T> dense_view(ops_handle_s *h, int N)
{
    const std::array<size_t, 5> o = dense_offsets(N, h->dense_ctas);
    DenseScratch<T> d;
    d.words = (N + 31) / 32;
    d.vals = reinterpret_cast<typename Acc<T>::S *>(h->dense);
    d.bits = reinterpret_cast<unsigned *>(h->dense + o[0]);
    d.tot = reinterpret_cast<typename Acc<T>::S *>(h->dense + o[1]);
    d.cnt = reinterpret_cast<int *>(h->dense + o[2]);
    d.pos = reinterpret_cast<int *>(h->dense + o[3]);
    return d;
}

int grid_for(long long work_items, int per_block, int cap)
{
    long long b = (work_items + per_block - 1) / per_block;
    return (int)std::max<long long>(1, std::min<long long>(b, cap));
}

// Classes whose rows a one-pass call computes in the counting phase: all but R8 (counted
// by k_setup; their numeric writes C directly in the second phase, next to the copy of the
// staged rows), D only if its whole-GPU sort fits the scratch budget, and E1 only if some
// E1 row is staged (not a column-window row; the split is made on the device, and without
// such rows the E1 class keeps its own list and two passes).
bool staged_class(const ops_handle_s *h, int c)
{
    return c != kClsR8 && (c != kClsD || h->stage_d) && (c != kClsE1 || h->stage_e1);
}

// Below this many staged products the set-up of a one-pass call (the offset scan, the
// copy into C) costs more than the counting kernels it saves.
constexpr unsigned long long kMinStageFlop = 1ull << 20;

// Values region of the staging area (after the columns of staged_flop entries).
template <typename T>
T *stage_vals(ops_handle_s *h)
{
    return reinterpret_cast<T *>(h->stage + align_up(sizeof(int) * (size_t)h->stage_entries, 256));
}

// Counting phase of a one-pass call: class c's numeric kernels write its rows' entries
// to the staging area at soff[r] and their counts to c_rpt, in place of the counting
// kernels.  The E1 rows it does not stage are counted as usual.
template <typename T, typename GA>
int launch_staged_class(ops_handle_s *h, const GA &gs, int c, const int *list, int n, cudaStream_t s)
{
    SpgemmArgs<T> g{};
    g.arpt = gs.arpt;
    g.acol = gs.acol;
    g.aval = static_cast<const T *>(h->op_aval);
    g.brpt = gs.brpt;
    g.bcol = gs.bcol;
    g.bval = static_cast<const T *>(h->op_bval);
    g.M = gs.M;
    g.K = gs.K;
    g.N = gs.N;
    g.row_flop = gs.row_flop;
    g.c_rpt = gs.c_rpt;
    g.info = gs.info;
    g.soff = h->soff;
    g.c_col = reinterpret_cast<int *>(h->stage);
    g.c_val = stage_vals<T>(h);
    const int sms = h->num_sms;
    const size_t M = (size_t)h->plan_M;
    int *xl = h->lists + (size_t)kNumClasses * M;
    switch (c) {
        case kClsR16:
            k_reg_rows<16, true, T><<<grid_for((n + 1) / 2, 8, sms * 8), 256, 0, s>>>(g, list, n);
            break;
        case kClsR32:
            k_reg_rows<32, true, T><<<grid_for(n, 8, sms * 8), 256, 0, s>>>(g, list, n);
            break;
        case kClsW: {
            using Sh = WsortShape<4>;
            const int grid = grid_for(n, Sh::kWarps, sms * 8);
            if (g.N <= (1 << (32 - Sh::kIdBits))) {
                k_wsort_rows<4, true, T, unsigned>
                    <<<grid, Sh::kThreads, Sh::smem<true, T, unsigned>(), s>>>(g, list, &h->info->counts[c]);
            } else {
                k_wsort_rows<4, true, T, unsigned long long>
                    <<<grid, Sh::kThreads, Sh::smem<true, T, unsigned long long>(), s>>>(g, list, &h->info->counts[c]);
            }
            break;
        }
        case kClsE1: {
            // the staged rows (not column-window rows) into the staging area: by warp sort
            // up to kE1OnePassFlopMax products, else (on an extra stream) by CTA
            // expand/sort/compress; the rest counted by the warp hash
            int *one = xl + kXlE1One * M;
            int *two = xl + kXlE1Two * M;
            int *one_large = xl + kXlE1OneLarge * M;
            k_split_list<3, PickStaged><<<grid_for(n, 256, sms * 4), 256, 0, s>>>(
                list, &h->info->counts[c], PickStaged{h->soff, g.row_flop}, one, (int)M, h->info->split1);
            OPS_CUDA(h, cudaGetLastError());
            ++h->launches;
            OPS_CUDA(h, cudaEventRecord(h->ev_x_fork[0], s));
            OPS_CUDA(h, cudaStreamWaitEvent(h->side_x[0], h->ev_x_fork[0], 0));
            launch_besc_e1<T>(g, one_large, &h->info->split1[2], &h->info->next[0][c], std::min(n, sms * 8),
                              h->side_x[0]);
            OPS_CUDA(h, cudaGetLastError());
            ++h->launches;
            SpgemmArgs<double> gc{};
            gc.arpt = g.arpt;
            gc.acol = g.acol;
            gc.brpt = g.brpt;
            gc.bcol = g.bcol;
            gc.M = g.M;
            gc.K = g.K;
            gc.N = g.N;
            gc.row_flop = g.row_flop;
            gc.c_rpt = g.c_rpt;
            gc.info = g.info;
            k_warp_rows<false, double, 2 * kEsc1FlopMax>
                <<<grid_for(n, kWarpRowsThreads / 32, sms * 3), kWarpRowsThreads,
                   warp_rows_smem<false, double, 2 * kEsc1FlopMax>(), h->side_x[0]>>>(gc, two, &h->info->split1[1]);
            OPS_CUDA(h, cudaGetLastError());
            ++h->launches;
            OPS_CUDA(h, cudaEventRecord(h->ev_x_join[0], h->side_x[0]));
            using Sh = WsortShape<16>;
            const int sgrid = grid_for(n, Sh::kWarps, sms * 4);
            if (g.N <= (1 << (32 - Sh::kIdBits))) {
                k_wsort_rows<16, true, T, unsigned>
                    <<<sgrid, Sh::kThreads, Sh::smem<true, T, unsigned>(), s>>>(g, one, &h->info->split1[0]);
            } else {
                k_wsort_rows<16, true, T, unsigned long long>
                    <<<sgrid, Sh::kThreads, Sh::smem<true, T, unsigned long long>(), s>>>(g, one, &h->info->split1[0]);
            }
            OPS_CUDA(h, cudaGetLastError());
            OPS_CUDA(h, cudaStreamWaitEvent(s, h->ev_x_join[0], 0));
            break;
        }
        case kClsE2: {
            // the counting phase's split and longest-first orders, then both numeric shapes
            int *mid_list = xl + kXlE2Mid * M;
            int *large_list = xl + kXlE2Large * M;
            k_split_list<2, PickE2><<<grid_for(n, 256, sms * 4), 256, 0, s>>>(
                list, &h->info->counts[c], PickE2{g.arpt, g.row_flop}, mid_list, (int)M, h->info->split2);
            OPS_CUDA(h, cudaGetLastError());
            ++h->launches;
            OPS_CUDA(h, cudaEventRecord(h->ev_x_fork[1], s));
            OPS_CUDA(h, cudaStreamWaitEvent(h->side_x[1], h->ev_x_fork[1], 0));
            if (n > 1) {
                k_sort_heavy_first<<<1, 1024, 0, h->side_x[1]>>>(large_list, &h->info->split2[1], h->row_flop);
                OPS_CUDA(h, cudaGetLastError());
                ++h->launches;
            }
            k_esc_rows<EscLarge, true, T><<<std::min(n, sms), EscLarge::kThreads, EscLarge::kNumericSmem,
                                            h->side_x[1]>>>(g, large_list, &h->info->split2[1], &h->info->next[0][c]);
            OPS_CUDA(h, cudaGetLastError());
            ++h->launches;
            OPS_CUDA(h, cudaEventRecord(h->ev_x_join[1], h->side_x[1]));
            if (n > 1) {
                k_sort_heavy_first<<<1, 1024, 0, s>>>(mid_list, &h->info->split2[0], h->row_flop);
                OPS_CUDA(h, cudaGetLastError());
                ++h->launches;
            }
            launch_besc<BescMid, true, T>(g, mid_list, &h->info->split2[0], &h->info->next_mid[0],
                                          std::min(n, sms * 4), s);
            OPS_CUDA(h, cudaGetLastError());
            OPS_CUDA(h, cudaStreamWaitEvent(s, h->ev_x_join[1], 0));
            break;
        }
        case kClsD: {  // whole-GPU expand/sort/compress, counts from its head scan
            const int st_d = run_d_rows<T>(h, g, list, n, true, s);
            if (st_d != OPS_OK) return st_d == OPS_NOT_SUPPORTED ? fail(h, OPS_CUDA_ERROR, "D-row scratch changed") : st_d;
            h->d_rows_path[0] = n;
            h->d_rows_path[1] = 0;
            break;
        }
        default:
            return fail(h, OPS_NOT_SUPPORTED, "class without a one-pass kernel");
    }
    return OPS_OK;
}

// One-pass set-up, once the class sizes are known: when the call has its values, one
// pass is on and the staged products fit the handle's staging budget, grows the staging
// area and turns the per-row product counts (k_setup's sflop) into staging offsets.
// Otherwise leaves h->staged false: two passes.
int prepare_stage(ops_handle_s *h, const DevInfo &hi, int M, cudaStream_t st)
{
    h->staged = false;
    const int vs = h->op_dtype == OPS_F64 ? 8 : (h->op_dtype == OPS_F32 ? 4 : 0);
    if (!h->one_pass || vs == 0 || M == 0 || hi.staged_flop == 0) return OPS_OK;
    if (h->one_pass == 1 && hi.staged_flop < kMinStageFlop) return OPS_OK;
    const unsigned long long entries = hi.staged_flop;
    const size_t total = align_up(sizeof(int) * (size_t)entries, 256) + align_up((size_t)vs * (size_t)entries, 256);
    if (entries > (unsigned long long)INT_MAX || total > h->stage_budget) return OPS_OK;
    if (total > h->stage_bytes) {
        if (h->stage) OPS_CUDA(h, cudaFreeAsync(h->stage, st));
        h->stage = nullptr;
        h->stage_bytes = 0;
        void *p = nullptr;
        if (cudaMallocFromPoolAsync(&p, total, h->pool, st) != cudaSuccess) {  // two passes instead
            (void)cudaGetLastError();
            return OPS_OK;
        }
        h->stage = static_cast<unsigned char *>(p);
        h->stage_bytes = total;
    }
    h->stage_entries = (long long)entries;
    // D rows are staged only if their whole-GPU sort fits the scratch budget (else they keep
    // two passes and the dense-row kernel may take them)
    h->stage_d = false;
    if (hi.counts[kClsD] > 0) {
        SpgemmArgs<double> gd{};
        gd.N = h->plan_N;
        gd.soff = h->soff;
        h->stage_d = run_d_rows<double>(h, gd, nullptr, hi.counts[kClsD], true, st, true) == OPS_OK;
        h->last_error.clear();
        if (!h->stage_d) {
            k_unstage_rows<<<grid_for(hi.counts[kClsD], 256, h->num_sms * 4), 256, 0, st>>>(
                h->lists + (size_t)kClsD * M, &h->info->counts[kClsD], h->soff);
            OPS_CUDA(h, cudaGetLastError());
            ++h->launches;
        }
    }
    size_t cb = h->cub_bytes;
    OPS_CUDA(h, cub::DeviceScan::ExclusiveSum(h->cub_tmp, cb, h->soff, h->soff, M + 1, st));
    ++h->launches;
    h->staged = true;
    h->stage_e1 = hi.e1_one > 0;
    h->stage_e1_all = hi.e1_one == hi.counts[kClsE1];
    return OPS_OK;
}

// Launch the kernels of every non-empty class, each on its own stream forked from `st`
// and joined back into it.  A re-binned class (E1 numeric, E2) first splits its list on
// the device and runs its second kernel on an extra stream forked from the class stream;
// the class stream joins it again, so the class's events span both kernels.
template <bool kNum, typename T>
int launch_classes(ops_handle_s *h, const SpgemmArgs<T> &g, cudaStream_t st)
{
    OPS_CUDA(h, cudaEventRecord(h->ev_fork, st));
    const int sms = h->num_sms;
    const size_t M = (size_t)h->plan_M;
    int *xl = h->lists + (size_t)kNumClasses * M;  // extra lists
    auto fork_x = [&](int x, cudaStream_t from) -> cudaStream_t {
        if (cudaEventRecord(h->ev_x_fork[x], from) != cudaSuccess) return nullptr;
        if (cudaStreamWaitEvent(h->side_x[x], h->ev_x_fork[x], 0) != cudaSuccess) return nullptr;
        return h->side_x[x];
    };
    auto join_x = [&](int x, cudaStream_t into) -> bool {
        return cudaEventRecord(h->ev_x_join[x], h->side_x[x]) == cudaSuccess &&
               cudaStreamWaitEvent(into, h->ev_x_join[x], 0) == cudaSuccess;
    };
    // heaviest classes first: their long kernels then overlap the light classes instead
    // of forming the tail of the phase
    constexpr int kOrder[kNumClasses] = {kClsE2, kClsD, kClsE1, kClsW, kClsR32, kClsR16, kClsR8};
    if (kNum && h->staged) {
        // one-pass call: the rows computed in the counting phase move from the staging
        // area into C, on the caller's stream while the remaining classes run on theirs
        const long long ranges = (h->plan_nnz + kPlaceRange - 1) / kPlaceRange;
        k_place_staged<T><<<grid_for(ranges, 8, sms * 8), 256, 0, st>>>(
            g.M, h->soff, g.c_rpt, reinterpret_cast<const int *>(h->stage), stage_vals<T>(h), g.c_col, g.c_val);
        OPS_CUDA(h, cudaGetLastError());
        ++h->launches;
    }
    for (int oi = 0; oi < kNumClasses; ++oi) {
        const int c = kOrder[oi];
        const int n = h->counts[c];
        if (n <= 0) continue;
        const bool staged = h->staged && staged_class(h, c);
        // R8 rows are counted inside k_setup; staged classes are done after the counting
        // phase, except the E1 rows left to two passes
        if (!kNum && c == kClsR8) continue;
        if (kNum && staged && (c != kClsE1 || h->stage_e1_all)) continue;
        cudaStream_t s = h->side[c];
        OPS_CUDA(h, cudaStreamWaitEvent(s, h->ev_fork, 0));
        const int *list = h->lists + (size_t)c * M;
        if (!kNum && c == kClsD && n > 1 && n <= kLptMax) {
            // longest rows first; the numeric phase reuses the ordered list
            k_sort_heavy_first<<<1, 1024, 0, s>>>(h->lists + (size_t)c * M, &h->info->counts[c], h->row_flop);
            OPS_CUDA(h, cudaGetLastError());
            ++h->launches;
        }
        if (h->timing >= 2) OPS_CUDA(h, cudaEventRecord(h->ev_k[kNum][c][0], s));
        if (staged && !kNum) {  // one-pass call: numeric into the staging area
            OPS_CHECK(h->op_dtype == OPS_F64 ? launch_staged_class<double>(h, g, c, list, n, s)
                                             : launch_staged_class<float>(h, g, c, list, n, s));
        } else
        switch (c) {
            case kClsR8:  // numeric only: walks the rows in order
                k_small_rows<T><<<grid_for(g.M, kSmallThreads, sms * 8), kSmallThreads, 0, s>>>(g, h->plan_th.r8);
                break;
            case kClsR16:
                k_reg_rows<16, kNum, T><<<grid_for((n + 1) / 2, 8, sms * 8), 256, 0, s>>>(g, list, n);
                break;
            case kClsR32:
                k_reg_rows<32, kNum, T><<<grid_for(n, 8, sms * 8), 256, 0, s>>>(g, list, n);
                break;
            case kClsW: {  // warp sort: products sorted in registers, no table
                using Sh = WsortShape<4>;
                const int grid = grid_for(n, Sh::kWarps, sms * 8);
                if (!kNum) {
                    k_wsort_rows<4, false, T, unsigned>
                        <<<grid, Sh::kThreads, Sh::smem<false, T, unsigned>(), s>>>(g, list, &h->info->counts[c]);
                } else if (g.N <= (1 << (32 - Sh::kIdBits))) {
                    k_wsort_rows<4, true, T, unsigned>
                        <<<grid, Sh::kThreads, Sh::smem<true, T, unsigned>(), s>>>(g, list, &h->info->counts[c]);
                } else {
                    k_wsort_rows<4, true, T, unsigned long long>
                        <<<grid, Sh::kThreads, Sh::smem<true, T, unsigned long long>(), s>>>(g, list,
                                                                                            &h->info->counts[c]);
                }
                break;
            }
            case kClsE1: {
                if (!kNum) {  // distinct-column count: one warp per row, table of 2*flop slots
                    k_warp_rows<false, T, 2 * kEsc1FlopMax>
                        <<<grid_for(n, kWarpRowsThreads / 32, sms * 3), kWarpRowsThreads,
                           warp_rows_smem<false, T, 2 * kEsc1FlopMax>(), s>>>(g, list, &h->info->counts[c]);
                    break;
                }
                // re-bin by output size: warp sort / warp hash on this stream,
                // expand/sort/compress on an extra stream (a one-pass call re-bins only
                // the rows it left to two passes)
                int *sort_list = xl + kXlE1Sort * M;
                int *hash_list = xl + kXlE1Hash * M;
                int *esc_list = xl + kXlE1Esc * M;
                const int *e1_list = staged ? xl + kXlE1Two * M : list;
                const int *e1_count = staged ? &h->info->split1[1] : &h->info->counts[c];
                k_split_list<3, PickE1><<<grid_for(n, 256, sms * 4), 256, 0, s>>>(
                    e1_list, e1_count, PickE1{g.c_rpt, g.row_flop, kWsortFlopMax}, sort_list, (int)M,
                    h->info->split);
                OPS_CUDA(h, cudaGetLastError());
                ++h->launches;
                cudaStream_t sx = fork_x(0, s);
                if (!sx) return fail(h, OPS_CUDA_ERROR, "stream fork failed");
                launch_besc_e1<T>(g, esc_list, &h->info->split[2], &h->info->next[1][c], std::min(n, sms * 8), sx);
                OPS_CUDA(h, cudaGetLastError());
                ++h->launches;
                if (!join_x(0, s)) return fail(h, OPS_CUDA_ERROR, "stream join failed");
                using Sh = WsortShape<16>;
                const int sgrid = grid_for(n, Sh::kWarps, sms * 4);
                if (g.N <= (1 << (32 - Sh::kIdBits))) {
                    k_wsort_rows<16, true, T, unsigned>
                        <<<sgrid, Sh::kThreads, Sh::smem<true, T, unsigned>(), s>>>(g, sort_list, &h->info->split[0]);
                } else {
                    k_wsort_rows<16, true, T, unsigned long long>
                        <<<sgrid, Sh::kThreads, Sh::smem<true, T, unsigned long long>(), s>>>(g, sort_list,
                                                                                              &h->info->split[0]);
                }
                OPS_CUDA(h, cudaGetLastError());
                ++h->launches;
                k_warp_rows<true, T, 2 * kSplitNnz>
                    <<<grid_for(n, kWarpRowsThreads / 32, sms * 4), kWarpRowsThreads,
                       warp_rows_smem<true, T, 2 * kSplitNnz>(), s>>>(g, hash_list, &h->info->split[1]);
                break;
            }
            case kClsE2: {
                // mid shape (3 CTAs per SM) on this stream, large shape (1 per SM) on an
                // extra stream; the split and the longest-first order are made once, by
                // the symbolic phase, and reused by numeric
                int *mid_list = xl + kXlE2Mid * M;
                int *large_list = xl + kXlE2Large * M;
                if (!kNum) {
                    k_split_list<2, PickE2><<<grid_for(n, 256, sms * 4), 256, 0, s>>>(
                        list, &h->info->counts[c], PickE2{g.arpt, g.row_flop}, mid_list, (int)M, h->info->split2);
                    OPS_CUDA(h, cudaGetLastError());
                    ++h->launches;
                }
                cudaStream_t sx = fork_x(1, s);
                if (!sx) return fail(h, OPS_CUDA_ERROR, "stream fork failed");
                if (!kNum && n > 1) {
                    k_sort_heavy_first<<<1, 1024, 0, sx>>>(large_list, &h->info->split2[1], h->row_flop);
                    OPS_CUDA(h, cudaGetLastError());
                    ++h->launches;
                }
                // large rows: radix-sort expand/sort/compress (for 8K-16K products the
                // 3 radix passes beat a 16K-key bitonic network); counting by hash table
                k_esc_rows<EscLarge, kNum, T>
                    <<<std::min(n, sms), EscLarge::kThreads, kNum ? EscLarge::kNumericSmem : EscLarge::kSymbolicSmem,
                       sx>>>(g, large_list, &h->info->split2[1], &h->info->next[kNum][c]);
                OPS_CUDA(h, cudaGetLastError());
                ++h->launches;
                if (!join_x(1, s)) return fail(h, OPS_CUDA_ERROR, "stream join failed");
                if (!kNum && n > 1) {
                    k_sort_heavy_first<<<1, 1024, 0, s>>>(mid_list, &h->info->split2[0], h->row_flop);
                    OPS_CUDA(h, cudaGetLastError());
                    ++h->launches;
                }
                if (kNum) {  // mid rows: bitonic expand/sort/compress
                    launch_besc<BescMid, true, T>(g, mid_list, &h->info->split2[0], &h->info->next_mid[1],
                                                  std::min(n, sms * 4), s);
                } else {  // counting by hash table
                    k_esc_rows<EscMid, false, T><<<std::min(n, sms * 4), EscMid::kThreads, EscMid::kSymbolicSmem, s>>>(
                        g, mid_list, &h->info->split2[0], &h->info->next_mid[0]);
                }
                break;
            }
            case kClsD: {
                // whole-GPU expand/sort/compress; the CTA-per-row dense kernel when the
                // packed keys or the scratch do not fit
                const int st_d = run_d_rows<T>(h, g, list, n, kNum, s);
                h->d_rows_path[0] = st_d == OPS_OK ? n : 0;
                h->d_rows_path[1] = st_d == OPS_NOT_SUPPORTED ? n : 0;
                if (st_d == OPS_NOT_SUPPORTED) {
                    OPS_CHECK(ensure_dense(h, g.N, n, s));
                    k_dense_rows<kNum, T><<<std::min(n, h->dense_ctas), kDenseRowsThreads, 0, s>>>(
                        g, list, n, dense_view<T>(h, g.N));
                } else if (st_d != OPS_OK) {
                    return st_d;
                }
                break;
            }
        }
        OPS_CUDA(h, cudaGetLastError());
        ++h->launches;
        if (h->timing >= 2) {
            OPS_CUDA(h, cudaEventRecord(h->ev_k[kNum][c][1], s));
            h->kmeasured[kNum][c] = true;
        }
        OPS_CUDA(h, cudaEventRecord(h->ev_join[c], s));
        OPS_CUDA(h, cudaStreamWaitEvent(st, h->ev_join[c], 0));
    }
    return OPS_OK;
}

int check_mat_args(ops_handle_s *h, int rows, int cols, const int *rpt, const int *col, long long nnz)
{
    if (rows < 0 || cols < 0 || nnz < 0) return fail(h, OPS_INVALID_ARGUMENT, "negative matrix size");
    if (nnz > INT_MAX) return fail(h, OPS_INT32_OVERFLOW, "input nnz exceeds INT32_MAX");
    if (!rpt && rows > 0) return fail(h, OPS_INVALID_ARGUMENT, "null row_ptr");
    if (!col && nnz > 0) return fail(h, OPS_INVALID_ARGUMENT, "null col_idx");
    return OPS_OK;
}

float ev_ms(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
        (void)cudaGetLastError();
        return 0.f;
    }
    return ms;
}

int dtype_size(int dtype) { return dtype == OPS_F64 ? 8 : (dtype == OPS_F32 ? 4 : 0); }

// Largest C (at one entry per product) that a one-pass ops_spgemm allocates before its
// entry count is known.
constexpr long long kEarlyAllocBytes = 256ll << 20;

// Status of the counting phase from its device results.
int count_status(ops_handle_s *h, const DevInfo &d)
{
    if (d.flags & kErrBadColumn) return fail(h, OPS_INVALID_CSR, "B has a column index outside [0, cols)");
    if (d.flags & kErrProbeLimit) return fail(h, OPS_PROBE_LIMIT, "symbolic hash table overflow");
    if (d.total_nnz > (unsigned long long)INT_MAX) return fail(h, OPS_INT32_OVERFLOW, "nnz(C) exceeds INT32_MAX");
    return OPS_OK;
}

// Counting phase: class sizes (one host sync), the classes' kernels, the row_ptr scan and
// nnz(C) (a second sync).  early_alloc (ops_spgemm): where C at one entry per product fits
// kEarlyAllocBytes and no row is a D row, the second sync is left out; *c_nnz is then -1,
// plan_nnz holds the product count (an upper bound of nnz(C)) and the phase's results
// reach h_info_count when the stream gets there, for the caller to read after its own
// sync.  No D row means no kernel indexes memory by a column of B, so the numeric phase
// may run before a bad column is reported, writing at most one entry per product.
int run_symbolic(ops_handle_s *h, const Mat &A, const Mat &B, int *c_rpt, long long *c_nnz, cudaStream_t st,
                 bool early_alloc = false)
{
    const int M = A.rows;
    OPS_CHECK(ensure_ws(h, std::max(M, 1), st));
    h->plan_valid = false;
    h->launches = 0;
    std::memset(h->kmeasured, 0, sizeof(h->kmeasured));
    if (h->timing) OPS_CUDA(h, cudaEventRecord(h->ev_t[0], st));
    OPS_CUDA(h, cudaMemsetAsync(h->info, 0, sizeof(DevInfo), st));
    OPS_CUDA(h, cudaMemsetAsync(c_rpt + M, 0, sizeof(int), st));
    // a one-pass call also gets the per-row products it may stage (made into offsets once
    // the staging area is known to fit)
    const bool want_stage = h->one_pass != 0 && h->op_dtype >= 0;
    if (want_stage) OPS_CUDA(h, cudaMemsetAsync(h->soff + M, 0, sizeof(int), st));
    if (h->timing) OPS_CUDA(h, cudaEventRecord(h->ev_t[1], st));
    if (M > 0) {
        k_setup<<<(M + kSetupThreads - 1) / kSetupThreads, kSetupThreads, 0, st>>>(
            A.rpt, A.col, B.rpt, B.col, M, A.cols, B.cols, h->row_flop, h->lists, c_rpt,
            want_stage ? h->soff : nullptr, h->info, h->th);
        OPS_CUDA(h, cudaGetLastError());
        ++h->launches;
    }
    OPS_CUDA(h, cudaMemcpyAsync(h->h_info, h->info, sizeof(DevInfo), cudaMemcpyDeviceToHost, st));
    if (h->timing) OPS_CUDA(h, cudaEventRecord(h->ev_t[2], st));
    OPS_CUDA(h, cudaStreamSynchronize(st));
    const DevInfo hi = *h->h_info;
    if (hi.flags & kErrBadColumn) return fail(h, OPS_INVALID_CSR, "A has a column index outside [0, cols)");
    if (hi.flags & kErrRowFlopOverflow)
        return fail(h, OPS_INT32_OVERFLOW, "a row of C has more than INT32_MAX intermediate products");
    std::memcpy(h->counts, hi.counts, sizeof(h->counts));
    h->plan_th = h->th;
    h->plan_M = M;
    h->plan_K = A.cols;
    h->plan_N = B.cols;
    h->plan_flop = (long long)hi.total_flop;
    h->plan_d_flop = (long long)hi.d_flop;
    h->plan_d_len_a = (long long)hi.d_len_a;
    h->staged = false;
    if (want_stage) OPS_CHECK(prepare_stage(h, hi, M, st));

    SpgemmArgs<double> g{};
    g.arpt = A.rpt;
    g.acol = A.col;
    g.brpt = B.rpt;
    g.bcol = B.col;
    g.M = M;
    g.K = A.cols;
    g.N = B.cols;
    g.row_flop = h->row_flop;
    g.c_rpt = c_rpt;
    g.info = h->info;
    OPS_CHECK((launch_classes<false, double>(h, g, st)));
    if (h->timing) OPS_CUDA(h, cudaEventRecord(h->ev_t[3], st));
    size_t cb = h->cub_bytes;
    OPS_CUDA(h, cub::DeviceScan::ExclusiveSum(h->cub_tmp, cb, c_rpt, c_rpt, M + 1, st));
    if (h->timing) OPS_CUDA(h, cudaEventRecord(h->ev_t[4], st));
    const int vs = h->op_dtype >= 0 ? dtype_size(h->op_dtype) : 0;
    if (early_alloc && vs > 0 && hi.counts[kClsD] == 0 &&
        (long long)hi.total_flop * (long long)(4 + vs) <= kEarlyAllocBytes) {
        OPS_CUDA(h, cudaMemcpyAsync(h->h_info_count, h->info, sizeof(DevInfo), cudaMemcpyDeviceToHost, st));
        *c_nnz = -1;
        h->plan_nnz = (long long)hi.total_flop;
    } else {
        OPS_CUDA(h, cudaMemcpyAsync(h->h_info, h->info, sizeof(DevInfo), cudaMemcpyDeviceToHost, st));
        OPS_CUDA(h, cudaStreamSynchronize(st));
        const DevInfo h2 = *h->h_info;
        OPS_CHECK(count_status(h, h2));
        *c_nnz = (long long)h2.total_nnz;
        h->plan_nnz = (long long)h2.total_nnz;
    }
    h->plan_arpt = A.rpt;
    h->plan_acol = A.col;
    h->plan_brpt = B.rpt;
    h->plan_bcol = B.col;
    h->plan_valid = true;
    return OPS_OK;
}

template <typename T>
int run_numeric(ops_handle_s *h, const Mat &A, const Mat &B, const int *c_rpt, int *c_col, T *c_val, cudaStream_t st)
{
    if (!h->plan_valid || h->plan_M != A.rows || h->plan_K != A.cols || h->plan_N != B.cols ||
        h->plan_arpt != A.rpt || h->plan_acol != A.col || h->plan_brpt != B.rpt || h->plan_bcol != B.col)
        return fail(h, OPS_NOT_SUPPORTED, "numeric phase without a matching symbolic phase on this handle");
    OPS_CUDA(h, cudaMemsetAsync(&h->info->flags, 0, sizeof(int), st));
    OPS_CUDA(h, cudaMemsetAsync(h->info->next[1], 0, sizeof(h->info->next[1]), st));
    OPS_CUDA(h, cudaMemsetAsync(h->info->split, 0, sizeof(h->info->split), st));
    OPS_CUDA(h, cudaMemsetAsync(&h->info->next_mid[1], 0, sizeof(int), st));
    SpgemmArgs<T> g{};
    g.arpt = A.rpt;
    g.acol = A.col;
    g.aval = static_cast<const T *>(A.val);
    g.brpt = B.rpt;
    g.bcol = B.col;
    g.bval = static_cast<const T *>(B.val);
    g.M = A.rows;
    g.K = A.cols;
    g.N = B.cols;
    g.row_flop = h->row_flop;
    g.c_rpt = const_cast<int *>(c_rpt);
    g.c_col = c_col;
    g.c_val = c_val;
    g.info = h->info;
    g.hash_slots = h->hash_slots;
    return launch_classes<true, T>(h, g, st);
}

int check_flags(ops_handle_s *h, cudaStream_t st)
{
    OPS_CUDA(h, cudaMemcpyAsync(&h->h_info->flags, &h->info->flags, sizeof(int), cudaMemcpyDeviceToHost, st));
    OPS_CUDA(h, cudaStreamSynchronize(st));
    const int f = h->h_info->flags;
    if (f & kErrCountMismatch) return fail(h, OPS_COUNT_MISMATCH, "numeric nnz differs from symbolic nnz");
    if (f & kErrProbeLimit) return fail(h, OPS_PROBE_LIMIT, "numeric hash table overflow");
    if (f & kErrBadColumn) return fail(h, OPS_INVALID_CSR, "column index outside [0, cols)");
    return OPS_OK;
}

void fill_timings(ops_handle_s *h, bool with_numeric)
{
    ops_timings &t = h->last_t;
    std::memset(&t, 0, sizeof(t));
    t.flop = h->plan_flop;
    t.nnz = h->plan_nnz;
    for (int c = 0; c < kNumClasses; ++c) t.class_rows[c] = h->counts[c];
    t.launches = h->launches;
    for (int ph = 0; ph < 2; ++ph)
        for (int c = 0; c < kNumClasses; ++c)
            t.kernel_ms[ph][c] = h->kmeasured[ph][c] ? ev_ms(h->ev_k[ph][c][0], h->ev_k[ph][c][1]) : 0.f;
    if (!h->timing) return;
    t.setup = ev_ms(h->ev_t[0], h->ev_t[1]) * 1e-3;
    t.symbolic_binning = ev_ms(h->ev_t[1], h->ev_t[2]) * 1e-3;
    t.symbolic = ev_ms(h->ev_t[2], h->ev_t[3]) * 1e-3;
    t.prefix = ev_ms(h->ev_t[3], h->ev_t[4]) * 1e-3;
    if (with_numeric) {
        t.allocate = ev_ms(h->ev_t[4], h->ev_t[5]) * 1e-3;
        t.numeric = ev_ms(h->ev_t[5], h->ev_t[6]) * 1e-3;
        t.total = ev_ms(h->ev_t[0], h->ev_t[6]) * 1e-3;
    } else {
        t.total = ev_ms(h->ev_t[0], h->ev_t[4]) * 1e-3;
    }
}

// Output arrays of ops_spgemm: the handle's pool (stream-ordered) or plain cudaMalloc.
cudaError_t out_alloc(ops_handle_s *h, void **p, size_t bytes, cudaStream_t st)
{
    if (h->out_malloc) return cudaMalloc(p, bytes);
    return cudaMallocFromPoolAsync(p, bytes, h->pool, st);
}

void out_free(ops_handle_s *h, void *p, cudaStream_t st)
{
    if (!p) return;
    if (h->out_malloc) {
        cudaStreamSynchronize(st);
        cudaFree(p);
    } else {
        cudaFreeAsync(p, st);
    }
}

}  // namespace

// ================================================================== C ABI ==========
extern "C" {

const char *ops_version(void) { return kVersion; }

const char *ops_status_string(int s)
{
    switch (s) {
        case OPS_OK: return "ok";
        case OPS_NONSQUARE: return "nonsquare";
        case OPS_INT32_OVERFLOW: return "int32_overflow";
        case OPS_OOM: return "oom";
        case OPS_CUDA_ERROR: return "cuda_error";
        case OPS_EXCEPTION: return "exception";
        case OPS_INVALID_ARGUMENT: return "invalid_argument";
        case OPS_INVALID_CSR: return "invalid_csr";
        case OPS_PROBE_LIMIT: return "probe_limit";
        case OPS_TIMEOUT: return "timeout";
        case OPS_NOT_SUPPORTED: return "not_supported";
        case OPS_COUNT_MISMATCH: return "count_mismatch";
    }
    return "unknown";
}

int ops_handle_create(ops_handle_t *out)
{
    if (!out) return OPS_INVALID_ARGUMENT;
    *out = nullptr;
    ops_handle_s *h = new (std::nothrow) ops_handle_s();
    if (!h) return OPS_EXCEPTION;
    cudaError_t e = cudaGetDevice(&h->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
    if (e == cudaSuccess) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = h->device;
        e = cudaMemPoolCreate(&h->pool, &props);
    }
    if (e == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        e = cudaMemPoolSetAttribute(h->pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    // the D rows' whole-GPU sort is a chain of about twenty short launches, the longest
    // path of a call that has D rows: its stream gets the highest priority, so its blocks
    // are scheduled ahead of the other classes' waiting blocks
    int prio_low = 0, prio_high = 0;
    if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    for (int c = 0; c < kNumClasses && e == cudaSuccess; ++c) {
        e = cudaStreamCreateWithPriority(&h->side[c], cudaStreamNonBlocking, c == kClsD ? prio_high : prio_low);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_join[c], cudaEventDisableTiming);
    }
    for (int x = 0; x < ops_handle_s::kNumExtra && e == cudaSuccess; ++x) {
        e = cudaStreamCreateWithFlags(&h->side_x[x], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_x_fork[x], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_x_join[x], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming);
    for (int i = 0; i < ops_handle_s::kNumEv && e == cudaSuccess; ++i) e = cudaEventCreate(&h->ev_t[i]);
    for (int ph = 0; ph < 2 && e == cudaSuccess; ++ph)
        for (int c = 0; c < kNumClasses && e == cudaSuccess; ++c)
            for (int k = 0; k < 2 && e == cudaSuccess; ++k) e = cudaEventCreate(&h->ev_k[ph][c][k]);
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void **>(&h->h_info), sizeof(DevInfo));
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void **>(&h->h_info_count), sizeof(DevInfo));
    if (e == cudaSuccess) {
        set_smem_attrs<double>();
        set_smem_attrs<float>();
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        ops_handle_destroy(h);
        return status_of(e);
    }
    *out = h;
    return OPS_OK;
}

int ops_handle_destroy(ops_handle_t h)
{
    if (!h) return OPS_OK;
    cudaDeviceSynchronize();
    for (ops_handle_s *s : h->spare) ops_handle_destroy(s);
    if (h->ws) cudaFree(h->ws);
    if (h->dense) cudaFree(h->dense);
    if (h->stage) cudaFree(h->stage);
    for (int c = 0; c < kNumClasses; ++c) {
        if (h->side[c]) cudaStreamDestroy(h->side[c]);
        if (h->ev_join[c]) cudaEventDestroy(h->ev_join[c]);
    }
    for (int x = 0; x < ops_handle_s::kNumExtra; ++x) {
        if (h->side_x[x]) cudaStreamDestroy(h->side_x[x]);
        if (h->ev_x_fork[x]) cudaEventDestroy(h->ev_x_fork[x]);
        if (h->ev_x_join[x]) cudaEventDestroy(h->ev_x_join[x]);
    }
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    for (int i = 0; i < ops_handle_s::kNumEv; ++i)
        if (h->ev_t[i]) cudaEventDestroy(h->ev_t[i]);
    for (int ph = 0; ph < 2; ++ph)
        for (int c = 0; c < kNumClasses; ++c)
            for (int k = 0; k < 2; ++k)
                if (h->ev_k[ph][c][k]) cudaEventDestroy(h->ev_k[ph][c][k]);
    if (h->h_info) cudaFreeHost(h->h_info);
    if (h->h_info_count) cudaFreeHost(h->h_info_count);
    if (h->pool) cudaMemPoolDestroy(h->pool);
    (void)cudaGetLastError();
    delete h;
    return OPS_OK;
}

int ops_handle_set_timing(ops_handle_t h, int enable)
{
    if (!h) return OPS_INVALID_ARGUMENT;
    h->timing = enable < 0 ? 0 : (enable > 2 ? 2 : enable);
    return OPS_OK;
}

int ops_handle_get_timings(ops_handle_t h, ops_timings *out)
{
    if (!h || !out) return OPS_INVALID_ARGUMENT;
    *out = h->last_t;
    return OPS_OK;
}

int ops_handle_set_dense_budget(ops_handle_t h, size_t bytes)
{
    if (!h) return OPS_INVALID_ARGUMENT;
    h->dense_budget = bytes;
    return OPS_OK;
}

int ops_handle_set_thresholds(ops_handle_t h, const int32_t *th, int n)
{
    if (!h || !th || n != 6) return OPS_INVALID_ARGUMENT;
    const Thresholds cap = default_thresholds();
    Thresholds t{th[0], th[1], th[2], th[3], th[4], th[5]};
    if (t.r8 < 0 || t.r8 > cap.r8 || t.r16 < 0 || t.r16 > cap.r16 || t.r32 < 0 || t.r32 > cap.r32 || t.w < 0 ||
        t.w > cap.w || t.e1 < 0 || t.e1 > cap.e1 || t.e2 < 0 || t.e2 > cap.e2)
        return fail(h, OPS_INVALID_ARGUMENT, "threshold above the compiled capacity of its class");
    h->th = t;
    h->plan_valid = false;
    return OPS_OK;
}

int ops_handle_get_thresholds(ops_handle_t h, int32_t *th, int n)
{
    if (!h || !th || n != 6) return OPS_INVALID_ARGUMENT;
    const Thresholds t = h->th;
    const int32_t v[6] = {t.r8, t.r16, t.r32, t.w, t.e1, t.e2};
    std::memcpy(th, v, sizeof(v));
    return OPS_OK;
}

int ops_handle_set_one_pass(ops_handle_t h, int mode)
{
    if (!h || mode < 0 || mode > 2) return OPS_INVALID_ARGUMENT;
    h->one_pass = mode;
    return OPS_OK;
}

int ops_handle_set_tuning(ops_handle_t h, const ops_tuning *t)
{
    if (!h || !t) return OPS_INVALID_ARGUMENT;
    if ((t->hash_slots != 2 && t->hash_slots != 4) || (t->batch_persistent != 0 && t->batch_persistent != 1) ||
        t->batch_warp_max < kBatchWarpMaxLo || t->batch_warp_max > kBatchWarpMaxHi)
        return fail(h, OPS_INVALID_ARGUMENT, "tuning value out of range");
    OPS_CHECK(ops_handle_set_thresholds(h, t->thresholds, 6));
    h->hash_slots = t->hash_slots;
    h->batch_persistent = t->batch_persistent;
    h->batch_warp_max = t->batch_warp_max;
    return OPS_OK;
}

int ops_handle_get_tuning(ops_handle_t h, ops_tuning *t)
{
    if (!h || !t) return OPS_INVALID_ARGUMENT;
    OPS_CHECK(ops_handle_get_thresholds(h, t->thresholds, 6));
    t->hash_slots = h->hash_slots;
    t->batch_persistent = h->batch_persistent;
    t->batch_warp_max = h->batch_warp_max;
    return OPS_OK;
}

int ops_handle_set_stage_budget(ops_handle_t h, size_t bytes)
{
    if (!h) return OPS_INVALID_ARGUMENT;
    h->stage_budget = bytes;
    return OPS_OK;
}

int ops_handle_set_output_malloc(ops_handle_t h, int use_cuda_malloc)
{
    if (!h) return OPS_INVALID_ARGUMENT;
    h->out_malloc = use_cuda_malloc != 0;
    return OPS_OK;
}

const char *ops_handle_last_error(ops_handle_t h) { return h ? h->last_error.c_str() : "null handle"; }

int ops_handle_subclass_rows(ops_handle_t h, int32_t *out, int n)
{
    if (!h || !out || n < 0) return OPS_INVALID_ARGUMENT;
    int v[10] = {};
    v[5] = h->d_rows_path[0];
    v[6] = h->d_rows_path[1];
    if (h->info) {
        DevInfo d{};
        OPS_CUDA(h, cudaMemcpy(&d, h->info, sizeof(DevInfo), cudaMemcpyDeviceToHost));
        // a one-pass call computes its staged E1 rows while counting (split1)
        v[0] = d.split[0] + d.split1[0];
        v[1] = d.split[1];
        v[2] = d.split[2] + d.split1[2];
        v[3] = d.split2[0];
        v[4] = d.split2[1];
        for (int i = 0; i < 3; ++i) v[7 + i] = d.rank_rows[i];
    }
    for (int i = 0; i < n && i < 10; ++i) out[i] = v[i];
    return OPS_OK;
}

int ops_spgemm_symbolic(ops_handle_t h, int32_t rows_a, int32_t cols_a, int32_t cols_b, const int32_t *a_rpt,
                        const int32_t *a_col, int64_t a_nnz, const int32_t *b_rpt, const int32_t *b_col, int64_t b_nnz,
                        int32_t *c_rpt, int64_t *c_nnz, void *stream)
{
    if (!h || !c_rpt || !c_nnz) return fail(h, OPS_INVALID_ARGUMENT, "null handle or output");
    try {
        h->last_error.clear();
        OPS_CHECK(check_mat_args(h, rows_a, cols_a, a_rpt, a_col, a_nnz));
        OPS_CHECK(check_mat_args(h, cols_a, cols_b, b_rpt, b_col, b_nnz));
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        const Mat A{rows_a, cols_a, a_rpt, a_col, nullptr};
        const Mat B{cols_a, cols_b, b_rpt, b_col, nullptr};
        h->op_dtype = -1;  // no values: two passes
        long long nnz = 0;
        OPS_CHECK(run_symbolic(h, A, B, c_rpt, &nnz, st));
        *c_nnz = nnz;
        fill_timings(h, false);
        return OPS_OK;
    } catch (...) {
        return fail(h, OPS_EXCEPTION, "exception in ops_spgemm_symbolic");
    }
}

int ops_spgemm_numeric(ops_handle_t h, int dtype, int32_t rows_a, int32_t cols_a, int32_t cols_b,
                       const int32_t *a_rpt, const int32_t *a_col, const void *a_val, const int32_t *b_rpt,
                       const int32_t *b_col, const void *b_val, const int32_t *c_rpt, int32_t *c_col, void *c_val,
                       void *stream)
{
    if (!h) return OPS_INVALID_ARGUMENT;
    if (dtype_size(dtype) == 0) return fail(h, OPS_INVALID_ARGUMENT, "unknown dtype");
    try {
        h->last_error.clear();
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        const Mat A{rows_a, cols_a, a_rpt, a_col, a_val};
        const Mat B{cols_a, cols_b, b_rpt, b_col, b_val};
        if (h->plan_nnz > 0 && (!c_col || !c_val || !a_val || !b_val))
            return fail(h, OPS_INVALID_ARGUMENT, "null values or output");
        if (dtype == OPS_F64)
            return run_numeric<double>(h, A, B, c_rpt, c_col, static_cast<double *>(c_val), st);
        return run_numeric<float>(h, A, B, c_rpt, c_col, static_cast<float *>(c_val), st);
    } catch (...) {
        return fail(h, OPS_EXCEPTION, "exception in ops_spgemm_numeric");
    }
}

int ops_spgemm_check(ops_handle_t h, void *stream)
{
    if (!h) return OPS_INVALID_ARGUMENT;
    return check_flags(h, static_cast<cudaStream_t>(stream));
}

int ops_spgemm(ops_handle_t h, int dtype, int32_t rows_a, int32_t cols_a, int32_t cols_b, const int32_t *a_rpt,
               const int32_t *a_col, const void *a_val, int64_t a_nnz, const int32_t *b_rpt, const int32_t *b_col,
               const void *b_val, int64_t b_nnz, int32_t **c_rpt, int32_t **c_col, void **c_val, int64_t *c_nnz,
               void *stream)
{
    if (!h || !c_rpt || !c_col || !c_val || !c_nnz) return fail(h, OPS_INVALID_ARGUMENT, "null handle or output");
    const int vs = dtype_size(dtype);
    if (vs == 0) return fail(h, OPS_INVALID_ARGUMENT, "unknown dtype");
    *c_rpt = nullptr;
    *c_col = nullptr;
    *c_val = nullptr;
    *c_nnz = 0;
    try {
        h->last_error.clear();
        OPS_CHECK(check_mat_args(h, rows_a, cols_a, a_rpt, a_col, a_nnz));
        OPS_CHECK(check_mat_args(h, cols_a, cols_b, b_rpt, b_col, b_nnz));
        if ((a_nnz > 0 && !a_val) || (b_nnz > 0 && !b_val)) return fail(h, OPS_INVALID_ARGUMENT, "null values");
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        const Mat A{rows_a, cols_a, a_rpt, a_col, a_val};
        const Mat B{cols_a, cols_b, b_rpt, b_col, b_val};
        // the values are known before the counting phase: the R16, R32 and W rows may run
        // their numeric kernels there (one pass); reset whichever way the call returns
        struct OnePassScope {
            ops_handle_s *h;
            ~OnePassScope()
            {
                h->op_dtype = -1;
                h->op_aval = h->op_bval = nullptr;
                h->staged = false;
            }
        } one_pass_scope{h};
        h->op_dtype = dtype;
        h->op_aval = a_val;
        h->op_bval = b_val;
        void *p = nullptr;
        OPS_CUDA(h, out_alloc(h, &p, sizeof(int) * ((size_t)rows_a + 1), st));
        int *rpt = static_cast<int *>(p);
        long long nnz = 0;
        int s = run_symbolic(h, A, B, rpt, &nnz, st, true);
        if (s != OPS_OK) {
            out_free(h, rpt, st);
            return s;
        }
        // nnz < 0: C allocated at one entry per product, its count read after the numeric
        // phase, with no host round trip between the two phases
        const bool early = nnz < 0;
        const long long cap = early ? h->plan_nnz : nnz;
        void *col = nullptr, *val = nullptr;
        cudaError_t e = out_alloc(h, &col, sizeof(int) * (size_t)std::max(cap, 1LL), st);
        if (e == cudaSuccess) e = out_alloc(h, &val, (size_t)vs * (size_t)std::max(cap, 1LL), st);
        if (h->timing && e == cudaSuccess) e = cudaEventRecord(h->ev_t[5], st);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            out_free(h, col, st);
            out_free(h, rpt, st);
            return fail(h, status_of(e), std::string("allocating C: ") + cudaGetErrorString(e));
        }
        s = dtype == OPS_F64 ? run_numeric<double>(h, A, B, rpt, static_cast<int *>(col), static_cast<double *>(val), st)
                             : run_numeric<float>(h, A, B, rpt, static_cast<int *>(col), static_cast<float *>(val), st);
        if (s == OPS_OK && h->timing) {
            e = cudaEventRecord(h->ev_t[6], st);
            if (e != cudaSuccess) s = fail(h, status_of(e), "event record");
        }
        if (s == OPS_OK) s = check_flags(h, st);
        if (early) {  // the stream has passed the counting phase's results (a sync above or
                      // on the error path below); they take precedence over the numeric's
            if (s != OPS_OK) cudaStreamSynchronize(st);
            const int sc = count_status(h, *h->h_info_count);
            if (sc != OPS_OK) s = sc;
            nnz = (long long)h->h_info_count->total_nnz;
            h->plan_nnz = nnz;
        }
        if (s != OPS_OK) {
            out_free(h, val, st);
            out_free(h, col, st);
            out_free(h, rpt, st);
            cudaStreamSynchronize(st);
            return s;
        }
        fill_timings(h, true);
        *c_rpt = rpt;
        *c_col = static_cast<int *>(col);
        *c_val = val;
        *c_nnz = nnz;
        return OPS_OK;
    } catch (...) {
        return fail(h, OPS_EXCEPTION, "exception in ops_spgemm");
    }
}

int ops_free(void *dptr, void *stream)
{
    if (!dptr) return OPS_OK;
    cudaError_t e = cudaFreeAsync(dptr, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return status_of(e);
    }
    return OPS_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ ops_flop -------
namespace {
__global__ void __launch_bounds__(256) k_flop64(const int *__restrict__ arpt, const int *__restrict__ acol,
                                                const int *__restrict__ brpt, int M, int K, long long *row_flop,
                                                unsigned long long *total, int *bad)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long s = 0;
    if (r < M) {
        for (int p = arpt[r]; p < arpt[r + 1]; ++p) {
            const int j = acol[p];
            if ((unsigned)j < (unsigned)K) s += (unsigned long long)(brpt[j + 1] - brpt[j]);
            else atomicOr(bad, 1);
        }
        if (row_flop) row_flop[r] = (long long)s;
    }
    block_add_u64(s, total);
}
}  // namespace

extern "C" int ops_flop(int32_t rows_a, int32_t cols_a, const int32_t *a_rpt, const int32_t *a_col,
                        const int32_t *b_rpt, int64_t *row_flop, int64_t *total, void *stream)
{
    if (rows_a < 0 || !total || (rows_a > 0 && (!a_rpt || !b_rpt))) return OPS_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    void *p = nullptr;
    cudaError_t e = cudaMallocAsync(&p, 16, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(p, 0, 16, st);
    unsigned long long *d_total = static_cast<unsigned long long *>(p);
    int *d_bad = reinterpret_cast<int *>(d_total + 1);
    if (e == cudaSuccess && rows_a > 0) {
        k_flop64<<<(rows_a + 255) / 256, 256, 0, st>>>(a_rpt, a_col, b_rpt, rows_a, cols_a,
                                                      reinterpret_cast<long long *>(row_flop), d_total, d_bad);
        e = cudaGetLastError();
    }
    unsigned long long h_res[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_res, p, 16, cudaMemcpyDeviceToHost, st);
    if (p) cudaFreeAsync(p, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return status_of(e);
    }
    if (h_res[1] & 1ull) return OPS_INVALID_CSR;
    *total = (int64_t)h_res[0];
    return OPS_OK;
}
