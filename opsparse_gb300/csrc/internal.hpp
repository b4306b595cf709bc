// internal.hpp — the handle and the error helpers shared by the library's translation
// units (not part of the C ABI).
#pragma once

#include <string>
#include <vector>

#include "common.cuh"
#include "opsparse_gb300.h"

using opsg::DevInfo;
using opsg::kNumClasses;

// Per-pattern state of the fixed-pattern backward (built on first use, kept on the handle).
struct BackwardPlan {
    bool valid = false;
    // key: the pattern it was built for
    int M = 0, K = 0, N = 0;
    long long nnz_a = 0, nnz_b = 0;
    const int *a_rpt = nullptr, *a_col = nullptr, *b_rpt = nullptr, *b_col = nullptr;
    const int *c_rpt = nullptr, *c_col = nullptr;
    bool with_map = false;      // product -> position map stored (else binary search per product)
    long long products = 0;
    unsigned char *mem = nullptr;
    size_t bytes = 0;
    long long *pos_base = nullptr;  // [nnz_a] first product index of each A entry
    int *pmap = nullptr;            // [products] position in C of each product
    int *at_ptr = nullptr;          // [K+1] columns of A (transpose row pointers)
    int *at_ent = nullptr;          // [nnz_a] A entries ordered by (column, row)
    int *arow = nullptr;            // [nnz_a] row of each A entry
};

struct ops_handle_s {
    int device = 0;
    int num_sms = 0;
    cudaMemPool_t pool = nullptr;
    // segment handles of released batches, taken by the next batch of this handle (their
    // streams, events and workspaces are made once)
    std::vector<ops_handle_s *> spare;
    cudaStream_t side[kNumClasses] = {};
    cudaEvent_t ev_fork = nullptr;
    cudaEvent_t ev_join[kNumClasses] = {};
    // extra streams for the second kernel of a re-binned class (E1 numeric, E2)
    static constexpr int kNumExtra = 2;
    cudaStream_t side_x[kNumExtra] = {};
    cudaEvent_t ev_x_fork[kNumExtra] = {};
    cudaEvent_t ev_x_join[kNumExtra] = {};
    static constexpr int kNumEv = 8;
    cudaEvent_t ev_t[kNumEv] = {};
    cudaEvent_t ev_k[2][kNumClasses][2] = {};  // [phase][class][start, end]
    bool kmeasured[2][kNumClasses] = {};
    int timing = 0;
    long long launches = 0;
    bool out_malloc = false;  // allocate C with cudaMalloc instead of the pool
    ops_timings last_t{};
    size_t dense_budget = size_t(4) << 30;

    // workspace (grow-only)
    unsigned char *ws = nullptr;
    size_t ws_bytes = 0;
    int ws_M = -1;
    int *lists = nullptr;
    int *row_flop = nullptr;
    DevInfo *info = nullptr;
    void *cub_tmp = nullptr;
    size_t cub_bytes = 0;
    DevInfo *h_info = nullptr;  // pinned host mirror
    DevInfo *h_info_count = nullptr;  // the counting phase's results, read at the end of a
                                      // call whose C was allocated before they were known

    // dense-row scratch, all-zero between kernels
    unsigned char *dense = nullptr;
    size_t dense_bytes = 0;
    int dense_ctas = 0;

    // one-pass numeric (ops_spgemm, where the values are known before the counting
    // phase): every row but the R8 rows, the D rows and the E1 column-window rows is
    // computed in the counting phase into a staging area
    // (grow-only) at the exclusive prefix of the staged rows' product counts, and moved
    // into C after the scan
    int one_pass = 1;              // 0 off, 1 on above kMinStageFlop staged products, 2 on
    int op_dtype = -1;             // value type of the call in progress, -1 = two passes
    const void *op_aval = nullptr, *op_bval = nullptr;
    bool staged = false;           // the counting phase of the call in progress stages
    bool stage_e1 = false;         // ... and some of its rows are E1 rows
    bool stage_e1_all = false;     // ... all of the E1 rows
    bool stage_d = false;          // ... and the D rows (whole-GPU sort)
    unsigned char *stage = nullptr;        // [columns | values] of stage_entries entries
    size_t stage_bytes = 0;
    long long stage_entries = 0;
    size_t stage_budget = size_t(2) << 30;  // larger staging areas fall back to two passes
    int *soff = nullptr;           // [M + 1] staged products per row, then their prefix (workspace)

    // plan of the last symbolic phase
    bool plan_valid = false;
    int plan_M = 0, plan_K = 0, plan_N = 0;
    const int *plan_arpt = nullptr, *plan_acol = nullptr, *plan_brpt = nullptr, *plan_bcol = nullptr;
    int counts[kNumClasses] = {};
    long long plan_flop = 0;
    long long plan_nnz = 0;
    int d_rows_path[2] = {};      // D rows of the last phase by [whole-GPU sort, dense kernel]
    long long plan_d_flop = 0;    // products of the D rows
    long long plan_d_len_a = 0;   // A entries of the D rows

    // batches: 1 = one setup kernel and one persistent kernel per row-size queue and phase,
    // over every problem's rows (batch_rows.cuh), where every row fits the queues; 0 =
    // per-segment pipeline.  batch_warp_max = the largest row (products) a warp takes.
    int batch_persistent = 1;
    int batch_warp_max = 512;
    int hash_slots = 4;  // slots per output entry of the E1 warp-hash numeric table (2 or 4)

    size_t map_budget = size_t(8) << 30;  // largest product map the backward may keep
    opsg::Thresholds th = opsg::default_thresholds();
    opsg::Thresholds plan_th = opsg::default_thresholds();  // thresholds the current plan was built with
    BackwardPlan bwd;

    std::string last_error;
};

namespace opsg_internal {

// D rows (more than the E2 capacity) by whole-GPU expand / stable radix sort / compress
// (gesc.cu).  Returns OPS_NOT_SUPPORTED, having launched nothing, when the products do
// not fit 32-bit positions or the scratch exceeds the handle's dense budget; the caller
// then uses the dense-row kernel.  numeric with g.soff set: a one-pass call, whose D rows
// are computed into the staging area and counted into c_rpt.  dry_run: only the check.
template <typename T>
int run_d_rows(ops_handle_s *h, const opsg::SpgemmArgs<T> &g, const int *list, int n, bool numeric, cudaStream_t s,
               bool dry_run = false);

inline int status_of(cudaError_t e) { return e == cudaErrorMemoryAllocation ? OPS_OOM : OPS_CUDA_ERROR; }

inline int fail(ops_handle_s *h, int status, const std::string &msg)
{
    if (h) h->last_error = msg;
    return status;
}

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace opsg_internal

#define OPS_CUDA(h, expr)                                                                                      \
    do {                                                                                                       \
        cudaError_t e_ = (expr);                                                                               \
        if (e_ != cudaSuccess) {                                                                               \
            (void)cudaGetLastError();                                                                          \
            return opsg_internal::fail((h), opsg_internal::status_of(e_),                                      \
                                       std::string(#expr) + ": " + cudaGetErrorString(e_));                    \
        }                                                                                                      \
    } while (0)

#define OPS_CHECK(expr)              \
    do {                             \
        int s_ = (expr);             \
        if (s_ != OPS_OK) return s_; \
    } while (0)
