/*
 * opsparse_gb300.h — C ABI of the GB300 CSR SpGEMM library (libopsparse_gb300.so).
 *
 * Plain pointers and sizes only.  Every matrix argument is a CSR triple of DEVICE
 * pointers: row_ptr (rows+1 int32), col_idx (nnz int32, ascending and unique within each
 * row) and values (nnz elements of the call's value type).  Every function returns an
 * ops_status (0 = success) and never throws.  Calls on one handle must not overlap;
 * use one handle per host thread.
 *
 * Correspondence with OpSparse's C++ API (paths relative to its source tree):
 *   ops_spgemm            <- opsparse_spgemm / opsparse_spgemm_reg
 *                            (include/opsparse/core_algo/spgemm/spgemm.hpp:12-17,
 *                             src/opsparse/core_algo/spgemm/spgemm.cu:16-126)
 *   ops_spgemm_symbolic   <- h_setup + h_symbolic_binning + h_symbolic + the row_ptr scan
 *                            (src/opsparse/core_algo/spgemm/spgemm_phases.cu:19-121, spgemm.cu:49)
 *   ops_spgemm_numeric    <- h_numeric_binning + h_numeric_full_occu
 *                            (spgemm_phases.cu:123-206)
 *   ops_flop              <- k_compute_flop (src/opsparse/numeric/compute_flop.cu:9-31)
 *   status codes 0..5     <- SpgemmStatus (include/opsparse/profile/perf.hpp:16-23)
 *   ops_timings           <- SpgemmTimings fields (include/opsparse/profile/spgemm_timings.hpp:6-30)
 *   ops_handle_*          <- SpgemmMeta (include/opsparse/core_algo/spgemm/meta.hpp:15-60),
 *                            but persistent: streams, pool and workspace survive across calls.
 */
#ifndef OPSPARSE_GB300_H_
#define OPSPARSE_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ops_handle_s *ops_handle_t;

/* Status codes.  0..5 have the numeric values of OpSparse's SpgemmStatus. */
enum ops_status {
    OPS_OK = 0,
    OPS_NONSQUARE = 1,         /* A.cols != B.rows */
    OPS_INT32_OVERFLOW = 2,    /* a row's products or nnz(C) exceed INT32_MAX */
    OPS_OOM = 3,               /* device allocation failed */
    OPS_CUDA_ERROR = 4,        /* any other CUDA error */
    OPS_EXCEPTION = 5,         /* unexpected host-side failure */
    OPS_INVALID_ARGUMENT = 6,  /* null pointer, negative size, unknown dtype, ... */
    OPS_INVALID_CSR = 7,       /* a column index outside [0, cols) or a malformed row_ptr */
    OPS_PROBE_LIMIT = 8,       /* an internal hash table overflowed (a library bug if seen) */
    OPS_TIMEOUT = 9,           /* a bounded device wait gave up */
    OPS_NOT_SUPPORTED = 10,    /* no plan / request outside what the library supports */
    OPS_COUNT_MISMATCH = 11    /* numeric found a different nnz than symbolic (library bug) */
};

/* Value types. */
enum ops_dtype { OPS_F64 = 0, OPS_F32 = 1 };

/* Per-call phase times in seconds (CUDA events), filled when timing is enabled on the
 * handle.  Field names follow OpSparse's SpgemmTimings. */
typedef struct {
    double setup;             /* workspace preparation */
    double symbolic_binning;  /* product count + row classification (one kernel) */
    double symbolic;          /* per-class symbolic kernels */
    double reduce;            /* always 0: no separate reduction phase */
    double numeric_binning;   /* always 0: numeric reuses the symbolic classification */
    double prefix;            /* row_ptr scan */
    double allocate;          /* C allocation */
    double numeric;           /* per-class numeric kernels */
    double cleanup;           /* always 0: workspace is kept on the handle */
    double total;
    int64_t flop;             /* intermediate products, sum over rows */
    int64_t nnz;              /* nnz(C) */
    int32_t class_rows[8];    /* rows per class: R8, R16, R32, W, E1, E2, D, - */
    int64_t launches;         /* library kernels launched by the call */
    float kernel_ms[2][8];    /* [symbolic, numeric][class] kernel times (timing level 2) */
} ops_timings;

/* -------------------------------------------------------------------- handle -- */
int ops_handle_create(ops_handle_t *handle);
int ops_handle_destroy(ops_handle_t handle);
/* Event timing: 0 off, 1 per phase, 2 per phase and per class kernel (events recorded on
 * each class's own stream around its kernel). */
int ops_handle_set_timing(ops_handle_t handle, int enable);
int ops_handle_get_timings(ops_handle_t handle, ops_timings *out);
/* Upper bound in bytes for the dense-row scratch (default 4 GiB). */
int ops_handle_set_dense_budget(ops_handle_t handle, size_t bytes);
/* Where ops_spgemm allocates C: 0 (default) = the handle's stream-ordered pool, release
 * with ops_free; 1 = cudaMalloc, release with cudaFree (what OpSparse's CSR::drelease
 * expects). */
int ops_handle_set_output_malloc(ops_handle_t handle, int use_cuda_malloc);
/* One pass in ops_spgemm, where the values are known before the counting phase.  mode 1
 * (default): when at least 2^20 products are eligible, the rows of the R16 to D classes
 * (see ops_handle_set_thresholds) are computed during the counting phase into a staging
 * area held by the handle and copied into C after the row_ptr scan, instead of reading A
 * and B again in a second pass.  Left to two passes: the R8 rows (counted while they are
 * classified, computed straight into C), the E1 rows whose products fall within 32768
 * consecutive columns (banded and stencil rows, which fold many products per output), and
 * the D rows when their whole-GPU sort would exceed the dense-row budget.  The staging area grows only and holds the eligible
 * products (column and value each), at most the staging budget (2 GiB unless
 * ops_handle_set_stage_budget says otherwise); beyond that, or if it cannot be allocated,
 * the call runs two passes.  mode 2: the same at any size.  mode 0: always two
 * passes.  Results are identical in every mode.  ops_spgemm_symbolic and
 * ops_spgemm_numeric always run two passes.  No OpSparse counterpart: its symbolic and
 * numeric kernels always run separately (core_algo/spgemm/spgemm.cu:16-62). */
int ops_handle_set_one_pass(ops_handle_t handle, int mode);
/* Every run-time choice of kernels and sizes, in one record: the autotuner's search space.
 * No OpSparse counterpart: its bin ranges, table sizes and threads per row are compile-time
 * constants (include/opsparse/utils/config.hpp:6-27, kernels/binning.cuh:21,105). */
typedef struct {
    int32_t thresholds[6];    /* row-class bounds, see ops_handle_set_thresholds */
    int32_t hash_slots;       /* slots per output entry of the E1 warp-hash numeric table (2 or 4,
                                 default 4) */
    int32_t batch_persistent; /* batches: 1 (default) = one setup kernel and one persistent
                                 kernel per row-size queue and phase over every problem's rows
                                 (where every row has at most 4,096 products and 1,280 A
                                 entries), 0 = per-segment pipeline */
    int32_t batch_warp_max;   /* threads per row in the persistent batch kernels: rows of at most
                                 this many products (128..512, default 512) get one warp
                                 (register sort), larger rows a 128-thread CTA (up to 1,024
                                 products) or a 256-thread CTA (up to 4,096) */
} ops_tuning;
int ops_handle_set_tuning(ops_handle_t handle, const ops_tuning *tuning);
int ops_handle_get_tuning(ops_handle_t handle, ops_tuning *tuning);
/* Upper bound in bytes for the one-pass staging area (default 2 GiB); a call whose staged
 * products need more runs two passes.  No OpSparse counterpart. */
int ops_handle_set_stage_budget(ops_handle_t handle, size_t bytes);
/* Row-class thresholds used by the next symbolic phase, as 6 int32 upper bounds on a
 * row's intermediate products: {R8, R16, R32, W, E1, E2} (defaults {8, 16, 32, 128, 1024,
 * 13312}, which are also the maxima; 0 switches a class off; rows above E2 use the dense
 * class).  Replaces OpSparse's compile-time bin ranges (kernels/binning.cuh:21,105). */
int ops_handle_set_thresholds(ops_handle_t handle, const int32_t *thresholds, int count);
int ops_handle_get_thresholds(ops_handle_t handle, int32_t *thresholds, int count);
/* Message for the last failing call on this handle ("" if none). */
const char *ops_handle_last_error(ops_handle_t handle);
/* Rows handled by each sub-kernel in the last call (synchronises the handle's device
 * counters to the host): out[0..2] = E1 numeric rows by warp sort, warp hash and
 * expand/sort/compress; out[3..4] = E2 rows by the mid and the large expand/sort/compress
 * shape; out[5..6] = D rows by the whole-GPU sort and by the dense-row kernel;
 * out[7..9] = expand rows of the numeric phase whose columns span fewer than 65,536
 * columns, by path: column-window rank with no repeated column, rank with repeated
 * columns re-folded, sort (more than 128 products in repeated columns).  Diagnostic; no
 * OpSparse counterpart. */
int ops_handle_subclass_rows(ops_handle_t handle, int32_t *out, int count);
const char *ops_status_string(int status);

/* ------------------------------------------------------------------- spgemm -- */
/* C = A * B in one call (drop-in for opsparse_spgemm).  A is rows_a x cols_a, B is
 * cols_a x cols_b.  On success *c_rpt, *c_col, *c_val hold device arrays allocated by
 * the library (ops_handle_set_output_malloc says how to release them) and *c_nnz
 * receives nnz(C).  Returns after the result is complete (the stream is synchronized).
 * dtype: OPS_F64 or OPS_F32.  c_col and c_val hold at least nnz(C) entries: where C at
 * one entry per intermediate product fits 256 MiB (and no row needs the whole-GPU sort),
 * they are allocated at that size before nnz(C) is known, which spares the call a host
 * round trip between its counting and numeric phases. */
int ops_spgemm(ops_handle_t handle, int dtype, int32_t rows_a, int32_t cols_a, int32_t cols_b,
               const int32_t *a_rpt, const int32_t *a_col, const void *a_val, int64_t a_nnz,
               const int32_t *b_rpt, const int32_t *b_col, const void *b_val, int64_t b_nnz,
               int32_t **c_rpt, int32_t **c_col, void **c_val, int64_t *c_nnz, void *stream);

/* Symbolic phase: fills the caller's c_rpt (rows_a + 1 int32, device) with C's row
 * pointers and returns nnz(C) in *c_nnz.  Keeps the row classification on the handle
 * for a following ops_spgemm_numeric on the same A and B.  Synchronizes the stream. */
int ops_spgemm_symbolic(ops_handle_t handle, int32_t rows_a, int32_t cols_a, int32_t cols_b,
                        const int32_t *a_rpt, const int32_t *a_col, int64_t a_nnz,
                        const int32_t *b_rpt, const int32_t *b_col, int64_t b_nnz,
                        int32_t *c_rpt, int64_t *c_nnz, void *stream);

/* Numeric phase: fills the caller's c_col / c_val (nnz(C) each) for the pattern from the
 * last ops_spgemm_symbolic on this handle (same A and B structure; values may differ).
 * Asynchronous: returns once the kernels are queued on `stream`. */
int ops_spgemm_numeric(ops_handle_t handle, int dtype, int32_t rows_a, int32_t cols_a, int32_t cols_b,
                       const int32_t *a_rpt, const int32_t *a_col, const void *a_val,
                       const int32_t *b_rpt, const int32_t *b_col, const void *b_val,
                       const int32_t *c_rpt, int32_t *c_col, void *c_val, void *stream);

/* Checks the device-side error flags raised by the last numeric phase (synchronizes the
 * stream).  Returns OPS_OK, OPS_PROBE_LIMIT or OPS_COUNT_MISMATCH. */
int ops_spgemm_check(ops_handle_t handle, void *stream);

/* ------------------------------------------------------------------ backward -- */
/* Gradients of loss = sum(dC .* C) for C = A * B with A's, B's and C's patterns fixed
 * (no counterpart in OpSparse).  c_rpt/c_col is C's pattern as produced by the forward
 * (ascending columns); dc_val holds dC on it.  Fills da_val (A's pattern) and/or db_val
 * (B's pattern); either may be NULL.  dA_ij = sum_k B_jk dC_ik folded over k in B's row
 * order; dB_jk = sum_i A_ij dC_ik folded over ascending i; FP64 uses one FMA per term,
 * FP32 the Dot2 compensated sum.  The first call for a pattern builds a plan on the handle
 * (A's transpose order and, if it fits the map budget, each product's position in C);
 * later calls with the same pattern pointers reuse it.  Asynchronous; ops_spgemm_check
 * reports OPS_COUNT_MISMATCH if C's pattern lacks a product of A and B. */
int ops_spgemm_backward(ops_handle_t handle, int dtype, int32_t rows_a, int32_t cols_a, int32_t cols_b,
                        const int32_t *a_rpt, const int32_t *a_col, const void *a_val, int64_t a_nnz,
                        const int32_t *b_rpt, const int32_t *b_col, const void *b_val, int64_t b_nnz,
                        const int32_t *c_rpt, const int32_t *c_col, const void *dc_val,
                        void *da_val, void *db_val, void *stream);
/* Largest product -> position map (4 bytes per intermediate product) the backward plan may
 * keep (default 8 GiB).  Above it, positions are searched in C's rows on every call. */
int ops_handle_set_map_budget(ops_handle_t handle, size_t bytes);
/* Products and map mode (1 = map kept) of the current backward plan. */
int ops_backward_plan_info(ops_handle_t handle, int64_t *products, int *with_map);

/* ------------------------------------------------------------------- batched -- */
/* Many independent products C_b = A_b * B_b (no counterpart in OpSparse).  Each item holds
 * device CSR arrays; A_b is rows x cols_a, B_b is cols_a x cols_b. */
typedef struct {
    int32_t rows, cols_a, cols_b;
    int64_t a_nnz, b_nnz;
    const int32_t *a_rpt, *a_col;
    const void *a_val;
    const int32_t *b_rpt, *b_col;
    const void *b_val;
} ops_batch_item;

typedef struct ops_batch_s *ops_batch_t;

/* Plans a batch: per-problem product counts, grouping into segments whose products fit
 * int32 and block-diagonal layout of each segment; then, where every row has at most
 * 4,096 products and 1,280 A entries (and ops_tuning.batch_persistent is on), one setup
 * kernel that puts every row of every problem into one of four row-size queues and one
 * persistent kernel per queue that counts them all; otherwise a row classification and
 * symbolic phase per segment.  Then each segment's scan and the allocation of every C_b.  The items' value
 * pointers are read by ops_batch_execute, which may be called repeatedly with new values
 * in the same arrays.  The handle's row-class thresholds are used.  Synchronizes. */
int ops_batch_create(ops_handle_t handle, int dtype, int32_t count, const ops_batch_item *items, ops_batch_t *batch,
                     void *stream);
/* Numeric phase of every problem: the value gathers and one persistent kernel per queue
 * (or the per-segment numeric phases).  use_graph = 1: the first call records the work on
 * `stream` (a created stream) as a CUDA graph and later calls replay it with a single
 * cudaGraphLaunch; use_graph = 0: plain launches.  Asynchronous. */
int ops_batch_execute(ops_batch_t batch, int use_graph, void *stream);
/* Device-side error flags of the last execute (synchronizes). */
int ops_batch_check(ops_batch_t batch, void *stream);
/* Device pointers of C_b (views into the batch's storage, valid until destroy). */
int ops_batch_result(ops_batch_t batch, int32_t index, int32_t **c_rpt, int32_t **c_col, void **c_val,
                     int64_t *c_nnz);
int ops_batch_info(ops_batch_t batch, int32_t *segments, int64_t *flop, int64_t *nnz);
/* How the batch was planned: *persistent = 1 when one setup kernel and one persistent kernel
 * per row-size queue and phase cover all its problems (ops_tuning.batch_persistent), with
 * the rows its warp-per-row and CTA-per-row queues hold; 0 (queues 0) when it runs segment
 * by segment.  Diagnostic. */
int ops_batch_queues(ops_batch_t batch, int32_t *persistent, int64_t *warp_rows, int64_t *cta_rows);
/* Releases the batch (synchronizes).  Its device memory returns to the handle's pool and
 * its per-segment handles to the handle, both reused by the handle's next batch; destroy
 * every batch before its handle. */
int ops_batch_destroy(ops_batch_t batch);

/* ----------------------------------------------------------------- autotuner -- */
/* Chooses every field of ops_tuning for a workload by coordinate descent: the row-class
 * thresholds, the warp-hash table's slots per output entry (hash-table size), the batch
 * plan (persistent kernels over row-size queues, or per segment) and the largest row a warp
 * takes in the persistent kernels (threads per row: a warp, or a 128- or 256-thread CTA
 * above it).  Each candidate is timed as complete batched runs of `items` (a representative
 * sample) with CUDA events, median of `reps` runs.  Installs the best tuning on the handle
 * (read it with ops_handle_get_tuning), returns its thresholds in best[6] and the time in
 * *best_ms.  Synchronizes.  No OpSparse counterpart: its tunables are compile-time
 * constants (include/opsparse/utils/config.hpp:6-27). */
int ops_autotune(ops_handle_t handle, int dtype, int32_t count, const ops_batch_item *items, int reps,
                 int32_t *best, float *best_ms, void *stream);
/* Tuning records persisted as JSON {"<key>": [values], ...}; key typically names the GPU and
 * the workload.  ops_tuning_store / lookup keep the 6 thresholds; ops_tuning_store_record /
 * lookup_record the whole ops_tuning (a thresholds-only record reads back with the other
 * fields at their defaults).  The lookups return OPS_NOT_SUPPORTED when the key is absent. */
int ops_tuning_store(const char *path, const char *key, const int32_t *thresholds);
int ops_tuning_lookup(const char *path, const char *key, int32_t *thresholds);
int ops_tuning_store_record(const char *path, const char *key, const ops_tuning *tuning);
int ops_tuning_lookup_record(const char *path, const char *key, ops_tuning *tuning);

/* Per-row intermediate-product counts (row_flop, rows_a int64, device; may be NULL) and
 * their sum (*total, host).  Synchronizes the stream. */
int ops_flop(int32_t rows_a, int32_t cols_a, const int32_t *a_rpt, const int32_t *a_col, const int32_t *b_rpt,
             int64_t *row_flop, int64_t *total, void *stream);

/* ops_flop without any device allocation, for callers that may not allocate device memory
 * at this point: serving loops that forbid the CUDA allocator once running, hosts that give
 * the library a fixed memory budget.  Same arguments and results as ops_flop.  Its scratch
 * is a 64 KiB array in the library's own device memory, shared by every call: rows_a above
 * 2,097,152 returns OPS_NOT_SUPPORTED; calls that overlap on the GPU race and must be
 * serialized; the first call on a device resolves the array's address (keep that call
 * before any stream capture, and do not use the library across cudaDeviceReset).
 * Synchronizes the stream.  No counterpart in OpSparse. */
int ops_flop_noalloc(int32_t rows_a, int32_t cols_a, const int32_t *a_rpt, const int32_t *a_col,
                     const int32_t *b_rpt, int64_t *row_flop, int64_t *total, void *stream);

/* Releases a device array that ops_spgemm allocated from the handle's pool
 * (stream-ordered on `stream`). */
int ops_free(void *dptr, void *stream);

/* Library version string. */
const char *ops_version(void);

#ifdef __cplusplus
}
#endif

#endif /* OPSPARSE_GB300_H_ */
