// spgemm.cpp — drop-in entry points (signatures of OpSparse's
// include/opsparse/core_algo/spgemm/spgemm.hpp:12-21) implemented over the C ABI of
// opsparse_gb300.h.  C's device arrays are allocated with cudaMalloc so that the
// caller's CSR::drelease()/cudaFree() releases them, as with the original library.
#include "opsparse/core_algo/spgemm/spgemm.hpp"

#include <climits>
#include <stdexcept>
#include <string>

#include "opsparse/numeric/compute_flop.hpp"
#include "opsparse/utils/tsc_timer.hpp"
#include "opsparse_gb300.h"

namespace opsparse {

SpgemmMeta::SpgemmMeta(CSR &C) { allocate_rpt(C); }

void SpgemmMeta::allocate_rpt(CSR &C)
{
    OPSPARSE_CHECK_CUDA(cudaMalloc(&C.d_rpt, sizeof(mint) * (static_cast<std::size_t>(C.M) + 1)));
}

void SpgemmMeta::allocate(CSR &C)
{
    M = C.M;
    N = C.N;
    (void)handle();
}

// The handle (streams, pool, workspace) is kept for the next call.
void SpgemmMeta::release() {}

ops_handle_s *SpgemmMeta::handle()
{
    if (!handle_) {
        const int s = ops_handle_create(&handle_);
        if (s != OPS_OK) {
            handle_ = nullptr;
            throw std::runtime_error(std::string("ops_handle_create: ") + ops_status_string(s));
        }
        ops_handle_set_output_malloc(handle_, 1);
    }
    return handle_;
}

SpgemmMeta::~SpgemmMeta()
{
    if (handle_) ops_handle_destroy(handle_);
    handle_ = nullptr;
}

namespace {

// Runs one C = A*B through the C ABI and publishes the result into C (device arrays).
int run(const CSR &A, const CSR &B, CSR &C, SpgemmMeta &meta, SpgemmTimings &timing, bool phase_timing)
{
    if (A.N != B.M) return OPS_NONSQUARE;
    ops_handle_s *h = meta.handle();
    ops_handle_set_timing(h, phase_timing ? 1 : 0);
    if (C.d_rpt) {  // a row_ptr pre-allocated by SpgemmMeta(CSR&) is replaced
        cudaFree(C.d_rpt);
        C.d_rpt = nullptr;
    }
    C.M = A.M;
    C.N = B.N;
    C.nnz = 0;
    int32_t *rpt = nullptr, *col = nullptr;
    void *val = nullptr;
    int64_t nnz = 0;
    const int s = ops_spgemm(h, OPS_F64, A.M, A.N, B.N, A.d_rpt, A.d_col, A.d_val, A.nnz, B.d_rpt, B.d_col, B.d_val,
                             B.nnz, &rpt, &col, &val, &nnz, meta.stream);
    if (s != OPS_OK) return s;
    C.d_rpt = rpt;
    C.d_col = col;
    C.d_val = static_cast<mdouble *>(val);
    C.nnz = static_cast<mint>(nnz);
    ops_timings t{};
    ops_handle_get_timings(h, &t);
    meta.M = C.M;
    meta.N = C.N;
    meta.total_nnz = t.nnz;
    mint off = 0;
    for (int c = 0; c < kNumBin; ++c) {
        meta.bin_size[c] = t.class_rows[c];
        meta.bin_offset[c] = off;
        off += t.class_rows[c];
    }
    if (phase_timing) {
        timing.setup = t.setup;
        timing.symbolic_binning = t.symbolic_binning;
        timing.symbolic = t.symbolic;
        timing.reduce = t.reduce;
        timing.numeric_binning = t.numeric_binning;
        timing.prefix = t.prefix;
        timing.allocate = t.allocate;
        timing.numeric = t.numeric;
        timing.cleanup = t.cleanup;
        timing.total = t.total;
    }
    return OPS_OK;
}

void throw_on(int s, ops_handle_s *h)
{
    if (s == OPS_OK) return;
    std::string msg = std::string("opsparse_spgemm: ") + ops_status_string(s);
    if (h) msg += std::string(" (") + ops_handle_last_error(h) + ")";
    throw std::runtime_error(msg);
}

}  // namespace

void opsparse_spgemm(const CSR &A, const CSR &B, CSR &C, SpgemmMeta &meta, SpgemmTimings &timing)
{
    throw_on(run(A, B, C, meta, timing, true), meta.handle());
}

void opsparse_spgemm_reg(const CSR &A, const CSR &B, CSR &C, SpgemmMeta &meta, SpgemmTimings &timing)
{
    const double t0 = fast_clock_time();
    const int s = run(A, B, C, meta, timing, false);
    throw_on(s, meta.handle());
    timing.total = fast_clock_time() - t0;
}

SpgemmStatus opsparse_spgemm_safe(const CSR &A, const CSR &B, CSR &C, SpgemmMeta &meta, SpgemmTimings &timing,
                                  SpgemmPerf &perf)
{
    perf.reset();
    if (A.N != B.M) {
        perf.status = SpgemmStatus::nonsquare;
        perf.error_msg = "A.N != B.M";
        return perf.status;
    }
    try {
        ops_handle_s *h = meta.handle();
        int64_t flop = 0;
        int s = ops_flop(A.M, A.N, A.d_rpt, A.d_col, B.d_rpt, nullptr, &flop, meta.stream);
        perf.total_flop = flop;
        query_cuda_memory(perf.free_before_bytes, perf.device_total_bytes);
        const double t0 = fast_clock_time();
        if (s == OPS_OK) s = run(A, B, C, meta, timing, false);
        timing.total = fast_clock_time() - t0;
        switch (s) {
            case OPS_OK: perf.status = SpgemmStatus::ok; break;
            case OPS_NONSQUARE: perf.status = SpgemmStatus::nonsquare; break;
            case OPS_INT32_OVERFLOW: perf.status = SpgemmStatus::int32_overflow; break;
            case OPS_OOM: perf.status = SpgemmStatus::oom; break;
            case OPS_CUDA_ERROR: perf.status = SpgemmStatus::cuda_error; break;
            default: perf.status = SpgemmStatus::exception; break;
        }
        if (s != OPS_OK) perf.error_msg = std::string(ops_status_string(s)) + ": " + ops_handle_last_error(h);
        else perf.c_nnz = C.nnz;
        query_cuda_memory(perf.free_after_bytes, perf.device_total_bytes);
        if (perf.free_before_bytes >= perf.free_after_bytes)
            perf.peak_used_bytes = perf.free_before_bytes - perf.free_after_bytes;
        return perf.status;
    } catch (const std::exception &e) {
        perf.status = SpgemmStatus::exception;
        perf.error_msg = e.what();
        return perf.status;
    }
}

void opsparse_spgemm_backward(const CSR &A, const CSR &B, const CSR &C, const mdouble *d_dC, mdouble *d_dA,
                              mdouble *d_dB, SpgemmMeta &meta)
{
    if (A.N != B.M) throw_on(OPS_NONSQUARE, nullptr);
    if (C.M != A.M || C.N != B.N) throw std::runtime_error("opsparse_spgemm_backward: C is not A*B's shape");
    ops_handle_s *h = meta.handle();
    int s = ops_spgemm_backward(h, OPS_F64, A.M, A.N, B.N, A.d_rpt, A.d_col, A.d_val, A.nnz, B.d_rpt, B.d_col,
                                B.d_val, B.nnz, C.d_rpt, C.d_col, d_dC, d_dA, d_dB, meta.stream);
    if (s == OPS_OK) s = ops_spgemm_check(h, meta.stream);  // synchronizes the stream
    throw_on(s, h);
}

}  // namespace opsparse
