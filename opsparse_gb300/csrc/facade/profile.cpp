// profile.cpp — SpgemmTimings printing/arithmetic and SpgemmPerf helpers (API of
// OpSparse's include/opsparse/profile/{spgemm_timings,perf}.hpp) plus the host flop
// counter (include/opsparse/numeric/compute_flop.hpp).
#include <cstdio>

#include "opsparse/core_ds/csr.hpp"
#include "opsparse/numeric/compute_flop.hpp"
#include "opsparse/profile/perf.hpp"
#include "opsparse/profile/spgemm_timings.hpp"

namespace opsparse {

#define OPSPARSE_TIMING_FIELDS(X) \
    X(setup) X(symbolic_binning) X(symbolic) X(reduce) X(numeric_binning) X(prefix) X(allocate) X(numeric) X(cleanup) X(total)

void SpgemmTimings::operator+=(const SpgemmTimings &b)
{
#define ADD_FIELD(f) f += b.f;
    OPSPARSE_TIMING_FIELDS(ADD_FIELD)
#undef ADD_FIELD
}

void SpgemmTimings::operator/=(double x)
{
#define DIV_FIELD(f) f /= x;
    OPSPARSE_TIMING_FIELDS(DIV_FIELD)
#undef DIV_FIELD
}

void SpgemmTimings::print(double total_flop) const
{
    const double g = total_flop / 1e9;
    std::printf("total flop %lf\n", total_flop);
    if (!measure_separate) return;
    std::printf("time(ms):\n");
#define PRINT_MS(f) std::printf("    %-16s %8.3lfms %6.2lf%%\n", #f, 1000 * f, total > 0 ? f / total * 100 : 0.0);
    OPSPARSE_TIMING_FIELDS(PRINT_MS)
#undef PRINT_MS
    std::printf("perf(Gflops):\n");
#define PRINT_GF(f) std::printf("    %-16s %6.2lf\n", #f, f > 0 ? g / f : 0.0);
    OPSPARSE_TIMING_FIELDS(PRINT_GF)
#undef PRINT_GF
}

void SpgemmTimings::reg_print(double total_flop) const { std::printf("%6.2lf\n", total > 0 ? total_flop / 1e9 / total : 0.0); }

void SpgemmTimings::perf_print(double total_flop) const
{
    const double g = total_flop / 1e9;
    std::printf("%6.2lf %6.2lf\n", symbolic > 0 ? g / symbolic : 0.0, numeric > 0 ? g / numeric : 0.0);
}

void SpgemmTimings::binning_print(double) const
{
    const double b = symbolic_binning + numeric_binning;
    std::printf("%.4le %.4lf\n", b, total > 0 ? 100 * b / total : 0.0);
}

const char *to_cstr(SpgemmStatus s)
{
    switch (s) {
        case SpgemmStatus::ok: return "ok";
        case SpgemmStatus::nonsquare: return "nonsquare";
        case SpgemmStatus::int32_overflow: return "int32_overflow";
        case SpgemmStatus::oom: return "oom";
        case SpgemmStatus::cuda_error: return "cuda_error";
        case SpgemmStatus::exception: return "exception";
    }
    return "unknown";
}

void SpgemmPerf::reset()
{
    status = SpgemmStatus::ok;
    device_total_bytes = free_before_bytes = free_after_bytes = peak_used_bytes = attempted_bytes = 0;
    total_flop = 0;
    c_nnz = -1;
    error_msg.clear();
}

void SpgemmPerf::snapshot_free(std::size_t &out_free) const
{
    std::size_t total = 0;
    query_cuda_memory(out_free, total);
}

void query_cuda_memory(std::size_t &free_bytes, std::size_t &total_bytes)
{
    if (cudaMemGetInfo(&free_bytes, &total_bytes) != cudaSuccess) {
        (void)cudaGetLastError();
        free_bytes = total_bytes = 0;
    }
}

long compute_flop(const mint *row_ptr_a, const mint *col_idx_a, const mint *row_ptr_b, mint M, mint *row_flop_out)
{
    long total = 0;
    for (mint i = 0; i < M; ++i) {
        long s = 0;
        for (mint p = row_ptr_a[i]; p < row_ptr_a[i + 1]; ++p) s += row_ptr_b[col_idx_a[p] + 1] - row_ptr_b[col_idx_a[p]];
        if (row_flop_out) row_flop_out[i] = static_cast<mint>(s);
        total += s;
    }
    return total;
}

long compute_flop(const CSR &A, const CSR &B, mint *row_flop) { return compute_flop(A.rpt, A.col, B.rpt, A.M, row_flop); }

long compute_flop(const CSR &A, const CSR &B) { return compute_flop(A.rpt, A.col, B.rpt, A.M, nullptr); }

}  // namespace opsparse
