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

// Same text as OpSparse's SpgemmTimings::print (src/opsparse/profile/spgemm_timings.cpp:35-70),
// so logs and scripts that read it keep working: the four phases it highlights keep their
// ANSI colour, the shares divide by `total`, and GFLOPS divide by each phase's time (inf
// for a phase this library does not have, as there).
void SpgemmTimings::print(double total_flop) const
{
    const double g = total_flop / 1e9;
    std::printf("total flop %lf\n", total_flop);
    if (!measure_separate) return;
    const double sum_total =
        setup + symbolic_binning + symbolic + numeric_binning + reduce + prefix + allocate + numeric + cleanup;
    struct Row {
        const char *label;
        double v;
        bool red;
    };
    const Row rows[] = {{"setup           ", setup, false},     {"symbolic_binning", symbolic_binning, true},
                        {"symbolic        ", symbolic, true},   {"reduce           ", reduce, false},
                        {"numeric_binning ", numeric_binning, true}, {"prefix          ", prefix, false},
                        {"allocate        ", allocate, false},  {"numeric         ", numeric, true},
                        {"cleanup         ", cleanup, false},   {"sum_total       ", sum_total, false},
                        {"total           ", total, false}};
    std::printf("time(ms):\n");
    for (const Row &r : rows) {
        if (r.red) std::printf("\e[1;31m    %s %8.3lfms %6.2lf%%\n\e[0m", r.label, 1000 * r.v, r.v / total * 100);
        else std::printf("    %s %8.3lfms %6.2lf%%\n", r.label, 1000 * r.v, r.v / total * 100);
    }
    std::printf("perf(Gflops):\n");
    const Row perf[] = {{"setup           ", setup, false},    {"symbolic_binning", symbolic_binning, false},
                        {"symbolic        ", symbolic, false}, {"reduce          ", reduce, false},
                        {"numeric_binning ", numeric_binning, false}, {"prefix          ", prefix, false},
                        {"allocate        ", allocate, false}, {"numeric         ", numeric, false},
                        {"cleanup         ", cleanup, false},  {"total           ", total, false}};
    for (const Row &r : perf) std::printf("    %s %6.2lf\n", r.label, g / r.v);
}

void SpgemmTimings::reg_print(double total_flop) const { std::printf("%6.2lf\n", total_flop / 1e9 / total); }

void SpgemmTimings::perf_print(double total_flop) const
{
    const double g = total_flop / 1e9;
    std::printf("%6.2lf %6.2lf\n", g / symbolic, g / numeric);
}

void SpgemmTimings::binning_print(double) const
{
    const double b = symbolic_binning + numeric_binning;
    std::printf("%.4le %.4lf\n", b, 100 * b / total);
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
