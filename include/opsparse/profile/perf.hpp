// perf.hpp — status and memory snapshot of one SpGEMM (same names and numeric values as
// OpSparse's include/opsparse/profile/perf.hpp:16-51).
#ifndef OPSPARSE_PROFILE_PERF_HPP_
#define OPSPARSE_PROFILE_PERF_HPP_

#include <cstddef>
#include <string>

namespace opsparse {

enum class SpgemmStatus {
    ok = 0,
    nonsquare = 1,
    int32_overflow = 2,
    oom = 3,
    cuda_error = 4,
    exception = 5,
};

const char *to_cstr(SpgemmStatus s);

struct SpgemmPerf {
    SpgemmStatus status = SpgemmStatus::ok;
    std::size_t device_total_bytes = 0;
    std::size_t free_before_bytes = 0;
    std::size_t free_after_bytes = 0;
    std::size_t peak_used_bytes = 0;
    std::size_t attempted_bytes = 0;
    long long total_flop = 0;
    long long c_nnz = 0;  // -1 if not reached
    std::string error_msg;

    void reset();
    void snapshot_free(std::size_t &out_free) const;
};

void query_cuda_memory(std::size_t &free_bytes, std::size_t &total_bytes);

}  // namespace opsparse

#endif  // OPSPARSE_PROFILE_PERF_HPP_
