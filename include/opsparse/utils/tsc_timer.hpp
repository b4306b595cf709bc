// tsc_timer.hpp — monotonic wall clock in seconds (name kept from OpSparse
// include/opsparse/utils/tsc_timer.hpp:10-19).
#ifndef OPSPARSE_UTILS_TSC_TIMER_HPP_
#define OPSPARSE_UTILS_TSC_TIMER_HPP_

#include <chrono>

namespace opsparse {

inline double fast_clock_time()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace opsparse

#endif  // OPSPARSE_UTILS_TSC_TIMER_HPP_
