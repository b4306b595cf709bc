// compute_flop.hpp — host intermediate-product counters (same signatures as the host
// functions of OpSparse's include/opsparse/numeric/compute_flop.hpp:11-18).  The device
// counter is ops_flop in opsparse_gb300.h.
#ifndef OPSPARSE_NUMERIC_COMPUTE_FLOP_HPP_
#define OPSPARSE_NUMERIC_COMPUTE_FLOP_HPP_

#include "opsparse/system/cuda_common.hpp"

namespace opsparse {

class CSR;

long compute_flop(const mint *row_ptr_a, const mint *col_idx_a, const mint *row_ptr_b, mint M, mint *row_flop_out);
long compute_flop(const CSR &A, const CSR &B, mint *row_flop);
long compute_flop(const CSR &A, const CSR &B);

}  // namespace opsparse

#endif  // OPSPARSE_NUMERIC_COMPUTE_FLOP_HPP_
