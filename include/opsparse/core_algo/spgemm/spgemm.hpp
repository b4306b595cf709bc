// spgemm.hpp — drop-in SpGEMM entry points, same signatures as OpSparse's
// include/opsparse/core_algo/spgemm/spgemm.hpp:12-21.
//
// A and B must be device-resident (d_rpt/d_col/d_val, e.g. after H2D()), columns sorted
// and unique within each row.  On return C.M, C.N, C.nnz are set and C.d_rpt/d_col/d_val
// hold cudaMalloc'ed arrays (release with C.release()/drelease()).  Synchronous.
#ifndef OPSPARSE_CORE_ALGO_SPGEMM_SPGEMM_HPP_
#define OPSPARSE_CORE_ALGO_SPGEMM_SPGEMM_HPP_

#include "opsparse/core_algo/spgemm/meta.hpp"
#include "opsparse/core_ds/csr.hpp"
#include "opsparse/profile/perf.hpp"
#include "opsparse/profile/spgemm_timings.hpp"

namespace opsparse {

// Full pipeline with every SpgemmTimings phase filled (CUDA-event times).
void opsparse_spgemm(const CSR &A, const CSR &B, CSR &C, SpgemmMeta &meta, SpgemmTimings &timing);

// Same result without per-phase timing (only total/numeric are filled).
void opsparse_spgemm_reg(const CSR &A, const CSR &B, CSR &C, SpgemmMeta &meta, SpgemmTimings &timing);

// Never throws: classifies failures into SpgemmStatus and records memory use in perf.
// Totals of intermediate products are 64-bit; only nnz(C) > INT32_MAX (C's int32 row
// pointers) or a single row with more than INT32_MAX products report int32_overflow.
SpgemmStatus opsparse_spgemm_safe(const CSR &A, const CSR &B, CSR &C, SpgemmMeta &meta, SpgemmTimings &timing,
                                  SpgemmPerf &perf);

// Gradients through C = A*B with A's, B's and C's sparsity patterns fixed (no counterpart
// in OpSparse, which has no backward).  C is the product opsparse_spgemm returned for these
// A and B (device arrays); d_dC holds dLoss/dC on C's pattern (C.nnz device values).  Fills
// d_dA (A.nnz device values, on A's pattern) and d_dB (B.nnz device values, on B's
// pattern); either may be null:
//     dA_ij = sum_k B_jk dC_ik  over k in B(j,:),    dB_jk = sum_i A_ij dC_ik  over i with A_ij != 0,
// each folded in a fixed order (ascending k, ascending i), so results are reproducible bit
// for bit.  The first call for a pattern builds a plan on meta's library handle (A's
// transpose order, each product's position in C); later calls on the same device arrays
// reuse it.  Synchronous; throws std::runtime_error on failure (C.nnz != the product's
// pattern, a product missing from C's pattern, CUDA errors).
void opsparse_spgemm_backward(const CSR &A, const CSR &B, const CSR &C, const mdouble *d_dC, mdouble *d_dA,
                              mdouble *d_dB, SpgemmMeta &meta);

}  // namespace opsparse

#endif  // OPSPARSE_CORE_ALGO_SPGEMM_SPGEMM_HPP_
