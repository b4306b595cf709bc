// meta.hpp — per-caller SpGEMM workspace of the drop-in API (compare OpSparse's
// include/opsparse/core_algo/spgemm/meta.hpp:15-60).  Here it owns one persistent
// library handle (streams, stream-ordered memory pool, workspace) that is reused by every
// call made with it; release() keeps the handle, the destructor frees it.  The bin
// bookkeeping members of the original are kept for source compatibility and mirror the
// row-class sizes of the last call.
#ifndef OPSPARSE_CORE_ALGO_SPGEMM_META_HPP_
#define OPSPARSE_CORE_ALGO_SPGEMM_META_HPP_

#include <cstddef>

#include "opsparse/system/cuda_common.hpp"
#include "opsparse/utils/config.hpp"

struct ops_handle_s;

namespace opsparse {

class CSR;

class SpgemmMeta {
   public:
    mint M = 0;
    mint N = 0;

    // row-class sizes and offsets of the last call (host), as OpSparse's bin_size/bin_offset
    mint bin_size[kNumBin] = {};
    mint bin_offset[kNumBin] = {};
    mint max_row_nnz = 0;   // largest per-row product count of the last call (clamped)
    long long total_nnz = 0;

    cudaStream_t stream = nullptr;  // stream the calls run on (default: legacy stream)

    SpgemmMeta() = default;
    SpgemmMeta(const SpgemmMeta &) = delete;
    SpgemmMeta &operator=(const SpgemmMeta &) = delete;
    explicit SpgemmMeta(CSR &C);

    void allocate_rpt(CSR &C);
    void allocate(CSR &C);
    void release();

    // The library handle, created on first use.
    ops_handle_s *handle();

    ~SpgemmMeta();

   private:
    ops_handle_s *handle_ = nullptr;
};

}  // namespace opsparse

#endif  // OPSPARSE_CORE_ALGO_SPGEMM_META_HPP_
