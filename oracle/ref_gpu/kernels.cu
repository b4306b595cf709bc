// kernels.cu — OpSparse's own SpGEMM kernels, compiled unchanged from its source tree into
// a cubin for sm_103a, so that the reference can be timed and checked on the GPU.
// TEST AND BENCHMARK INFRASTRUCTURE ONLY (oracle/ref_gpu/Makefile builds it into
// oracle/_ref/, which is not part of the library).  The kernels come from:
//   include/opsparse/core_algo/spgemm/kernels/binning.cuh, symbolic.cuh, numeric.cuh
//   src/opsparse/numeric/compute_flop.cu (k_compute_flop)
// The template instances below are the ones OpSparse's host drivers launch
// (src/opsparse/core_algo/spgemm/spgemm_phases.cu:55-199).
#include "opsparse/core_algo/spgemm/kernels/binning.cuh"
#include "opsparse/core_algo/spgemm/kernels/numeric.cuh"
#include "opsparse/core_algo/spgemm/kernels/symbolic.cuh"
#include "opsparse/numeric/compute_flop.cu"

namespace opsparse {
// Taking the addresses makes the compiler emit these instances.
void *const kRefGpuInstances[] = {
    (void *)k_symbolic_shared_hash_tb<8192>,
    (void *)k_symbolic_shared_hash_tb<4096>,
    (void *)k_symbolic_shared_hash_tb<2048>,
    (void *)k_symbolic_shared_hash_tb<1024>,
    (void *)k_symbolic_shared_hash_tb<512>,
    (void *)k_numeric_shared_hash_tb_full_occu<4096, 1024>,
    (void *)k_numeric_shared_hash_tb_full_occu<2048, 512>,
    (void *)k_numeric_shared_hash_tb_full_occu<1024, 256>,
    (void *)k_numeric_shared_hash_tb_full_occu<512, 128>,
    (void *)k_numeric_shared_hash_tb_full_occu<256, 64>,
    (void *)k_symbolic_binning,
    (void *)k_symbolic_binning2,
    (void *)k_binning_small,
    (void *)k_numeric_binning,
    (void *)k_numeric_binning2,
};
}  // namespace opsparse
