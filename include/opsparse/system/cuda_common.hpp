// cuda_common.hpp — index/value types and CUDA error helpers of the drop-in C++ API.
// Same names as OpSparse's include/opsparse/system/cuda_common.hpp:13-65 (mint, mdouble,
// check_cuda, d2h/h2d/d2d, cuda_runtime_warmup, OPSPARSE_CHECK_CUDA); cuSPARSE is not used.
#ifndef OPSPARSE_SYSTEM_CUDA_COMMON_HPP_
#define OPSPARSE_SYSTEM_CUDA_COMMON_HPP_

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdio>
#include <stdexcept>
#include <string>

namespace opsparse {

using mint = int;
using mdouble = double;

inline bool expect_true(bool x) { return __builtin_expect(x, 1); }
inline bool expect_false(bool x) { return __builtin_expect(x, 0); }

// Prints the CUDA error and throws (a std::runtime_error carrying the same text).
inline void check_cuda(cudaError_t err, const char *file, int line)
{
    if (expect_false(err != cudaSuccess)) {
        std::printf("%s in %s at line %d\n", cudaGetErrorString(err), file, line);
        throw std::runtime_error(std::string(cudaGetErrorString(err)) + " at " + file + ":" + std::to_string(line));
    }
}

template <typename T>
inline void d2h(T *dst, const T *src, std::size_t bytes)
{
    check_cuda(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost), __FILE__, __LINE__);
}

template <typename T>
inline void h2d(T *dst, const T *src, std::size_t bytes)
{
    check_cuda(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice), __FILE__, __LINE__);
}

template <typename T>
inline void d2d(T *dst, const T *src, std::size_t bytes)
{
    check_cuda(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToDevice), __FILE__, __LINE__);
}

// Forces CUDA context creation before any timed work.
inline void cuda_runtime_warmup()
{
    void *d = nullptr;
    check_cuda(cudaMalloc(&d, 4), __FILE__, __LINE__);
    check_cuda(cudaFree(d), __FILE__, __LINE__);
    check_cuda(cudaDeviceSynchronize(), __FILE__, __LINE__);
}

}  // namespace opsparse

#define OPSPARSE_CHECK_CUDA(err) (::opsparse::check_cuda((err), __FILE__, __LINE__))

#endif  // OPSPARSE_SYSTEM_CUDA_COMMON_HPP_
