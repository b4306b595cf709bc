// cuda_emul.hpp — a minimal CPU execution model for CUDA kernel source, used only to run
// OpSparse's own SpGEMM kernels (include/opsparse/core_algo/spgemm/kernels/*.cuh and
// src/opsparse/numeric/compute_flop.cu) on the host so that their outputs can pin the
// oracle.  TEST INFRASTRUCTURE ONLY.
//
// Model: a launch runs its blocks one after another.  Each CUDA thread of a block is a
// ucontext fiber with its own stack; __syncthreads() suspends the fiber until every
// live fiber of the block has reached a barrier (fibers that returned count as
// arrived).  __shared__ variables become thread_local: all fibers run on the one OS
// thread, so they share them exactly like a CUDA block shares shared memory.  Fibers
// never preempt each other, so the atomics below are plain read-modify-writes.
// Supports 1-D grids and blocks, which is all OpSparse uses.
#pragma once

#include <cuda_runtime.h>
#include <cusparse.h>
#include <ucontext.h>

#include <functional>
#include <vector>

#undef __global__
#undef __device__
#undef __host__
#undef __shared__
#undef __forceinline__
#undef __launch_bounds__
#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __shared__ thread_local
#define __launch_bounds__(...)

namespace emu {

struct Fiber {
    ucontext_t ctx;
    std::vector<char> stack;
    uint3 tid;
    bool done = false;
    bool at_barrier = false;
};

extern Fiber *g_cur;
extern uint3 g_block_idx, g_block_dim, g_grid_dim;

void syncthreads();
// Runs body() once per thread of a grid x block launch.
void launch(unsigned grid, unsigned block, const std::function<void()> &body);

}  // namespace emu

#undef threadIdx
#undef blockIdx
#undef blockDim
#undef gridDim
#define threadIdx (::emu::g_cur->tid)
#define blockIdx (::emu::g_block_idx)
#define blockDim (::emu::g_block_dim)
#define gridDim (::emu::g_grid_dim)

inline void __syncthreads() { emu::syncthreads(); }

inline int atomicCAS(int *p, int cmp, int val)
{
    const int old = *p;
    if (old == cmp) *p = val;
    return old;
}

inline int atomicAdd(int *p, int v)
{
    const int old = *p;
    *p = old + v;
    return old;
}

inline double atomicAdd(double *p, double v)
{
    const double old = *p;
    *p = old + v;
    return old;
}

inline int atomicMax(int *p, int v)
{
    const int old = *p;
    if (v > old) *p = v;
    return old;
}
