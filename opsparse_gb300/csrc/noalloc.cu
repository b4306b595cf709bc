// noalloc.cu — intermediate-product count that allocates no device memory.
//
// Some callers of this library cannot allocate device memory at the point where they count
// products: serving or real-time loops that forbid the CUDA allocator once they are running
// (cudaMalloc can synchronize the whole device, and cudaMallocAsync changes the state of a
// memory pool another component may own), and hosts that hand the library a fixed memory
// budget up front and account for every byte themselves.  ops_flop (spgemm.cu) takes a
// small device temporary from cudaMallocAsync on every call; ops_flop_noalloc below
// computes the same result with its scratch in a file-scope __device__ array instead, and
// calls no allocating function (no cudaMalloc, cudaFree or allocating library routine).
//
// The scratch holds one 64-bit partial sum per CTA of the flop kernel, the total, a
// completion ticket and an error flag: kNoAllocMaxBlocks partials cap the input at
// kNoAllocMaxRows = 8192 * 256 = 2,097,152 rows of A; larger inputs are refused with
// OPS_NOT_SUPPORTED.  Every GPU that loads the library keeps this 64 KiB array until the
// process exits.
//
// Set-up: the first call on each device looks up the array's device address with
// cudaGetSymbolAddress (with that device current) and keeps it for later calls; make that
// first call before any stream capture.  Like the library's handles, the kept address does
// not survive cudaDeviceReset: do not call the library across a device reset.  All calls
// share the one array and it keeps the previous call's contents, so each call clears the
// words that must start at zero; calls whose work overlaps on the GPU (two streams, or two
// host threads) race on it and must be serialized by the caller.  The call reads the total
// back to the host and synchronizes its stream before it returns.
#include <cstdint>

#include "common.cuh"
#include "opsparse_gb300.h"

namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocMaxBlocks = 8192;
constexpr long long kNoAllocMaxRows = (long long)kNoAllocMaxBlocks * kNoAllocThreads;

// Per-CTA partial sums, the total, the completion ticket and the error flag.
struct NoAllocScratch {
    unsigned long long partial[kNoAllocMaxBlocks];
    unsigned long long total;
    unsigned int ticket;      // must be 0 when a launch starts
    unsigned int bad_column;  // must be 0 when a launch starts
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Same per-row count as k_flop64, but each CTA writes its partial sum to the scratch and
// the last CTA to finish (completion ticket) adds the partials in CTA order, so the total
// needs no atomics on a shared word and no second launch.
__global__ void __launch_bounds__(kNoAllocThreads) k_flop64_noalloc(const int *__restrict__ arpt,
                                                                    const int *__restrict__ acol,
                                                                    const int *__restrict__ brpt, int M, int K,
                                                                    long long *row_flop, NoAllocScratch *scratch)
{
    __shared__ unsigned long long s_part[kNoAllocThreads / 32];
    __shared__ bool s_last;
    const int r = blockIdx.x * kNoAllocThreads + threadIdx.x;
    unsigned long long s = 0;
    if (r < M) {
        for (int p = arpt[r]; p < arpt[r + 1]; ++p) {
            const int j = acol[p];
            if ((unsigned)j < (unsigned)K) s += (unsigned long long)(brpt[j + 1] - brpt[j]);
            else atomicOr(&scratch->bad_column, 1u);
        }
        if (row_flop) row_flop[r] = (long long)s;
    }
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) s += __shfl_xor_sync(opsg::kFull, s, d);
    if (opsg::lane_id() == 0) s_part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < kNoAllocThreads / 32; ++w) t += s_part[w];
        scratch->partial[blockIdx.x] = t;
        __threadfence();
        s_last = atomicAdd(&scratch->ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
        __threadfence();
        unsigned long long t = 0;
        for (unsigned b = 0; b < gridDim.x; ++b) t += ((volatile unsigned long long *)scratch->partial)[b];
        scratch->total = t;
    }
}

// Device address of g_noalloc_scratch on the current device, looked up on every call: an
// address kept from an earlier call would be stale after a reset of the device's context.
cudaError_t noalloc_scratch(NoAllocScratch **out)
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    *out = static_cast<NoAllocScratch *>(p);
    return cudaSuccess;
}

}  // namespace

extern "C" int ops_flop_noalloc(int32_t rows_a, int32_t cols_a, const int32_t *a_rpt, const int32_t *a_col,
                                const int32_t *b_rpt, int64_t *row_flop, int64_t *total, void *stream)
{
    if (rows_a < 0 || !total || (rows_a > 0 && (!a_rpt || !b_rpt))) return OPS_INVALID_ARGUMENT;
    if ((long long)rows_a > kNoAllocMaxRows) return OPS_NOT_SUPPORTED;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    NoAllocScratch *scratch = nullptr;
    cudaError_t e = noalloc_scratch(&scratch);
    // the total, the ticket and the error flag must start at zero (the partials are
    // overwritten by every launch); the array keeps the previous call's contents
    if (e == cudaSuccess)
        e = cudaMemsetAsync(&scratch->total, 0, sizeof(unsigned long long) + 2 * sizeof(unsigned int), st);
    if (e == cudaSuccess && rows_a > 0) {
        const int blocks = (rows_a + kNoAllocThreads - 1) / kNoAllocThreads;
        k_flop64_noalloc<<<blocks, kNoAllocThreads, 0, st>>>(a_rpt, a_col, b_rpt, rows_a, cols_a,
                                                            reinterpret_cast<long long *>(row_flop), scratch);
        e = cudaGetLastError();
    }
    unsigned long long h_total = 0;
    unsigned int h_bad = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_total, &scratch->total, sizeof(h_total), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_bad, &scratch->bad_column, sizeof(h_bad), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? OPS_OOM : OPS_CUDA_ERROR;
    }
    if (h_bad) return OPS_INVALID_CSR;
    *total = (int64_t)h_total;
    return OPS_OK;
}
