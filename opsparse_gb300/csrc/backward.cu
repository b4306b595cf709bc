// backward.cu — gradients of loss = sum(dC .* C) for C = A*B on fixed sparsity patterns.
// OpSparse has no backward pass; this is new.
//
//   dA_ij = sum_{k in B(j,:)} B_jk * dC_ik      (one value per entry of A)
//   dB_jk = sum_{i : j in A(i,:)} A_ij * dC_ik   (one value per entry of B)
//
// Both re-walk the forward's product enumeration (i, j in A(i,:), k in B(j,:)); every
// product needs the position of (i, k) in C's row i.  Each value is folded in a fixed
// order with the same accumulation policy as the forward (FP64: one FMA per term; FP32:
// Dot2): dA over k in B's row order, dB over i ascending.  dB is computed per entry of B
// over the A entries of column j (a stable transpose of A), so no atomics are needed and
// results are deterministic.
//
// Plan (built once per pattern, kept on the handle):
//   arow[p]     row of A entry p;
//   pos_base[p] index of A entry p's first product in the global (row, A entry, B entry)
//               enumeration = exclusive scan of the B-row lengths over A's entries;
//   at_ptr/at_ent  A's entries ordered by (column, row): CUB radix sort by column, which
//               is stable, over entries in row-major order;
//   pmap[q]     position in C of product q, found once by binary search in C's sorted
//               row — only when products * 4 bytes fits the handle's map budget.  Without
//               it every product's position is searched again on each call.
#include <cub/cub.cuh>

#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "internal.hpp"

using namespace opsg;
using namespace opsg_internal;

namespace {

// First index in a[0, n) with a[idx] >= key.
__device__ __forceinline__ int lower_bound_i32(const int *__restrict__ a, int n, int key)
{
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(a + mid) < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Position of (i, key) in C, or -1 (and an error flag) if C's row i lacks the key.
__device__ __forceinline__ int c_position(const int *__restrict__ c_rpt, const int *__restrict__ c_col, int i,
                                          int key, int *flags)
{
    const int c0 = __ldg(c_rpt + i);
    const int n = __ldg(c_rpt + i + 1) - c0;
    const int t = lower_bound_i32(c_col + c0, n, key);
    if (t >= n || __ldg(c_col + c0 + t) != key) {
        atomicOr(flags, kErrCountMismatch);
        return -1;
    }
    return c0 + t;
}

__global__ void k_blen_of_a(const int *__restrict__ acol, const int *__restrict__ brpt, long long nnz,
                            long long *__restrict__ out)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < nnz; p += (long long)gridDim.x * blockDim.x) {
        const int j = __ldg(acol + p);
        out[p] = __ldg(brpt + j + 1) - __ldg(brpt + j);
    }
}

__global__ void k_iota(int *out, long long n)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x)
        out[p] = (int)p;
}

// arow[p] = row of A entry p; one warp per row.
__global__ void k_expand_rows(const int *__restrict__ arpt, int M, int *__restrict__ arow)
{
    const long long w0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long i = w0; i < M; i += nw) {
        const int a0 = __ldg(arpt + i), a1 = __ldg(arpt + i + 1);
        for (int p = a0 + lane_id(); p < a1; p += 32) arow[p] = (int)i;
    }
}

// at_ptr[j] = first position of column j in the column-sorted key array.
__global__ void k_col_starts(const int *__restrict__ sorted_cols, long long nnz, int K, int *__restrict__ at_ptr)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p <= nnz; p += (long long)gridDim.x * blockDim.x) {
        const int cur = p < nnz ? __ldg(sorted_cols + p) : K;
        const int prev = p > 0 ? __ldg(sorted_cols + p - 1) : -1;
        for (int j = prev + 1; j <= cur; ++j) at_ptr[j] = (int)p;
    }
}

// pmap[pos_base[p] + t] = position in C of product (row(p), B entry brpt[j]+t); one warp
// per row of A, products walked in chunks of 32.
__global__ void __launch_bounds__(256) k_build_pmap(const int *__restrict__ arpt, const int *__restrict__ acol,
                                                     const int *__restrict__ brpt, const int *__restrict__ bcol, int M,
                                                     const int *__restrict__ c_rpt, const int *__restrict__ c_col,
                                                     const long long *__restrict__ pos_base, int *__restrict__ pmap,
                                                     int *flags)
{
    const long long w0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long i = w0; i < M; i += nw) {
        const int a0 = __ldg(arpt + i), a1 = __ldg(arpt + i + 1);
        warp_products<false, double>(a0, a1, 32, acol, nullptr, brpt, [&](bool valid, int k, double, int p) {
            if (valid) {
                const int j = __ldg(acol + p);
                const int pos = c_position(c_rpt, c_col, (int)i, __ldg(bcol + k), flags);
                pmap[__ldg(pos_base + p) + (k - __ldg(brpt + j))] = pos;
            }
        });
    }
}

// dA: one warp per row of A, lanes over the row's entries, each folding its B row in order.
template <typename T, bool kMap>
__global__ void __launch_bounds__(256) k_grad_a(const int *__restrict__ arpt, const int *__restrict__ acol, int M,
                                                 const int *__restrict__ brpt, const int *__restrict__ bcol,
                                                 const T *__restrict__ bval, const int *__restrict__ c_rpt,
                                                 const int *__restrict__ c_col, const T *__restrict__ dc,
                                                 const long long *__restrict__ pos_base, const int *__restrict__ pmap,
                                                 T *__restrict__ da, int *flags)
{
    using AccT = Acc<T>;
    const long long w0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long i = w0; i < M; i += nw) {
        const int a0 = __ldg(arpt + i), a1 = __ldg(arpt + i + 1);
        for (int p = a0 + lane_id(); p < a1; p += 32) {
            const int j = __ldg(acol + p);
            const int b0 = __ldg(brpt + j), b1 = __ldg(brpt + j + 1);
            typename AccT::S s = AccT::zero();
            const long long base = kMap ? __ldg(pos_base + p) : 0;
            for (int q = b0; q < b1; ++q) {
                int pos;
                if (kMap) pos = __ldg(pmap + base + (q - b0));
                else pos = c_position(c_rpt, c_col, (int)i, __ldg(bcol + q), flags);
                const T d = pos >= 0 ? __ldg(dc + pos) : T(0);
                s = AccT::step(s, __ldg(bval + q), d);
            }
            da[p] = AccT::fin(s);
        }
    }
}

// dB: one warp per row j of B, lanes over the row's entries, each folding the A entries
// of column j in ascending row order.
template <typename T, bool kMap>
__global__ void __launch_bounds__(256) k_grad_b(int K, const int *__restrict__ brpt, const int *__restrict__ bcol,
                                                 const T *__restrict__ aval, const int *__restrict__ at_ptr,
                                                 const int *__restrict__ at_ent, const int *__restrict__ arow,
                                                 const int *__restrict__ c_rpt, const int *__restrict__ c_col,
                                                 const T *__restrict__ dc, const long long *__restrict__ pos_base,
                                                 const int *__restrict__ pmap, T *__restrict__ db, int *flags)
{
    using AccT = Acc<T>;
    const long long w0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long j = w0; j < K; j += nw) {
        const int b0 = __ldg(brpt + j), b1 = __ldg(brpt + j + 1);
        const int e0 = __ldg(at_ptr + j), e1 = __ldg(at_ptr + j + 1);
        for (int q = b0 + lane_id(); q < b1; q += 32) {
            const int key = kMap ? 0 : __ldg(bcol + q);
            typename AccT::S s = AccT::zero();
            for (int e = e0; e < e1; ++e) {
                const int p = __ldg(at_ent + e);
                int pos;
                if (kMap) pos = __ldg(pmap + __ldg(pos_base + p) + (q - b0));
                else pos = c_position(c_rpt, c_col, __ldg(arow + p), key, flags);
                const T d = pos >= 0 ? __ldg(dc + pos) : T(0);
                s = AccT::step(s, __ldg(aval + p), d);
            }
            db[q] = AccT::fin(s);
        }
    }
}

int grid_of(long long work, int per_block, int cap)
{
    const long long b = (work + per_block - 1) / per_block;
    return (int)std::max<long long>(1, std::min<long long>(b, cap));
}

// Builds (or reuses) the plan for this pattern.
int build_plan(ops_handle_s *h, int M, int K, int N, const int *a_rpt, const int *a_col, long long nnz_a,
               const int *b_rpt, const int *b_col, long long nnz_b, const int *c_rpt, const int *c_col,
               cudaStream_t st)
{
    BackwardPlan &pl = h->bwd;
    if (pl.valid && pl.M == M && pl.K == K && pl.N == N && pl.nnz_a == nnz_a && pl.nnz_b == nnz_b &&
        pl.a_rpt == a_rpt && pl.a_col == a_col && pl.b_rpt == b_rpt && pl.b_col == b_col && pl.c_rpt == c_rpt &&
        pl.c_col == c_col)
        return OPS_OK;
    if (pl.mem) {
        OPS_CUDA(h, cudaFreeAsync(pl.mem, st));
        pl.mem = nullptr;
    }
    pl.valid = false;
    const int sms = h->num_sms;
    const size_t na = (size_t)std::max<long long>(nnz_a, 1);
    // temporaries: B-row length per A entry (int64), sort keys/values, CUB scratch
    size_t sort_tmp = 0, scan_tmp = 0;
    OPS_CUDA(h, cub::DeviceRadixSort::SortPairs(nullptr, sort_tmp, (int *)nullptr, (int *)nullptr, (int *)nullptr,
                                                (int *)nullptr, (int)na, 0, std::max(1, ceil_log2(std::max(K, 2))),
                                                st));
    OPS_CUDA(h, cub::DeviceScan::ExclusiveSum(nullptr, scan_tmp, (long long *)nullptr, (long long *)nullptr,
                                              (int)na + 1, st));
    const size_t tmp_bytes = align_up(8 * (na + 1), 256) + align_up(4 * na, 256) * 2 + align_up(sort_tmp, 256) +
                             align_up(scan_tmp, 256);
    void *tp = nullptr;
    OPS_CUDA(h, cudaMallocFromPoolAsync(&tp, tmp_bytes, h->pool, st));
    unsigned char *t = static_cast<unsigned char *>(tp);
    long long *blen = reinterpret_cast<long long *>(t);
    t += align_up(8 * (na + 1), 256);
    int *sorted_cols = reinterpret_cast<int *>(t);
    t += align_up(4 * na, 256);
    int *iota = reinterpret_cast<int *>(t);
    t += align_up(4 * na, 256);
    void *sort_scratch = t;
    t += align_up(sort_tmp, 256);
    void *scan_scratch = t;

    // persistent plan arrays (map added below once the product count is known)
    const size_t base_bytes = align_up(8 * (na + 1), 256) + align_up(4 * ((size_t)K + 1), 256) +
                              align_up(4 * na, 256) * 2;
    void *pp = nullptr;
    OPS_CUDA(h, cudaMallocFromPoolAsync(&pp, base_bytes, h->pool, st));
    unsigned char *m = static_cast<unsigned char *>(pp);
    pl.mem = m;
    pl.bytes = base_bytes;
    pl.pos_base = reinterpret_cast<long long *>(m);
    m += align_up(8 * (na + 1), 256);
    pl.at_ptr = reinterpret_cast<int *>(m);
    m += align_up(4 * ((size_t)K + 1), 256);
    pl.at_ent = reinterpret_cast<int *>(m);
    m += align_up(4 * na, 256);
    pl.arow = reinterpret_cast<int *>(m);

    OPS_CUDA(h, cudaMemsetAsync(blen + na, 0, sizeof(long long), st));
    if (nnz_a > 0) {
        k_blen_of_a<<<grid_of(nnz_a, 256, sms * 16), 256, 0, st>>>(a_col, b_rpt, nnz_a, blen);
        k_iota<<<grid_of(nnz_a, 256, sms * 16), 256, 0, st>>>(iota, nnz_a);
        OPS_CUDA(h, cudaGetLastError());
    }
    OPS_CUDA(h, cub::DeviceScan::ExclusiveSum(scan_scratch, scan_tmp, blen, pl.pos_base, (int)na + 1, st));
    if (M > 0) {
        k_expand_rows<<<grid_of(M, 8, sms * 8), 256, 0, st>>>(a_rpt, M, pl.arow);
        OPS_CUDA(h, cudaGetLastError());
    }
    if (nnz_a > 0)
        OPS_CUDA(h, cub::DeviceRadixSort::SortPairs(sort_scratch, sort_tmp, a_col, sorted_cols, iota, pl.at_ent,
                                                    (int)nnz_a, 0, std::max(1, ceil_log2(std::max(K, 2))), st));
    k_col_starts<<<grid_of(nnz_a + 1, 256, sms * 16), 256, 0, st>>>(sorted_cols, nnz_a, K, pl.at_ptr);
    OPS_CUDA(h, cudaGetLastError());
    long long products = 0;
    OPS_CUDA(h, cudaMemcpyAsync(&products, pl.pos_base + na - (nnz_a > 0 ? 0 : 1), sizeof(long long),
                                cudaMemcpyDeviceToHost, st));
    OPS_CUDA(h, cudaStreamSynchronize(st));
    if (nnz_a == 0) products = 0;
    pl.products = products;
    pl.with_map = products > 0 && products <= INT_MAX && (size_t)products * 4 <= h->map_budget;
    pl.pmap = nullptr;
    if (pl.with_map) {
        void *mp = nullptr;
        cudaError_t e = cudaMallocFromPoolAsync(&mp, (size_t)products * 4, h->pool, st);
        if (e == cudaSuccess) {
            pl.pmap = static_cast<int *>(mp);
            OPS_CUDA(h, cudaMemsetAsync(&h->info->flags, 0, sizeof(int), st));
            k_build_pmap<<<grid_of(M, 8, sms * 8), 256, 0, st>>>(a_rpt, a_col, b_rpt, b_col, M, c_rpt, c_col,
                                                                 pl.pos_base, pl.pmap, &h->info->flags);
            OPS_CUDA(h, cudaGetLastError());
        } else {
            (void)cudaGetLastError();
            pl.with_map = false;  // no room: search positions on every call instead
        }
    }
    OPS_CUDA(h, cudaFreeAsync(tp, st));
    pl.M = M;
    pl.K = K;
    pl.N = N;
    pl.nnz_a = nnz_a;
    pl.nnz_b = nnz_b;
    pl.a_rpt = a_rpt;
    pl.a_col = a_col;
    pl.b_rpt = b_rpt;
    pl.b_col = b_col;
    pl.c_rpt = c_rpt;
    pl.c_col = c_col;
    pl.valid = true;
    return OPS_OK;
}

template <typename T>
int run_backward(ops_handle_s *h, int M, int K, const int *a_rpt, const int *a_col, const T *a_val,
                 const int *b_rpt, const int *b_col, const T *b_val, const int *c_rpt, const int *c_col, const T *dc,
                 T *da, T *db, cudaStream_t st)
{
    const BackwardPlan &pl = h->bwd;
    const int sms = h->num_sms;
    int *flags = &h->info->flags;
    if (da && M > 0) {
        if (pl.with_map)
            k_grad_a<T, true><<<grid_of(M, 8, sms * 8), 256, 0, st>>>(a_rpt, a_col, M, b_rpt, b_col, b_val, c_rpt, c_col,
                                                                      dc, pl.pos_base, pl.pmap, da, flags);
        else
            k_grad_a<T, false><<<grid_of(M, 8, sms * 8), 256, 0, st>>>(a_rpt, a_col, M, b_rpt, b_col, b_val, c_rpt,
                                                                       c_col, dc, pl.pos_base, pl.pmap, da, flags);
        OPS_CUDA(h, cudaGetLastError());
    }
    if (db && K > 0) {
        if (pl.with_map)
            k_grad_b<T, true><<<grid_of(K, 8, sms * 8), 256, 0, st>>>(K, b_rpt, b_col, a_val, pl.at_ptr, pl.at_ent,
                                                                      pl.arow, c_rpt, c_col, dc, pl.pos_base, pl.pmap,
                                                                      db, flags);
        else
            k_grad_b<T, false><<<grid_of(K, 8, sms * 8), 256, 0, st>>>(K, b_rpt, b_col, a_val, pl.at_ptr, pl.at_ent,
                                                                       pl.arow, c_rpt, c_col, dc, pl.pos_base, pl.pmap,
                                                                       db, flags);
        OPS_CUDA(h, cudaGetLastError());
    }
    return OPS_OK;
}

}  // namespace

extern "C" int ops_spgemm_backward(ops_handle_t h, int dtype, int32_t rows_a, int32_t cols_a, int32_t cols_b,
                                   const int32_t *a_rpt, const int32_t *a_col, const void *a_val, int64_t a_nnz,
                                   const int32_t *b_rpt, const int32_t *b_col, const void *b_val, int64_t b_nnz,
                                   const int32_t *c_rpt, const int32_t *c_col, const void *dc_val, void *da_val,
                                   void *db_val, void *stream)
{
    if (!h) return OPS_INVALID_ARGUMENT;
    if (dtype != OPS_F64 && dtype != OPS_F32) return fail(h, OPS_INVALID_ARGUMENT, "unknown dtype");
    if (rows_a < 0 || cols_a < 0 || cols_b < 0 || a_nnz < 0 || b_nnz < 0 || a_nnz > INT_MAX || b_nnz > INT_MAX)
        return fail(h, OPS_INVALID_ARGUMENT, "bad matrix sizes");
    if ((rows_a > 0 && (!a_rpt || !c_rpt)) || (cols_a > 0 && !b_rpt) || (a_nnz > 0 && (!a_col || !a_val)) ||
        (b_nnz > 0 && (!b_col || !b_val)) || !dc_val)
        return fail(h, OPS_INVALID_ARGUMENT, "null input");
    try {
        h->last_error.clear();
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        if (!h->info) {  // the handle has not run a forward yet: create its workspace
            void *p = nullptr;
            OPS_CUDA(h, cudaMallocFromPoolAsync(&p, 256, h->pool, st));
            h->ws = static_cast<unsigned char *>(p);
            h->ws_M = 0;
            h->info = reinterpret_cast<DevInfo *>(h->ws);
        }
        OPS_CHECK(build_plan(h, rows_a, cols_a, cols_b, a_rpt, a_col, a_nnz, b_rpt, b_col, b_nnz, c_rpt, c_col, st));
        OPS_CUDA(h, cudaMemsetAsync(&h->info->flags, 0, sizeof(int), st));
        int s;
        if (dtype == OPS_F64)
            s = run_backward<double>(h, rows_a, cols_a, a_rpt, a_col, static_cast<const double *>(a_val), b_rpt, b_col,
                                     static_cast<const double *>(b_val), c_rpt, c_col,
                                     static_cast<const double *>(dc_val), static_cast<double *>(da_val),
                                     static_cast<double *>(db_val), st);
        else
            s = run_backward<float>(h, rows_a, cols_a, a_rpt, a_col, static_cast<const float *>(a_val), b_rpt, b_col,
                                    static_cast<const float *>(b_val), c_rpt, c_col, static_cast<const float *>(dc_val),
                                    static_cast<float *>(da_val), static_cast<float *>(db_val), st);
        return s;
    } catch (...) {
        return fail(h, OPS_EXCEPTION, "exception in ops_spgemm_backward");
    }
}

extern "C" int ops_handle_set_map_budget(ops_handle_t h, size_t bytes)
{
    if (!h) return OPS_INVALID_ARGUMENT;
    h->map_budget = bytes;
    h->bwd.valid = false;
    return OPS_OK;
}

extern "C" int ops_backward_plan_info(ops_handle_t h, int64_t *products, int *with_map)
{
    if (!h || !products || !with_map) return OPS_INVALID_ARGUMENT;
    *products = h->bwd.valid ? h->bwd.products : 0;
    *with_map = h->bwd.valid && h->bwd.with_map ? 1 : 0;
    return OPS_OK;
}
