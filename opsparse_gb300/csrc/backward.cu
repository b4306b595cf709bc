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

// The position in C of product (row i, B entry q) of A entry p: from the map, or by a
// binary search of C's row i.
template <bool kMap>
__device__ __forceinline__ int prod_pos(const int *__restrict__ pmap, long long base, int t,
                                        const int *__restrict__ c_rpt, const int *__restrict__ c_col, int i, int key,
                                        int *flags)
{
    if constexpr (kMap) return __ldg(pmap + base + t);
    return c_position(c_rpt, c_col, i, key, flags);
}

constexpr int kGradBatch = 8;      // chain steps whose operands are loaded together
constexpr int kGradShortMax = 64;  // dA chains longer than this are folded by a warp

// dA, chains of at most kGradShortMax terms: one thread per A entry p = (i, j), folding
// B row j in order, kGradBatch terms' operands loaded ahead of their FMAs.  Longer chains
// are listed for k_grad_a_long.
template <typename T, bool kMap>
__global__ void __launch_bounds__(256) k_grad_a_short(const int *__restrict__ acol, long long nnz_a,
                                                       const int *__restrict__ arow, const int *__restrict__ brpt,
                                                       const int *__restrict__ bcol, const T *__restrict__ bval,
                                                       const int *__restrict__ c_rpt, const int *__restrict__ c_col,
                                                       const T *__restrict__ dc, const long long *__restrict__ pos_base,
                                                       const int *__restrict__ pmap, T *__restrict__ da,
                                                       int *__restrict__ long_list, int *long_count, int *flags)
{
    using AccT = Acc<T>;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < nnz_a;
         p += (long long)gridDim.x * blockDim.x) {
        const int j = __ldg(acol + p);
        const int b0 = __ldg(brpt + j), b1 = __ldg(brpt + j + 1);
        if (b1 - b0 > kGradShortMax) {
            long_list[atomicAdd(long_count, 1)] = (int)p;
            continue;
        }
        const long long base = kMap ? __ldg(pos_base + p) : 0;
        const int i = kMap ? 0 : __ldg(arow + p);
        typename AccT::S s = AccT::zero();
        for (int q0 = b0; q0 < b1; q0 += kGradBatch) {
            int pos[kGradBatch];
            T bv[kGradBatch], d[kGradBatch];
#pragma unroll
            for (int u = 0; u < kGradBatch; ++u)
                pos[u] = q0 + u < b1 ? prod_pos<kMap>(pmap, base, q0 + u - b0, c_rpt, c_col, i,
                                                      kMap ? 0 : __ldg(bcol + q0 + u), flags)
                                     : -1;
#pragma unroll
            for (int u = 0; u < kGradBatch; ++u) {
                bv[u] = q0 + u < b1 ? __ldg(bval + q0 + u) : T(0);
                d[u] = pos[u] >= 0 ? __ldg(dc + pos[u]) : T(0);
            }
#pragma unroll
            for (int u = 0; u < kGradBatch; ++u)
                if (q0 + u < b1) s = AccT::step(s, bv[u], d[u]);
        }
        da[p] = AccT::fin(s);
    }
}

// dA, long chains: one warp per listed A entry.  The lanes load the operands of the next
// two batches of 32 terms (positions and B values coalesced, dC gathered in parallel)
// while lane 0 folds the current 32 from shared memory, in order.
template <typename T, bool kMap>
__global__ void __launch_bounds__(256) k_grad_a_long(const int *__restrict__ acol, const int *__restrict__ arow,
                                                      const int *__restrict__ brpt, const int *__restrict__ bcol,
                                                      const T *__restrict__ bval, const int *__restrict__ c_rpt,
                                                      const int *__restrict__ c_col, const T *__restrict__ dc,
                                                      const long long *__restrict__ pos_base,
                                                      const int *__restrict__ pmap, T *__restrict__ da,
                                                      const int *__restrict__ long_list, const int *long_count,
                                                      int *flags)
{
    using AccT = Acc<T>;
    __shared__ T s_b[256 / 32][2][32];
    __shared__ T s_d[256 / 32][2][32];
    const int lane = lane_id();
    const int warp = threadIdx.x >> 5;
    const int count = *long_count;
    const long long w0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long it = w0; it < count; it += nw) {
        const int p = __ldg(long_list + it);
        const int j = __ldg(acol + p);
        const int b0 = __ldg(brpt + j), b1 = __ldg(brpt + j + 1);
        const long long base = kMap ? __ldg(pos_base + p) : 0;
        const int i = kMap ? 0 : __ldg(arow + p);
        auto gather = [&](int q, T &bv, T &d) {
            bv = T(0);
            d = T(0);
            if (q < b1) {
                const int pos = prod_pos<kMap>(pmap, base, q - b0, c_rpt, c_col, i, kMap ? 0 : __ldg(bcol + q), flags);
                bv = __ldg(bval + q);
                d = pos >= 0 ? __ldg(dc + pos) : T(0);
            }
        };
        T nb, nd, nb2, nd2;
        gather(b0 + lane, nb, nd);
        gather(b0 + 32 + lane, nb2, nd2);
        typename AccT::S s = AccT::zero();
        int buf = 0;
        for (int q = b0; q < b1; q += 32) {
            s_b[warp][buf][lane] = nb;
            s_d[warp][buf][lane] = nd;
            __syncwarp();
            nb = nb2;
            nd = nd2;
            gather(q + 64 + lane, nb2, nd2);
            if (lane == 0) {
                const int m = min(32, b1 - q);
                for (int u = 0; u < m; ++u) s = AccT::step(s, s_b[warp][buf][u], s_d[warp][buf][u]);
            }
            buf ^= 1;
        }
        if (lane == 0) da[p] = AccT::fin(s);
        __syncwarp();
    }
}

// dB: one warp per row j of B, lanes over the row's entries q, each folding the A entries
// of column j in ascending row order.  All lanes walk the same column entries, so the
// warp loads 32 of them at once (one per lane) and shares them by shuffle; each lane then
// loads kGradBatch terms' positions and dC values ahead of its FMAs.
template <typename T, bool kMap>
__global__ void __launch_bounds__(256) k_grad_b(int K, const int *__restrict__ brpt, const int *__restrict__ bcol,
                                                 const T *__restrict__ aval, const int *__restrict__ at_ptr,
                                                 const int *__restrict__ at_ent, const int *__restrict__ arow,
                                                 const int *__restrict__ c_rpt, const int *__restrict__ c_col,
                                                 const T *__restrict__ dc, const long long *__restrict__ pos_base,
                                                 const int *__restrict__ pmap, T *__restrict__ db, int *flags)
{
    using AccT = Acc<T>;
    const int lane = lane_id();
    const long long w0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long j = w0; j < K; j += nw) {
        const int b0 = __ldg(brpt + j), b1 = __ldg(brpt + j + 1);
        const int e0 = __ldg(at_ptr + j), e1 = __ldg(at_ptr + j + 1);
        for (int qb = b0; qb < b1; qb += 32) {
            const int q = qb + lane;
            const bool qv = q < b1;
            const int key = (!kMap && qv) ? __ldg(bcol + q) : 0;
            typename AccT::S s = AccT::zero();
            for (int eb = e0; eb < e1; eb += 32) {
                // one column entry per lane: its A entry, row, value and product base
                int pe = 0, re = 0;
                long long be = 0;
                T ae = T(0);
                if (eb + lane < e1) {
                    pe = __ldg(at_ent + eb + lane);
                    ae = __ldg(aval + pe);
                    if (kMap) be = __ldg(pos_base + pe);
                    else re = __ldg(arow + pe);
                }
                const int m = min(32, e1 - eb);
                for (int t0 = 0; t0 < m; t0 += kGradBatch) {
                    int pos[kGradBatch];
                    T a[kGradBatch], d[kGradBatch];
#pragma unroll
                    for (int u = 0; u < kGradBatch; ++u) {
                        const int src = min(t0 + u, 31);
                        const long long bu = kMap ? __shfl_sync(kFull, be, src) : 0;
                        const int ru = kMap ? 0 : __shfl_sync(kFull, re, src);
                        a[u] = shfl(ae, src);
                        pos[u] = (qv && t0 + u < m) ? prod_pos<kMap>(pmap, bu, q - b0, c_rpt, c_col, ru, key, flags)
                                                    : -1;
                    }
#pragma unroll
                    for (int u = 0; u < kGradBatch; ++u) d[u] = pos[u] >= 0 ? __ldg(dc + pos[u]) : T(0);
#pragma unroll
                    for (int u = 0; u < kGradBatch; ++u)
                        if (t0 + u < m) s = AccT::step(s, a[u], d[u]);
                }
            }
            if (qv) db[q] = AccT::fin(s);
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
    if (da && pl.nnz_a > 0) {
        // thread per A entry for short chains; the long ones are listed and get a warp each
        int *long_list = nullptr;
        OPS_CUDA(h, cudaMallocFromPoolAsync(reinterpret_cast<void **>(&long_list), sizeof(int) * pl.nnz_a, h->pool,
                                            st));
        OPS_CUDA(h, cudaMemsetAsync(&h->info->d_cursor, 0, sizeof(int), st));
        const int g1 = grid_of(pl.nnz_a, 256, sms * 16);
        if (pl.with_map) {
            k_grad_a_short<T, true><<<g1, 256, 0, st>>>(a_col, pl.nnz_a, pl.arow, b_rpt, b_col, b_val, c_rpt, c_col, dc,
                                                        pl.pos_base, pl.pmap, da, long_list, &h->info->d_cursor, flags);
            k_grad_a_long<T, true><<<sms * 8, 256, 0, st>>>(a_col, pl.arow, b_rpt, b_col, b_val, c_rpt, c_col, dc,
                                                            pl.pos_base, pl.pmap, da, long_list, &h->info->d_cursor,
                                                            flags);
        } else {
            k_grad_a_short<T, false><<<g1, 256, 0, st>>>(a_col, pl.nnz_a, pl.arow, b_rpt, b_col, b_val, c_rpt, c_col,
                                                         dc, pl.pos_base, pl.pmap, da, long_list, &h->info->d_cursor,
                                                         flags);
            k_grad_a_long<T, false><<<sms * 8, 256, 0, st>>>(a_col, pl.arow, b_rpt, b_col, b_val, c_rpt, c_col, dc,
                                                             pl.pos_base, pl.pmap, da, long_list, &h->info->d_cursor,
                                                             flags);
        }
        OPS_CUDA(h, cudaGetLastError());
        OPS_CUDA(h, cudaFreeAsync(long_list, st));
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
