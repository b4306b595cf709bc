// gesc.cu — rows with more products than a CTA can sort in shared memory ("D" rows:
// more than 13,312), by expand / sort / compress over the whole GPU.  Replaces OpSparse's
// global-memory hash fallback for its heaviest rows (kernels/symbolic.cuh:263-325,
// kernels/numeric.cuh:304-393), and this library's CTA-per-row dense kernel.
//
//   1. The D rows' A entries are concatenated (scan of their lengths) and every entry's
//      products get consecutive positions (scan of its B row lengths), so the expansion
//      writes product t of the concatenation at position t: row-major, ascending j.
//   2. Key of a product: (D-row index << cb) | column — 32 bits when they fit.  Numeric
//      carries (A position, B position) as the value.
//   3. One stable radix sort (CUB DeviceRadixSort over exactly db + cb bits) makes the
//      products of each output entry adjacent, still in ascending j: the order the
//      oracle folds them in.
//   4. Symbolic: count the run heads of each row.  Numeric: number the heads (scan),
//      record where each run starts, and fold each run with one FMA per product — by
//      one thread for runs of at most 32 products, by a warp for longer runs (the lanes
//      gather the operands of the next two batches of 32 while lane 0 folds the current
//      32 from shared memory: a run is a chain of dependent FMAs, and a dependent FP64
//      FMA costs about 64 cycles on GB300).  Runs of more than kBlockFoldMin products
//      fold in kFoldBlocks blocks, lane b the b-th, merged in lane order by lane 0 — the
//      fixed blocked order the oracle uses for such entries — so the longest chain is
//      at most kBlockFoldMin FMAs.  C entry h of
//      D row d goes to row_ptr[row] + h - (heads of the earlier D rows).
#include <cub/cub.cuh>

#include <algorithm>

#include "internal.hpp"

namespace {

using namespace opsg;
using opsg_internal::align_up;
using opsg_internal::fail;
using opsg_internal::status_of;

constexpr int kThreads = 256;
constexpr int kShortRun = 32;  // longer runs are folded by a warp

int grid_of(long long items, int per_block, int cap)
{
    const long long b = (items + per_block - 1) / per_block;
    return (int)std::max<long long>(1, std::min<long long>(b, cap));
}

// Last d in [0, n) with dA[d] <= e (dA[0] == 0, dA non-decreasing).
__device__ __forceinline__ int d_row_of(const int *__restrict__ dA, int n, int e)
{
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(dA + mid) <= e) lo = mid;
        else hi = mid;
    }
    return lo;
}

// dlen[d] = A-row length of D row d (dlen[n] = 0); symbolic: zero the rows' nnz, which
// the count kernel accumulates; numeric: dnnz[d] = nnz of the row (dnnz[n] = 0).
__global__ void k_d_prep(const int *__restrict__ list, int n, const int *__restrict__ arpt, int *c_rpt,
                         int *__restrict__ dlen, int *__restrict__ dnnz, bool numeric)
{
    for (int d = blockIdx.x * blockDim.x + threadIdx.x; d <= n; d += gridDim.x * blockDim.x) {
        if (d == n) {
            dlen[n] = 0;
            if (numeric) dnnz[n] = 0;
            continue;
        }
        const int r = list[d];
        dlen[d] = arpt[r + 1] - arpt[r];
        if (numeric)
            dnnz[d] = c_rpt[r + 1] - c_rpt[r];
        else
            c_rpt[r] = 0;
    }
}

// elen[e] = length of the B row of concatenated A entry e (elen[ea] = 0).
__global__ void k_d_elen(const int *__restrict__ list, int n, const int *__restrict__ dA, const int *__restrict__ arpt,
                         const int *__restrict__ acol, const int *__restrict__ brpt, int *__restrict__ elen)
{
    const int ea = dA[n];
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e <= ea; e += gridDim.x * blockDim.x) {
        if (e == ea) {
            elen[ea] = 0;
            continue;
        }
        const int d = d_row_of(dA, n, e);
        const int j = __ldg(acol + __ldg(arpt + __ldg(list + d)) + (e - __ldg(dA + d)));
        elen[e] = __ldg(brpt + j + 1) - __ldg(brpt + j);
    }
}

// One warp per 32 concatenated A entries; product t of the concatenation is written at
// position t (epos: exclusive scan of elen), four chunks of 32 in flight.
template <bool kNum, typename KT>
__global__ void __launch_bounds__(kThreads) k_d_expand(const int *__restrict__ list, int n, const int *__restrict__ dA,
                                                       const int *__restrict__ epos, const int *__restrict__ arpt,
                                                       const int *__restrict__ acol, const int *__restrict__ brpt,
                                                       const int *__restrict__ bcol, int N, int cb,
                                                       KT *__restrict__ keys, unsigned long long *__restrict__ vals,
                                                       int *flags)
{
    const int lane = lane_id();
    const int ea = dA[n];
    const long long warp0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    bool bad = false;
    for (long long w = warp0; w * 32 < ea; w += nwarps) {
        const int e = (int)(w * 32) + lane;
        int d = 0, pa = 0, b0 = 0, bl = 0, at = 0;
        if (e < ea) {
            d = d_row_of(dA, n, e);
            pa = __ldg(arpt + __ldg(list + d)) + (e - __ldg(dA + d));
            const int j = __ldg(acol + pa);
            b0 = __ldg(brpt + j);
            bl = __ldg(brpt + j + 1) - b0;
            at = __ldg(epos + e);
        }
        int incl = bl;
#pragma unroll
        for (int s = 1; s < 32; s <<= 1) {
            const int t = __shfl_up_sync(kFull, incl, s);
            if (lane >= s) incl += t;
        }
        const int wtot = __shfl_sync(kFull, incl, 31);
        const int base = __shfl_sync(kFull, at, 0);  // the window's products are contiguous
        for (int c = 0; c < wtot; c += 32 * 4) {
            int kk[4], col[4], od[4], opa[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int p = c + u * 32 + lane;
                int lo = 0;
#pragma unroll
                for (int step = 16; step >= 1; step >>= 1) {
                    const int vv = __shfl_sync(kFull, incl, lo + step - 1);
                    if (vv <= p) lo += step;
                }
                const int o_incl = __shfl_sync(kFull, incl, lo);
                const int o_bl = __shfl_sync(kFull, bl, lo);
                const int o_b0 = __shfl_sync(kFull, b0, lo);
                od[u] = __shfl_sync(kFull, d, lo);
                opa[u] = __shfl_sync(kFull, pa, lo);
                kk[u] = o_b0 + (p - (o_incl - o_bl));
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) col[u] = (c + u * 32 + lane < wtot) ? __ldg(bcol + kk[u]) : 0;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int p = c + u * 32 + lane;
                if (p >= wtot) continue;
                if ((unsigned)col[u] >= (unsigned)N) {
                    bad = true;
                    col[u] = 0;
                }
                keys[base + p] = ((KT)od[u] << cb) | (KT)(unsigned)col[u];
                if constexpr (kNum) vals[base + p] = ((unsigned long long)(unsigned)opa[u] << 32) | (unsigned)kk[u];
            }
        }
    }
    if (bad) atomicOr(flags, kErrBadColumn);
}

// Symbolic: count the run heads (distinct (row, column) keys) of each D row.
template <typename KT>
__global__ void __launch_bounds__(kThreads) k_d_count(const KT *__restrict__ keys, long long total, int cb,
                                                      const int *__restrict__ list, int *c_rpt,
                                                      unsigned long long *total_nnz)
{
    const int lane = lane_id();
    unsigned long long mine = 0;
    for (long long t0 = (long long)blockIdx.x * blockDim.x; t0 < total; t0 += (long long)gridDim.x * blockDim.x) {
        const long long t = t0 + threadIdx.x;
        bool head = false;
        int d = -1;
        if (t < total) {
            const KT k = keys[t];
            head = t == 0 || k != keys[t - 1];
            d = (int)(k >> cb);
        }
        const unsigned grp = __match_any_sync(kFull, head ? d : -1);
        const unsigned hb = __ballot_sync(kFull, head);
        if (head && lane == __ffs(grp) - 1) atomicAdd(&c_rpt[list[d]], __popc(hb & grp));
        mine += head ? 1u : 0u;
    }
    mine = warp_sum_u64(mine);
    if (lane == 0 && mine) atomicAdd(total_nnz, mine);
}

// Numeric: flag[t] = 1 if element t starts a run.
template <typename KT>
__global__ void k_d_flags(const KT *__restrict__ keys, long long total, unsigned *__restrict__ flag)
{
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x)
        flag[t] = (t == 0 || keys[t] != keys[t - 1]) ? 1u : 0u;
}

// Numeric: hstart[h] = first element of run h; hstart[H] = total.
template <typename KT>
__global__ void k_d_starts(const KT *__restrict__ keys, const unsigned *__restrict__ hidx, long long total,
                           const int *__restrict__ hcum, int n, unsigned *__restrict__ hstart)
{
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x)
        if (t == 0 || keys[t] != keys[t - 1]) hstart[hidx[t]] = (unsigned)t;
    if (blockIdx.x == 0 && threadIdx.x == 0) hstart[hcum[n]] = (unsigned)total;
}

// Writes C entry h (run h of D row d, column col); a one-pass call writes it to the row's
// staging slot (soff) instead.
template <typename T>
__device__ __forceinline__ void d_write(int h, int d, int col, typename Acc<T>::S s, const int *__restrict__ hcum,
                                        const int *__restrict__ list, const int *__restrict__ c_rpt,
                                        const int *__restrict__ soff, int *c_col, T *c_val, int *flags)
{
    const int r = __ldg(list + d);
    const int *base = soff ? soff : c_rpt;
    const int off = __ldg(base + r);
    const int pos = off + (h - __ldg(hcum + d));
    if (pos < off || pos >= __ldg(base + r + 1)) {
        atomicOr(flags, kErrCountMismatch);
        return;
    }
    c_col[pos] = col;
    c_val[pos] = Acc<T>::fin(s);
}

// Numeric, runs of at most kShortRun products: one thread per run, four products'
// operands loaded together.  Longer runs are listed for k_d_fold_long.
template <typename T, typename KT>
__global__ void __launch_bounds__(kThreads) k_d_fold_short(const KT *__restrict__ keys,
                                                           const unsigned long long *__restrict__ vals,
                                                           const unsigned *__restrict__ hstart,
                                                           const int *__restrict__ hcum, int n, int cb,
                                                           const int *__restrict__ list, const T *__restrict__ aval,
                                                           const T *__restrict__ bval, const int *__restrict__ c_rpt,
                                                           const int *__restrict__ soff, int *__restrict__ c_col,
                                                           T *__restrict__ c_val, unsigned *__restrict__ long_runs,
                                                           int *long_count, int *flags)
{
    using AccT = Acc<T>;
    const int H = hcum[n];
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < H; h += gridDim.x * blockDim.x) {
        const unsigned t0 = hstart[h], t1 = hstart[h + 1];
        if (t1 - t0 > (unsigned)kShortRun) {
            long_runs[atomicAdd(long_count, 1)] = (unsigned)h;
            continue;
        }
        typename AccT::S s = AccT::zero();
        for (unsigned q = t0; q < t1; q += 4) {
            T av[4], bv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                av[u] = T(0);
                bv[u] = T(0);
                if (q + u < t1) {
                    const unsigned long long v = vals[q + u];
                    av[u] = __ldg(aval + (int)(v >> 32));
                    bv[u] = __ldg(bval + (int)(v & 0xffffffffu));
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (q + u < t1) s = AccT::step(s, av[u], bv[u]);
        }
        const KT k0 = keys[t0];
        d_write<T>(h, (int)(k0 >> cb), (int)(k0 & ((KT(1) << cb) - 1)), s, hcum, list, c_rpt, soff, c_col, c_val,
                   flags);
    }
}

// Numeric, long runs: one warp per run.  The lanes gather the operands of the next two
// batches of 32 products while lane 0 folds the current 32 from shared memory, in order.
template <typename T, typename KT>
__global__ void __launch_bounds__(kThreads) k_d_fold_long(const KT *__restrict__ keys,
                                                          const unsigned long long *__restrict__ vals,
                                                          const unsigned *__restrict__ hstart,
                                                          const int *__restrict__ hcum, int cb,
                                                          const int *__restrict__ list, const T *__restrict__ aval,
                                                          const T *__restrict__ bval, const int *__restrict__ c_rpt,
                                                          const int *__restrict__ soff, int *__restrict__ c_col,
                                                          T *__restrict__ c_val, const unsigned *__restrict__ long_runs,
                                                          const int *long_count, int *flags)
{
    using AccT = Acc<T>;
    __shared__ T s_a[kThreads / 32][2][32];
    __shared__ T s_b[kThreads / 32][2][32];
    const int lane = lane_id();
    const int warp = threadIdx.x >> 5;
    const int count = *long_count;
    const long long warp0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long i = warp0; i < count; i += nwarps) {
        const int h = (int)long_runs[i];
        const unsigned t0 = hstart[h], t1 = hstart[h + 1];
        auto gather = [&](unsigned q, T &a, T &b) {
            a = T(0);
            b = T(0);
            if (q < t1) {
                const unsigned long long v = vals[q];
                a = __ldg(aval + (int)(v >> 32));
                b = __ldg(bval + (int)(v & 0xffffffffu));
            }
        };
        if (t1 - t0 > (unsigned)kBlockFoldMin) {
            // blocked entry: lane b folds products [t0 + b c, t0 + (b + 1) c), eight
            // products' operands in flight; lane 0 merges the lanes' states in order
            static_assert(kFoldBlocks == 32, "a lane per block");
            const unsigned c = (t1 - t0 + kFoldBlocks - 1) / kFoldBlocks;
            const unsigned q0 = t0 + (unsigned)lane * c;
            const unsigned q1 = min(t1, q0 + c);
            typename AccT::S s = AccT::zero();
            for (unsigned q = q0; q < q1; q += 8) {
                T a8[8], b8[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    a8[u] = T(0);
                    b8[u] = T(0);
                    if (q + u < q1) {
                        const unsigned long long v = vals[q + u];
                        a8[u] = __ldg(aval + (int)(v >> 32));
                        b8[u] = __ldg(bval + (int)(v & 0xffffffffu));
                    }
                }
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    if (q + u < q1) s = AccT::step(s, a8[u], b8[u]);
            }
            typename AccT::S tot = s;
            for (int b = 1; b < kFoldBlocks; ++b) {
                const typename AccT::S o = AccT::shfl(s, b);
                if (lane == 0) tot = AccT::merge(tot, o);
            }
            if (lane == 0) {
                const KT k0 = keys[t0];
                d_write<T>(h, (int)(k0 >> cb), (int)(k0 & ((KT(1) << cb) - 1)), tot, hcum, list, c_rpt, soff, c_col,
                           c_val, flags);
            }
            __syncwarp();
            continue;
        }
        // two batches in flight ahead of the fold: a batch's gather (two dependent loads)
        // takes about as long as 32 dependent FP64 FMAs (~64 cycles each on this GPU)
        T na, nb, na2, nb2;
        gather(t0 + lane, na, nb);
        gather(t0 + 32 + lane, na2, nb2);
        typename AccT::S s = AccT::zero();
        int buf = 0;
        for (unsigned q = t0; q < t1; q += 32) {
            s_a[warp][buf][lane] = na;
            s_b[warp][buf][lane] = nb;
            __syncwarp();
            na = na2;
            nb = nb2;
            gather(q + 64 + lane, na2, nb2);
            if (lane == 0) {
                const int m = (int)min(32u, t1 - q);
                if (m == 32) {  // operands to registers first: the chain waits only on the FMAs
                    T ra[32], rb[32];
#pragma unroll
                    for (int u = 0; u < 32; ++u) {
                        ra[u] = s_a[warp][buf][u];
                        rb[u] = s_b[warp][buf][u];
                    }
#pragma unroll
                    for (int u = 0; u < 32; ++u) s = AccT::step(s, ra[u], rb[u]);
                } else {
                    for (int u = 0; u < m; ++u) s = AccT::step(s, s_a[warp][buf][u], s_b[warp][buf][u]);
                }
            }
            buf ^= 1;
        }
        if (lane == 0) {
            const KT k0 = keys[t0];
            d_write<T>(h, (int)(k0 >> cb), (int)(k0 & ((KT(1) << cb) - 1)), s, hcum, list, c_rpt, soff, c_col,
                       c_val, flags);
        }
        __syncwarp();
    }
}

// One-pass call: the D rows' output counts come from the head scan itself.  Row d's
// products start at sorted position epos[dA[d]] (the sort keeps rows in order), so the
// heads before it are hidx there; hcum[d] = those heads, c_rpt[row] = the row's heads, and
// nnz(C) gains all of them.
__global__ void k_d_stage_counts(const int *__restrict__ list, int n, const int *__restrict__ dA,
                                 const int *__restrict__ epos, const unsigned *__restrict__ hidx,
                                 const unsigned *__restrict__ flag, long long total, int *__restrict__ hcum,
                                 int *c_rpt, unsigned long long *total_nnz)
{
    const int all = (int)(hidx[total - 1] + flag[total - 1]);
    auto heads_before = [&](int d) {
        const int p = d < n ? __ldg(epos + __ldg(dA + d)) : (int)total;
        return p < total ? (int)hidx[p] : all;
    };
    for (int d = blockIdx.x * blockDim.x + threadIdx.x; d <= n; d += gridDim.x * blockDim.x) {
        const int h0 = heads_before(d);
        hcum[d] = h0;
        if (d < n) c_rpt[list[d]] = heads_before(d + 1) - h0;
        else atomicAdd(total_nnz, (unsigned long long)all);
    }
}

template <typename T, typename KT>
int run_d_rows_keyed(ops_handle_s *h, const SpgemmArgs<T> &g, const int *list, int n, bool numeric, cudaStream_t s,
                     int cb, int bits, bool dry_run)
{
    const bool staged = numeric && g.soff != nullptr;  // one-pass call: counts found here
    const long long total = h->plan_d_flop;
    const long long ea_max = h->plan_d_len_a;  // concatenated A entries

    size_t cub_sort = 0, cub_scan = 0, cub_small = 0;
    {
        cub::DoubleBuffer<KT> kb(nullptr, nullptr);
        cub::DoubleBuffer<unsigned long long> vb(nullptr, nullptr);
        if (numeric)
            OPS_CUDA(h, cub::DeviceRadixSort::SortPairs(nullptr, cub_sort, kb, vb, (int)total, 0, bits, s));
        else
            OPS_CUDA(h, cub::DeviceRadixSort::SortKeys(nullptr, cub_sort, kb, (int)total, 0, bits, s));
        OPS_CUDA(h, cub::DeviceScan::ExclusiveSum(nullptr, cub_scan, (unsigned *)nullptr, (unsigned *)nullptr,
                                                  (int)std::max<long long>(total, ea_max + 1), s));
        OPS_CUDA(h, cub::DeviceScan::ExclusiveSum(nullptr, cub_small, (int *)nullptr, (int *)nullptr, n + 1, s));
    }
    const size_t cub_bytes = std::max(cub_sort, std::max(cub_scan, cub_small));
    const size_t kbytes = align_up(sizeof(KT) * (size_t)total, 256);
    const size_t vbytes = numeric ? align_up(sizeof(unsigned long long) * (size_t)total, 256) : 0;
    const size_t hbytes = numeric ? align_up(sizeof(unsigned) * ((size_t)total + 1), 256) : 0;
    const size_t ebytes = align_up(sizeof(int) * (size_t)(ea_max + 1), 256);
    const size_t sbytes = align_up(sizeof(int) * (size_t)(n + 1), 256);
    const size_t need = 2 * kbytes + 2 * vbytes + 2 * hbytes + 2 * ebytes + 4 * sbytes + align_up(cub_bytes, 256);
    if (need > h->dense_budget) return OPS_NOT_SUPPORTED;
    if (dry_run) return OPS_OK;

    void *mem = nullptr;
    OPS_CUDA(h, cudaMallocFromPoolAsync(&mem, need, h->pool, s));
    unsigned char *p = static_cast<unsigned char *>(mem);
    auto take = [&](size_t b) {
        unsigned char *q = p;
        p += b;
        return q;
    };
    KT *k0 = reinterpret_cast<KT *>(take(kbytes));
    KT *k1 = reinterpret_cast<KT *>(take(kbytes));
    auto *v0 = numeric ? reinterpret_cast<unsigned long long *>(take(vbytes)) : nullptr;
    auto *v1 = numeric ? reinterpret_cast<unsigned long long *>(take(vbytes)) : nullptr;
    unsigned *flag = numeric ? reinterpret_cast<unsigned *>(take(hbytes)) : nullptr;
    unsigned *hidx = numeric ? reinterpret_cast<unsigned *>(take(hbytes)) : nullptr;
    int *elen = reinterpret_cast<int *>(take(ebytes));
    int *epos = reinterpret_cast<int *>(take(ebytes));
    int *dlen = reinterpret_cast<int *>(take(sbytes));
    int *dA = reinterpret_cast<int *>(take(sbytes));
    int *dnnz = reinterpret_cast<int *>(take(sbytes));
    int *hcum = reinterpret_cast<int *>(take(sbytes));
    void *cub_tmp = take(align_up(cub_bytes, 256));
    const int sms = h->num_sms;
    int st = OPS_OK;
    auto check = [&](cudaError_t e, const char *what) {
        if (e != cudaSuccess && st == OPS_OK) {
            (void)cudaGetLastError();
            st = fail(h, status_of(e), std::string(what) + ": " + cudaGetErrorString(e));
        }
        return st == OPS_OK;
    };
    auto launched = [&](const char *what) {
        ++h->launches;
        return check(cudaGetLastError(), what);
    };
    size_t b = cub_bytes;

    k_d_prep<<<grid_of(n + 1, kThreads, sms * 4), kThreads, 0, s>>>(list, n, g.arpt, g.c_rpt, dlen, dnnz,
                                                                      numeric && !staged);
    if (launched("k_d_prep")) check(cub::DeviceScan::ExclusiveSum(cub_tmp, b = cub_bytes, dlen, dA, n + 1, s), "D-row scan");
    if (st == OPS_OK) {
        k_d_elen<<<grid_of(ea_max + 1, kThreads, sms * 8), kThreads, 0, s>>>(list, n, dA, g.arpt, g.acol, g.brpt, elen);
        if (launched("k_d_elen"))
            check(cub::DeviceScan::ExclusiveSum(cub_tmp, b = cub_bytes, elen, epos, (int)ea_max + 1, s), "product scan");
    }
    if (st == OPS_OK) {
        const int grid = grid_of(ea_max / 32 + 1, kThreads / 32, sms * 8);
        if (numeric)
            k_d_expand<true, KT><<<grid, kThreads, 0, s>>>(list, n, dA, epos, g.arpt, g.acol, g.brpt, g.bcol, g.N, cb,
                                                            k0, v0, &g.info->flags);
        else
            k_d_expand<false, KT><<<grid, kThreads, 0, s>>>(list, n, dA, epos, g.arpt, g.acol, g.brpt, g.bcol, g.N, cb,
                                                             k0, nullptr, &g.info->flags);
        launched("k_d_expand");
    }
    cub::DoubleBuffer<KT> keys(k0, k1);
    cub::DoubleBuffer<unsigned long long> vals(v0, v1);
    if (st == OPS_OK) {
        check(numeric ? cub::DeviceRadixSort::SortPairs(cub_tmp, b = cub_bytes, keys, vals, (int)total, 0, bits, s)
                      : cub::DeviceRadixSort::SortKeys(cub_tmp, b = cub_bytes, keys, (int)total, 0, bits, s),
              "stable radix sort of the D-row products");
    }
    const int grid = grid_of(total, kThreads, sms * 16);
    if (st == OPS_OK && !numeric) {
        k_d_count<KT><<<grid, kThreads, 0, s>>>(keys.Current(), total, cb, list, g.c_rpt, &g.info->total_nnz);
        launched("k_d_count");
    }
    if (st == OPS_OK && numeric) {
        k_d_flags<KT><<<grid, kThreads, 0, s>>>(keys.Current(), total, flag);
        if (launched("k_d_flags"))
            check(cub::DeviceScan::ExclusiveSum(cub_tmp, b = cub_bytes, flag, hidx, (int)total, s), "head scan");
        if (st == OPS_OK && staged) {
            k_d_stage_counts<<<grid_of(n + 1, kThreads, sms * 4), kThreads, 0, s>>>(
                list, n, dA, epos, hidx, flag, total, hcum, g.c_rpt, &g.info->total_nnz);
            launched("k_d_stage_counts");
        } else if (st == OPS_OK) {
            check(cub::DeviceScan::ExclusiveSum(cub_tmp, b = cub_bytes, dnnz, hcum, n + 1, s), "row nnz scan");
        }
        unsigned *hstart = flag;                                                   // free after the scan
        unsigned *long_runs = reinterpret_cast<unsigned *>(vals.Alternate());    // free after the sort
        if (st == OPS_OK) {
            k_d_starts<KT><<<grid, kThreads, 0, s>>>(keys.Current(), hidx, total, hcum, n, hstart);
            launched("k_d_starts");
        }
        if (st == OPS_OK) check(cudaMemsetAsync(&g.info->d_cursor, 0, sizeof(int), s), "long-run counter");
        if (st == OPS_OK) {
            k_d_fold_short<T, KT><<<grid, kThreads, 0, s>>>(keys.Current(), vals.Current(), hstart, hcum, n, cb, list,
                                                           g.aval, g.bval, g.c_rpt, g.soff, g.c_col, g.c_val,
                                                           long_runs, &g.info->d_cursor, &g.info->flags);
            launched("k_d_fold_short");
        }
        if (st == OPS_OK) {
            k_d_fold_long<T, KT><<<sms * 8, kThreads, 0, s>>>(keys.Current(), vals.Current(), hstart, hcum, cb, list,
                                                             g.aval, g.bval, g.c_rpt, g.soff, g.c_col, g.c_val,
                                                             long_runs, &g.info->d_cursor, &g.info->flags);
            launched("k_d_fold_long");
        }
    }
    check(cudaFreeAsync(mem, s), "scratch release");
    return st;
}

}  // namespace

namespace opsg_internal {

template <typename T>
int run_d_rows(ops_handle_s *h, const SpgemmArgs<T> &g, const int *list, int n, bool numeric, cudaStream_t s,
               bool dry_run)
{
    const long long total = h->plan_d_flop;
    const int db = ceil_log2(std::max(n, 2));
    const int cb = ceil_log2(std::max(g.N, 2));
    if (total <= 0 || total > (long long)INT_MAX - 1 || h->plan_d_len_a <= 0 ||
        h->plan_d_len_a > (long long)INT_MAX - 1)
        return OPS_NOT_SUPPORTED;
    if (db + cb <= 32) return run_d_rows_keyed<T, unsigned>(h, g, list, n, numeric, s, cb, db + cb, dry_run);
    return run_d_rows_keyed<T, unsigned long long>(h, g, list, n, numeric, s, cb, db + cb, dry_run);
}

template int run_d_rows<double>(ops_handle_s *, const SpgemmArgs<double> &, const int *, int, bool, cudaStream_t,
                                bool);
template int run_d_rows<float>(ops_handle_s *, const SpgemmArgs<float> &, const int *, int, bool, cudaStream_t,
                               bool);

}  // namespace opsg_internal
