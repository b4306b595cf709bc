// kernels.cuh — the SpGEMM kernels (setup/binning, symbolic and numeric per row class).
//
// Correspondence with OpSparse (paths relative to its source tree):
//   k_setup            <- k_compute_flop (src/opsparse/numeric/compute_flop.cu:9-31) fused with
//                         k_symbolic_binning/k_symbolic_binning2 (kernels/binning.cuh:11-81):
//                         one pass computes each row's product count and appends the row to its
//                         class list, with no host round trip between count and scatter.
//   k_reg_rows<G>      <- k_symbolic_shared_hash_pwarp / k_numeric_shared_hash_pwarp
//                         (kernels/symbolic.cuh:9-72, kernels/numeric.cuh:9-107): rows with at
//                         most G products are handled by G lanes in registers (match_any
//                         de-duplication, no table, no sort pass).
//   k_warp_rows        <- k_*_shared_hash_tb for the small bins (symbolic.cuh:74-130,
//                         numeric.cuh:109-205): one warp per row, table in shared memory.
//   k_esc_rows (esc.cuh) <- the same kernels for the middle/large bins and
//                         k_*_max_shared_hash_tb (symbolic.cuh:132-261, numeric.cuh:207-302).
//   k_dense_rows       <- the global-hash fallback (symbolic.cuh:263-325, numeric.cuh:304-393):
//                         one CTA per row over a dense accumulator and bitmap in HBM, which
//                         also yields ascending columns without a sort.
//   k_small_rows       <- k_numeric_shared_hash_pwarp for rows of at most 8 products: one
//                         thread per row, a sorting network in registers.
//   k_place_staged     no counterpart: copies the rows a one-pass call computed while
//                         counting from the staging area into C.
//
// Numeric values are folded in ascending j for every output entry (see common.cuh), so
// all classes produce the same bits as the CPU oracle.
#pragma once

#include <climits>

#include "common.cuh"

namespace opsg {

// Sum of one u64 per thread over the warp, added to *dst by lane 0: no block barrier,
// so warps of one CTA that finish early do not wait for the others.
__device__ __forceinline__ void warp_add_u64(unsigned long long v, unsigned long long *dst)
{
    v = warp_sum_u64(v);
    if (lane_id() == 0 && v) atomicAdd(dst, v);
}

// Sum of one u64 per thread over the block, added to *dst by one thread.  Every thread
// of the block must call it.
__device__ __forceinline__ void block_add_u64(unsigned long long v, unsigned long long *dst)
{
    __shared__ unsigned long long s_part[32];
    v = warp_sum_u64(v);
    const int warp = threadIdx.x >> 5;
    if (lane_id() == 0) s_part[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_part[w];
        if (t) atomicAdd(dst, t);
    }
    __syncthreads();
}

constexpr int kFoldUnroll = 4;  // fold steps whose operands are loaded together

// Folds the runs [hs, he) owned by the calling thread (run h covers the sorted positions
// [head(h), end(h)); runs of skip_len or more products are left to the caller): the
// concatenation of the runs is walked one product per step, the operands of kFoldUnroll
// steps loaded together (load(t, a, b, k) gives product t's operands and its B index),
// and each completed run is passed to write(h, t, k, s) with one of its positions and B
// indices.  A warp-wide FP64 FMA costs the same however few lanes are active, so packing
// the steps makes a warp issue about as many FMAs as its busiest lane has products,
// where one run per lane per step would issue kFoldUnroll per run.
template <typename T, typename Head, typename End, typename Load, typename Write>
__device__ __forceinline__ void fold_own_runs(int hs, int he, int skip_len, Head head, End end, Load load,
                                              Write write)
{
    using AccT = Acc<T>;
    using S = typename AccT::S;
    int h = hs, t = 0, e = 0;  // current run, next position, end of the run
    auto next_run = [&]() {    // from run h on: the first run to fold, or h == he
        for (; h < he; ++h) {
            t = head(h);
            e = end(h);
            if (e - t < skip_len) return;
        }
    };
    next_run();
    S s = AccT::zero();
    while (h < he) {
        T av[kFoldUnroll], bv[kFoldUnroll];
        int hu[kFoldUnroll], pu[kFoldUnroll], ku[kFoldUnroll];
#pragma unroll
        for (int u = 0; u < kFoldUnroll; ++u) {
            hu[u] = -1;
            pu[u] = 0;
            ku[u] = 0;
            av[u] = T(0);
            bv[u] = T(0);
            if (h < he) {
                hu[u] = h;
                pu[u] = t;
                load(t, av[u], bv[u], ku[u]);
                if (++t == e) {
                    ++h;
                    next_run();
                }
            }
        }
#pragma unroll
        for (int u = 0; u < kFoldUnroll; ++u) {
            if (hu[u] >= 0) {
                s = AccT::step(s, av[u], bv[u]);
                const int hn = u + 1 < kFoldUnroll ? hu[u + 1] : (h < he ? h : -1);
                if (hn != hu[u]) {  // run hu[u] is complete
                    write(hu[u], pu[u], ku[u], s);
                    s = AccT::zero();
                }
            }
        }
    }
}

// ==================================================================================
// Setup: per-row product count, validation of A's columns, class assignment, and the
// scatter of row ids into per-class lists (lists[c * M + i]).  One thread per row for
// rows of at most 8 A entries, whose loads are issued all at once (8 column loads, then
// 16 row-pointer loads); longer rows are summed cooperatively by their warp, 8 loads in
// flight per lane.  Rows with no products get nnz 0 immediately and join no list.
// ==================================================================================
constexpr int kSetupThreads = 512;
constexpr int kSetupUnroll = 8;

static __global__ void __launch_bounds__(kSetupThreads) k_setup(const int *__restrict__ arpt, const int *__restrict__ acol,
                                                        const int *__restrict__ brpt, const int *__restrict__ bcol,
                                                        int M, int K, int N, int *__restrict__ row_flop,
                                                        int *__restrict__ lists, int *__restrict__ c_rownnz,
                                                        int *__restrict__ sflop, DevInfo *info, Thresholds th)
{
    static_assert(kSmallFlopMax == kSetupUnroll, "R8 rows are gathered from the light-row registers");
    __shared__ int s_cnt[kNumClasses];
    __shared__ int s_base[kNumClasses];
    __shared__ unsigned long long s_flop[kSetupThreads / 32];
    __shared__ unsigned long long s_sflop[kSetupThreads / 32];
    __shared__ int s_e1one;
    __shared__ unsigned s_small[kSetupThreads / 32];
    __shared__ int s_flags;
    const int lane = lane_id();
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x < kNumClasses) s_cnt[threadIdx.x] = 0;
    if (threadIdx.x == 0) {
        s_flags = 0;
        s_e1one = 0;
    }
    __syncthreads();

    const int r = blockIdx.x * kSetupThreads + threadIdx.x;
    const bool in = r < M;
    int a0 = 0, a1 = 0;
    if (in) {
        a0 = arpt[r];
        a1 = arpt[r + 1];
    }
    const int lenA = a1 - a0;
    long long flop = 0;
    bool bad = false;
    const bool light = in && lenA <= kSetupUnroll;
    int b0[kSetupUnroll], bl[kSetupUnroll];
    {
        int jj[kSetupUnroll];
#pragma unroll
        for (int u = 0; u < kSetupUnroll; ++u) jj[u] = (light && u < lenA) ? __ldg(acol + a0 + u) : -1;
#pragma unroll
        for (int u = 0; u < kSetupUnroll; ++u) {
            b0[u] = 0;
            bl[u] = 0;
            if (jj[u] >= 0 && jj[u] < K) {
                b0[u] = __ldg(brpt + jj[u]);
                bl[u] = __ldg(brpt + jj[u] + 1) - b0[u];
            } else if (light && u < lenA) {
                bad = true;
            }
            flop += bl[u];
        }
    }
    unsigned heavy = __ballot_sync(kFull, in && !light);
    while (heavy) {
        const int t = __ffs(heavy) - 1;
        heavy &= heavy - 1u;
        const int h0 = __shfl_sync(kFull, a0, t);
        const int h1 = __shfl_sync(kFull, a1, t);
        unsigned long long s = 0;
        bool hb = false;
        for (int p0 = h0; p0 < h1; p0 += 32 * kSetupUnroll) {
            int jj[kSetupUnroll];
#pragma unroll
            for (int u = 0; u < kSetupUnroll; ++u) {
                const int p = p0 + u * 32 + lane;
                jj[u] = p < h1 ? __ldg(acol + p) : -1;
            }
            int lo[kSetupUnroll], hi[kSetupUnroll];
#pragma unroll
            for (int u = 0; u < kSetupUnroll; ++u) {
                const bool ok = (unsigned)jj[u] < (unsigned)K;
                hb |= (p0 + u * 32 + lane < h1) && !ok;
                lo[u] = ok ? __ldg(brpt + jj[u]) : 0;
                hi[u] = ok ? __ldg(brpt + jj[u] + 1) : 0;
            }
#pragma unroll
            for (int u = 0; u < kSetupUnroll; ++u) s += (unsigned long long)(hi[u] - lo[u]);
        }
        s = warp_sum_u64(s);
        hb = __any_sync(kFull, hb);
        if (lane == t) {
            flop = (long long)s;
            bad = hb;
        }
    }
    if (bad) atomicOr(&s_flags, kErrBadColumn);
    if (flop > INT_MAX) atomicOr(&s_flags, kErrRowFlopOverflow);
    const int f32 = flop > INT_MAX ? INT_MAX : (int)flop;

    int cls = -1;
    unsigned small_nnz = 0;
    if (in) {
        row_flop[r] = f32;
        if (flop == 0) {
            c_rownnz[r] = 0;
        } else if (!bad && flop <= th.r8 && lenA <= th.r8) {
            // R8 row: its symbolic phase happens here.  Product t (t < flop <= 8) is
            // entry b0[u] + t - pre[u] of the B row of the A entry u that covers it; the
            // <= 8 column keys are loaded together and the distinct ones counted in
            // registers.  These rows join no list; the numeric phase walks them in row
            // order (k_small_rows).
            cls = kClsR8;
            int kt[kSmallFlopMax];
#pragma unroll
            for (int t = 0; t < kSmallFlopMax; ++t) kt[t] = 0;
            int pre = 0;
#pragma unroll
            for (int u = 0; u < kSetupUnroll; ++u) {
#pragma unroll
                for (int t = 0; t < kSmallFlopMax; ++t)
                    if (t >= pre && t < pre + bl[u]) kt[t] = b0[u] + t - pre;
                pre += bl[u];
            }
            int key[kSmallFlopMax];
#pragma unroll
            for (int t = 0; t < kSmallFlopMax; ++t) key[t] = t < f32 ? __ldg(bcol + kt[t]) : -1;
#pragma unroll
            for (int t = 0; t < kSmallFlopMax; ++t) {
                if (t >= f32) continue;
                bool dup = (unsigned)key[t] >= (unsigned)N;
                if (dup) atomicOr(&s_flags, kErrBadColumn);
#pragma unroll
                for (int q = 0; q < t; ++q) dup |= key[q] == key[t];
                small_nnz += dup ? 0u : 1u;
            }
            c_rownnz[r] = (int)small_nnz;
        } else if (flop <= th.r16 && lenA <= 16) {
            cls = kClsR16;
        } else if (flop <= th.r32 && lenA <= 32) {
            cls = kClsR32;
        } else if (flop <= th.w) {
            cls = kClsW;
        } else if (flop <= th.e1 && lenA <= kEsc1AMax) {
            cls = kClsE1;
        } else if (flop <= th.e2 && lenA <= kEsc2AMax) {
            cls = kClsE2;
        } else {
            cls = kClsD;
            atomicAdd(&info->d_len_a, (unsigned long long)lenA);
            atomicAdd(&info->d_flop, (unsigned long long)flop);
        }
    }

    // Per-class positions: warp rank -> block rank -> global base.
    int my_off = 0;
#pragma unroll
    for (int c = 0; c < kNumClasses; ++c) {
        const unsigned mk = __ballot_sync(kFull, cls == c);
        if (mk) {
            const int leader = __ffs(mk) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(&s_cnt[c], __popc(mk));
            base = __shfl_sync(kFull, base, leader);
            if (cls == c) my_off = base + __popc(mk & lanemask_lt());
        }
    }
    // products a one-pass call may compute in the counting phase (every class but R8, whose
    // count is made here and whose numeric runs straight into C, and the E1 column-window
    // rows), for the prefix that places them in the staging area
    int staged = 0;
    if (sflop) {
        staged = cls > kClsR8 ? f32 : 0;
        if (cls == kClsE1 && f32 >= 16 * lenA) {
            // a column-window row keeps two passes: span of its B rows' first and last
            // columns (B rows are sorted; lenA <= 64 here)
            int cmin = INT_MAX, cmax = -1;
            if (light) {
#pragma unroll
                for (int u = 0; u < kSetupUnroll; ++u) {
                    if (u < lenA && bl[u] > 0) {
                        cmin = min(cmin, __ldg(bcol + b0[u]));
                        cmax = max(cmax, __ldg(bcol + b0[u] + bl[u] - 1));
                    }
                }
            } else {
                for (int p = a0; p < a1; ++p) {
                    const int j = __ldg(acol + p);
                    if ((unsigned)j >= (unsigned)K) continue;  // reported above
                    const int q0 = __ldg(brpt + j), q1 = __ldg(brpt + j + 1);
                    if (q1 > q0) {
                        cmin = min(cmin, __ldg(bcol + q0));
                        cmax = max(cmax, __ldg(bcol + q1 - 1));
                    }
                }
            }
            if (cmax >= cmin && cmax - cmin < kWinBits) staged = 0;
        }
        if (in) sflop[r] = staged;
        if (cls == kClsE1 && staged) atomicAdd(&s_e1one, 1);
    }
    const unsigned long long wsf = warp_sum_u64((unsigned long long)staged);
    unsigned long long wf = warp_sum_u64((unsigned long long)flop);
    const unsigned wmax = __reduce_max_sync(kFull, (unsigned)f32);
    const unsigned wsmall = __reduce_add_sync(kFull, small_nnz);
    if (lane == 0) {
        s_flop[warp] = wf;
        s_sflop[warp] = wsf;
        s_small[warp] = wsmall;
    }
    __syncthreads();
    if (threadIdx.x < kNumClasses) {
        const int n = s_cnt[threadIdx.x];
        s_base[threadIdx.x] = n ? atomicAdd(&info->counts[threadIdx.x], n) : 0;
    }
    if (threadIdx.x == 32) {
        unsigned long long t = 0;
        for (int w = 0; w < kSetupThreads / 32; ++w) t += s_flop[w];
        if (t) atomicAdd(&info->total_flop, t);
        unsigned long long ts = 0;
        for (int w = 0; w < kSetupThreads / 32; ++w) ts += s_sflop[w];
        if (ts) atomicAdd(&info->staged_flop, ts);
        if (s_e1one) atomicAdd(&info->e1_one, s_e1one);
        unsigned long long sn = 0;
        for (int w = 0; w < kSetupThreads / 32; ++w) sn += s_small[w];
        if (sn) atomicAdd(&info->total_nnz, sn);
        if (s_flags) atomicOr(&info->flags, s_flags);
    }
    if (lane == 0 && wmax) atomicMax(&info->max_flop, (int)wmax);
    __syncthreads();
    if (cls > kClsR8) lists[(size_t)cls * M + s_base[cls] + my_off] = r;
}

// ==================================================================================
// Numeric phase of the R8 rows (<= 8 products, <= 8 A entries), one thread per row in
// row order: no list, coalesced row metadata, nothing in shared memory.  Each level of
// loads is issued at once (A entries, then B row pointers, then the <= 8 products), the
// products are sorted in registers by (column, product index) with a 19-comparator
// network — equal columns keep ascending j — and each run is folded with one FMA per
// product, so a warp issues at most 8 FMA instructions per 32 rows.
// ==================================================================================
constexpr int kSmallThreads = 256;

template <typename K, typename T>
__device__ __forceinline__ void cmp_swap3(K &ka, T &aa, T &ba, K &kb, T &ab, T &bb)
{
    const bool sw = kb < ka;
    const K k = sw ? kb : ka;
    kb = sw ? ka : kb;
    ka = k;
    const T a = sw ? ab : aa;
    ab = sw ? aa : ab;
    aa = a;
    const T b = sw ? bb : ba;
    bb = sw ? ba : bb;
    ba = b;
}

template <typename T>
__global__ void __launch_bounds__(kSmallThreads, 4) k_small_rows(SpgemmArgs<T> g, int r8)
{
    using AccT = Acc<T>;
    constexpr int U = kSmallFlopMax;
    static_assert(U == 8, "the sorting network is for 8 keys");
    for (int r = blockIdx.x * kSmallThreads + threadIdx.x; r < g.M; r += gridDim.x * kSmallThreads) {
        const int flop = __ldg(g.row_flop + r);
        const int a0 = __ldg(g.arpt + r);
        const int lenA = __ldg(g.arpt + r + 1) - a0;
        if (flop == 0 || flop > r8 || lenA > r8) continue;
        int jj[U];
        T av[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            jj[u] = u < lenA ? __ldg(g.acol + a0 + u) : 0;
            av[u] = u < lenA ? __ldg(g.aval + a0 + u) : T(0);
        }
        int b0[U], bl[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            b0[u] = u < lenA ? __ldg(g.brpt + jj[u]) : 0;
            bl[u] = u < lenA ? __ldg(g.brpt + jj[u] + 1) - b0[u] : 0;
        }
        // product t is entry b0[u] + t - pre[u] of the B row of the A entry u covering it
        int kt[U];
        T at[U];
#pragma unroll
        for (int t = 0; t < U; ++t) {
            kt[t] = 0;
            at[t] = T(0);
        }
        int pre = 0;
#pragma unroll
        for (int u = 0; u < U; ++u) {
#pragma unroll
            for (int t = 0; t < U; ++t) {
                if (t >= pre && t < pre + bl[u]) {
                    kt[t] = b0[u] + t - pre;
                    at[t] = av[u];
                }
            }
            pre += bl[u];
        }
        unsigned long long key[U];
        T bt[U];
#pragma unroll
        for (int t = 0; t < U; ++t) {
            const bool v = t < flop;
            key[t] = v ? (((unsigned long long)(unsigned)__ldg(g.bcol + kt[t]) << 3) | (unsigned)t) : ~0ull;
            bt[t] = v ? __ldg(g.bval + kt[t]) : T(0);
        }
#define OPSG_CS(i, j) cmp_swap3(key[i], at[i], bt[i], key[j], at[j], bt[j])
        OPSG_CS(0, 2); OPSG_CS(1, 3); OPSG_CS(4, 6); OPSG_CS(5, 7);
        OPSG_CS(0, 4); OPSG_CS(1, 5); OPSG_CS(2, 6); OPSG_CS(3, 7);
        OPSG_CS(0, 1); OPSG_CS(2, 3); OPSG_CS(4, 5); OPSG_CS(6, 7);
        OPSG_CS(2, 4); OPSG_CS(3, 5);
        OPSG_CS(1, 4); OPSG_CS(3, 6);
        OPSG_CS(1, 2); OPSG_CS(3, 4); OPSG_CS(5, 6);
#undef OPSG_CS
        const int off = __ldg(g.c_rpt + r);
        const int n_expect = __ldg(g.c_rpt + r + 1) - off;
        typename AccT::S acc = AccT::zero();
        int pos = 0;
#pragma unroll
        for (int m = 0; m < U; ++m) {
            if (m < flop) {
                acc = AccT::step(acc, at[m], bt[m]);
                const bool last = m + 1 == flop || (m + 1 < U && (key[m + 1] >> 3) != (key[m] >> 3));
                if (last) {
                    if (pos < n_expect) {
                        g.c_col[off + pos] = (int)(key[m] >> 3);
                        g.c_val[off + pos] = AccT::fin(acc);
                    }
                    ++pos;
                    acc = AccT::zero();
                }
            }
        }
        if (pos != n_expect) atomicOr(&g.info->flags, kErrCountMismatch);
    }
}

// ==================================================================================
// R classes: G lanes per row (G = 8, 16, 32), all of the row's products in one chunk.
// Lane q of a group holds product q; duplicates are found with __match_any_sync, the
// lowest lane of each match group is its leader.  Symbolic: nnz = number of leaders.
// Numeric: each leader folds its group in lane order (= ascending j), ranks itself
// among the group's leaders by column, and writes C directly in sorted position.
// Grid-stride over the class list; every lane of a warp runs the same trip count.
// ==================================================================================
template <int G, bool kNum, typename T>
__global__ void __launch_bounds__(256) k_reg_rows(SpgemmArgs<T> g, const int *__restrict__ list, int count)
{
    using AccT = Acc<T>;
    using S = typename AccT::S;
    constexpr int kGroups = 32 / G;
    const int lane = lane_id();
    const int q = lane & (G - 1);
    const unsigned gmask = (G == 32) ? kFull : (((1u << G) - 1u) << (lane & ~(G - 1)));
    const long long warp0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    unsigned long long nnz_acc = 0;

    for (long long w = warp0; w * kGroups < count; w += nwarps) {
        const long long gid = w * kGroups + lane / G;
        const bool active = gid < count;
        int r = 0, a0 = 0, lenA = 0;
        if (active) {
            r = __ldg(list + gid);
            a0 = __ldg(g.arpt + r);
            lenA = __ldg(g.arpt + r + 1) - a0;
        }
        int b0 = 0, bl = 0;
        T av = T(0);
        if (q < lenA) {
            const int j = __ldg(g.acol + a0 + q);
            b0 = __ldg(g.brpt + j);
            bl = __ldg(g.brpt + j + 1) - b0;
            if (kNum) av = __ldg(g.aval + a0 + q);
        }
        int incl = bl;
#pragma unroll
        for (int d = 1; d < G; d <<= 1) {
            const int t = __shfl_up_sync(kFull, incl, d, G);
            if (q >= d) incl += t;
        }
        const int flop = __shfl_sync(kFull, incl, G - 1, G);
        const bool valid = q < flop;
        int lo = 0;
#pragma unroll
        for (int step = G / 2; step >= 1; step >>= 1) {
            const int v = __shfl_sync(kFull, incl, lo + step - 1, G);
            if (v <= q) lo += step;
        }
        const int o_incl = __shfl_sync(kFull, incl, lo, G);
        const int o_bl = __shfl_sync(kFull, bl, lo, G);
        const int o_b0 = __shfl_sync(kFull, b0, lo, G);
        const int k = o_b0 + (q - (o_incl - o_bl));
        const int col = valid ? __ldg(g.bcol + k) : kEmpty;
        if (__any_sync(kFull, valid && (unsigned)col >= (unsigned)g.N) && lane == 0)
            atomicOr(&g.info->flags, kErrBadColumn);  // B column outside [0, N)
        const unsigned m = __match_any_sync(kFull, col) & gmask;
        const bool leader = valid && (lane == __ffs(m) - 1);

        if constexpr (!kNum) {
            const unsigned lb = __ballot_sync(kFull, leader) & gmask;
            if (active && q == 0) {
                g.c_rpt[r] = __popc(lb);
                nnz_acc += (unsigned long long)__popc(lb);
            }
        } else {
            const T o_av = shfl(av, lo + (lane & ~(G - 1)));
            const T bv = valid ? __ldg(g.bval + k) : T(0);
            S s = fold_group<T>(AccT::zero(), leader ? m : 0u, o_av, bv);
            int rank = 0;
#pragma unroll
            for (int t = 0; t < G; ++t) {
                const int ct = __shfl_sync(kFull, col, t, G);
                const int lt = __shfl_sync(kFull, (int)leader, t, G);
                rank += (lt && ct < col) ? 1 : 0;
            }
            if (g.soff) {  // one-pass: staging slot of the row, count as symbolic
                if (leader) {
                    const int pos = __ldg(g.soff + r) + rank;
                    g.c_col[pos] = col;
                    g.c_val[pos] = AccT::fin(s);
                }
                const unsigned lb = __ballot_sync(kFull, leader) & gmask;
                if (active && q == 0) {
                    g.c_rpt[r] = __popc(lb);
                    nnz_acc += (unsigned long long)__popc(lb);
                }
            } else if (leader) {
                const int pos = __ldg(g.c_rpt + r) + rank;
                g.c_col[pos] = col;
                g.c_val[pos] = AccT::fin(s);
            }
        }
    }
    if (!kNum || g.soff) warp_add_u64(nnz_acc, &g.info->total_nnz);
}

// Takes a class list's rows out of a one-pass call's staging (their staged product counts
// to zero, before the counts are scanned into offsets).
static __global__ void k_unstage_rows(const int *__restrict__ list, const int *count_ptr, int *soff)
{
    const int count = *count_ptr;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) soff[list[i]] = 0;
}

// Moves the staged rows of a one-pass call into C.  Row r was staged if soff[r + 1] >
// soff[r] (its staging slot holds up to its product count); its c_rpt[r + 1] - c_rpt[r]
// entries go to C from c_rpt[r] on.  C's entries are cut into ranges of kPlaceRange; a
// warp finds the row holding its range's first entry by a 32-way search of c_rpt (four
// rounds of one load per lane for a million rows), then takes 32 rows at a time and walks
// the concatenation of their entries inside the range, each lane locating its entry's row
// by a binary search over the warp's prefix of counts, kPlaceUnroll chunks' loads in
// flight together.  Every warp copies about the same number of entries, however the row
// lengths are spread; C is written contiguously and the staging area read almost so (its
// slots follow row order).
constexpr int kPlaceUnroll = 8;
constexpr int kPlaceRange = 1024;

template <typename T>
__global__ void __launch_bounds__(256) k_place_staged(int M, const int *__restrict__ soff,
                                                      const int *__restrict__ c_rpt, const int *__restrict__ scol,
                                                      const T *__restrict__ sval, int *__restrict__ c_col,
                                                      T *__restrict__ c_val)
{
    const int lane = lane_id();
    const long long warp0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    const int nnz = __ldg(c_rpt + M);
    for (long long q = warp0; q * kPlaceRange < nnz; q += nwarps) {
        const int p0 = (int)(q * kPlaceRange);
        const int p1 = min(nnz, p0 + kPlaceRange);
        // row of entry p0: c_rpt[lo] <= p0 < c_rpt[hi]
        int lo = 0, hi = M;
        while (hi - lo > 1) {
            const int step = (hi - lo + 31) / 32;
            const long long idx = (long long)lo + (long long)(lane + 1) * step;
            const int v = idx < hi ? __ldg(c_rpt + idx) : INT_MAX;
            const int k = __popc(__ballot_sync(kFull, v <= p0));
            const int nlo = lo + k * step;
            hi = (int)min((long long)hi, (long long)nlo + step);
            lo = nlo;
        }
        for (int r0 = lo; r0 < M; r0 += 32) {
            const int r = r0 + lane;
            int so = 0, o = 0, o1 = 0, n = 0, src0 = 0, dst0 = 0;
            if (r < M) {  // the row's four words are loaded together
                so = __ldg(soff + r);
                const int so1 = __ldg(soff + r + 1);
                o = __ldg(c_rpt + r);
                o1 = __ldg(c_rpt + r + 1);
                const int e0 = max(o, p0), e1 = min(o1, p1);
                if (so1 > so && e1 > e0) {
                    n = e1 - e0;
                    src0 = so + (e0 - o);
                    dst0 = e0;
                }
            }
            int incl = n;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int t = __shfl_up_sync(kFull, incl, d);
                if (lane >= d) incl += t;
            }
            const int total = __shfl_sync(kFull, incl, 31);
            for (int base = 0; base < total; base += 32 * kPlaceUnroll) {
                int src[kPlaceUnroll], dst[kPlaceUnroll];
#pragma unroll
                for (int u = 0; u < kPlaceUnroll; ++u) {
                    const int e = base + u * 32 + lane;
                    int l = 0;  // lanes whose entries end at or before e
#pragma unroll
                    for (int step = 16; step >= 1; step >>= 1) {
                        const int v = __shfl_sync(kFull, incl, l + step - 1);
                        if (v <= e) l += step;
                    }
                    l = min(l, 31);
                    const int first = __shfl_sync(kFull, incl, l) - __shfl_sync(kFull, n, l);
                    const int s0 = __shfl_sync(kFull, src0, l);
                    const int d0 = __shfl_sync(kFull, dst0, l);
                    src[u] = e < total ? s0 + (e - first) : -1;
                    dst[u] = d0 + (e - first);
                }
                int cv[kPlaceUnroll];
                T vv[kPlaceUnroll];
#pragma unroll
                for (int u = 0; u < kPlaceUnroll; ++u) {
                    cv[u] = src[u] >= 0 ? __ldg(scol + src[u]) : 0;
                    vv[u] = src[u] >= 0 ? __ldg(sval + src[u]) : T(0);
                }
#pragma unroll
                for (int u = 0; u < kPlaceUnroll; ++u) {
                    if (src[u] >= 0) {
                        c_col[dst[u]] = cv[u];
                        c_val[dst[u]] = vv[u];
                    }
                }
            }
            // done once this window of rows reaches the end of the range
            if (__shfl_sync(kFull, r < M ? o1 : INT_MAX, 31) >= p1) break;
        }
    }
}

// ==================================================================================
// Warp-per-row hash kernel (W class, and E1 rows whose outputs are few): one warp per
// row, open-addressing table of nextpow2(2*n) <= TMAX slots in shared memory (n = flop in
// symbolic, nnz in numeric).  The row count is read from device memory (count_ptr) so
// lists split on the device need no host round trip.  Products are visited
// in j-major chunks of 32 by warp_products; within a chunk, match groups are folded by
// their leader, and chunks are separated by __syncwarp, so each slot sees its
// contributions in ascending j.  Numeric then compacts the table and places each entry
// at its rank among the row's columns.
// ==================================================================================
// Writes the n compacted (column, value) entries of a warp-hash row to C in column order:
// keys (column << 8 | slot) are sorted in registers by the warp bitonic network.
template <int PER, typename T, typename KT>
__device__ __forceinline__ void warp_table_sort_write(const SpgemmArgs<T> &g, const int *keys,
                                                      const typename Acc<T>::S *vals, int n, int off)
{
    const int lane = lane_id();
    KT x[PER];
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = i * 32 + lane;  // any arrangement will do: the network sorts it
        x[i] = e < n ? (((KT)(unsigned)keys[e] << 8) | (KT)(unsigned)e) : ~KT(0);
    }
    warp_bitonic_blocked<PER, KT>(x);
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = lane * PER + i;
        if (e < n) {
            g.c_col[off + e] = (int)(x[i] >> 8);
            g.c_val[off + e] = Acc<T>::fin(vals[x[i] & 255u]);
        }
    }
}

constexpr int kWarpRowsThreads = 256;
constexpr int kCountUnroll = 4;  // symbolic: chunks whose column loads are issued together

// Column-window rows (symbolic): a row whose products all fall within kWinBits consecutive
// columns (banded and stencil matrices) is counted over a bitmap of that window instead of
// a hash table.  Marking a column is one shared-memory OR whose result nobody waits for
// (no probing, no dependent second access); the row's words are then swept once to count
// the set bits and clear them, so the bitmap is all-zero between window rows.
constexpr int kWinWords = kWinBits / 32;

template <bool kNum, typename T, int TMAX>
constexpr size_t warp_rows_per_warp()
{
    constexpr size_t hash = (size_t)TMAX * (sizeof(int) + (kNum ? sizeof(typename Acc<T>::S) : 0));
    constexpr size_t win = kNum ? 0 : (size_t)kWinWords * 4;
    return hash > win ? hash : win;
}

template <bool kNum, typename T, int TMAX>
constexpr size_t warp_rows_smem()
{
    return (size_t)(kWarpRowsThreads / 32) * warp_rows_per_warp<kNum, T, TMAX>();
}

// Column window of a row whose B rows are long: [cmin, cmax] from the first and last
// column of each B row (B rows are sorted).  cmax < cmin when the row has no products.
template <typename T>
__device__ __forceinline__ void row_window(const SpgemmArgs<T> &g, int a0, int a1, int &cmin, int &cmax)
{
    const int lane = lane_id();
    cmin = INT_MAX;
    cmax = -1;
    for (int wa = a0; wa < a1; wa += 32) {
        const int q = wa + lane;
        if (q < a1) {
            const int j = __ldg(g.acol + q);
            const int b0 = __ldg(g.brpt + j), b1 = __ldg(g.brpt + j + 1);
            if (b1 > b0) {
                cmin = min(cmin, __ldg(g.bcol + b0));
                cmax = max(cmax, __ldg(g.bcol + b1 - 1));
            }
        }
    }
    cmin = __reduce_min_sync(kFull, cmin);
    cmax = __reduce_max_sync(kFull, cmax);
}

// Sets the bits of the row's columns (offsets from cmin, at most span).  Returns true on
// every lane if a column fell outside [cmin, cmin + span] (a B row out of order).
template <typename T>
// Counting needs no order, so each lane walks whole B rows of its own (one per A entry,
// four columns' loads in flight), with no per-row broadcast of the B row's extent.
__device__ __forceinline__ bool window_mark(const SpgemmArgs<T> &g, int a0, int a1, int cmin, int span,
                                            unsigned *bits)
{
    const int lane = lane_id();
    bool bad = false;
    for (int q = a0 + lane; q < a1; q += 32) {
        const int j = __ldg(g.acol + q);
        const int b1 = __ldg(g.brpt + j + 1);
        for (int p = __ldg(g.brpt + j); p < b1; p += 4) {
            int col[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) col[u] = p + u < b1 ? __ldg(g.bcol + p + u) : 0;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (p + u >= b1) break;
                const int o = col[u] - cmin;
                if ((unsigned)o <= (unsigned)span) atomicOr(bits + (o >> 5), 1u << (o & 31));
                else bad = true;
            }
        }
    }
    __syncwarp();
    return __any_sync(kFull, bad);
}

// Counts the set bits of bitmap words [0, nw) and clears them, four words (one 16-byte
// shared access) per lane step.  Words past nw up to the next multiple of four are zero
// (never marked), and nw <= kWinWords, a multiple of four.  Returns the count on every lane.
__device__ __forceinline__ int window_sweep(unsigned *bits, int nw)
{
    uint4 *b4 = reinterpret_cast<uint4 *>(bits);
    int cnt = 0;
    for (int w = lane_id(); w < (nw + 3) >> 2; w += 32) {
        const uint4 x = b4[w];
        cnt += __popc(x.x) + __popc(x.y) + __popc(x.z) + __popc(x.w);
        b4[w] = make_uint4(0u, 0u, 0u, 0u);
    }
    return (int)__reduce_add_sync(kFull, (unsigned)cnt);
}

__device__ __forceinline__ void window_store_count(int *c_rpt, int r, int total, unsigned long long &nnz_acc)
{
    if (lane_id() == 0) {
        c_rpt[r] = total;
        nnz_acc += (unsigned long long)total;
    }
    __syncwarp();
}

// Distinct-column count of one window row, written to c_rpt[r].  All lanes call it.
template <typename T>
__device__ __forceinline__ void window_count_row(const SpgemmArgs<T> &g, int r, int a0, int a1, int cmin, int cmax,
                                                 unsigned *bits, unsigned long long &nnz_acc)
{
    const bool bad = window_mark<T>(g, a0, a1, cmin, cmax - cmin, bits) || cmin < 0 || cmax >= g.N;
    if (bad && lane_id() == 0) atomicOr(&g.info->flags, kErrBadColumn);
    window_store_count(g.c_rpt, r, window_sweep(bits, ((cmax - cmin) >> 5) + 1), nnz_acc);
}

// B-row quads (16-byte loads) a lane has in flight in the short-row window count.
constexpr int kWinQuads = 8;

// Marks the columns of one batch of a lane's B row: quads v[u] hold columns q0 + 4u .. +3;
// those below b0 (first quad only, lo = b0 - q0) or from b1 on are not the row's.
__device__ __forceinline__ void window_mark_quads(const int4 (&v)[kWinQuads], int q0, int lo, int b1, int cmin,
                                                  unsigned span, unsigned *bits, bool &bad)
{
#pragma unroll
    for (int u = 0; u < kWinQuads; ++u) {
        const int e[4] = {v[u].x, v[u].y, v[u].z, v[u].w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if ((u != 0 || k >= lo) && q0 + 4 * u + k < b1) {
                const unsigned o = (unsigned)(e[k] - cmin);
                if (o <= span) atomicOr(bits + (o >> 5), 1u << (o & 31));
                else bad = true;
            }
        }
    }
}

// Loads one batch of a lane's B row: the quads at q0, q0 + 4, ... that start before b1.
// vec: 16-byte loads (B's column array is 16-byte aligned and the lane's last quad ends
// inside it); otherwise the row's columns one by one.
__device__ __forceinline__ void window_load_quads(const int *__restrict__ bcol, int q0, int b0, int b1, bool vec,
                                                  int4 (&v)[kWinQuads])
{
#pragma unroll
    for (int u = 0; u < kWinQuads; ++u) {
        const int q = q0 + 4 * u;
        if (q < b1) {
            if (vec) {
                v[u] = __ldg(reinterpret_cast<const int4 *>(bcol + q));
            } else {
                v[u].x = q >= b0 ? __ldg(bcol + q) : 0;
                v[u].y = q + 1 >= b0 && q + 1 < b1 ? __ldg(bcol + q + 1) : 0;
                v[u].z = q + 2 >= b0 && q + 2 < b1 ? __ldg(bcol + q + 2) : 0;
                v[u].w = q + 3 < b1 ? __ldg(bcol + q + 3) : 0;
            }
        }
    }
}

// Column-window count of a row with at most 32 A entries, a lane per A entry.  The lane's
// B row is read as 16-byte quads, up to kWinQuads in flight, issued together with the
// loads of its first and last column that give the window: a stencil row (B rows of 27
// columns) takes three dependent round trips to L2 (A's column, B's row extent, B's
// columns), where finding the window before reading the B rows takes at least four.
// Returns false, having marked nothing, when the products do not fit a window of WBITS
// columns (bits holds WBITS / 32 words).
template <typename T, int WBITS = kWinBits>
__device__ __forceinline__ bool window_row_short(const SpgemmArgs<T> &g, int r, int a0, int a1, int nnz_b,
                                                 bool bcol16, unsigned *bits, bool &clean,
                                                 unsigned long long &nnz_acc)
{
    static_assert(WBITS % 128 == 0, "whole 16-byte sweep steps");
    const int lane = lane_id();
    int b0 = 0, b1 = 0;
    if (a0 + lane < a1) {
        const int j = __ldg(g.acol + a0 + lane);
        b0 = __ldg(g.brpt + j);
        b1 = __ldg(g.brpt + j + 1);
    }
    const int q0 = b0 & ~3;
    const bool vec = bcol16 && ((b1 + 3) & ~3) <= nnz_b;
    int4 v[kWinQuads];
    window_load_quads(g.bcol, q0, b0, b1, vec, v);
    const int cmin = __reduce_min_sync(kFull, b1 > b0 ? __ldg(g.bcol + b0) : INT_MAX);
    const int cmax = __reduce_max_sync(kFull, b1 > b0 ? __ldg(g.bcol + b1 - 1) : -1);
    if (!(cmax >= cmin && cmax - cmin < WBITS)) return false;
    if (!clean) {
        for (int i = lane; i < WBITS / 32; i += 32) bits[i] = 0u;
        __syncwarp();
        clean = true;
    }
    const unsigned span = (unsigned)(cmax - cmin);
    bool bad = cmin < 0 || cmax >= g.N;
    window_mark_quads(v, q0, b0 - q0, b1, cmin, span, bits, bad);
    for (int q = q0 + 4 * kWinQuads; q < b1; q += 4 * kWinQuads) {
        window_load_quads(g.bcol, q, b0, b1, vec, v);
        window_mark_quads(v, q, 0, b1, cmin, span, bits, bad);
    }
    __syncwarp();
    if (__any_sync(kFull, bad) && lane == 0) atomicOr(&g.info->flags, kErrBadColumn);
    window_store_count(g.c_rpt, r, window_sweep(bits, (int)(span >> 5) + 1), nnz_acc);
    return true;
}

template <bool kNum, typename T, int TMAX>
__global__ void __launch_bounds__(kWarpRowsThreads) k_warp_rows(SpgemmArgs<T> g, const int *__restrict__ list,
                                                                const int *count_ptr)
{
    using AccT = Acc<T>;
    using S = typename AccT::S;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = lane_id();
    const int warp = threadIdx.x >> 5;
    const int count = *count_ptr;
    unsigned char *wbase = smem_raw + (size_t)warp * warp_rows_per_warp<kNum, T, TMAX>();
    S *vals = reinterpret_cast<S *>(wbase);
    int *keys = reinterpret_cast<int *>(wbase + (kNum ? sizeof(S) * TMAX : 0));
    unsigned *wbits = reinterpret_cast<unsigned *>(wbase);  // window layout (symbolic)
    bool win_clean = false;  // the window bitmap is all-zero (no hash row has used the space since)
    const long long warp0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    unsigned long long nnz_acc = 0;
    int nnz_b = 0;
    bool bcol16 = false;
    if constexpr (!kNum) {
        nnz_b = __ldg(g.brpt + g.K);
        bcol16 = ((size_t)g.bcol & 15) == 0;
    }

    // the next row's number is loaded a row ahead
    int r = warp0 < count ? __ldg(list + warp0) : 0, r_next = 0;
    for (long long it = warp0; it < count; it += nwarps, r = r_next) {
        r_next = it + nwarps < count ? __ldg(list + it + nwarps) : 0;
        const int a0 = __ldg(g.arpt + r);
        const int a1 = __ldg(g.arpt + r + 1);
        int n_expect = 0, off = 0;
        if constexpr (kNum) {
            off = __ldg(g.c_rpt + r);
            n_expect = __ldg(g.c_rpt + r + 1) - off;
        } else {
            n_expect = __ldg(g.row_flop + r);
        }
        // numeric knows the row's output count: hash_slots (default 4) slots per output
        // where the table has room (fewer probe collisions), at least 2
        const int log_ts = kNum ? min(ceil_log2_c(TMAX), max(5, ceil_log2((g.hash_slots ? g.hash_slots : 4) *
                                                                           max(n_expect, 1))))
                                : max(5, ceil_log2(2 * max(n_expect, 1)));
        const int row_products = kNum ? __ldg(g.row_flop + r) : n_expect;
        const bool rowwise = row_products >= 16 * (a1 - a0);
        if (!kNum && rowwise && a1 - a0 <= 32) {
            // long B rows: do all the products fit a window of kWinBits columns?
            if (window_row_short<T>(g, r, a0, a1, nnz_b, bcol16, wbits, win_clean, nnz_acc)) continue;
        } else if (!kNum && rowwise) {
            int cmin, cmax;
            row_window<T>(g, a0, a1, cmin, cmax);
            if (cmax >= cmin && cmax - cmin < kWinBits) {
                if (!win_clean) {
                    for (int i = lane; i < kWinWords; i += 32) wbits[i] = 0u;
                    __syncwarp();
                    win_clean = true;
                }
                window_count_row<T>(g, r, a0, a1, cmin, cmax, wbits, nnz_acc);
                continue;
            }
        }
        win_clean = false;  // the hash table below reuses the space
        for (int i = lane; i < (1 << log_ts); i += 32) {
            keys[i] = kEmpty;
            if constexpr (kNum) vals[i] = AccT::zero();
        }
        __syncwarp();
        int cnt = 0;
        if constexpr (!kNum) {
            // counting is order-free: kUnroll chunks of 32 products have their column
            // loads in flight together before the claims
            for (int wa = a0; wa < a1; wa += 32) {
                const int q = wa + lane;
                int b0 = 0, bl = 0;
                if (q < a1) {
                    const int j = __ldg(g.acol + q);
                    b0 = __ldg(g.brpt + j);
                    bl = __ldg(g.brpt + j + 1) - b0;
                }
                int incl = bl;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const int t = __shfl_up_sync(kFull, incl, d);
                    if (lane >= d) incl += t;
                }
                const int wtot = __shfl_sync(kFull, incl, 31);
                for (int c = 0; c < wtot; c += 32 * kCountUnroll) {
                    int col[kCountUnroll];
#pragma unroll
                    for (int u = 0; u < kCountUnroll; ++u) {
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
                        col[u] = p < wtot ? __ldg(g.bcol + o_b0 + (p - (o_incl - o_bl))) : kEmpty;
                    }
#pragma unroll
                    for (int u = 0; u < kCountUnroll; ++u) {
                        if (col[u] == kEmpty) continue;
                        bool is_new = false;
                        table_claim(keys, col[u], log_ts, &is_new, &g.info->flags);
                        cnt += is_new ? 1 : 0;
                    }
                }
            }
        } else if (rowwise) {
            // long B rows: one B row per step, every lane owns a distinct key; four
            // B rows' operands are loaded ahead of their steps
            warp_rowwise_products_pf<4, kNum, T>(a0, a1, g.acol, g.aval, g.brpt, g.bcol, g.bval,
                                                 [&](bool valid, int col, T bv, T av) {
                                                     if (valid) {
                                                         bool is_new = false;
                                                         const int slot =
                                                             table_claim(keys, col, log_ts, &is_new, &g.info->flags);
                                                         cnt += is_new ? 1 : 0;
                                                         if constexpr (kNum) {
                                                             if (slot >= 0) vals[slot] = AccT::step(vals[slot], av, bv);
                                                         }
                                                     }
                                                     __syncwarp();
                                                 });
        } else
        warp_products<kNum, T>(a0, a1, 32, g.acol, g.aval, g.brpt, [&](bool valid, int k, T av, int) {
            const int col = valid ? __ldg(g.bcol + k) : kEmpty;
            const unsigned m = __match_any_sync(kFull, col);
            const bool leader = valid && (lane == __ffs(m) - 1);
            int slot = -1;
            if (leader) {
                bool is_new = false;
                slot = table_claim(keys, col, log_ts, &is_new, &g.info->flags);
                cnt += is_new ? 1 : 0;
            }
            if constexpr (kNum) {
                const T bv = valid ? __ldg(g.bval + k) : T(0);
                S s = slot >= 0 ? vals[slot] : AccT::zero();
                s = fold_group<T>(s, slot >= 0 ? m : 0u, av, bv);
                if (slot >= 0) vals[slot] = s;
            }
            __syncwarp();
        });
        if constexpr (!kNum) {
            const int tot = (int)__reduce_add_sync(kFull, (unsigned)cnt);
            if (lane == 0) {
                g.c_rpt[r] = tot;
                nnz_acc += (unsigned long long)tot;
            }
        } else {
            // In-place compaction: block b of 32 slots writes to positions < 32*(b+1).
            int n = 0;
            for (int base = 0; base < (1 << log_ts); base += 32) {
                const int kk = keys[base + lane];
                const S vv = vals[base + lane];
                const bool occ = kk != kEmpty;
                const unsigned bal = __ballot_sync(kFull, occ);
                __syncwarp();
                if (occ) {
                    const int pos = n + __popc(bal & lanemask_lt());
                    keys[pos] = kk;
                    vals[pos] = vv;
                }
                n += __popc(bal);
                __syncwarp();
            }
            if (n != n_expect && lane == 0) atomicOr(&g.info->flags, kErrCountMismatch);
            const int nw = min(n, n_expect);
            if (nw <= 32) {  // rank among at most 32 keys
                for (int e = lane; e < nw; e += 32) {
                    const int ke = keys[e];
                    int rank = 0;
                    for (int t = 0; t < nw; ++t) rank += keys[t] < ke ? 1 : 0;
                    g.c_col[off + rank] = ke;
                    g.c_val[off + rank] = AccT::fin(vals[e]);
                }
            } else if (g.N <= (1 << 24)) {  // (column << 8 | slot) fits 32 bits
                if (nw <= 128)
                    warp_table_sort_write<4, T, unsigned>(g, keys, vals, nw, off);
                else if (nw <= 256)
                    warp_table_sort_write<8, T, unsigned>(g, keys, vals, nw, off);
            } else if (nw <= 128) {
                warp_table_sort_write<4, T, unsigned long long>(g, keys, vals, nw, off);
            } else if (nw <= 256) {
                warp_table_sort_write<8, T, unsigned long long>(g, keys, vals, nw, off);
            } else {  // not reached: numeric rows here have at most TMAX/2 outputs
                if (lane == 0) atomicOr(&g.info->flags, kErrCountMismatch);
            }
            __syncwarp();
        }
    }
    if constexpr (!kNum) warp_add_u64(nnz_acc, &g.info->total_nnz);
}

// ==================================================================================
// CTA-chunk walk of a row's products in j-major order, used by the D numeric kernel.  A windows of NT entries are scanned block-wide; the window's products are
// processed NT at a time (thread t holds product c+t).  `claim(valid, col, leader,
// lane_members)` runs in parallel; then the warps apply their match groups one warp at
// a time (warp 0 first), so contributions from different warps reach a slot in
// ascending j.  `apply(warp-converged)` is called by the active warp only.
// Loop trip counts depend only on block-uniform values, so every thread reaches every
// barrier.
// ==================================================================================
template <int NT, typename T>
struct ChunkSmem {
    int incl[NT];
    int b0[NT];
    T av[NT];
    int warp_sums[32];
};

template <int NT, typename T, typename FClaim, typename FApply>
__device__ __forceinline__ void block_products_ordered(int a0, int a1, const SpgemmArgs<T> &g, ChunkSmem<NT, T> &cs,
                                                       FClaim &&claim, FApply &&apply)
{
    const int tid = threadIdx.x;
    const int lane = lane_id();
    const int warp = tid >> 5;
    constexpr int kWarps = NT / 32;
    for (int wa = a0; wa < a1; wa += NT) {
        const int q = wa + tid;
        int b0 = 0, bl = 0;
        T av = T(0);
        if (q < a1) {
            const int j = __ldg(g.acol + q);
            b0 = __ldg(g.brpt + j);
            bl = __ldg(g.brpt + j + 1) - b0;
            av = __ldg(g.aval + q);
        }
        int wtot = 0;
        const int incl = block_inclusive_scan(bl, cs.warp_sums, &wtot);
        cs.incl[tid] = incl;
        cs.b0[tid] = b0;
        cs.av[tid] = av;
        __syncthreads();
        for (unsigned c = 0; c < (unsigned)wtot; c += NT) {
            const int p = (int)(c + tid);
            const bool valid = (unsigned)p < (unsigned)wtot;
            int lo = 0;
#pragma unroll
            for (int step = NT / 2; step >= 1; step >>= 1) {
                if (cs.incl[lo + step - 1] <= p) lo += step;
            }
            const int o_excl = lo ? cs.incl[lo - 1] : 0;
            const int k = cs.b0[lo] + (p - o_excl);
            const T oav = cs.av[lo];
            const int col = valid ? __ldg(g.bcol + k) : kEmpty;
            const T bv = valid ? __ldg(g.bval + k) : T(0);
            const unsigned m = __match_any_sync(kFull, col);
            const bool leader = valid && (lane == __ffs(m) - 1);
            const int slot = claim(valid, col, leader);
            for (int w = 0; w < kWarps; ++w) {
                __syncthreads();
                if (warp == w) apply(slot, slot >= 0 ? m : 0u, oav, bv);
            }
        }
        __syncthreads();
    }
}

// ==================================================================================
// D class: one CTA (512 threads) per row, dense accumulator over all N columns plus a
// bitmap, both private to the CTA and kept all-zero between rows (each row clears what
// it touched).  Symbolic: atomicOr on the bitmap counts first insertions.  Numeric:
// ordered CTA-chunk walk into vals[col]; then the bitmap words between the row's
// smallest and largest column are split into contiguous per-thread pieces, counted,
// scanned and walked in order, which emits ascending columns with no sort.  Rows of more
// than kBlockFoldMin A entries first count each column's products (cnt); the walk folds
// an entry of more than kBlockFoldMin products in blocks (vals = the current block,
// tot = the merged earlier blocks, pos = products folded), as every other path does.
// ==================================================================================
constexpr int kDenseRowsThreads = 512;

template <typename T>
struct DenseScratch {
    typename Acc<T>::S *vals;  // gridDim.x * N
    unsigned *bits;            // gridDim.x * words
    typename Acc<T>::S *tot;   // gridDim.x * N: merged earlier blocks of a blocked entry
    int *cnt;                  // gridDim.x * N: products per column (rows of long entries)
    int *pos;                  // gridDim.x * N: products of a blocked entry folded so far
    int words;                 // ceil(N / 32)
};

template <bool kNum, typename T>
__global__ void __launch_bounds__(kDenseRowsThreads) k_dense_rows(SpgemmArgs<T> g, const int *__restrict__ list,
                                                                  int count, DenseScratch<T> ds)
{
    using AccT = Acc<T>;
    using S = typename AccT::S;
    constexpr int NT = kDenseRowsThreads;
    __shared__ ChunkSmem<NT, T> cs;
    __shared__ int s_red[3][32];
    const int tid = threadIdx.x;
    const int lane = lane_id();
    const int warp = tid >> 5;
    constexpr int kWarps = NT / 32;
    S *vals = ds.vals + (size_t)blockIdx.x * (size_t)g.N;
    unsigned *bits = ds.bits + (size_t)blockIdx.x * (size_t)ds.words;
    S *totc = ds.tot + (size_t)blockIdx.x * (size_t)g.N;
    int *cntc = ds.cnt + (size_t)blockIdx.x * (size_t)g.N;
    int *posc = ds.pos + (size_t)blockIdx.x * (size_t)g.N;
    const unsigned N = (unsigned)g.N;
    unsigned long long nnz_acc = 0;

    for (int it = blockIdx.x; it < count; it += gridDim.x) {
        const int r = __ldg(list + it);
        const int a0 = __ldg(g.arpt + r);
        const int a1 = __ldg(g.arpt + r + 1);
        int cnt = 0, kmin = INT_MAX, kmax = -1;
        if constexpr (!kNum) {
            warp_products<false, T>(a0 + warp * 32, a1, NT, g.acol, g.aval, g.brpt, [&](bool valid, int k, T, int) {
                if (valid) {
                    const int col = __ldg(g.bcol + k);
                    if ((unsigned)col < N) {
                        const unsigned bit = 1u << (col & 31);
                        const unsigned old = atomicOr(bits + (col >> 5), bit);
                        cnt += (old & bit) ? 0 : 1;
                        kmin = min(kmin, col);
                        kmax = max(kmax, col);
                    } else {
                        atomicOr(&g.info->flags, kErrBadColumn);
                    }
                }
            });
        } else {
            const bool long_row = a1 - a0 > kBlockFoldMin;  // may hold entries folded in blocks
            if (long_row) {
                warp_products<false, T>(a0 + warp * 32, a1, NT, g.acol, g.aval, g.brpt, [&](bool valid, int k, T, int) {
                    if (valid) {
                        const int col = __ldg(g.bcol + k);
                        if ((unsigned)col < N) atomicAdd(cntc + col, 1);
                    }
                });
                __syncthreads();
            }
            block_products_ordered<NT, T>(
                a0, a1, g, cs,
                [&](bool valid, int col, bool leader) -> int {
                    if (!leader) return -1;
                    if ((unsigned)col >= N) return -1;
                    atomicOr(bits + (col >> 5), 1u << (col & 31));
                    kmin = min(kmin, col);
                    kmax = max(kmax, col);
                    return col;
                },
                [&](int slot, unsigned members, T a, T b) {
                    if (!long_row) {
                        S s = slot >= 0 ? vals[slot] : AccT::zero();
                        s = fold_group<T>(s, members, a, b);
                        if (slot >= 0) vals[slot] = s;
                        return;
                    }
                    S cur = AccT::zero(), acc_tot = AccT::zero();
                    int pos = 0, c = 0;
                    if (slot >= 0) {
                        cur = vals[slot];
                        const int m = cntc[slot];
                        if (m > kBlockFoldMin) {
                            c = (m + kFoldBlocks - 1) / kFoldBlocks;
                            pos = posc[slot];
                            acc_tot = totc[slot];
                        }
                    }
                    fold_group_blocked<T>(cur, acc_tot, pos, c, members, a, b);
                    if (slot >= 0) {
                        vals[slot] = cur;
                        if (c) {
                            posc[slot] = pos;
                            totc[slot] = acc_tot;
                        }
                    }
                });
        }
        // Block reduction of (cnt, kmin, kmax).
        cnt = (int)__reduce_add_sync(kFull, (unsigned)cnt);
        kmin = __reduce_min_sync(kFull, kmin);
        kmax = __reduce_max_sync(kFull, kmax);
        if (lane == 0) {
            s_red[0][warp] = cnt;
            s_red[1][warp] = kmin;
            s_red[2][warp] = kmax;
        }
        __syncthreads();
        if (warp == 0) {
            int c = lane < kWarps ? s_red[0][lane] : 0;
            int lo = lane < kWarps ? s_red[1][lane] : INT_MAX;
            int hi = lane < kWarps ? s_red[2][lane] : -1;
            c = (int)__reduce_add_sync(kFull, (unsigned)c);
            lo = __reduce_min_sync(kFull, lo);
            hi = __reduce_max_sync(kFull, hi);
            if (lane == 0) {
                s_red[0][0] = c;
                s_red[1][0] = lo;
                s_red[2][0] = hi;
            }
        }
        __syncthreads();
        const int tot = s_red[0][0];
        const int lo = s_red[1][0], hi = s_red[2][0];
        const int w0 = hi >= 0 ? (lo >> 5) : 0;
        const int nwords = hi >= 0 ? (hi >> 5) - w0 + 1 : 0;
        if constexpr (!kNum) {
            if (tid == 0) {
                g.c_rpt[r] = tot;
                nnz_acc += (unsigned long long)tot;
            }
            for (int w = tid; w < nwords; w += NT) bits[w0 + w] = 0u;
            __syncthreads();
        } else {
            const int off = __ldg(g.c_rpt + r);
            const int n_expect = __ldg(g.c_rpt + r + 1) - off;
            const int per = (nwords + NT - 1) / NT;
            const int wb = min(nwords, tid * per);
            const int we = min(nwords, wb + per);
            int mine = 0;
            for (int w = wb; w < we; ++w) mine += __popc(bits[w0 + w]);
            int total = 0;
            const int incl = block_inclusive_scan(mine, cs.warp_sums, &total);
            if (tid == 0 && total != n_expect) atomicOr(&g.info->flags, kErrCountMismatch);
            int pos = incl - mine;
            const bool long_row = a1 - a0 > kBlockFoldMin;
            for (int w = wb; w < we; ++w) {
                unsigned word = bits[w0 + w];
                if (word) bits[w0 + w] = 0u;
                while (word) {
                    const int b = __ffs(word) - 1;
                    word &= word - 1u;
                    const int col = ((w0 + w) << 5) + b;
                    S v = vals[col];
                    if (long_row) {
                        if (cntc[col] > kBlockFoldMin) {  // the last block merged into the others
                            v = AccT::merge(totc[col], v);
                            totc[col] = AccT::zero();
                            posc[col] = 0;
                        }
                        cntc[col] = 0;
                    }
                    if (pos < n_expect) {
                        g.c_col[off + pos] = col;
                        g.c_val[off + pos] = AccT::fin(v);
                    }
                    vals[col] = AccT::zero();
                    ++pos;
                }
            }
            __syncthreads();
        }
    }
    if constexpr (!kNum) warp_add_u64(nnz_acc, &g.info->total_nnz);
}

}  // namespace opsg
