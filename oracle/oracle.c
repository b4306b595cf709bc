/*
 * oracle.c — CPU restatement of OpSparse's CSR SpGEMM C = A*B.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links, loads or calls this file:
 * it is the checker used by tests/, by __graft_entry__.smoke() and by the CPU
 * baseline leg of bench.py.
 *
 * What it restates (paths are relative to the OpSparse source tree):
 *  - orc_flop: the per-row intermediate-product count of
 *    src/opsparse/numeric/compute_flop.cu:33-52 (row_flop[i] = sum over j in A(i,:)
 *    of nnz(B(j,:)); total returned as 64-bit).
 *  - orc_symbolic: the distinct-column count per row that the symbolic hash
 *    kernels produce (include/opsparse/core_algo/spgemm/kernels/symbolic.cuh:9-325)
 *    followed by the exclusive scan into row_ptr (src/opsparse/core_algo/spgemm/spgemm.cu:49).
 *  - orc_spgemm_f64: the numeric result of kernels/numeric.cuh:9-393.  The structure of
 *    C is the structural union of the B rows selected by A's row (entries whose products
 *    cancel to 0.0 are kept, numeric.cuh:183-192), with ascending columns per row
 *    (the rank sort of numeric.cuh:196-204).  Each value is accumulated in a FIXED order:
 *    contributions in ascending j (A's column order), each folded in with one fused
 *    multiply-add, c = fma(a_ij, b_jk, c), starting from +0.0.  An entry with more than
 *    ORC_BLOCK_FOLD_MIN (2,560) contributions — possible only where A's row has more
 *    entries than that, since a B row holds a column once — is folded in ORC_BLOCKS (32)
 *    consecutive blocks of c = ceil(m / 32) of its m contributions, each block the same
 *    fma chain from +0.0, and the block sums added in block order,
 *    ((s_0 + s_1) + s_2) + ...  The reference itself adds in a run-dependent order
 *    (atomicAdd), so its values agree with this only to rounding; the GB300 library uses
 *    this exact order and is compared bit-for-bit.
 *  - orc_spgemm_f32: the same structure for FP32 values, each entry accumulated with the
 *    compensated dot product "Dot2" of Ogita, Rump and Oishi (Accurate Sum and Dot
 *    Product, SIAM J. Sci. Comput. 26(6), 2005): TwoProduct via fmaf, TwoSum, and a
 *    running compensation term, rounded to float once at the end.
 *  - orc_backward_f64: gradients of loss = sum(W .* C) on fixed patterns,
 *    dA_ij = sum_k B_jk dC_ik and dB_jk = sum_i A_ij dC_ik (no reference counterpart).
 *  - orc_omp_symbolic / orc_omp_numeric_f64: OpenMP row-wise Gustavson hash SpGEMM (two
 *    phases, per-thread open-addressing tables), the timed CPU baseline.  Same summation order as
 *    orc_spgemm_f64 (plain ascending j for every entry), so its output is bit-identical to
 *    it wherever no entry has more than ORC_BLOCK_FOLD_MIN contributions.
 *
 * Pinning: flop counts, structure and values are checked against the reference's own
 * kernels and host compute_flop, compiled from its sources and run on the CPU
 * (oracle/ref_emul/, through the golden fixtures tests/golden/*.npz that
 * tests/golden/make_golden.py made with them), and against the same kernels on the GPU
 * (oracle/ref_gpu/); also against an independent implementation (scipy.sparse) and the
 * known sizes of the Laplacian and 27-point configurations.
 *
 * Build: gcc -O2 -fopenmp -ffp-contract=off -shared -fPIC (oracle/Makefile).  Contraction
 * must stay off: every rounding step above is spelled out explicitly.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------- flop count ---- */
/* compute_flop.cu:33-52 — per-row product counts, 64-bit total. */
int64_t orc_flop(int32_t M, const int32_t *arpt, const int32_t *acol, const int32_t *brpt, int64_t *row_flop)
{
    int64_t total = 0;
#pragma omp parallel for reduction(+ : total) schedule(static)
    for (int32_t i = 0; i < M; i++) {
        int64_t s = 0;
        for (int32_t p = arpt[i]; p < arpt[i + 1]; p++) {
            const int32_t j = acol[p];
            s += (int64_t)(brpt[j + 1] - brpt[j]);
        }
        if (row_flop) row_flop[i] = s;
        total += s;
    }
    return total;
}

/* -------------------------------------------------------------- symbolic ---- */
/* Distinct columns per row (dense marker, one per thread); writes crpt[0..M] as the
 * exclusive scan and returns nnz(C) as 64-bit. */
int64_t orc_symbolic(int32_t M, int32_t N, const int32_t *arpt, const int32_t *acol, const int32_t *brpt,
                     const int32_t *bcol, int64_t *crpt)
{
    int64_t *cnt = (int64_t *)calloc((size_t)M + 1, sizeof(int64_t));
#pragma omp parallel
    {
        int32_t *mark = (int32_t *)malloc((size_t)(N > 0 ? N : 1) * sizeof(int32_t));
        for (int32_t k = 0; k < N; k++) mark[k] = -1;
#pragma omp for schedule(dynamic, 256)
        for (int32_t i = 0; i < M; i++) {
            int64_t c = 0;
            for (int32_t p = arpt[i]; p < arpt[i + 1]; p++) {
                const int32_t j = acol[p];
                for (int32_t q = brpt[j]; q < brpt[j + 1]; q++) {
                    const int32_t k = bcol[q];
                    if (mark[k] != i) {
                        mark[k] = i;
                        c++;
                    }
                }
            }
            cnt[i] = c;
        }
        free(mark);
    }
    int64_t run = 0;
    for (int32_t i = 0; i < M; i++) {
        crpt[i] = run;
        run += cnt[i];
    }
    crpt[M] = run;
    free(cnt);
    return run;
}

/* ------------------------------------------------------------ numeric f64 ---- */
static int cmp_i32(const void *a, const void *b)
{
    const int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

#define ORC_BLOCK_FOLD_MIN 2560 /* entries with more contributions fold in blocks */
#define ORC_BLOCKS 32

/* Block of contribution t (0-based) of an entry with m contributions. */
static inline int64_t orc_block_of(int64_t t, int64_t m)
{
    return t / ((m + ORC_BLOCKS - 1) / ORC_BLOCKS);
}

/* Per-thread scratch of the long-entry rows: contributions and block slot per column. */
typedef struct {
    int32_t *cnt, *slot, *pos;
} orc_long_scratch;

static orc_long_scratch orc_long_alloc(int32_t N)
{
    orc_long_scratch ls;
    const size_t n = (size_t)(N > 0 ? N : 1);
    ls.cnt = (int32_t *)malloc(n * sizeof(int32_t));
    ls.slot = (int32_t *)malloc(n * sizeof(int32_t));
    ls.pos = (int32_t *)malloc(n * sizeof(int32_t));
    return ls;
}

static void orc_long_free(orc_long_scratch *ls)
{
    free(ls->cnt);
    free(ls->slot);
    free(ls->pos);
}

/* Distinct columns of row i into cols (first-touch order) with their contribution counts;
 * entries with more than ORC_BLOCK_FOLD_MIN get consecutive slots.  Returns the number of
 * distinct columns; *nlong receives the number of slots. */
static int64_t orc_long_count(int32_t i, const int32_t *arpt, const int32_t *acol, const int32_t *brpt,
                              const int32_t *bcol, int32_t *mark, int32_t *cols, orc_long_scratch *ls,
                              int64_t *nlong)
{
    int64_t n = 0, nl = 0;
    for (int32_t p = arpt[i]; p < arpt[i + 1]; p++) {
        const int32_t j = acol[p];
        for (int32_t q = brpt[j]; q < brpt[j + 1]; q++) {
            const int32_t k = bcol[q];
            if (mark[k] != i) {
                mark[k] = i;
                ls->cnt[k] = 0;
                cols[n++] = k;
            }
            ls->cnt[k]++;
        }
    }
    for (int64_t t = 0; t < n; t++) {
        const int32_t k = cols[t];
        ls->pos[k] = 0;
        ls->slot[k] = ls->cnt[k] > ORC_BLOCK_FOLD_MIN ? (int32_t)nl++ : -1;
    }
    *nlong = nl;
    return n;
}

/* Fills ccol/cval given crpt from orc_symbolic.  Dense accumulator per thread; the
 * first touch of column k starts its sum at +0.0 and every contribution is folded in
 * with fma() in ascending j. */
void orc_spgemm_f64(int32_t M, int32_t N, const int32_t *arpt, const int32_t *acol, const double *aval,
                    const int32_t *brpt, const int32_t *bcol, const double *bval, const int64_t *crpt, int32_t *ccol,
                    double *cval)
{
#pragma omp parallel
    {
        int32_t *mark = (int32_t *)malloc((size_t)(N > 0 ? N : 1) * sizeof(int32_t));
        double *acc = (double *)malloc((size_t)(N > 0 ? N : 1) * sizeof(double));
        orc_long_scratch ls = orc_long_alloc(N);
        for (int32_t k = 0; k < N; k++) mark[k] = -1;
#pragma omp for schedule(dynamic, 256)
        for (int32_t i = 0; i < M; i++) {
            int64_t n = 0;
            int32_t *cols = ccol + crpt[i];
            if (arpt[i + 1] - arpt[i] > ORC_BLOCK_FOLD_MIN) {
                /* a row that may hold long entries: count first, then fold */
                int64_t nl = 0;
                n = orc_long_count(i, arpt, acol, brpt, bcol, mark, cols, &ls, &nl);
                double *part = (double *)calloc((size_t)(nl > 0 ? nl : 1) * ORC_BLOCKS, sizeof(double));
                for (int64_t t = 0; t < n; t++) acc[cols[t]] = 0.0;
                for (int32_t p = arpt[i]; p < arpt[i + 1]; p++) {
                    const int32_t j = acol[p];
                    const double a = aval[p];
                    for (int32_t q = brpt[j]; q < brpt[j + 1]; q++) {
                        const int32_t k = bcol[q];
                        if (ls.slot[k] >= 0) {
                            double *pb = part + (size_t)ls.slot[k] * ORC_BLOCKS + orc_block_of(ls.pos[k]++, ls.cnt[k]);
                            *pb = fma(a, bval[q], *pb);
                        } else {
                            acc[k] = fma(a, bval[q], acc[k]);
                        }
                    }
                }
                for (int64_t t = 0; t < n; t++) {
                    const int32_t k = cols[t];
                    if (ls.slot[k] < 0) continue;
                    const double *pb = part + (size_t)ls.slot[k] * ORC_BLOCKS;
                    double s = pb[0];
                    for (int b = 1; b < ORC_BLOCKS; b++) s = s + pb[b];
                    acc[k] = s;
                }
                free(part);
            } else {
                for (int32_t p = arpt[i]; p < arpt[i + 1]; p++) {
                    const int32_t j = acol[p];
                    const double a = aval[p];
                    for (int32_t q = brpt[j]; q < brpt[j + 1]; q++) {
                        const int32_t k = bcol[q];
                        if (mark[k] != i) {
                            mark[k] = i;
                            acc[k] = 0.0;
                            cols[n++] = k;
                        }
                        acc[k] = fma(a, bval[q], acc[k]);
                    }
                }
            }
            qsort(cols, (size_t)n, sizeof(int32_t), cmp_i32);
            for (int64_t t = 0; t < n; t++) cval[crpt[i] + t] = acc[cols[t]];
        }
        free(mark);
        free(acc);
        orc_long_free(&ls);
    }
}

/* ------------------------------------------------------------ numeric f32 ---- */
/* Dot2 state: s = running sum, c = running compensation. */
typedef struct {
    float s, c;
} dot2_t;

static inline dot2_t dot2_step(dot2_t st, float a, float b)
{
    const float h = a * b;           /* TwoProduct: h + r == a*b exactly */
    const float r = fmaf(a, b, -h);
    const float s = st.s + h;        /* TwoSum(st.s, h): s + q == st.s + h exactly */
    const float z = s - st.s;
    const float q = (st.s - (s - z)) + (h - z);
    dot2_t out;
    out.s = s;
    out.c = st.c + (q + r);
    return out;
}

/* Two Dot2 states of consecutive blocks combined: TwoSum of the sums, the compensations
 * added, then the TwoSum error. */
static inline dot2_t dot2_merge(dot2_t u, dot2_t v)
{
    const float s = u.s + v.s;
    const float z = s - u.s;
    const float q = (u.s - (s - z)) + (v.s - z);
    dot2_t out;
    out.s = s;
    out.c = (u.c + v.c) + q;
    return out;
}

void orc_spgemm_f32(int32_t M, int32_t N, const int32_t *arpt, const int32_t *acol, const float *aval,
                    const int32_t *brpt, const int32_t *bcol, const float *bval, const int64_t *crpt, int32_t *ccol,
                    float *cval)
{
#pragma omp parallel
    {
        int32_t *mark = (int32_t *)malloc((size_t)(N > 0 ? N : 1) * sizeof(int32_t));
        dot2_t *acc = (dot2_t *)malloc((size_t)(N > 0 ? N : 1) * sizeof(dot2_t));
        orc_long_scratch ls = orc_long_alloc(N);
        for (int32_t k = 0; k < N; k++) mark[k] = -1;
#pragma omp for schedule(dynamic, 256)
        for (int32_t i = 0; i < M; i++) {
            int64_t n = 0;
            int32_t *cols = ccol + crpt[i];
            if (arpt[i + 1] - arpt[i] > ORC_BLOCK_FOLD_MIN) {
                int64_t nl = 0;
                n = orc_long_count(i, arpt, acol, brpt, bcol, mark, cols, &ls, &nl);
                dot2_t *part = (dot2_t *)calloc((size_t)(nl > 0 ? nl : 1) * ORC_BLOCKS, sizeof(dot2_t));
                for (int64_t t = 0; t < n; t++) {
                    acc[cols[t]].s = 0.0f;
                    acc[cols[t]].c = 0.0f;
                }
                for (int32_t p = arpt[i]; p < arpt[i + 1]; p++) {
                    const int32_t j = acol[p];
                    const float a = aval[p];
                    for (int32_t q = brpt[j]; q < brpt[j + 1]; q++) {
                        const int32_t k = bcol[q];
                        if (ls.slot[k] >= 0) {
                            dot2_t *pb = part + (size_t)ls.slot[k] * ORC_BLOCKS + orc_block_of(ls.pos[k]++, ls.cnt[k]);
                            *pb = dot2_step(*pb, a, bval[q]);
                        } else {
                            acc[k] = dot2_step(acc[k], a, bval[q]);
                        }
                    }
                }
                for (int64_t t = 0; t < n; t++) {
                    const int32_t k = cols[t];
                    if (ls.slot[k] < 0) continue;
                    const dot2_t *pb = part + (size_t)ls.slot[k] * ORC_BLOCKS;
                    dot2_t st = pb[0];
                    for (int b = 1; b < ORC_BLOCKS; b++) st = dot2_merge(st, pb[b]);
                    acc[k] = st;
                }
                free(part);
            } else {
                for (int32_t p = arpt[i]; p < arpt[i + 1]; p++) {
                    const int32_t j = acol[p];
                    const float a = aval[p];
                    for (int32_t q = brpt[j]; q < brpt[j + 1]; q++) {
                        const int32_t k = bcol[q];
                        if (mark[k] != i) {
                            mark[k] = i;
                            acc[k].s = 0.0f;
                            acc[k].c = 0.0f;
                            cols[n++] = k;
                        }
                        acc[k] = dot2_step(acc[k], a, bval[q]);
                    }
                }
            }
            qsort(cols, (size_t)n, sizeof(int32_t), cmp_i32);
            for (int64_t t = 0; t < n; t++) cval[crpt[i] + t] = acc[cols[t]].s + acc[cols[t]].c;
        }
        free(mark);
        free(acc);
        orc_long_free(&ls);
    }
}

/* ------------------------------------------------------------- backward ---- */
/* dA_ij = sum_k B_jk dC_ik over A's pattern; dB_jk = sum_i A_ij dC_ik over B's pattern.
 * dC is given on C's pattern (ccol sorted per row).  dA is accumulated per A entry
 * in ascending k with fma; dB is accumulated in ascending (i, k) order. */
void orc_backward_f64(int32_t M, int32_t N, int32_t K, const int32_t *arpt, const int32_t *acol, const double *aval,
                      const int32_t *brpt, const int32_t *bcol, const double *bval, const int64_t *crpt,
                      const int32_t *ccol, const double *dcval, double *daval, double *dbval)
{
    (void)K;
    /* dA: row-parallel, dense scatter of dC row. */
#pragma omp parallel
    {
        double *dense = (double *)calloc((size_t)(N > 0 ? N : 1), sizeof(double));
#pragma omp for schedule(dynamic, 256)
        for (int32_t i = 0; i < M; i++) {
            for (int64_t t = crpt[i]; t < crpt[i + 1]; t++) dense[ccol[t]] = dcval[t];
            for (int32_t p = arpt[i]; p < arpt[i + 1]; p++) {
                const int32_t j = acol[p];
                double s = 0.0;
                for (int32_t q = brpt[j]; q < brpt[j + 1]; q++) s = fma(bval[q], dense[bcol[q]], s);
                daval[p] = s;
            }
            for (int64_t t = crpt[i]; t < crpt[i + 1]; t++) dense[ccol[t]] = 0.0;
        }
        free(dense);
    }
    /* dB: sequential over i, scatter-adding into B's entries through a dense copy of
     * row i of dC. */
    int64_t nnzb = brpt[K];
    for (int64_t q = 0; q < nnzb; q++) dbval[q] = 0.0;
    double *dense = (double *)calloc((size_t)(N > 0 ? N : 1), sizeof(double));
    for (int32_t i = 0; i < M; i++) {
        for (int64_t t = crpt[i]; t < crpt[i + 1]; t++) dense[ccol[t]] = dcval[t];
        for (int32_t p = arpt[i]; p < arpt[i + 1]; p++) {
            const int32_t j = acol[p];
            const double a = aval[p];
            for (int32_t q = brpt[j]; q < brpt[j + 1]; q++) dbval[q] = fma(a, dense[bcol[q]], dbval[q]);
        }
        for (int64_t t = crpt[i]; t < crpt[i + 1]; t++) dense[ccol[t]] = 0.0;
    }
    free(dense);
}

/* ------------------------------------------------ OpenMP hash Gustavson ---- */
/* Row-wise Gustavson with open-addressing hash tables (one per thread), two phases:
 * symbolic count -> scan -> numeric accumulate + per-row sort.  Returns nnz(C).
 * orc_omp_symbolic then orc_omp_numeric_f64. */
static inline uint32_t orc_hash(uint32_t k) { return k * 2654435761u; }

static inline int64_t next_pow2(int64_t x)
{
    int64_t p = 16;
    while (p < x) p <<= 1;
    return p;
}

/* Symbolic phase: distinct columns per row through a per-thread hash table sized to
 * the row's product count; writes crpt[0..M] (exclusive scan) and returns nnz(C). */
int64_t orc_omp_symbolic(int32_t M, const int32_t *arpt, const int32_t *acol, const int32_t *brpt,
                         const int32_t *bcol, int64_t *crpt)
{
    int64_t maxflop = 0;
#pragma omp parallel for reduction(max : maxflop) schedule(static)
    for (int32_t i = 0; i < M; i++) {
        int64_t s = 0;
        for (int32_t p = arpt[i]; p < arpt[i + 1]; p++) s += brpt[acol[p] + 1] - brpt[acol[p]];
        crpt[i] = s; /* flop, replaced by the count below */
        if (s > maxflop) maxflop = s;
    }
    const int64_t tmax = next_pow2(2 * maxflop);
#pragma omp parallel
    {
        int32_t *keys = (int32_t *)malloc((size_t)tmax * sizeof(int32_t));
#pragma omp for schedule(dynamic, 64)
        for (int32_t i = 0; i < M; i++) {
            const int64_t ts = next_pow2(2 * crpt[i]);
            const uint32_t mask = (uint32_t)(ts - 1);
            for (int64_t t = 0; t < ts; t++) keys[t] = -1;
            int64_t c = 0;
            for (int32_t p = arpt[i]; p < arpt[i + 1]; p++) {
                const int32_t j = acol[p];
                for (int32_t q = brpt[j]; q < brpt[j + 1]; q++) {
                    const int32_t k = bcol[q];
                    uint32_t h = orc_hash((uint32_t)k) & mask;
                    while (keys[h] != -1 && keys[h] != k) h = (h + 1) & mask;
                    if (keys[h] == -1) {
                        keys[h] = k;
                        c++;
                    }
                }
            }
            crpt[i] = c;
        }
        free(keys);
    }
    int64_t run = 0;
    for (int32_t i = 0; i < M; i++) {
        const int64_t c = crpt[i];
        crpt[i] = run;
        run += c;
    }
    crpt[M] = run;
    return run;
}

/* Numeric phase: accumulate each row in a hash table (fma, ascending j), then emit the
 * occupied slots in ascending column order. */
void orc_omp_numeric_f64(int32_t M, const int32_t *arpt, const int32_t *acol, const double *aval, const int32_t *brpt,
                         const int32_t *bcol, const double *bval, const int64_t *crpt, int32_t *ccol, double *cval)
{
    int64_t maxn = 0;
    for (int32_t i = 0; i < M; i++)
        if (crpt[i + 1] - crpt[i] > maxn) maxn = crpt[i + 1] - crpt[i];
    const int64_t tmax = next_pow2(2 * maxn);
#pragma omp parallel
    {
        int32_t *keys = (int32_t *)malloc((size_t)tmax * sizeof(int32_t));
        double *vals = (double *)malloc((size_t)tmax * sizeof(double));
#pragma omp for schedule(dynamic, 64)
        for (int32_t i = 0; i < M; i++) {
            const int64_t n = crpt[i + 1] - crpt[i];
            const int64_t ts = next_pow2(2 * n);
            const uint32_t mask = (uint32_t)(ts - 1);
            for (int64_t t = 0; t < ts; t++) keys[t] = -1;
            for (int32_t p = arpt[i]; p < arpt[i + 1]; p++) {
                const int32_t j = acol[p];
                const double a = aval[p];
                for (int32_t q = brpt[j]; q < brpt[j + 1]; q++) {
                    const int32_t k = bcol[q];
                    uint32_t h = orc_hash((uint32_t)k) & mask;
                    while (keys[h] != -1 && keys[h] != k) h = (h + 1) & mask;
                    if (keys[h] == -1) {
                        keys[h] = k;
                        vals[h] = 0.0;
                    }
                    vals[h] = fma(a, bval[q], vals[h]);
                }
            }
            /* gather occupied slots, insertion-sort by column (rows are short on average;
             * long rows fall back to qsort) */
            int32_t *oc = ccol + crpt[i];
            double *ov = cval + crpt[i];
            int64_t m = 0;
            for (int64_t t = 0; t < ts; t++)
                if (keys[t] != -1) oc[m++] = keys[t];
            qsort(oc, (size_t)m, sizeof(int32_t), cmp_i32);
            for (int64_t t = 0; t < m; t++) {
                const int32_t k = oc[t];
                uint32_t h = orc_hash((uint32_t)k) & mask;
                while (keys[h] != k) h = (h + 1) & mask;
                ov[t] = vals[h];
            }
        }
        free(keys);
        free(vals);
    }
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
