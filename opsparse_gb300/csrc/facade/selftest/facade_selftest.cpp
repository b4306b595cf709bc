// facade_selftest.cpp — drives the drop-in C++ API the way OpSparse's own benchmark drivers
// do (benchmarks/opsparse_profile.cu:10-48, opsparse_reg.cu:46-117): load MatrixMarket
// files through CSR, H2D, SpGEMM through opsparse_spgemm / _reg / _safe, print the timings,
// D2H, release.  Used by the GPU tests, which compare what it writes with the oracle.
//
//   facade_selftest                                  self-contained check on a generated
//                                                    symmetric 2-D Laplacian file
//   facade_selftest run A.mtx B.mtx|- OUTDIR [dC.bin]
//       loads A (and B; "-" means B = A, as the reference's drivers do), multiplies through
//       every entry point, and writes OUTDIR/A.bin, B.bin and C.bin.  With dC.bin (C.nnz
//       doubles) it also runs opsparse_spgemm_backward and writes OUTDIR/dA.bin, dB.bin.
//
// .bin layout: int64 M, N, nnz, then rpt (M+1 int32), col (nnz int32), val (nnz double);
// dA.bin / dB.bin hold the values only.  Exit status 0 and "FACADE_SELFTEST OK" on success.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#include "opsparse/core_algo/spgemm/spgemm.hpp"
#include "opsparse/numeric/compute_flop.hpp"

using namespace opsparse;

static int failures = 0;
#define EXPECT(cond)                                                      \
    do {                                                                  \
        if (!(cond)) {                                                    \
            std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #cond);   \
            ++failures;                                                   \
        }                                                                 \
    } while (0)

// Host reference: row-wise, ascending j, one fma per product, ascending columns.
static void host_spgemm(const CSR &A, const CSR &B, std::vector<int> &rpt, std::vector<int> &col,
                        std::vector<double> &val)
{
    rpt.assign(A.M + 1, 0);
    col.clear();
    val.clear();
    for (int i = 0; i < A.M; ++i) {
        std::map<int, double> acc;
        for (int p = A.rpt[i]; p < A.rpt[i + 1]; ++p) {
            const int j = A.col[p];
            for (int q = B.rpt[j]; q < B.rpt[j + 1]; ++q) {
                auto it = acc.find(B.col[q]);
                if (it == acc.end()) it = acc.emplace(B.col[q], 0.0).first;
                it->second = std::fma(A.val[p], B.val[q], it->second);
            }
        }
        for (auto &kv : acc) {
            col.push_back(kv.first);
            val.push_back(kv.second);
        }
        rpt[i + 1] = static_cast<int>(col.size());
    }
}

static void write_laplacian_mtx(const std::string &path, int n)
{
    // symmetric 2-D Laplacian, lower triangle only, 1-based
    std::ofstream f(path);
    int entries = 0;
    for (int i = 0; i < n * n; ++i) {
        entries += 1;
        if (i % n) entries += 1;
        if (i >= n) entries += 1;
    }
    f << "%%MatrixMarket matrix coordinate real symmetric\n% test file\n";
    f << n * n << " " << n * n << " " << entries << "\n";
    for (int i = 0; i < n * n; ++i) {
        if (i >= n) f << i + 1 << " " << i - n + 1 << " -1\n";
        if (i % n) f << i + 1 << " " << i << " -1\n";
        f << i + 1 << " " << i + 1 << " 4\n";
    }
}

static bool same_product(const CSR &A, const CSR &B, CSR &C)
{
    C.D2H();
    std::vector<int> rpt, col;
    std::vector<double> val;
    host_spgemm(A, B, rpt, col, val);
    if (C.nnz != static_cast<int>(col.size())) return false;
    int bad = 0;
    for (int i = 0; i <= A.M; ++i) bad += C.rpt[i] != rpt[i];
    for (int p = 0; p < C.nnz; ++p) bad += (C.col[p] != col[p]) || (C.val[p] != val[p]);
    return bad == 0;
}

static bool same_host(const CSR &X, const CSR &Y)
{
    if (X.M != Y.M || X.N != Y.N || X.nnz != Y.nnz) return false;
    return std::memcmp(X.rpt, Y.rpt, sizeof(mint) * (X.M + 1)) == 0 &&
           std::memcmp(X.col, Y.col, sizeof(mint) * X.nnz) == 0 &&
           std::memcmp(X.val, Y.val, sizeof(mdouble) * X.nnz) == 0;
}

static void write_csr(const std::string &path, const CSR &X)
{
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) {
        std::printf("FAIL cannot write %s\n", path.c_str());
        ++failures;
        return;
    }
    const long long hdr[3] = {X.M, X.N, X.nnz};
    std::fwrite(hdr, sizeof(hdr), 1, f);
    std::fwrite(X.rpt, sizeof(mint), static_cast<size_t>(X.M) + 1, f);
    std::fwrite(X.col, sizeof(mint), static_cast<size_t>(X.nnz), f);
    std::fwrite(X.val, sizeof(mdouble), static_cast<size_t>(X.nnz), f);
    std::fclose(f);
}

static void write_values(const std::string &path, const std::vector<double> &v)
{
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) {
        ++failures;
        return;
    }
    std::fwrite(v.data(), sizeof(double), v.size(), f);
    std::fclose(f);
}

static size_t free_bytes()
{
    size_t fr = 0, tot = 0;
    query_cuda_memory(fr, tot);
    return fr;
}

// Everything the reference's drivers do with A and B, checked as it goes; C goes to
// outdir/C.bin when outdir is given.
static void exercise(CSR &A, CSR &B, const std::string &outdir, const std::string &dc_path)
{
    A.H2D();
    B.H2D();
    const long flop = compute_flop(A, B);
    EXPECT(flop >= 0);
    cuda_runtime_warmup();
    SpgemmMeta meta;
    CSR C0;
    {
        // opsparse_profile.cu: one warm-up call, then timed calls with C.release() between
        SpgemmTimings timing, acc;
        opsparse_spgemm(A, B, C0, meta, timing);
        C0.release();
        for (int it = 0; it < 3; ++it) {
            opsparse_spgemm(A, B, C0, meta, timing);
            acc += timing;
            if (it < 2) C0.release();
        }
        acc /= 3;
        EXPECT(acc.total > 0);
        acc.print(2.0 * flop);
        C0.D2H();
    }
    {
        // opsparse_reg.cu: the fused variant, timing.total only
        CSR C;
        SpgemmTimings timing;
        for (int it = 0; it < 3; ++it) {
            opsparse_spgemm_reg(A, B, C, meta, timing);
            if (it < 2) C.release();
        }
        EXPECT(timing.total > 0);
        std::printf("PERF,reg,");
        timing.reg_print(2.0 * flop);
        C.D2H();
        EXPECT(same_host(C, C0));
        C.release();
    }
    {
        CSR C;
        SpgemmTimings timing;
        SpgemmPerf perf;
        const SpgemmStatus st = opsparse_spgemm_safe(A, B, C, meta, timing, perf);
        std::printf("STATUS,%s\n", to_cstr(st));
        EXPECT(st == SpgemmStatus::ok);
        EXPECT(perf.total_flop == flop);
        EXPECT(perf.c_nnz == C0.nnz);
        EXPECT(perf.error_msg.empty());
        C.D2H();
        EXPECT(same_host(C, C0));
        C.release();
        // a slice of A whose column count differs from B's row count
        if (A.N > 1) {
            CSR S(A, A.M, A.N - 1, 0, 0);
            S.H2D();
            CSR C2;
            const SpgemmStatus st2 = opsparse_spgemm_safe(S, B, C2, meta, timing, perf);
            std::printf("STATUS,%s\n", to_cstr(st2));
            EXPECT(st2 == SpgemmStatus::nonsquare);
            EXPECT(C2.d_rpt == nullptr && C2.d_col == nullptr && C2.d_val == nullptr);
            S.release();
        }
    }
    {
        // C's arrays come from cudaMalloc and go back with C.release(): repeated calls
        // leave the device's free memory where it was
        CSR C;
        SpgemmTimings timing;
        opsparse_spgemm(A, B, C, meta, timing);
        C.release();
        const size_t before = free_bytes();
        for (int it = 0; it < 5; ++it) {
            opsparse_spgemm(A, B, C, meta, timing);
            EXPECT(C.d_rpt && (C.nnz == 0 || (C.d_col && C.d_val)));
            C.release();
            EXPECT(C.d_rpt == nullptr && C.d_col == nullptr && C.d_val == nullptr);
        }
        const size_t after = free_bytes();
        std::printf("MEMORY,free_before,%zu,free_after,%zu\n", before, after);
        EXPECT(after + (size_t(4) << 20) >= before);
        EXPECT(cudaGetLastError() == cudaSuccess);
    }
    if (!outdir.empty()) {
        write_csr(outdir + "/A.bin", A);
        write_csr(outdir + "/B.bin", B);
        write_csr(outdir + "/C.bin", C0);
    }
    if (!dc_path.empty()) {
        std::vector<double> dc(static_cast<size_t>(C0.nnz));
        FILE *f = std::fopen(dc_path.c_str(), "rb");
        EXPECT(f != nullptr);
        if (f) {
            EXPECT(std::fread(dc.data(), sizeof(double), dc.size(), f) == dc.size());
            std::fclose(f);
        }
        // C0's device arrays are still the product's (D2H only made host copies)
        mdouble *d_dc = nullptr, *d_da = nullptr, *d_db = nullptr;
        OPSPARSE_CHECK_CUDA(cudaMalloc(&d_dc, sizeof(mdouble) * std::max<size_t>(dc.size(), 1)));
        OPSPARSE_CHECK_CUDA(cudaMalloc(&d_da, sizeof(mdouble) * std::max<size_t>(A.nnz, 1)));
        OPSPARSE_CHECK_CUDA(cudaMalloc(&d_db, sizeof(mdouble) * std::max<size_t>(B.nnz, 1)));
        if (!dc.empty()) h2d(d_dc, dc.data(), sizeof(mdouble) * dc.size());
        std::vector<double> da(A.nnz), db(B.nnz), da2(A.nnz), db2(B.nnz);
        for (int rep = 0; rep < 2; ++rep) {  // the second call reuses the plan on the handle
            opsparse_spgemm_backward(A, B, C0, d_dc, d_da, d_db, meta);
            std::vector<double> &xa = rep ? da2 : da, &xb = rep ? db2 : db;
            if (A.nnz) d2h(xa.data(), d_da, sizeof(mdouble) * A.nnz);
            if (B.nnz) d2h(xb.data(), d_db, sizeof(mdouble) * B.nnz);
        }
        EXPECT(std::memcmp(da.data(), da2.data(), sizeof(double) * da.size()) == 0);
        EXPECT(std::memcmp(db.data(), db2.data(), sizeof(double) * db.size()) == 0);
        // dA only: d_dB may be null
        opsparse_spgemm_backward(A, B, C0, d_dc, d_da, nullptr, meta);
        if (A.nnz) d2h(da2.data(), d_da, sizeof(mdouble) * A.nnz);
        EXPECT(std::memcmp(da.data(), da2.data(), sizeof(double) * da.size()) == 0);
        cudaFree(d_dc);
        cudaFree(d_da);
        cudaFree(d_db);
        if (!outdir.empty()) {
            write_values(outdir + "/dA.bin", da);
            write_values(outdir + "/dB.bin", db);
        }
    }
    C0.release();
    A.release();
    B.release();
}

static int selfcheck()
{
    const std::string path = "/tmp/opsparse_facade_selftest.mtx";
    write_laplacian_mtx(path, 48);
    CSR A(path);
    std::remove(path.c_str());
    EXPECT(A.M == 48 * 48 && A.N == 48 * 48);
    EXPECT(A.nnz == 5 * 48 * 48 - 4 * 48);
    CSR B;
    B = A;
    {
        CSR Ad(A), Bd(B);
        Ad.H2D();
        Bd.H2D();
        SpgemmMeta meta;
        CSR C;
        SpgemmTimings timing;
        opsparse_spgemm(Ad, Bd, C, meta, timing);
        EXPECT(same_product(A, B, C));
        CSR C2;
        opsparse_spgemm(Ad, Bd, C2, meta, timing);
        C2.D2H();
        EXPECT(C == C2);  // the reference's tolerant comparison
        C.release();
        C2.release();
    }
    exercise(A, B, "", "");
    return 0;
}

int main(int argc, char **argv)
{
    try {
        if (argc >= 5 && std::string(argv[1]) == "run") {
            CSR A(argv[2]);
            CSR B;
            if (std::string(argv[3]) == "-") B = A;
            else B.construct(argv[3]);
            exercise(A, B, argv[4], argc >= 6 ? argv[5] : "");
        } else if (argc == 1) {
            selfcheck();
        } else {
            std::printf("usage: facade_selftest [run A.mtx B.mtx|- OUTDIR [dC.bin]]\n");
            return 2;
        }
    } catch (const std::exception &e) {
        std::printf("FAIL exception: %s\n", e.what());
        ++failures;
    }
    if (failures) {
        std::printf("FACADE_SELFTEST FAILED (%d)\n", failures);
        return 1;
    }
    std::printf("FACADE_SELFTEST OK\n");
    return 0;
}
