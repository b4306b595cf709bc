// facade_selftest.cpp — exercises the drop-in C++ API the way OpSparse's own benchmark
// drivers do (benchmarks/opsparse_profile.cu, opsparse_reg.cu): load a MatrixMarket file,
// H2D, SpGEMM through opsparse_spgemm / _reg / _safe, D2H, compare, release.
// Exit status 0 and "FACADE_SELFTEST OK" on success.
#include <cmath>
#include <cstdio>
#include <cstdlib>
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

static void write_mtx(const std::string &path, int n)
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

static void check_product(const CSR &A, const CSR &B, CSR &C)
{
    C.D2H();
    std::vector<int> rpt, col;
    std::vector<double> val;
    host_spgemm(A, B, rpt, col, val);
    EXPECT(C.nnz == static_cast<int>(col.size()));
    if (C.nnz != static_cast<int>(col.size())) return;
    int bad = 0;
    for (int i = 0; i <= A.M; ++i) bad += C.rpt[i] != rpt[i];
    for (int p = 0; p < C.nnz; ++p) bad += (C.col[p] != col[p]) || (C.val[p] != val[p]);
    EXPECT(bad == 0);
}

int main(int argc, char **argv)
{
    const std::string path = argc > 1 ? argv[1] : "/tmp/opsparse_facade_selftest.mtx";
    write_mtx(path, 48);
    CSR A(path);
    EXPECT(A.M == 48 * 48 && A.N == 48 * 48);
    EXPECT(A.nnz == 5 * 48 * 48 - 4 * 48);
    CSR B;
    B = A;
    A.H2D();
    B.H2D();
    const long flop = compute_flop(A, B);
    EXPECT(flop > 0);

    cuda_runtime_warmup();
    SpgemmMeta meta;
    {
        CSR C;
        SpgemmTimings timing;
        opsparse_spgemm(A, B, C, meta, timing);
        check_product(A, B, C);
        EXPECT(timing.total > 0);
        timing.print(2.0 * flop);
        C.release();
    }
    {
        CSR C;
        SpgemmTimings timing, acc;
        for (int it = 0; it < 3; ++it) {
            opsparse_spgemm_reg(A, B, C, meta, timing);
            acc += timing;
            if (it < 2) C.release();
        }
        acc /= 3;
        check_product(A, B, C);
        C.release();
    }
    {
        CSR C;
        SpgemmTimings timing;
        SpgemmPerf perf;
        const SpgemmStatus st = opsparse_spgemm_safe(A, B, C, meta, timing, perf);
        EXPECT(st == SpgemmStatus::ok);
        EXPECT(perf.total_flop == flop);
        EXPECT(perf.c_nnz == C.nnz);
        std::printf("STATUS,%s\n", to_cstr(st));
        check_product(A, B, C);
        C.release();
        // sub-matrix slice: 100 x 2304 times the full B is non-square against A
        CSR S(A, 100, A.N - 1, 0, 0);
        S.H2D();
        CSR C2;
        EXPECT(opsparse_spgemm_safe(S, B, C2, meta, timing, perf) == SpgemmStatus::nonsquare);
        S.release();
    }
    {
        // operator== on identical products
        CSR C1, C2;
        SpgemmTimings timing;
        opsparse_spgemm(A, B, C1, meta, timing);
        opsparse_spgemm(A, B, C2, meta, timing);
        C1.D2H();
        C2.D2H();
        EXPECT(C1 == C2);
        C1.release();
        C2.release();
    }
    A.release();
    B.release();
    std::remove(path.c_str());
    if (failures) {
        std::printf("FACADE_SELFTEST FAILED (%d)\n", failures);
        return 1;
    }
    std::printf("FACADE_SELFTEST OK\n");
    return 0;
}
