// ref_driver.cpp — runs OpSparse's own SpGEMM kernels on the CPU (through cuda_emul.hpp)
// in the order and launch shapes of its host phase drivers, to produce reference outputs
// that pin the oracle.  TEST INFRASTRUCTURE ONLY; built by oracle/ref_emul/Makefile into
// oracle/_ref/ from the OpSparse sources, never shipped.
//
// The kernels are compiled from OpSparse's headers unchanged:
//   include/opsparse/core_algo/spgemm/kernels/binning.cuh, symbolic.cuh, numeric.cuh,
//   src/opsparse/numeric/compute_flop.cu (k_compute_flop and the host compute_flop).
// The host sequence below restates (paths relative to the OpSparse tree):
//   opsparse_spgemm                   src/opsparse/core_algo/spgemm/spgemm.cu:16-62
//   h_setup / h_compute_flop          src/opsparse/core_algo/spgemm/spgemm_phases.cu:12-26
//   h_symbolic_binning                spgemm_phases.cu:28-50
//   h_symbolic                        spgemm_phases.cu:52-121
//   h_numeric_binning                 spgemm_phases.cu:123-146
//   h_numeric_full_occu               spgemm_phases.cu:148-206
//   SpgemmMeta workspace layout       src/opsparse/core_algo/spgemm/meta.cu:16-48
// Device memory is host memory; cudaMemcpy/cudaMemset become assignments; the CUB scan
// becomes a sequential exclusive scan; the eight streams run one after another.
#include "opsparse/core_algo/spgemm/kernels/binning.cuh"
#include "opsparse/core_algo/spgemm/kernels/numeric.cuh"
#include "opsparse/core_algo/spgemm/kernels/symbolic.cuh"
#include "opsparse/numeric/compute_flop.cu"

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

using namespace opsparse;

// Backing store of the kernels' `extern __shared__ mint shared_mem[]` (the largest
// dynamic allocation OpSparse launches with is 98,304 bytes, spgemm_phases.cu:71-74,150-155).
namespace opsparse {
thread_local mint shared_mem[98304 / sizeof(mint)];
}

namespace {

struct RefResult {
    std::vector<mint> rpt, col;
    std::vector<mdouble> val;
    mint bin_size_sym[kNumBin] = {};
    mint bin_size_num[kNumBin] = {};
    mint fail_rows = 0;
} g_res;

void exclusive_scan(mint *a, mint n)
{
    mint run = 0;
    for (mint i = 0; i < n; ++i) {
        const mint v = a[i];
        a[i] = run;
        run += v;
    }
}

// bin_size -> bin_offset on the host, as in spgemm_phases.cu:37-41 / :131-135
void offsets(const mint *bin_size, mint *bin_offset)
{
    bin_offset[0] = 0;
    for (int i = 0; i < kNumBin - 1; ++i) bin_offset[i + 1] = bin_offset[i] + bin_size[i];
}

}  // namespace

extern "C" int ref_spgemm(int M, int K, int N, const int *arpt, const int *acol, const double *aval, const int *brpt,
                          const int *bcol, const double *bval)
{
    (void)K;
    const mint BS = 1024;
    const mint GS = div_up(M, BS);
    std::vector<mint> crpt(M + 1, 0);
    std::vector<mint> bins(std::max(M, 1));
    mint d_bin_size[kNumBin] = {}, d_bin_offset[kNumBin] = {};
    mint d_max_row_nnz = 0, d_total_nnz = 0;
    mint bin_size[kNumBin] = {}, bin_offset[kNumBin] = {};

    // ---- h_setup: row flop into C.rpt[i], max into C.rpt[M]
    crpt[M] = 0;
    emu::launch(GS, BS, [&] { k_compute_flop(arpt, acol, brpt, M, crpt.data(), crpt.data() + M); });
    mint max_flop = crpt[M];

    // ---- h_symbolic_binning
    std::memset(d_bin_size, 0, sizeof(d_bin_size));
    if (max_flop <= 26) {
        emu::launch(GS, BS, [&] { k_binning_small(bins.data(), M); });
        bin_size[0] = M;
        for (int i = 1; i < kNumBin; ++i) bin_size[i] = 0;
        bin_offset[0] = 0;
        for (int i = 1; i < kNumBin; ++i) bin_offset[i] = M;
    } else {
        emu::launch(GS, BS, [&] { k_symbolic_binning(crpt.data(), M, d_bin_size); });
        std::memcpy(bin_size, d_bin_size, sizeof(bin_size));
        std::memset(d_bin_size, 0, sizeof(d_bin_size));
        offsets(bin_size, bin_offset);
        std::memcpy(d_bin_offset, bin_offset, sizeof(bin_offset));
        emu::launch(GS, BS, [&] { k_symbolic_binning2(crpt.data(), M, bins.data(), d_bin_size, d_bin_offset); });
    }
    std::memcpy(g_res.bin_size_sym, bin_size, sizeof(bin_size));

    // ---- h_symbolic (launch order 5, 7, 6, 0, [7 fail], 4, 3, 2, 1)
    mint *d_bins = bins.data();
    if (bin_size[5])
        emu::launch(bin_size[5], 1024, [&] {
            k_symbolic_shared_hash_tb<8192>(arpt, acol, brpt, bcol, d_bins + bin_offset[5], crpt.data());
        });
    std::vector<mint> fail_bins;
    mint fail_bin_size = 0;
    if (bin_size[7]) {
        fail_bins.assign(bin_size[7] + 1, 0);
        fail_bins[bin_size[7]] = 0;
        emu::launch(bin_size[7], 1024, [&] {
            k_symbolic_max_shared_hash_tb_with_fail(arpt, acol, brpt, bcol, d_bins + bin_offset[7], fail_bins.data(),
                                                    fail_bins.data() + bin_size[7], crpt.data());
        });
    }
    if (bin_size[6])
        emu::launch(bin_size[6], 1024, [&] {
            k_symbolic_large_shared_hash_tb(arpt, acol, brpt, bcol, d_bins + bin_offset[6], crpt.data());
        });
    if (bin_size[0])
        emu::launch(div_up(bin_size[0], kPwarpRows), kPwarpRows * kPwarp, [&] {
            k_symbolic_shared_hash_pwarp(arpt, acol, brpt, bcol, d_bins + bin_offset[0], bin_size[0], crpt.data());
        });
    if (bin_size[7]) {
        fail_bin_size = fail_bins[bin_size[7]];
        if (fail_bin_size) {
            const mint max_tsize = max_flop * kSymbolicScaleLarge;
            std::vector<mint> pool((size_t)fail_bin_size * (size_t)max_tsize);
            emu::launch(fail_bin_size, 1024, [&] {
                k_symbolic_global_hash_tb(arpt, acol, brpt, bcol, fail_bins.data(), crpt.data(), pool.data(),
                                          max_tsize);
            });
        }
    }
    g_res.fail_rows = fail_bin_size;
    if (bin_size[4])
        emu::launch(bin_size[4], 512, [&] {
            k_symbolic_shared_hash_tb<4096>(arpt, acol, brpt, bcol, d_bins + bin_offset[4], crpt.data());
        });
    if (bin_size[3])
        emu::launch(bin_size[3], 256, [&] {
            k_symbolic_shared_hash_tb<2048>(arpt, acol, brpt, bcol, d_bins + bin_offset[3], crpt.data());
        });
    if (bin_size[2])
        emu::launch(bin_size[2], 128, [&] {
            k_symbolic_shared_hash_tb<1024>(arpt, acol, brpt, bcol, d_bins + bin_offset[2], crpt.data());
        });
    if (bin_size[1])
        emu::launch(bin_size[1], 64, [&] {
            k_symbolic_shared_hash_tb<512>(arpt, acol, brpt, bcol, d_bins + bin_offset[1], crpt.data());
        });

    // ---- h_numeric_binning (bins by row nnz; sum and max of row nnz)
    std::memset(d_bin_size, 0, sizeof(d_bin_size));
    d_max_row_nnz = 0;
    d_total_nnz = 0;
    emu::launch(GS, BS, [&] { k_numeric_binning(crpt.data(), M, d_bin_size, &d_total_nnz, &d_max_row_nnz); });
    std::memcpy(bin_size, d_bin_size, sizeof(bin_size));
    const mint max_row_nnz = d_max_row_nnz;
    const mint total_nnz = d_total_nnz;
    if (max_row_nnz <= 16) {
        emu::launch(GS, BS, [&] { k_binning_small(bins.data(), M); });
        bin_size[0] = M;
        for (int i = 1; i < kNumBin; ++i) bin_size[i] = 0;
        bin_offset[0] = 0;
        for (int i = 1; i < kNumBin; ++i) bin_offset[i] = M;
    } else {
        std::memset(d_bin_size, 0, sizeof(d_bin_size));
        offsets(bin_size, bin_offset);
        std::memcpy(d_bin_offset, bin_offset, sizeof(bin_offset));
        emu::launch(GS, BS, [&] { k_numeric_binning2(crpt.data(), M, bins.data(), d_bin_size, d_bin_offset); });
    }
    std::memcpy(g_res.bin_size_num, bin_size, sizeof(bin_size));

    // ---- allocate C, exclusive scan of row nnz over M+1 entries
    std::vector<mint> ccol(std::max(total_nnz, 1));
    std::vector<mdouble> cval(std::max(total_nnz, 1));
    exclusive_scan(crpt.data(), M + 1);

    // ---- h_numeric_full_occu (launch order 6, 7, 5, 0, 4, 3, 2, 1)
    if (bin_size[6])
        emu::launch(bin_size[6], 1024, [&] {
            k_numeric_max_shared_hash_tb_half_occu(arpt, acol, aval, brpt, bcol, bval, d_bins + bin_offset[6],
                                                   crpt.data(), ccol.data(), cval.data());
        });
    if (bin_size[7]) {
        const mint max_tsize = max_row_nnz * kNumericScaleLarge;
        std::vector<mint> pool((size_t)bin_size[7] * (size_t)max_tsize * ((sizeof(mint) + sizeof(mdouble)) / sizeof(mint)));
        emu::launch(bin_size[7], 1024, [&] {
            k_numeric_global_hash_tb_full_occu(arpt, acol, aval, brpt, bcol, bval, d_bins + bin_offset[7], max_tsize,
                                               pool.data(), crpt.data(), ccol.data(), cval.data());
        });
    }
    if (bin_size[5])
        emu::launch(bin_size[5], 1024, [&] {
            k_numeric_shared_hash_tb_full_occu<4096, 1024>(arpt, acol, aval, brpt, bcol, bval, d_bins + bin_offset[5],
                                                           crpt.data(), ccol.data(), cval.data());
        });
    if (bin_size[0])
        emu::launch(div_up(bin_size[0], kNumericPwarpRows), kNumericPwarpRows * kNumericPwarp, [&] {
            k_numeric_shared_hash_pwarp(arpt, acol, aval, brpt, bcol, bval, d_bins + bin_offset[0], bin_size[0],
                                        crpt.data(), ccol.data(), cval.data());
        });
    if (bin_size[4])
        emu::launch(bin_size[4], 512, [&] {
            k_numeric_shared_hash_tb_full_occu<2048, 512>(arpt, acol, aval, brpt, bcol, bval, d_bins + bin_offset[4],
                                                          crpt.data(), ccol.data(), cval.data());
        });
    if (bin_size[3])
        emu::launch(bin_size[3], 256, [&] {
            k_numeric_shared_hash_tb_full_occu<1024, 256>(arpt, acol, aval, brpt, bcol, bval, d_bins + bin_offset[3],
                                                          crpt.data(), ccol.data(), cval.data());
        });
    if (bin_size[2])
        emu::launch(bin_size[2], 128, [&] {
            k_numeric_shared_hash_tb_full_occu<512, 128>(arpt, acol, aval, brpt, bcol, bval, d_bins + bin_offset[2],
                                                         crpt.data(), ccol.data(), cval.data());
        });
    if (bin_size[1])
        emu::launch(bin_size[1], 64, [&] {
            k_numeric_shared_hash_tb_full_occu<256, 64>(arpt, acol, aval, brpt, bcol, bval, d_bins + bin_offset[1],
                                                        crpt.data(), ccol.data(), cval.data());
        });
    (void)N;
    g_res.rpt.swap(crpt);
    ccol.resize(total_nnz);
    cval.resize(total_nnz);
    g_res.col.swap(ccol);
    g_res.val.swap(cval);
    return total_nnz;
}

// Copies the last result out (rpt: M+1, col/val: nnz) and the bin histograms (8 + 8) and
// the number of rows that took the global-hash fallback.
extern "C" void ref_fetch(int *rpt, int *col, double *val, int *bins_sym, int *bins_num, int *fail_rows)
{
    std::copy(g_res.rpt.begin(), g_res.rpt.end(), rpt);
    std::copy(g_res.col.begin(), g_res.col.end(), col);
    std::copy(g_res.val.begin(), g_res.val.end(), val);
    std::copy(g_res.bin_size_sym, g_res.bin_size_sym + kNumBin, bins_sym);
    std::copy(g_res.bin_size_num, g_res.bin_size_num + kNumBin, bins_num);
    *fail_rows = g_res.fail_rows;
}

// The reference's own host flop counter (compute_flop.cu:33-52).
extern "C" long ref_compute_flop(const int *arpt, const int *acol, const int *brpt, int M, int *row_flop)
{
    return compute_flop(arpt, acol, brpt, M, row_flop);
}
