// ref_gpu.cu — runs OpSparse's own SpGEMM kernels on the GPU (from the cubin that
// oracle/ref_gpu/Makefile compiles out of OpSparse's sources) in the order, launch
// shapes, streams, allocations and host synchronisations of its host code.  TEST AND
// BENCHMARK INFRASTRUCTURE ONLY: it pins this library against the reference on the same
// GPU and times the reference with its own protocol.  Built on the GPU machine by
// __graft_entry__.build() into oracle/_ref/libref_gpu.so; needs no OpSparse source.
//
// Host code restated (paths relative to the OpSparse tree):
//   opsparse_spgemm                        src/opsparse/core_algo/spgemm/spgemm.cu:16-62
//   h_compute_flop, h_setup                src/opsparse/core_algo/spgemm/spgemm_phases.cu:12-26
//   h_symbolic_binning                     spgemm_phases.cu:28-50
//   h_symbolic                             spgemm_phases.cu:52-121
//   h_numeric_binning                      spgemm_phases.cu:123-146
//   h_numeric_full_occu                    spgemm_phases.cu:148-206
//   SpgemmMeta allocate / release / copies src/opsparse/core_algo/spgemm/meta.cu:12-95
//   tunables                               include/opsparse/utils/config.hpp:6-27
#include <cub/cub.cuh>
#include <cuda.h>
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

namespace {

// OpSparse's tunables (include/opsparse/utils/config.hpp:6-27)
constexpr int kNumBin = 8;
constexpr int kPwarp = 4, kPwarpRows = 256;
constexpr int kNumericPwarp = 8, kNumericPwarpRows = 128;
constexpr int kSymbolicScaleLarge = 1;
constexpr int kNumericScaleLarge = 2;

int div_up(int a, int b) { return (a + b - 1) / b; }

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

enum K {
    kComputeFlop,
    kSymBinning,
    kSymBinning2,
    kBinningSmall,
    kNumBinning,
    kNumBinning2,
    kSymTb8192,
    kSymTb4096,
    kSymTb2048,
    kSymTb1024,
    kSymTb512,
    kSymMaxWithFail,
    kSymLarge,
    kSymPwarp,
    kSymGlobal,
    kNumTb4096,
    kNumTb2048,
    kNumTb1024,
    kNumTb512,
    kNumTb256,
    kNumMaxHalf,
    kNumGlobal,
    kNumPwarp,
    kNumKernels
};

// Itanium-mangled name fragments that identify each kernel in the cubin's entry list
const char *kKey[kNumKernels] = {
    "14k_compute_flopE",
    "18k_symbolic_binningE",
    "19k_symbolic_binning2E",
    "15k_binning_smallE",
    "17k_numeric_binningE",
    "18k_numeric_binning2E",
    "25k_symbolic_shared_hash_tbILi8192EE",
    "25k_symbolic_shared_hash_tbILi4096EE",
    "25k_symbolic_shared_hash_tbILi2048EE",
    "25k_symbolic_shared_hash_tbILi1024EE",
    "25k_symbolic_shared_hash_tbILi512EE",
    "39k_symbolic_max_shared_hash_tb_with_failE",
    "31k_symbolic_large_shared_hash_tbE",
    "28k_symbolic_shared_hash_pwarpE",
    "25k_symbolic_global_hash_tbE",
    "34k_numeric_shared_hash_tb_full_occuILi4096ELi1024EE",
    "34k_numeric_shared_hash_tb_full_occuILi2048ELi512EE",
    "34k_numeric_shared_hash_tb_full_occuILi1024ELi256EE",
    "34k_numeric_shared_hash_tb_full_occuILi512ELi128EE",
    "34k_numeric_shared_hash_tb_full_occuILi256ELi64EE",
    "38k_numeric_max_shared_hash_tb_half_occuE",
    "34k_numeric_global_hash_tb_full_occuE",
    "27k_numeric_shared_hash_pwarpE",
};

CUmodule g_mod = nullptr;
CUfunction g_fn[kNumKernels] = {};
std::string g_err;

bool fail(const std::string &m)
{
    if (g_err.empty()) g_err = m;
    return false;
}

#define RCHK(x)                                                                   \
    do {                                                                          \
        cudaError_t e_ = (x);                                                     \
        if (e_ != cudaSuccess) return fail(std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

bool launch(K k, int grid, int block, unsigned smem, cudaStream_t s, std::vector<void *> args)
{
    if (grid <= 0) return true;
    const CUresult r = cuLaunchKernel(g_fn[k], (unsigned)grid, 1, 1, (unsigned)block, 1, 1, smem, (CUstream)s,
                                      args.data(), nullptr);
    if (r != CUDA_SUCCESS) return fail(std::string("launch of ") + kKey[k] + " failed: " + std::to_string((int)r));
    return true;
}

// SpgemmMeta (include/opsparse/core_algo/spgemm/meta.hpp:15-60, meta.cu:16-48)
struct Meta {
    int M = 0;
    cudaStream_t stream[kNumBin] = {};
    size_t cub_storage_size = 0;
    int *d_combined = nullptr, *combined = nullptr;
    int *d_bins = nullptr, *d_bin_size = nullptr, *d_max_row_nnz = nullptr, *d_total_nnz = nullptr,
        *d_bin_offset = nullptr, *d_cub_storage = nullptr;
    int *bin_size = nullptr, *max_row_nnz = nullptr, *total_nnz = nullptr, *bin_offset = nullptr;
    void *d_global_mem_pool = nullptr;
    size_t global_mem_pool_size = 0;
    bool global_mem_pool_malloced = false;

    bool allocate(int *c_rpt)
    {
        for (int i = 0; i < kNumBin; i++) RCHK(cudaStreamCreate(stream + i));
        RCHK(cub::DeviceScan::ExclusiveSum(nullptr, cub_storage_size, c_rpt, c_rpt, M + 1));
        const size_t d_combined_size = (size_t)M + 2 * kNumBin + 2 + cub_storage_size / sizeof(int);
        RCHK(cudaMalloc(&d_combined, d_combined_size * sizeof(int)));
        combined = static_cast<int *>(std::malloc((2 * kNumBin + 2) * sizeof(int)));
        d_bins = d_combined;
        d_bin_size = d_combined + M;
        d_max_row_nnz = d_bin_size + kNumBin;
        d_total_nnz = d_bin_size + kNumBin + 1;
        d_bin_offset = d_total_nnz + 1;
        d_cub_storage = d_bin_offset + 1;
        bin_size = combined;
        max_row_nnz = bin_size + kNumBin;
        total_nnz = bin_size + kNumBin + 1;
        bin_offset = bin_size + kNumBin + 2;
        return true;
    }
    void release()
    {
        if (d_combined) cudaFree(d_combined);
        d_combined = nullptr;
        for (int i = 0; i < kNumBin; i++)
            if (stream[i]) cudaStreamDestroy(stream[i]);
        std::memset(stream, 0, sizeof(stream));
        std::free(combined);
        combined = nullptr;
    }
    bool offsets_h2d()
    {
        bin_offset[0] = 0;
        for (int i = 0; i < kNumBin - 1; i++) bin_offset[i + 1] = bin_offset[i] + bin_size[i];
        RCHK(cudaMemcpyAsync(d_bin_offset, bin_offset, kNumBin * sizeof(int), cudaMemcpyHostToDevice, stream[0]));
        return true;
    }
    void small_bins()
    {
        bin_size[0] = M;
        for (int i = 1; i < kNumBin; i++) bin_size[i] = 0;
        bin_offset[0] = 0;
        for (int i = 1; i < kNumBin; i++) bin_offset[i] = M;
    }
};

struct Out {
    int nnz = 0;
    int *rpt = nullptr, *col = nullptr;
    double *val = nullptr;
    double t[9] = {};  // setup, symbolic_binning, symbolic, numeric_binning, allocate, prefix, numeric, cleanup, total
    int bins_sym[kNumBin] = {}, bins_num[kNumBin] = {};
    int fail_rows = 0;
};

bool spgemm(int M, const int *arpt, const int *acol, const double *aval, const int *brpt, const int *bcol,
            const double *bval, Out &o)
{
    Meta meta;
    meta.M = M;
    const int BS = 1024, GS = div_up(M, BS);
    double t0 = now_s(), t1 = t0;

    // ---- h_setup (spgemm_phases.cu:19-26)
    int *crpt = nullptr;
    RCHK(cudaMalloc(&crpt, (M + 1) * sizeof(int)));
    cudaMemset(crpt + M, 0, sizeof(int));
    int *crpt_m = crpt + M;
    if (!launch(kComputeFlop, GS, BS, 0, 0, {&arpt, &acol, &brpt, &M, &crpt, &crpt_m})) return false;
    if (!meta.allocate(crpt)) return false;
    RCHK(cudaMemcpy(meta.max_row_nnz, crpt + M, sizeof(int), cudaMemcpyDeviceToHost));
    RCHK(cudaDeviceSynchronize());
    o.t[0] = now_s() - t0;

    // ---- h_symbolic_binning (spgemm_phases.cu:28-50)
    t0 = now_s();
    RCHK(cudaMemsetAsync(meta.d_bin_size, 0, (kNumBin + 2) * sizeof(int), meta.stream[0]));
    if (*meta.max_row_nnz <= 26) {
        if (!launch(kBinningSmall, GS, BS, 0, 0, {&meta.d_bins, &M})) return false;
        meta.small_bins();
    } else {
        if (!launch(kSymBinning, GS, BS, 0, meta.stream[0], {&crpt, &M, &meta.d_bin_size})) return false;
        RCHK(cudaMemcpyAsync(meta.bin_size, meta.d_bin_size, kNumBin * sizeof(int), cudaMemcpyDeviceToHost,
                             meta.stream[0]));
        RCHK(cudaMemsetAsync(meta.d_bin_size, 0, kNumBin * sizeof(int), meta.stream[0]));
        if (!meta.offsets_h2d()) return false;
        if (!launch(kSymBinning2, GS, BS, 0, meta.stream[0],
                    {&crpt, &M, &meta.d_bins, &meta.d_bin_size, &meta.d_bin_offset}))
            return false;
    }
    RCHK(cudaDeviceSynchronize());
    o.t[1] = now_s() - t0;
    std::memcpy(o.bins_sym, meta.bin_size, sizeof(o.bins_sym));

    // ---- h_symbolic (spgemm_phases.cu:52-121)
    t0 = now_s();
    int *bs = meta.bin_size, *bo = meta.bin_offset;
    auto bins_of = [&](int b) { return meta.d_bins + bo[b]; };
    int *bp = nullptr;
    if (bs[5]) {
        bp = bins_of(5);
        if (!launch(kSymTb8192, bs[5], 1024, 0, meta.stream[5], {&arpt, &acol, &brpt, &bcol, &bp, &crpt})) return false;
    }
    int *d_fail_bins = nullptr, *d_fail_bin_size = nullptr;
    int fail_bin_size = 0;
    const bool fail_in_cub = bs[7] && bs[7] + 1 <= (int)(meta.cub_storage_size / sizeof(int));
    if (bs[7]) {
        if (fail_in_cub) {
            d_fail_bins = meta.d_cub_storage;
        } else {
            RCHK(cudaMalloc(&d_fail_bins, (bs[7] + 1) * sizeof(int)));
        }
        d_fail_bin_size = d_fail_bins + bs[7];
        RCHK(cudaMemsetAsync(d_fail_bin_size, 0, sizeof(int), meta.stream[7]));
        cuFuncSetAttribute(g_fn[kSymMaxWithFail], CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, 98304);
        bp = bins_of(7);
        if (!launch(kSymMaxWithFail, bs[7], 1024, 98304, meta.stream[7],
                    {&arpt, &acol, &brpt, &bcol, &bp, &d_fail_bins, &d_fail_bin_size, &crpt}))
            return false;
    }
    if (bs[6]) {
        bp = bins_of(6);
        if (!launch(kSymLarge, bs[6], 1024, 0, meta.stream[6], {&arpt, &acol, &brpt, &bcol, &bp, &crpt})) return false;
    }
    if (bs[0]) {
        bp = bins_of(0);
        int n0 = bs[0];
        if (!launch(kSymPwarp, div_up(bs[0], kPwarpRows), kPwarpRows * kPwarp, 0, meta.stream[0],
                    {&arpt, &acol, &brpt, &bcol, &bp, &n0, &crpt}))
            return false;
    }
    if (bs[7]) {
        RCHK(cudaMemcpyAsync(&fail_bin_size, d_fail_bin_size, sizeof(int), cudaMemcpyDeviceToHost, meta.stream[7]));
        RCHK(cudaStreamSynchronize(meta.stream[7]));
        if (fail_bin_size) {
            int max_tsize = *meta.max_row_nnz * kSymbolicScaleLarge;
            meta.global_mem_pool_size = (size_t)fail_bin_size * max_tsize * sizeof(int);
            RCHK(cudaMalloc(&meta.d_global_mem_pool, meta.global_mem_pool_size));
            meta.global_mem_pool_malloced = true;
            int *pool = static_cast<int *>(meta.d_global_mem_pool);
            if (!launch(kSymGlobal, fail_bin_size, 1024, 0, meta.stream[7],
                        {&arpt, &acol, &brpt, &bcol, &d_fail_bins, &crpt, &pool, &max_tsize}))
                return false;
        }
    }
    o.fail_rows = fail_bin_size;
    const K sym_tb[4] = {kSymTb4096, kSymTb2048, kSymTb1024, kSymTb512};
    const int sym_bs[4] = {512, 256, 128, 64};
    for (int b = 4; b >= 1; --b) {
        if (!bs[b]) continue;
        bp = bins_of(b);
        if (!launch(sym_tb[4 - b], bs[b], sym_bs[4 - b], 0, meta.stream[b], {&arpt, &acol, &brpt, &bcol, &bp, &crpt}))
            return false;
    }
    if (bs[7] && !fail_in_cub) RCHK(cudaFree(d_fail_bins));
    RCHK(cudaDeviceSynchronize());
    o.t[2] = now_s() - t0;

    // ---- h_numeric_binning (spgemm_phases.cu:123-146)
    t0 = now_s();
    RCHK(cudaMemsetAsync(meta.d_bin_size, 0, (kNumBin + 2) * sizeof(int), meta.stream[0]));
    if (!launch(kNumBinning, GS, BS, 0, meta.stream[0],
                {&crpt, &M, &meta.d_bin_size, &meta.d_total_nnz, &meta.d_max_row_nnz}))
        return false;
    RCHK(cudaMemcpyAsync(meta.bin_size, meta.d_bin_size, (kNumBin + 2) * sizeof(int), cudaMemcpyDeviceToHost,
                         meta.stream[0]));
    RCHK(cudaStreamSynchronize(meta.stream[0]));
    if (*meta.max_row_nnz <= 16) {
        if (!launch(kBinningSmall, GS, BS, 0, 0, {&meta.d_bins, &M})) return false;
        meta.small_bins();
    } else {
        RCHK(cudaMemsetAsync(meta.d_bin_size, 0, kNumBin * sizeof(int), meta.stream[0]));
        if (!meta.offsets_h2d()) return false;
        if (!launch(kNumBinning2, GS, BS, 0, meta.stream[0],
                    {&crpt, &M, &meta.d_bins, &meta.d_bin_size, &meta.d_bin_offset}))
            return false;
    }
    RCHK(cudaDeviceSynchronize());
    o.t[3] = now_s() - t0;
    std::memcpy(o.bins_num, meta.bin_size, sizeof(o.bins_num));

    // ---- allocate C (spgemm.cu:42-46)
    t0 = now_s();
    const int nnz = *meta.total_nnz;
    int *ccol = nullptr;
    double *cval = nullptr;
    RCHK(cudaMalloc(&cval, (size_t)nnz * sizeof(double)));
    RCHK(cudaMalloc(&ccol, (size_t)nnz * sizeof(int)));
    o.t[4] = now_s() - t0;

    // ---- row_ptr scan (spgemm.cu:48-51)
    t0 = now_s();
    RCHK(cub::DeviceScan::ExclusiveSum(meta.d_cub_storage, meta.cub_storage_size, crpt, crpt, M + 1));
    RCHK(cudaDeviceSynchronize());
    o.t[5] = now_s() - t0;

    // ---- h_numeric_full_occu (spgemm_phases.cu:148-206)
    t0 = now_s();
    if (bs[6]) {
        cuFuncSetAttribute(g_fn[kNumMaxHalf], CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, 98304);
        bp = bins_of(6);
        if (!launch(kNumMaxHalf, bs[6], 1024, 98304, meta.stream[6],
                    {&arpt, &acol, &aval, &brpt, &bcol, &bval, &bp, &crpt, &ccol, &cval}))
            return false;
    }
    if (bs[7]) {
        int max_tsize = *meta.max_row_nnz * kNumericScaleLarge;
        const size_t global_size = (size_t)bs[7] * max_tsize * (sizeof(int) + sizeof(double));
        if (meta.global_mem_pool_malloced) {
            if (global_size > meta.global_mem_pool_size) {
                RCHK(cudaFree(meta.d_global_mem_pool));
                RCHK(cudaMalloc(&meta.d_global_mem_pool, global_size));
            }
        } else {
            RCHK(cudaMalloc(&meta.d_global_mem_pool, global_size));
            meta.global_mem_pool_size = global_size;
            meta.global_mem_pool_malloced = true;
        }
        int *pool = static_cast<int *>(meta.d_global_mem_pool);
        bp = bins_of(7);
        if (!launch(kNumGlobal, bs[7], 1024, 0, meta.stream[7],
                    {&arpt, &acol, &aval, &brpt, &bcol, &bval, &bp, &max_tsize, &pool, &crpt, &ccol, &cval}))
            return false;
    }
    if (bs[5]) {
        bp = bins_of(5);
        if (!launch(kNumTb4096, bs[5], 1024, 0, meta.stream[5],
                    {&arpt, &acol, &aval, &brpt, &bcol, &bval, &bp, &crpt, &ccol, &cval}))
            return false;
    }
    if (bs[0]) {
        bp = bins_of(0);
        int n0 = bs[0];
        if (!launch(kNumPwarp, div_up(bs[0], kNumericPwarpRows), kNumericPwarpRows * kNumericPwarp, 0, meta.stream[0],
                    {&arpt, &acol, &aval, &brpt, &bcol, &bval, &bp, &n0, &crpt, &ccol, &cval}))
            return false;
    }
    const K num_tb[4] = {kNumTb2048, kNumTb1024, kNumTb512, kNumTb256};
    const int num_bs[4] = {512, 256, 128, 64};
    for (int b = 4; b >= 1; --b) {
        if (!bs[b]) continue;
        bp = bins_of(b);
        if (!launch(num_tb[4 - b], bs[b], num_bs[4 - b], 0, meta.stream[b],
                    {&arpt, &acol, &aval, &brpt, &bcol, &bval, &bp, &crpt, &ccol, &cval}))
            return false;
    }
    if (meta.global_mem_pool_malloced) RCHK(cudaFree(meta.d_global_mem_pool));
    RCHK(cudaDeviceSynchronize());
    o.t[6] = now_s() - t0;

    // ---- meta.release (spgemm.cu:57-59)
    t0 = now_s();
    meta.release();
    o.t[7] = now_s() - t0;
    o.t[8] = now_s() - t1;
    o.nnz = nnz;
    o.rpt = crpt;
    o.col = ccol;
    o.val = cval;
    return true;
}

}  // namespace

extern "C" {

// Loads the cubin and resolves every kernel by its mangled name.  Returns 0 on success.
int refgpu_init(const char *cubin, const char *names)
{
    g_err.clear();
    if (cudaFree(nullptr) != cudaSuccess) return fail("no CUDA device"), 1;
    if (!g_mod && cuModuleLoad(&g_mod, cubin) != CUDA_SUCCESS) return fail(std::string("cannot load ") + cubin), 1;
    std::ifstream in(names);
    std::vector<std::string> all;
    for (std::string line; std::getline(in, line);)
        if (!line.empty()) all.push_back(line);
    for (int k = 0; k < kNumKernels; ++k) {
        std::string found;
        for (const auto &n : all)
            if (n.find(kKey[k]) != std::string::npos) found = n;
        if (found.empty() || cuModuleGetFunction(&g_fn[k], g_mod, found.c_str()) != CUDA_SUCCESS)
            return fail(std::string("kernel not found: ") + kKey[k]), 1;
    }
    return 0;
}

const char *refgpu_error() { return g_err.c_str(); }

// One opsparse_spgemm call on device CSR inputs.  C's arrays are cudaMalloc'ed (free
// them with refgpu_free); t[9] receives OpSparse's SpgemmTimings fields in seconds, bins
// the symbolic and numeric bin sizes (2 x 8), fail_rows the rows that took the
// global-hash fallback.  Returns nnz(C), or -1 on error (refgpu_error).
long long refgpu_spgemm(int M, const int *arpt, const int *acol, const double *aval, const int *brpt, const int *bcol,
                        const double *bval, int **rpt, int **col, double **val, double *t, int *bins, int *fail_rows)
{
    g_err.clear();
    Out o;
    if (!spgemm(M, arpt, acol, aval, brpt, bcol, bval, o)) return -1;
    *rpt = o.rpt;
    *col = o.col;
    *val = o.val;
    std::memcpy(t, o.t, sizeof(o.t));
    std::memcpy(bins, o.bins_sym, sizeof(o.bins_sym));
    std::memcpy(bins + kNumBin, o.bins_num, sizeof(o.bins_num));
    *fail_rows = o.fail_rows;
    return o.nnz;
}

void refgpu_free(void *p) { cudaFree(p); }

}  // extern "C"
