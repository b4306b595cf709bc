// csr.cpp — the drop-in CSR container (API of OpSparse include/opsparse/core_ds/csr.hpp:10-37,
// behaviour of src/opsparse/core_ds/csr.cu:30-352).
#include "opsparse/core_ds/csr.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <numeric>
#include <sstream>
#include <stdexcept>
#include <vector>

#include "opsparse/io/matrix_market.hpp"

namespace opsparse {

void CSR::hrelease()
{
    delete[] rpt;
    delete[] col;
    delete[] val;
    rpt = nullptr;
    col = nullptr;
    val = nullptr;
}

void CSR::drelease()
{
    // cudaFree(nullptr) is a no-op; errors are reported like OpSparse's check_cuda.
    OPSPARSE_CHECK_CUDA(cudaFree(d_rpt));
    OPSPARSE_CHECK_CUDA(cudaFree(d_col));
    OPSPARSE_CHECK_CUDA(cudaFree(d_val));
    d_rpt = nullptr;
    d_col = nullptr;
    d_val = nullptr;
}

void CSR::release()
{
    hrelease();
    drelease();
}

CSR::~CSR()
{
    hrelease();
    cudaFree(d_rpt);
    cudaFree(d_col);
    cudaFree(d_val);
}

void CSR::H2D()
{
    drelease();
    OPSPARSE_CHECK_CUDA(cudaMalloc(&d_rpt, sizeof(mint) * (static_cast<std::size_t>(M) + 1)));
    OPSPARSE_CHECK_CUDA(cudaMalloc(&d_col, sizeof(mint) * static_cast<std::size_t>(nnz)));
    OPSPARSE_CHECK_CUDA(cudaMalloc(&d_val, sizeof(mdouble) * static_cast<std::size_t>(nnz)));
    h2d(d_rpt, rpt, sizeof(mint) * (static_cast<std::size_t>(M) + 1));
    if (nnz) {
        h2d(d_col, col, sizeof(mint) * static_cast<std::size_t>(nnz));
        h2d(d_val, val, sizeof(mdouble) * static_cast<std::size_t>(nnz));
    }
}

void CSR::D2H()
{
    hrelease();
    rpt = new mint[static_cast<std::size_t>(M) + 1];
    col = new mint[static_cast<std::size_t>(nnz)];
    val = new mdouble[static_cast<std::size_t>(nnz)];
    d2h(rpt, d_rpt, sizeof(mint) * (static_cast<std::size_t>(M) + 1));
    if (nnz) {
        d2h(col, d_col, sizeof(mint) * static_cast<std::size_t>(nnz));
        d2h(val, d_val, sizeof(mdouble) * static_cast<std::size_t>(nnz));
    }
}

static void copy_host(CSR &dst, const CSR &src)
{
    dst.M = src.M;
    dst.N = src.N;
    dst.nnz = src.nnz;
    dst.rpt = new mint[static_cast<std::size_t>(src.M) + 1];
    dst.col = new mint[static_cast<std::size_t>(src.nnz)];
    dst.val = new mdouble[static_cast<std::size_t>(src.nnz)];
    std::memcpy(dst.rpt, src.rpt, sizeof(mint) * (static_cast<std::size_t>(src.M) + 1));
    std::memcpy(dst.col, src.col, sizeof(mint) * static_cast<std::size_t>(src.nnz));
    std::memcpy(dst.val, src.val, sizeof(mdouble) * static_cast<std::size_t>(src.nnz));
}

CSR::CSR(const CSR &A) { copy_host(*this, A); }

CSR &CSR::operator=(const CSR &A)
{
    if (this == &A) return *this;
    release();
    copy_host(*this, A);
    return *this;
}

// Rows [M_start, M_start+M_) and columns [N_start, N_start+N_) of A, re-indexed from 0.
CSR::CSR(const CSR &A, mint M_, mint N_, mint M_start, mint N_start)
{
    if (M_ + M_start > A.M || N_ + N_start > A.N) throw std::runtime_error("matrix subsect out of range");
    M = M_;
    N = N_;
    std::vector<mint> keep_col;
    std::vector<mdouble> keep_val;
    rpt = new mint[static_cast<std::size_t>(M) + 1];
    rpt[0] = 0;
    for (mint i = 0; i < M; ++i) {
        const mint r = i + M_start;
        for (mint p = A.rpt[r]; p < A.rpt[r + 1]; ++p) {
            const mint c = A.col[p] - N_start;
            if (c >= 0 && c < N) {
                keep_col.push_back(c);
                keep_val.push_back(A.val[p]);
            }
        }
        rpt[i + 1] = static_cast<mint>(keep_col.size());
    }
    nnz = rpt[M];
    col = new mint[keep_col.size()];
    val = new mdouble[keep_val.size()];
    std::copy(keep_col.begin(), keep_col.end(), col);
    std::copy(keep_val.begin(), keep_val.end(), val);
}

// Structure must match exactly; values within 1e-9 absolute or 1e-9 relative.  Throws if
// nnz differs or more than 10 mismatches are seen; returns false on any mismatch.
bool CSR::operator==(const CSR &rhs)
{
    if (nnz != rhs.nnz) {
        std::printf("nnz not equal %d %d\n", nnz, rhs.nnz);
        throw std::runtime_error("nnz not equal");
    }
    if (M != rhs.M || N != rhs.N) throw std::runtime_error("dimension not same");
    const double eps = 1e-9;
    int errors = 0;
    for (mint i = 0; i <= M; ++i) {
        if (rpt[i] != rhs.rpt[i]) {
            std::printf("rpt not equal at %d rows, %d != %d\n", i, rpt[i], rhs.rpt[i]);
            if (++errors > 10) throw std::runtime_error("matrix compare: error num exceed threshold");
        }
    }
    for (mint p = 0; p < nnz; ++p) {
        const double d = std::fabs(val[p] - rhs.val[p]);
        if (col[p] != rhs.col[p] || !(d < eps || d < eps * std::fabs(val[p]))) {
            std::printf("entry %d differs: col %d/%d val %.18le/%.18le\n", p, col[p], rhs.col[p], val[p], rhs.val[p]);
            if (++errors > 10) throw std::runtime_error("matrix compare: error num exceed threshold");
        }
    }
    return errors == 0;
}

CSR::CSR(const std::string &mtx_file) { construct(mtx_file); }

// MatrixMarket coordinate file -> CSR (1-based indices converted to 0-based).  Symmetric
// and skew-symmetric files are expanded; entries are ordered by (row, col); the result
// must have strictly ascending, in-range columns per row.
void CSR::construct(const std::string &mtx_file)
{
    std::ifstream in(mtx_file);
    if (!in) throw std::runtime_error("unable to open file \"" + mtx_file + "\" for reading");
    io::MatrixMarketBanner banner;
    io::read_mm_banner(in, banner);
    std::string line;
    do {
        if (!std::getline(in, line)) throw std::runtime_error("missing MatrixMarket size line");
    } while (!line.empty() && line[0] == '%');
    std::vector<std::string> tok;
    io::tokenize(tok, line);
    if (tok.size() != 3) throw std::runtime_error("invalid MatrixMarket coordinate format");
    long long rows = std::stoll(tok[0]), cols = std::stoll(tok[1]), entries = std::stoll(tok[2]);
    if (rows < 0 || cols < 0 || entries < 0 || rows > 0x7fffffff || cols > 0x7fffffff)
        throw std::runtime_error("MatrixMarket size out of range");
    const bool pattern = banner.type == "pattern";
    const bool complex_ = banner.type == "complex";
    const bool sym = banner.symmetry != "general";
    const bool skew = banner.symmetry == "skew-symmetric";
    std::vector<long long> key;
    std::vector<mdouble> v;
    key.reserve(static_cast<std::size_t>(sym ? 2 * entries : entries));
    v.reserve(key.capacity());
    for (long long e = 0; e < entries; ++e) {
        long long i, j;
        double x = 1.0, im = 0.0;
        if (!(in >> i >> j)) throw std::runtime_error("read nnz not equal to declared nnz " + std::to_string(e));
        if (!pattern && !(in >> x)) throw std::runtime_error("missing value in MatrixMarket entry");
        if (complex_ && !(in >> im)) throw std::runtime_error("missing imaginary part in MatrixMarket entry");
        --i;
        --j;
        if (i < 0 || i >= rows || j < 0 || j >= cols) throw std::runtime_error("csr col_index out of range");
        key.push_back(i * cols + j);
        v.push_back(x);
        if (sym && i != j) {
            key.push_back(j * cols + i);
            v.push_back(skew ? -x : x);
        }
    }
    std::vector<std::size_t> order(key.size());
    std::iota(order.begin(), order.end(), std::size_t(0));
    std::stable_sort(order.begin(), order.end(), [&](std::size_t a, std::size_t b) { return key[a] < key[b]; });
    release();
    M = static_cast<mint>(rows);
    N = static_cast<mint>(cols);
    if (key.size() > 0x7fffffffull) throw std::runtime_error("MatrixMarket nnz exceeds INT32_MAX");
    nnz = static_cast<mint>(key.size());
    rpt = new mint[static_cast<std::size_t>(M) + 1]();
    col = new mint[static_cast<std::size_t>(nnz)];
    val = new mdouble[static_cast<std::size_t>(nnz)];
    for (std::size_t t = 0; t < order.size(); ++t) {
        const long long k = key[order[t]];
        rpt[k / cols + 1]++;
        col[t] = static_cast<mint>(k % cols);
        val[t] = v[order[t]];
    }
    for (mint i = 0; i < M; ++i) rpt[i + 1] += rpt[i];
    for (mint i = 0; i < M; ++i)
        for (mint p = rpt[i]; p + 1 < rpt[i + 1]; ++p)
            if (!(col[p] < col[p + 1])) throw std::runtime_error("csr col_index not in assending order");
}

}  // namespace opsparse
