// matrix_market.hpp — MatrixMarket banner parsing (same names as OpSparse's
// include/opsparse/io/matrix_market.hpp:11-65): coordinate storage; real, integer,
// pattern and complex (real part) values; general, symmetric and skew-symmetric layout.
#ifndef OPSPARSE_IO_MATRIX_MARKET_HPP_
#define OPSPARSE_IO_MATRIX_MARKET_HPP_

#include <algorithm>
#include <cctype>
#include <istream>
#include <stdexcept>
#include <string>
#include <vector>

namespace opsparse::io {

struct MatrixMarketBanner {
    std::string matrix;    // "matrix"
    std::string storage;   // "coordinate"
    std::string type;      // "real", "integer", "pattern", "complex"
    std::string symmetry;  // "general", "symmetric", "skew-symmetric"
};

// Splits str at any of the delimiter characters, dropping empty fields.
inline void tokenize(std::vector<std::string> &tokens, const std::string &str, const std::string &delimiters = "\n\r\t ")
{
    tokens.clear();
    std::size_t pos = 0;
    while (pos < str.size()) {
        const std::size_t b = str.find_first_not_of(delimiters, pos);
        if (b == std::string::npos) break;
        const std::size_t e = str.find_first_of(delimiters, b);
        tokens.push_back(str.substr(b, e == std::string::npos ? std::string::npos : e - b));
        if (e == std::string::npos) break;
        pos = e;
    }
}

inline std::string lowercase(std::string s)
{
    std::transform(s.begin(), s.end(), s.begin(), [](unsigned char c) { return static_cast<char>(std::tolower(c)); });
    return s;
}

template <typename Stream>
inline void read_mm_banner(Stream &input, MatrixMarketBanner &banner)
{
    std::string line;
    std::vector<std::string> t;
    std::getline(input, line);
    tokenize(t, line);
    if (t.size() != 5 || t[0] != "%%MatrixMarket") throw std::runtime_error("invalid MatrixMarket banner");
    banner.matrix = lowercase(t[1]);
    banner.storage = lowercase(t[2]);
    banner.type = lowercase(t[3]);
    banner.symmetry = lowercase(t[4]);
    if (banner.matrix != "matrix") throw std::runtime_error("not impl matrix type: " + banner.matrix);
    if (banner.storage != "coordinate") throw std::runtime_error("not impl storage type " + banner.storage);
    if (banner.type != "real" && banner.type != "integer" && banner.type != "pattern" && banner.type != "complex")
        throw std::runtime_error("invalid MatrixMarket data type [" + banner.type + "]");
    if (banner.symmetry != "general" && banner.symmetry != "symmetric" && banner.symmetry != "skew-symmetric")
        throw std::runtime_error("invalid or unsupported MatrixMarket symmetry [" + banner.symmetry + "]");
}

}  // namespace opsparse::io

#endif  // OPSPARSE_IO_MATRIX_MARKET_HPP_
