// config.hpp — tunables of the drop-in API (compare OpSparse include/opsparse/utils/config.hpp:6-33).
// kNumBin keeps OpSparse's value, so arrays a caller sizes with it stay the same size.  The
// GB300 library sorts rows into seven classes by their intermediate-product count ("flop");
// they fill the first seven bins (SpgemmMeta::bin_size), and the eighth stays empty.  The
// class bounds below are the defaults; ops_handle_set_thresholds changes them at run time.
#ifndef OPSPARSE_UTILS_CONFIG_HPP_
#define OPSPARSE_UTILS_CONFIG_HPP_

namespace opsparse {

inline constexpr int kNumBin = 8;           // bins in SpgemmMeta; classes R8, R16, R32, W, E1, E2, D, (empty)
inline constexpr int kWarpSize = 32;
inline constexpr int kRegFlopMax = 32;      // R8/R16/R32: 8, 16 or 32 lanes per row, registers only
inline constexpr int kWarpFlopMax = 128;    // W: one warp per row, register bitonic sort
inline constexpr int kEsc1FlopMax = 1024;   // E1: warp sort, warp hash table or CTA expand/sort/compress
inline constexpr int kEsc2FlopMax = 13312;  // E2: CTA expand/sort/compress; above: whole-GPU sort (D)

template <typename Int>
inline constexpr Int div_up(Int a, Int b)
{
    return (a + b - 1) / b;
}

}  // namespace opsparse

#endif  // OPSPARSE_UTILS_CONFIG_HPP_
