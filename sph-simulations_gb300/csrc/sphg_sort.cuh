// sphg_sort.cuh -- host interface of the radix sort in sphg_sort.cu.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sphg {

int sort_num_tiles(int64_t n);
// 32-bit words of scratch radix_sort_pairs needs for n keys: digit histograms,
// tile counters, an error word, and the look-back words of every tile and pass.
size_t sort_scratch_words(int64_t n);
constexpr size_t sort_scratch_words_c(int64_t n) {
  return (size_t)4 * 256 + 256 + (size_t)4 * 256 * (size_t)((n + 2047) / 2048);
}
// The word radix_sort_pairs sets to 1 when a look-back wait gave up (never cleared by it).
uint32_t* sort_error_word(uint32_t* scratch);

// Stable sort of (keys_in, vals_in) on the low `bits` bits; vals_in == nullptr
// means the identity 0..n-1.  keys_tmp/vals_tmp are ping-pong buffers of n
// entries (unused for bits <= 8).  The result lands in keys_out/vals_out.
// No buffer may alias another.  When epoch is not null the first pass
// increments *epoch once (the step epoch of the cell-range table).  hist, when
// not null, holds the digit histograms of all passes already ([4][256], digit
// d of pass p at p*256 + d, summed over all keys); otherwise they are computed.
// When *skip (device word, read by the kernels) is non-zero the kernels return
// at once: the step's incremental re-sort produced the result instead.
// clear_err: zero the error word first (stand-alone sorts, whose callers have
// no handle that reports it).  n must not exceed kSortMaxKeys.
cudaError_t radix_sort_pairs(const uint32_t* keys_in, const uint32_t* vals_in,
                             uint32_t* keys_out, uint32_t* vals_out, uint32_t* keys_tmp,
                             uint32_t* vals_tmp, uint32_t* scratch, int64_t n, int bits,
                             cudaStream_t stream, uint32_t* epoch = nullptr,
                             const uint32_t* hist = nullptr, const uint32_t* skip = nullptr,
                             bool clear_err = false);
// Largest n the sort accepts: a look-back word keeps a running count in 30 bits
// under its two flag bits.
constexpr int64_t kSortMaxKeys = ((int64_t)1 << 30) - 1;
constexpr int kSortMaxPasses = 4;

}  // namespace sphg
