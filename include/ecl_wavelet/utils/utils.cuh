/*
 * Drop-in utilities of the GB300 wavelet tree (mirrors the public names of
 * include/ecl_wavelet/utils/utils.cuh in mfranzreb/ECL_wavelet: the query
 * record, the integer helpers the tree walk depends on, and shareVar).
 */
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>

#ifndef WS
#define WS 32
#endif

namespace ecl {

/* One rank or select query: index_ is the position (rank) or the 1-based
 * occurrence number (select); symbol_ the symbol.  16 bytes for every T. */
template <typename T>
struct RankSelectQuery {
  size_t index_;
  T symbol_;
};

namespace utils {

static constexpr uint8_t kMinAlphabetSize = 2;

template <typename T>
__host__ __device__ inline bool isPowTwo(T const n) {
  static_assert(std::is_integral<T>::value && std::is_unsigned<T>::value,
                "T must be an unsigned integral type.");
  return (n & (n - 1)) == 0;
}

/* n/2 for powers of two, else the largest power of two below n; 0 for 0. */
template <typename T>
__host__ __device__ inline T getPrevPowTwo(T n) {
  static_assert(std::is_integral<T>::value && std::is_unsigned<T>::value,
                "T must be an unsigned integral type.");
  if (n == 0) return 0;
  if (isPowTwo(n)) return n >> 1;
  uint64_t const v = n;
#ifdef __CUDA_ARCH__
  return static_cast<T>(uint64_t(1) << (63 - __clzll(static_cast<long long>(v))));
#else
  return static_cast<T>(uint64_t(1) << (63 - __builtin_clzll(v)));
#endif
}

template <typename T>
__host__ __device__ inline T powTwo(T n) {
  return static_cast<T>(uint64_t(1) << n);
}

template <typename T>
__host__ __device__ inline uint8_t ceilLog2(T n) {
  uint64_t const v = n;
#ifdef __CUDA_ARCH__
  uint8_t const hi = 63 - __clzll(static_cast<long long>(v));
#else
  uint8_t const hi = 63 - __builtin_clzll(v);
#endif
  return isPowTwo<uint64_t>(v) ? hi : hi + 1;
}

template <typename T>
__host__ __device__ inline bool getBit(uint8_t const i, T const c) {
  return (c >> i) & 1;
}

/* Shares var from the (first) lane where condition holds to all lanes of
 * mask. */
template <typename T>
__device__ inline void shareVar(bool condition, T& var, uint32_t const mask) {
  __syncwarp(mask);
  uint32_t src = __ballot_sync(mask, condition);
  if (src != 0) var = __shfl_sync(mask, var, __ffs(src) - 1);
}

}  // namespace utils
}  // namespace ecl
