/*
 * Drop-in ecl::BitArray of the GB300 wavelet tree: a non-owning view of the
 * packed bit arrays a tree (or a standalone RankSelect) keeps in device
 * memory.  Same public names and bit layout as
 * include/ecl_wavelet/bitarray/bit_array.cuh in mfranzreb/ECL_wavelet: bit
 * i of an array is bit i%32 of word i/32, each array starts on a 32-word
 * boundary.  Passed by value into kernels.
 */
#pragma once
#include <cstdint>

#include "ecl_wavelet/detail/device_ops.cuh"
#include "ecl_wavelet/utils/utils.cuh"

namespace ecl {

class BitArray {
 public:
  BitArray() = default;
  __host__ BitArray(detail::RSView const& v, uint64_t const* host_bits)
      : v_(v), host_bits_(host_bits) {}

  __device__ bool access(size_t array_index, size_t index) const {
    return ecl::detail::rs_bit(v_, v_.meta[array_index], index);
  }
  __device__ bool access(size_t array_index, size_t index,
                         size_t offset) const {
    return (v_.words[offset + (index >> 5)] >> (index & 31)) & 1u;
  }
  __device__ uint32_t word(size_t array_index, size_t index) const {
    return v_.words[v_.meta[array_index].word_off + index];
  }
  __device__ uint32_t word(size_t, size_t index, size_t offset) const {
    return v_.words[offset + index];
  }
  /* index must be even: words index and index+1 as one uint64. */
  __device__ uint64_t twoWords(size_t array_index, size_t index) const {
    return reinterpret_cast<uint64_t const*>(
        v_.words)[(v_.meta[array_index].word_off + index) / 2];
  }
  __device__ uint64_t twoWords(size_t, size_t index, size_t offset) const {
    return reinterpret_cast<uint64_t const*>(v_.words)[(offset + index) / 2];
  }
  __device__ uint32_t wordAtBit(size_t array_index, size_t index) const {
    return word(array_index, index / 32);
  }
  __device__ uint32_t partialWord(uint32_t w, uint8_t bit_index) const {
    return bit_index >= 32 ? w : (w & ((1u << bit_index) - 1u));
  }
  __device__ uint64_t partialTwoWords(uint64_t w, uint8_t bit_index) const {
    return bit_index >= 64 ? w : (w & ((uint64_t(1) << bit_index) - 1));
  }
  __device__ size_t getOffset(size_t array_index) const {
    return v_.meta[array_index].word_off;
  }
  __host__ __device__ size_t size(size_t array_index) const {
#ifdef __CUDA_ARCH__
    return v_.meta[array_index].bits;
#else
    return host_bits_[array_index];
#endif
  }
  __device__ size_t sizeInWords(size_t array_index) const {
    return (v_.meta[array_index].bits + 31) / 32;
  }
  __host__ __device__ uint8_t numArrays() const {
    return static_cast<uint8_t>(v_.num_arrays);
  }
  __host__ __device__ detail::RSView const& view() const { return v_; }

 private:
  detail::RSView v_{};
  uint64_t const* host_bits_ = nullptr;  // host copy owned by the tree
};

}  // namespace ecl
