/*
 * Drop-in ecl::BitArray of the GB300 wavelet tree.  Same public names and
 * bit layout as include/ecl_wavelet/bitarray/bit_array.cuh in
 * mfranzreb/ECL_wavelet: bit i of an array is bit i%32 of word i/32, each
 * array starts on a 32-word boundary.
 *
 * Either a non-owning view of the arrays a tree or a RankSelect keeps in
 * device memory, or (BitArray(sizes[, init_value]), bit_array.cuh:61,70)
 * the owner of new arrays on the current GPU, allocated by libewt.so
 * (ewt_bitarray_create), which the caller's kernels fill with writeWord /
 * writeWordAtBit and then move into a RankSelect.  Copies are shallow and
 * non-owning (as the reference's copy constructor), so the object can be
 * passed by value into kernels; copy assignment is deleted.
 */
#pragma once
#include <cstdint>
#include <stdexcept>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "ewt.h"
#include "ecl_wavelet/detail/device_ops.cuh"
#include "ecl_wavelet/utils/utils.cuh"

namespace ecl {

class RankSelect;

class BitArray {
 public:
  BitArray() = default;
  /* Non-owning view (used by RankSelect and WaveletTree). */
  __host__ BitArray(detail::RSView const& v, uint64_t const* host_bits)
      : v_(v), host_bits_(host_bits) {}

  /* sizes.size() arrays (at most 255) of sizes[a] bits each on the current
   * GPU, every bit zero (the reference leaves them uninitialised). */
  __host__ explicit BitArray(std::vector<size_t> const& sizes)
      : BitArray(sizes, false) {}
  /* The same with every bit set to init_value. */
  __host__ BitArray(std::vector<size_t> const& sizes, bool const init_value)
      : own_bits_(sizes.begin(), sizes.end()), owns_(true) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
      throw std::runtime_error("no CUDA device for the bit arrays");
    int const st = ewt_bitarray_create(
        own_bits_.data(), static_cast<uint32_t>(own_bits_.size()),
        init_value ? 1 : 0, dev, &handle_);
    if (st != EWT_OK) throw std::runtime_error(ewt_last_error());
    ewt_rs_get_device_view(handle_, &v_, sizeof(v_));
    host_bits_ = own_bits_.data();
  }

  BitArray& operator=(BitArray const&) = delete;
  __host__ BitArray(BitArray const& o) : v_(o.v_), host_bits_(o.host_bits_) {}
  __host__ BitArray(BitArray&& o) noexcept { take(std::move(o)); }
  __host__ BitArray& operator=(BitArray&& o) noexcept {
    if (this != &o) {
      release();
      take(std::move(o));
    }
    return *this;
  }
  __host__ ~BitArray() { release(); }

  /* Upper bound of the device bytes of num_arrays arrays of size bits. */
  __host__ static size_t getNeededGPUMemory(size_t const size,
                                            uint8_t const num_arrays) {
    uint64_t b = 0;
    ewt_needed_memory(EWT_MEM_BITARRAY, size, num_arrays, 0, &b);
    return b;
  }

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
  /* Writes word `index` of an array (its bit j is bit 32 * index + j). */
  __device__ void writeWord(size_t array_index, size_t index,
                            uint32_t value) {
    const_cast<uint32_t*>(v_.words)[v_.meta[array_index].word_off + index] =
        value;
  }
  /* Writes the word holding bit `index` of an array. */
  __device__ void writeWordAtBit(size_t array_index, size_t index,
                                 uint32_t value) {
    writeWord(array_index, index / 32, value);
  }
  __device__ void writeWordAtBit(size_t, size_t index, uint32_t value,
                                 size_t offset) {
    const_cast<uint32_t*>(v_.words)[offset + index / 32] = value;
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
  friend class RankSelect;
  __host__ void take(BitArray&& o) {
    v_ = o.v_;
    handle_ = o.handle_;
    owns_ = o.owns_;
    own_bits_ = std::move(o.own_bits_);
    host_bits_ = owns_ ? own_bits_.data() : o.host_bits_;
    o.handle_ = nullptr;
    o.owns_ = false;
  }
  __host__ void release() {
    if (owns_ && handle_) ewt_rs_free(handle_);
    handle_ = nullptr;
    owns_ = false;
  }

  detail::RSView v_{};
  uint64_t const* host_bits_ = nullptr;  // host copy of the array sizes
  ewt_rs* handle_ = nullptr;              // owned arrays (sizes constructors)
  std::vector<uint64_t> own_bits_;
  bool owns_ = false;
};

}  // namespace ecl
