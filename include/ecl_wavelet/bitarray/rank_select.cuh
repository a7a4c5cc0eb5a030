/*
 * Drop-in ecl::RankSelect of the GB300 wavelet tree.
 *
 * Same public names as include/ecl_wavelet/bitarray/rank_select.cuh in
 * mfranzreb/ECL_wavelet: RSConfig, RankResult, the device rank<NumThreads,
 * GetBit, Value> / select<Value, NumThreads> calls and the index getters.
 * A RankSelect is either a member of a WaveletTree (a non-owning view) or a
 * standalone object built over caller bit arrays through libewt.so
 * (ewt_rs_build), which then owns the device memory.  Copies are shallow
 * and non-owning, so the object can be passed by value into kernels.
 *
 * With NumThreads > 1 an aligned group of NumThreads lanes answers one
 * query together, as in the reference: all of them call with the same
 * arguments and all of them get the answer; the block's words are split
 * among the lanes and select's searches probe NumThreads candidates per
 * round (detail::rs_rank1_coop / rs_select_coop).
 */
#pragma once
#include <cstdint>
#include <stdexcept>
#include <vector>

#include "ewt.h"
#include "ecl_wavelet/bitarray/bit_array.cuh"

namespace ecl {

struct RSConfig {
  static constexpr size_t L2_BIT_SIZE = 512;
  static constexpr size_t NUM_L2_PER_L1 = 128;
  static constexpr size_t L1_BIT_SIZE = NUM_L2_PER_L1 * L2_BIT_SIZE;
  static constexpr size_t L2_WORD_SIZE = L2_BIT_SIZE / 32;
  static constexpr size_t L1_WORD_SIZE = L1_BIT_SIZE / 32;
  static constexpr size_t SELECT_SAMPLE_RATE = 4096;
  using L1_TYPE = uint64_t;
  using L2_TYPE = uint16_t;
};

struct RankResult {
  size_t rank;
  bool bit;
};

class RankSelect {
 public:
  BitArray bit_array_;

  RankSelect() noexcept = default;

  /* Non-owning view (used by WaveletTree). */
  __host__ RankSelect(detail::RSView const& v, uint64_t const* host_bits)
      : bit_array_(v, host_bits), is_copy_(true) {}

  /* Standalone, from bit arrays the caller created with BitArray(sizes[,
   * init_value]) and filled on the device: takes them over and builds the
   * counts and samples in place (all device work is waited for first).
   * Throws std::runtime_error on failure (the reference's constructor is
   * noexcept and aborts). */
  __host__ RankSelect(BitArray&& bit_array, uint32_t const GPU_index)
      : is_copy_(false) {
    (void)GPU_index;  // the arrays stay on the GPU they were created on
    if (!bit_array.owns_ || !bit_array.handle_)
      throw std::runtime_error(
          "RankSelect(BitArray&&) needs a BitArray that owns its arrays");
    host_bits_ = std::move(bit_array.own_bits_);
    handle_ = bit_array.handle_;
    bit_array.handle_ = nullptr;
    bit_array.owns_ = false;
    int const st = ewt_rs_build_in_place(handle_);
    if (st != EWT_OK) throw std::runtime_error(ewt_last_error());
    detail::RSView v;
    ewt_rs_get_device_view(handle_, &v, sizeof(v));
    bit_array_ = BitArray(v, host_bits_.data());
  }

  /* Standalone: bit arrays given as packed words (host or device memory),
   * one array after the other, ceil(bits[a]/32) words each. */
  __host__ RankSelect(uint32_t const* words, std::vector<size_t> const& bits,
                      uint32_t GPU_index)
      : host_bits_(bits.begin(), bits.end()), is_copy_(false) {
    std::vector<uint64_t> b(bits.begin(), bits.end());
    int const st = ewt_rs_build(words, b.data(),
                                static_cast<uint32_t>(b.size()),
                                static_cast<int>(GPU_index), &handle_);
    if (st != EWT_OK) throw std::runtime_error(ewt_last_error());
    detail::RSView v;
    ewt_rs_get_device_view(handle_, &v, sizeof(v));
    bit_array_ = BitArray(v, host_bits_.data());
  }

  __host__ RankSelect(RankSelect const& o)
      : bit_array_(o.bit_array_), handle_(o.handle_), is_copy_(true) {}
  RankSelect& operator=(RankSelect const&) = delete;
  __host__ RankSelect& operator=(RankSelect&& o) noexcept {
    if (this != &o) {
      release();
      bit_array_ = BitArray(o.bit_array_);  // a non-owning copy
      handle_ = o.handle_;
      host_bits_ = std::move(o.host_bits_);
      is_copy_ = o.is_copy_;
      if (!host_bits_.empty())
        bit_array_ = BitArray(o.bit_array_.view(), host_bits_.data());
      o.is_copy_ = true;
      o.handle_ = nullptr;
    }
    return *this;
  }
  __host__ ~RankSelect() { release(); }

  /* Number of Value bits in [0, index) of one array; with GetBit also the
   * bit at index (false when index == size). */
  template <int NumThreads, bool GetBit, int Value>
  __device__ auto rank(uint8_t array_index, size_t index, size_t /*offset*/) {
    static_assert(Value == 0 || Value == 1, "Value must be 0 or 1.");
    static_assert(NumThreads >= 1 && NumThreads <= 32 && 32 % NumThreads == 0,
                  "NumThreads must divide 32");
    detail::RSView const& v = bit_array_.view();
    detail::ArrayMeta const m = v.meta[array_index];
    bool bit = false;
    size_t r1;
    if constexpr (NumThreads > 1)
      r1 = detail::rs_rank1_coop<GetBit>(detail::LaneGroup<NumThreads>(), v, m,
                                         index, &bit);
    else
      r1 = detail::rs_rank1<GetBit>(v, m, index, &bit);
    size_t const r = Value ? r1 : index - r1;
    if constexpr (GetBit) {
      return RankResult{r, bit};
    } else {
      return r;
    }
  }

  /* Position of the i-th (1-based) Value bit, or the array size. */
  template <uint32_t Value, int NumThreads, bool UseSamples = true>
  __device__ size_t select(uint32_t array_index, size_t i,
                           size_t /*BA_offset*/) {
    static_assert(Value == 0 || Value == 1, "Value must be 0 or 1.");
    static_assert(NumThreads >= 1 && NumThreads <= 32 && 32 % NumThreads == 0,
                  "NumThreads must divide 32");
    detail::RSView const& v = bit_array_.view();
    if constexpr (NumThreads > 1)
      return detail::rs_select_coop<int(Value)>(detail::LaneGroup<NumThreads>(), v,
                                                v.meta[array_index], i);
    else
      return detail::rs_select<int(Value)>(v, v.meta[array_index], i);
  }

  __device__ size_t getNumL1Blocks(uint32_t a) const {
    return bit_array_.view().meta[a].num_l1;
  }
  __device__ size_t getNumL2Blocks(uint32_t a) const {
    detail::ArrayMeta const& m = bit_array_.view().meta[a];
    return (m.num_l1 - 1) * RSConfig::NUM_L2_PER_L1 + m.num_last_l2;
  }
  __device__ size_t getNumLastL2Blocks(uint32_t a) const {
    return bit_array_.view().meta[a].num_last_l2;
  }
  template <uint32_t Value>
  __device__ size_t getTotalNumVals(uint32_t a) const {
    detail::ArrayMeta const& m = bit_array_.view().meta[a];
    return Value ? m.ones : m.bits - m.ones;
  }
  template <uint32_t Value>
  __device__ size_t getSelectSample(uint32_t a, size_t index) const {
    detail::RSView const& v = bit_array_.view();
    return Value ? v.s1[v.meta[a].s1_off + index]
                 : v.s0[v.meta[a].s0_off + index];
  }
  /* Upper bound of the device bytes of num_arrays arrays of size bits with
   * their rank/select support. */
  __host__ static size_t getNeededGPUMemory(size_t const size,
                                            uint8_t const num_arrays) {
    uint64_t b = 0;
    ewt_needed_memory(EWT_MEM_RANKSELECT, size, num_arrays, 0, &b);
    return b;
  }

  __device__ RSConfig::L1_TYPE getL1Entry(uint32_t a, size_t index) const {
    detail::RSView const& v = bit_array_.view();
    return v.l1[v.meta[a].l1_off + index];
  }
  __device__ size_t getL2Entry(uint32_t a, size_t index) const {
    detail::RSView const& v = bit_array_.view();
    return v.l2[v.meta[a].l2_off + index];
  }

 private:
  void release() {
    if (!is_copy_ && handle_) ewt_rs_free(handle_);
    handle_ = nullptr;
  }
  ewt_rs* handle_ = nullptr;
  std::vector<uint64_t> host_bits_;
  bool is_copy_ = true;
};

}  // namespace ecl
