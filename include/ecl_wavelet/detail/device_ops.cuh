/*
 * Device-side data views and query primitives of the GB300 wavelet tree.
 *
 * Shared by the library's own kernels (libewt.so) and by the drop-in C++
 * headers, so a user kernel that receives an ecl::WaveletTree<T> by value
 * runs exactly the code the batch kernels run.
 *
 * Format (kept identical to mfranzreb/ECL_wavelet so exports compare
 * byte-for-byte):
 *   - a bit array stores bit i in bit i%32 of uint32 word i/32
 *     (include/ecl_wavelet/bitarray/bit_array.cuh:39-46); each array starts
 *     on a 32-word (128-byte) boundary (src/bitarray/bit_array.cu:62-68);
 *   - L1: uint64 count of ones before every 65,536-bit block; L2: uint16
 *     count of ones since the enclosing L1 block, per 512-bit block; select
 *     samples: position of every 4096-th one / zero
 *     (include/ecl_wavelet/bitarray/rank_select.cuh:44-64).
 */
#pragma once
#include <cstdint>

#ifndef __CUDACC__
#error "device_ops.cuh must be compiled by nvcc"
#endif

namespace ecl {
namespace detail {

constexpr uint64_t kL1Bits = 65536;
constexpr uint64_t kL2Bits = 512;
constexpr uint64_t kL2PerL1 = 128;
constexpr uint64_t kL2Words = kL2Bits / 32;
constexpr uint64_t kSampleRate = 4096;
constexpr uint32_t kMaxLevels = 64;

/* Per bit array bookkeeping; one entry per level of a tree. */
struct ArrayMeta {
  uint64_t word_off;    // first word of the array inside RSView::words
  uint64_t bits;        // array length in bits
  uint64_t l1_off;      // first L1 entry
  uint64_t l2_off;      // first L2 entry
  uint64_t s0_off;      // first zero-sample
  uint64_t s1_off;      // first one-sample
  uint64_t ones;        // total number of ones
  uint64_t num_l1;      // number of L1 blocks
  uint64_t num_last_l2; // L2 blocks inside the last L1 block
  uint64_t rb_off;      // first rank block (32-byte sector) of the array
  uint64_t rbh_off;     // first high-count entry of the array
  uint64_t ds0_off;     // first dense zero-sample (rank-block index, u32)
  uint64_t ds1_off;     // first dense one-sample
};

/* Query-side rank blocks: each 32-byte block (one DRAM sector) holds the low
 * 32 bits of the number of ones before its first bit followed by 224 bits of
 * the array, so a rank reads one sector.  The high part comes from a small
 * table with the full count before every 2^24-th block (within 2^24 blocks
 * the count grows by less than 2^32, so the low word fixes it; arrays shorter
 * than 2^24 blocks never read the table).  An auxiliary copy next to the
 * reference-format arrays, which stay the source of truth for exports and
 * select. */
constexpr uint64_t kRankBlockBits = 224;
constexpr uint64_t kRankBlockWords = kRankBlockBits / 32;
constexpr uint32_t kRankHighShift = 24;

/* Dense select samples (query side, next to the rank blocks): for every
 * R-th zero / one (R = 2^sel_shift; entry j covers the (j*R+1)-th) the index
 * of the rank block holding it, relative to the array's first block.  A
 * select reads two neighbouring entries, which bracket its block, and then
 * one or two rank blocks; sel_shift = 0 means none were built and select
 * uses the reference-format samples and counts. */
constexpr uint32_t kDefaultSelShift = 8;

/* rb_off / ds0_off of an array without rank blocks / dense samples (binary
 * levels that group levels cover); rank and select then use L1/L2. */
constexpr uint64_t kNoBlocks = ~uint64_t(0);

/* A set of bit arrays with rank/select support, all in device memory. */
struct RSView {
  const uint32_t* words;
  const uint64_t* l1;
  const uint16_t* l2;
  const uint64_t* s0;
  const uint64_t* s1;
  const ArrayMeta* meta;  // device array of num_arrays entries
  const uint4* rb;        // rank blocks (2 uint4 per block), may be null
  const uint64_t* rbh;    // high counts of the rank blocks
  const uint32_t* ds;     // dense select samples (ArrayMeta::ds0/ds1_off)
  uint32_t num_arrays;
  uint32_t sel_shift;     // log2 of the dense sample rate; 0 = none
};

/* Group levels of power-of-two alphabets (query side, no reference
 * counterpart).  A group level covers w = 2 or 3 consecutive binary levels
 * starting at level l: in level-l order it holds each symbol's w-bit digit
 * (bits l .. l+w-1 counted from the top), so one read resolves w binary
 * levels.  Storage: 32-byte blocks; a block holds, before its digits, the
 * counts of digits 0 .. 2^w - 2 since the start of its superblock (uint16;
 * the last digit's follows), and a superblock table holds the 2^w digit
 * counts before every superblock (uint64).
 *   w = 2 (quad): bits 0..47 counts, bits 64..255 96 digits (digit t at bit
 *         64 + 2t), 512 blocks per superblock (49,152 digits);
 *   w = 3 (octal): three 42-bit planes (bit 2, 1, 0 of each digit; digit t
 *         at bit t) in the low bits of words 1..3, counts of digits 0..3 in
 *         word 0 and of digits 4..6 in bits 42..57 of words 1..3; 512 blocks
 *         per superblock (21,504 digits).
 * Dense select samples per digit name the block holding every R-th
 * occurrence (uint32); node_ranks[group][node][digit] = occurrences of the
 * digit before the node. */
template <int W> struct GroupShape;
template <> struct GroupShape<2> {
  static constexpr uint32_t kDigits = 96, kSbBlocks = 512;
};
template <> struct GroupShape<3> {
  static constexpr uint32_t kDigits = 42, kSbBlocks = 512;
};
constexpr uint32_t kQuadDigits = GroupShape<2>::kDigits;
constexpr uint32_t kQuadSbBlocks = GroupShape<2>::kSbBlocks;
constexpr uint64_t kQuadSbDigits = uint64_t(kQuadDigits) * kQuadSbBlocks;

struct GroupLevel {
  uint64_t blk_off;     // first block (2 uint4 each)
  uint64_t sb_off;      // first superblock-table word (2^width per superblock)
  uint64_t ds_off[8];   // first dense sample of each digit
  uint64_t total[8];    // occurrences of each digit
  uint64_t nr_off;      // first node-rank entry (2^width per node)
  uint64_t num_blocks;  // n / digits-per-block + 1 (position n is addressable)
  uint32_t width;       // digit bits: 2 or 3
  uint32_t start;       // first binary level of the group
  uint32_t sel_shift;   // log2 of its dense sample rate (0: no samples)
  uint32_t reserved;
};

struct GroupView {
  const uint4* blocks;
  const uint64_t* sb;
  const uint32_t* ds;          // null: select searches the superblocks
  const uint64_t* node_ranks;
  const GroupLevel* levels;     // device array of num entries
  uint32_t num;                // group levels (0: the tree has none)
  uint32_t covered;            // binary levels they cover (the rest: binary)
};

/* Everything a query walk needs; trivially copyable into a kernel. */
struct TreeView {
  RSView rs;
  const uint64_t* counts;          // C[c]: symbols smaller than c, sigma entries
  const uint64_t* node_ranks;      // rank0 at every node start, num_ranks
  const uint64_t* node_base;       // node starts on levels < l, levels + 1
  const uint64_t* nodes_at_level;  // node starts on level l, levels
  const uint64_t* code_len;        // short codes of symbols >= codes_start
  const uint64_t* code_bits;
  const void* alphabet;            // sorted original symbols, elem_size each
  uint64_t n;
  uint64_t sigma;
  uint64_t codes_start;
  uint64_t num_ranks;
  uint64_t num_nodes_until_last_level;
  uint32_t levels;
  uint32_t elem_size;
  uint32_t is_pow2;
  uint32_t is_min;
  GroupView groups;                 // group (octal / quad) levels over the binary ones
};

/* ---------------------------------------------------------------------- */
__device__ __forceinline__ uint32_t popc32(uint32_t x) { return __popc(x); }

__device__ __forceinline__ bool is_pow2_u64(uint64_t n) {
  return (n & (n - 1)) == 0;
}

/* n/2 for powers of two, else the largest power of two below n
 * (semantics of utils.cuh:123-146 getPrevPowTwo). */
__device__ __forceinline__ uint64_t prev_pow2_u64(uint64_t n) {
  if (n == 0) return 0;
  if (is_pow2_u64(n)) return n >> 1;
  return uint64_t(1) << (63 - __clzll(static_cast<long long>(n)));
}

/* Position (0-based) of the r-th (1-based) set bit of x; r <= popc(x). */
__device__ __forceinline__ uint32_t select_in_word(uint32_t x, uint32_t r) {
  uint32_t pos = 0;
  uint32_t c = __popc(x & 0xFFFFu);
  if (r > c) { r -= c; x >>= 16; pos += 16; }
  c = __popc(x & 0xFFu);
  if (r > c) { r -= c; x >>= 8; pos += 8; }
  c = __popc(x & 0xFu);
  if (r > c) { r -= c; x >>= 4; pos += 4; }
  c = __popc(x & 0x3u);
  if (r > c) { r -= c; x >>= 2; pos += 2; }
  c = x & 1u;
  if (r > c) pos += 1;
  return pos;
}

__device__ __forceinline__ bool rs_bit(const RSView& v, const ArrayMeta& m,
                                       uint64_t pos) {
  return (__ldg(v.words + m.word_off + (pos >> 5)) >> (pos & 31)) & 1u;
}

/* Ones before rank block k of an array whose header holds the low word lo:
 * the high part comes from the high-count table for k >= 2^24. */
__device__ __forceinline__ uint64_t rb_ones_before(const RSView& v,
                                                   const ArrayMeta& m,
                                                   uint64_t k, uint32_t lo) {
  uint64_t const hj = k >> kRankHighShift;
  if (!hj) return lo;
  uint64_t const h = __ldg(v.rbh + m.rbh_off + hj);
  return h + static_cast<uint32_t>(lo - static_cast<uint32_t>(h));
}

/* Ones in [0, pos) of one array, pos <= bits; with GetBit also the bit at
 * pos (false for pos == bits).  Loads the L1 entry, the L2 entry and the
 * 128-bit chunks of the 512-bit block up to pos, all independent. */
template <bool GetBit>
__device__ __forceinline__ uint64_t rs_rank1(const RSView& v,
                                             const ArrayMeta& m, uint64_t pos,
                                             bool* bit) {
  if (pos >= m.bits) {
    if (GetBit) *bit = false;
    return m.ones;
  }
  if (v.rb && m.rb_off != kNoBlocks) {
    // One 32-byte block: low word of the ones before it + 7 data words.
    uint64_t const blk = pos / kRankBlockBits;
    uint32_t const off = static_cast<uint32_t>(pos - blk * kRankBlockBits);
    uint4 const* line = v.rb + (m.rb_off + blk) * 2;
    uint32_t const wi = off >> 5;
    uint4 const q0 = __ldg(line);
    uint4 const q1 = __ldg(line + 1);
    uint32_t const w[kRankBlockWords] = {q0.y, q0.z, q0.w, q1.x,
                                         q1.y, q1.z, q1.w};
    uint32_t acc = 0, cur = 0;
#pragma unroll
    for (uint32_t j = 0; j < kRankBlockWords; ++j) {
      acc += j < wi ? __popc(w[j]) : 0u;
      cur = j == wi ? w[j] : cur;
    }
    acc += __popc(cur & ((1u << (off & 31)) - 1u));
    if (GetBit) *bit = (cur >> (off & 31)) & 1u;
    return rb_ones_before(v, m, blk, q0.x) + acc;
  }
  uint64_t const b2 = pos >> 9;
  uint64_t r = __ldg(v.l1 + m.l1_off + (pos >> 16));
  r += __ldg(v.l2 + m.l2_off + b2);
  uint4 const* blk =
      reinterpret_cast<uint4 const*>(v.words + m.word_off + b2 * kL2Words);
  uint32_t const off = static_cast<uint32_t>(pos & 511);
  uint32_t const last = off >> 7;
  uint32_t acc = 0;
#pragma unroll
  for (uint32_t j = 0; j < 4; ++j) {
    if (j < last) {
      uint4 const q = __ldg(blk + j);
      acc += __popc(q.x) + __popc(q.y) + __popc(q.z) + __popc(q.w);
    } else if (j == last && (GetBit || (off & 127) != 0)) {
      uint4 const q = __ldg(blk + j);
      uint32_t const o = off & 127;
      uint32_t const wi = o >> 5;
      uint32_t const w = wi == 0 ? q.x : wi == 1 ? q.y : wi == 2 ? q.z : q.w;
      acc += (wi > 0 ? __popc(q.x) : 0) + (wi > 1 ? __popc(q.y) : 0) +
             (wi > 2 ? __popc(q.z) : 0);
      acc += __popc(w & ((1u << (o & 31)) - 1u));
      if (GetBit) *bit = (w >> (o & 31)) & 1u;
    }
  }
  return r + acc;
}

/* rs_select through the dense samples and rank blocks, 0 < i <= total:
 * two sample entries bracket the rank block holding the i-th `Value` bit;
 * a binary search over block headers narrows wider brackets to two blocks,
 * both read at once; the block whose count before it is below i holds it. */
template <int Value>
__device__ __forceinline__ uint64_t rs_select_dense(const RSView& v,
                                                    const ArrayMeta& m,
                                                    uint64_t i, uint64_t total) {
  uint32_t const* S = v.ds + (Value ? m.ds1_off : m.ds0_off);
  uint32_t const sh = v.sel_shift;
  uint64_t const j = (i - 1) >> sh;
  uint64_t const nblk = (m.bits + kRankBlockBits - 1) / kRankBlockBits;
  // entries name blocks of this array; the clamps keep every read inside it
  uint64_t lo = min(uint64_t(__ldg(S + j)), nblk - 1);
  uint64_t hi = ((j + 1) << sh) < total ? __ldg(S + j + 1) : nblk - 1;
  hi = min(max(hi, lo), nblk - 1);
  uint4 const* rb = v.rb + m.rb_off * 2;
  // value bits before block k given its header word
  auto before = [&](uint64_t k, uint32_t h) -> uint64_t {
    uint64_t const ones = rb_ones_before(v, m, k, h);
    return Value ? ones : k * kRankBlockBits - ones;
  };
  while (hi - lo > 16) {  // wide brackets only (sparse values)
    uint64_t const mid = (lo + hi + 1) >> 1;
    uint32_t const h = __ldg(reinterpret_cast<uint32_t const*>(rb + mid * 2));
    if (before(mid, h) < i) lo = mid; else hi = mid - 1;
  }
  // from the interpolated block, one block at a time (query throughput
  // follows the sectors read): the block holding the i-th value bit has
  // fewer than i of them before it and at least i up to its end
  uint64_t t = hi - lo > 1 && hi - lo <= 16
                   ? lo + (((hi - lo) * ((i - 1) - (j << sh))) >> sh)
                   : lo;
  uint4 b0, b1;
  uint64_t bt = 0;
  for (uint32_t guard = 0; guard < 24; ++guard) {
    b0 = __ldg(rb + t * 2);
    b1 = __ldg(rb + t * 2 + 1);
    bt = before(t, b0.x);
    if (bt >= i && t > lo) {  // it lies before this block
      hi = t - 1;
      --t;
      continue;
    }
    if (t < hi) {  // t is a full block
      uint32_t const ones_in = __popc(b0.y) + __popc(b0.z) + __popc(b0.w) +
                               __popc(b1.x) + __popc(b1.y) + __popc(b1.z) + __popc(b1.w);
      uint32_t const in = Value ? ones_in : uint32_t(kRankBlockBits) - ones_in;
      if (bt + in < i) {  // after it
        lo = t + 1;
        ++t;
        continue;
      }
    }
    break;
  }
  uint32_t r = static_cast<uint32_t>(i - bt);  // 1 ..= kRankBlockBits
  uint32_t const w[kRankBlockWords] = {b0.y, b0.z, b0.w, b1.x,
                                       b1.y, b1.z, b1.w};
  uint32_t sel = 0, wj = 0;
  bool found = false;
#pragma unroll
  for (uint32_t q = 0; q < kRankBlockWords; ++q) {
    uint32_t const x = Value ? w[q] : ~w[q];
    uint32_t const c = __popc(x);
    if (!found) {
      if (r <= c) {
        found = true;
        sel = x;
        wj = q;
      } else {
        r -= c;
      }
    }
  }
  if (!found) return m.bits;  // not reached for valid structures
  return t * kRankBlockBits + wj * 32 + select_in_word(sel, r);
}

/* Position of the i-th (1-based) `Value` bit, or bits when there are fewer
 * (or i == 0).  With dense samples: rs_select_dense.  Otherwise sample
 * bracket -> L1 binary search -> L2 binary search in the bracketed range ->
 * scan of the 512-bit block -> in-word select. */
template <int Value>
__device__ __forceinline__ uint64_t rs_select(const RSView& v,
                                              const ArrayMeta& m, uint64_t i) {
  uint64_t const total = Value ? m.ones : m.bits - m.ones;
  if (i == 0 || i > total) return m.bits;
  if (v.sel_shift && m.ds0_off != kNoBlocks)
    return rs_select_dense<Value>(v, m, i, total);
  uint64_t const* S = Value ? v.s1 + m.s1_off : v.s0 + m.s0_off;
  uint64_t const q = i / kSampleRate;
  uint64_t const lo = q ? __ldg(S + q - 1) : 0;
  uint64_t const hi = (q + 1) * kSampleRate <= total ? __ldg(S + q) : m.bits - 1;
  uint64_t const* L1 = v.l1 + m.l1_off;
  uint64_t b_lo = lo >> 16, b_hi = hi >> 16;
  // Invariant: values before block b_lo < i.
  while (b_lo < b_hi) {
    uint64_t const mid = (b_lo + b_hi + 1) >> 1;
    uint64_t const x = __ldg(L1 + mid);
    uint64_t const before = Value ? x : (mid << 16) - x;
    if (before < i) b_lo = mid; else b_hi = mid - 1;
  }
  uint64_t const b = b_lo;
  uint64_t const xb = __ldg(L1 + b);
  uint64_t rem = i - (Value ? xb : (b << 16) - xb);
  uint64_t const first = b * kL2PerL1;
  uint64_t const num_l2 = (m.num_l1 - 1) * kL2PerL1 + m.num_last_l2;
  uint64_t k_lo = ((lo >> 16) == b) ? (lo >> 9) : first;
  uint64_t k_hi = first + kL2PerL1 - 1;
  if (k_hi > num_l2 - 1) k_hi = num_l2 - 1;
  if ((hi >> 16) == b && (hi >> 9) < k_hi) k_hi = hi >> 9;
  uint16_t const* L2 = v.l2 + m.l2_off;
  while (k_lo < k_hi) {
    uint64_t const mid = (k_lo + k_hi + 1) >> 1;
    uint32_t const x = __ldg(L2 + mid);
    uint64_t const before = Value ? x : ((mid - first) << 9) - x;
    if (before < rem) k_lo = mid; else k_hi = mid - 1;
  }
  uint32_t const xk = __ldg(L2 + k_lo);
  rem -= Value ? xk : ((k_lo - first) << 9) - xk;
  uint4 const* blk =
      reinterpret_cast<uint4 const*>(v.words + m.word_off + k_lo * kL2Words);
  uint4 qs[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) qs[j] = __ldg(blk + j);
  uint32_t r = static_cast<uint32_t>(rem);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    uint32_t ws[4] = {qs[j].x, qs[j].y, qs[j].z, qs[j].w};
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      uint32_t const w = Value ? ws[t] : ~ws[t];
      uint32_t const c = __popc(w);
      if (r <= c) {
        return (k_lo * kL2Words + j * 4 + t) * 32 + select_in_word(w, r);
      }
      r -= c;
    }
  }
  return m.bits;  // not reached for valid structures
}

/* ---- cooperative rank/select (NumThreads lanes per query) -------------
 * The lanes of an aligned group of N lanes (N divides 32) answer one query
 * together, as RankSelect::rank<N, ...> / select<Value, N> of the reference
 * (rank_select.cuh:125-208, 224-523): every lane of the group calls with
 * the same arguments and every lane gets the answer.  Searches probe N
 * candidates per dependent round instead of one; the words of a block are
 * split among the lanes and combined with shuffles inside the group. */
template <int N>
struct LaneGroup {
  static_assert(N >= 1 && N <= 32 && (32 % N) == 0, "N must divide 32");
  uint32_t t, base, mask;
  __device__ __forceinline__ LaneGroup() {
    uint32_t const lane = threadIdx.x & 31u;
    t = lane % N;
    base = lane - t;
    mask = N == 32 ? 0xFFFFFFFFu : ((1u << N) - 1u) << base;
  }
  /* bit j set when lane j of the group has p */
  __device__ __forceinline__ uint32_t ballot(bool p) const {
    return (__ballot_sync(mask, p) & mask) >> base;
  }
  template <class V>
  __device__ __forceinline__ V sum(V v) const {
#pragma unroll
    for (int o = N / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o, N);
    return v;
  }
  __device__ __forceinline__ uint32_t exclusive_sum(uint32_t v) const {
    uint32_t inc = v;
#pragma unroll
    for (int o = 1; o < N; o <<= 1) {
      uint32_t const y = __shfl_up_sync(mask, inc, o, N);
      if (t >= uint32_t(o)) inc += y;
    }
    return inc - v;
  }
  template <class V>
  __device__ __forceinline__ V from(V v, uint32_t src) const {
    return __shfl_sync(mask, v, src, N);
  }
};

/* The largest x in [lo, hi] with pred(x), for pred true at lo and monotone
 * (true up to the answer, false after): each round the lanes probe N
 * evenly spaced candidates above lo, so the bracket shrinks N-fold per
 * dependent round. */
template <int N, class Pred>
__device__ __forceinline__ uint64_t coop_last_true(LaneGroup<N> const& g,
                                                   uint64_t lo, uint64_t hi,
                                                   Pred pred) {
  while (lo < hi) {
    uint64_t const step = (hi - lo + N - 1) / N;
    uint64_t const x = lo + 1 + g.t * step;
    uint32_t const ok = g.ballot(x <= hi && pred(x));
    uint32_t const cnt = __popc(ok);  // a prefix of the probes: monotone
    uint64_t const nlo = cnt ? lo + 1 + (cnt - 1) * step : lo;
    uint64_t const nhi = cnt < N ? lo + cnt * step : hi;  // below probe cnt
    lo = nlo;
    hi = nhi < hi ? nhi : hi;
  }
  return lo;
}

/* Position of the r-th (1-based) `Value` bit among W words at w (bit 0 of
 * word 0 = position base), r within their count; the lanes take contiguous
 * runs of words.  Returns `none` when the words hold fewer. */
template <int Value, int N>
__device__ __forceinline__ uint64_t coop_select_in_words(
    LaneGroup<N> const& g, uint32_t const* __restrict__ w, uint32_t W,
    uint32_t r, uint64_t base, uint64_t none) {
  uint32_t const per = (W + N - 1) / N;
  uint32_t const j0 = min(W, g.t * per), j1 = min(W, j0 + per);
  uint32_t c = 0;
  for (uint32_t j = j0; j < j1; ++j) {
    uint32_t const x = Value ? __ldg(w + j) : ~__ldg(w + j);
    c += __popc(x);
  }
  uint32_t const ex = g.exclusive_sum(c);
  bool const mine = r > ex && r <= ex + c;
  uint32_t pos = 0;
  if (mine) {
    uint32_t rr = r - ex;
    for (uint32_t j = j0; j < j1; ++j) {
      uint32_t const x = Value ? __ldg(w + j) : ~__ldg(w + j);
      uint32_t const pc = __popc(x);
      if (rr <= pc) {
        pos = j * 32 + select_in_word(x, rr);
        break;
      }
      rr -= pc;
    }
  }
  uint32_t const who = g.ballot(mine);
  if (!who) return none;
  return base + g.from(pos, __ffs(who) - 1);
}

/* rs_rank1 by a lane group: the block's words split among the lanes. */
template <bool GetBit, int N>
__device__ __forceinline__ uint64_t rs_rank1_coop(LaneGroup<N> const& g,
                                                  const RSView& v,
                                                  const ArrayMeta& m,
                                                  uint64_t pos, bool* bit) {
  if (pos >= m.bits) {
    if (GetBit) *bit = false;
    return m.ones;
  }
  uint32_t const* w;
  uint32_t W, off;
  uint64_t before;
  if (v.rb && m.rb_off != kNoBlocks) {  // header word + 7 data words
    uint64_t const blk = pos / kRankBlockBits;
    off = static_cast<uint32_t>(pos - blk * kRankBlockBits);
    uint32_t const* line = reinterpret_cast<uint32_t const*>(v.rb + (m.rb_off + blk) * 2);
    before = rb_ones_before(v, m, blk, __ldg(line));
    w = line + 1;
    W = kRankBlockWords;
  } else {  // L1 + L2 entry, then the 512-bit block
    uint64_t const b2 = pos >> 9;
    before = __ldg(v.l1 + m.l1_off + (pos >> 16)) + __ldg(v.l2 + m.l2_off + b2);
    off = static_cast<uint32_t>(pos & 511);
    w = v.words + m.word_off + b2 * kL2Words;
    W = kL2Words;
  }
  uint32_t const wi = off >> 5;
  uint32_t acc = 0;
  bool hold = false, bv = false;
  for (uint32_t j = g.t; j < W && j <= wi; j += N) {
    uint32_t const x = __ldg(w + j);
    if (j < wi) {
      acc += __popc(x);
    } else {
      acc += __popc(x & ((1u << (off & 31)) - 1u));
      hold = true;
      bv = (x >> (off & 31)) & 1u;
    }
  }
  acc = g.sum(acc);
  if (GetBit) *bit = g.ballot(hold && bv) != 0;
  return before + acc;
}

/* rs_select by a lane group: the same brackets as rs_select, searched N
 * candidates per round, then the block's words split among the lanes. */
template <int Value, int N>
__device__ __forceinline__ uint64_t rs_select_coop(LaneGroup<N> const& g,
                                                   const RSView& v,
                                                   const ArrayMeta& m,
                                                   uint64_t i) {
  uint64_t const total = Value ? m.ones : m.bits - m.ones;
  if (i == 0 || i > total) return m.bits;
  if (v.sel_shift && m.ds0_off != kNoBlocks) {
    uint32_t const* S = v.ds + (Value ? m.ds1_off : m.ds0_off);
    uint32_t const sh = v.sel_shift;
    uint64_t const j = (i - 1) >> sh;
    uint64_t const nblk = (m.bits + kRankBlockBits - 1) / kRankBlockBits;
    uint64_t lo = min(uint64_t(__ldg(S + j)), nblk - 1);
    uint64_t hi = ((j + 1) << sh) < total ? __ldg(S + j + 1) : nblk - 1;
    hi = min(max(hi, lo), nblk - 1);
    uint4 const* rb = v.rb + m.rb_off * 2;
    auto before = [&](uint64_t k) -> uint64_t {
      uint32_t const h = __ldg(reinterpret_cast<uint32_t const*>(rb + k * 2));
      uint64_t const ones = rb_ones_before(v, m, k, h);
      return Value ? ones : k * kRankBlockBits - ones;
    };
    uint64_t const t =
        coop_last_true(g, lo, hi, [&](uint64_t k) { return before(k) < i; });
    uint32_t const* line = reinterpret_cast<uint32_t const*>(rb + t * 2);
    return coop_select_in_words<Value>(g, line + 1, kRankBlockWords,
                                       static_cast<uint32_t>(i - before(t)),
                                       t * kRankBlockBits, m.bits);
  }
  uint64_t const* S = Value ? v.s1 + m.s1_off : v.s0 + m.s0_off;
  uint64_t const q = i / kSampleRate;
  uint64_t const lo = q ? __ldg(S + q - 1) : 0;
  uint64_t const hi = (q + 1) * kSampleRate <= total ? __ldg(S + q) : m.bits - 1;
  uint64_t const* L1 = v.l1 + m.l1_off;
  auto before1 = [&](uint64_t b) -> uint64_t {
    uint64_t const x = __ldg(L1 + b);
    return Value ? x : (b << 16) - x;
  };
  uint64_t const b =
      coop_last_true(g, lo >> 16, hi >> 16, [&](uint64_t x) { return before1(x) < i; });
  uint64_t const rem = i - before1(b);
  uint64_t const first = b * kL2PerL1;
  uint64_t const num_l2 = (m.num_l1 - 1) * kL2PerL1 + m.num_last_l2;
  uint64_t const k_lo = ((lo >> 16) == b) ? (lo >> 9) : first;
  uint64_t k_hi = first + kL2PerL1 - 1;
  if (k_hi > num_l2 - 1) k_hi = num_l2 - 1;
  if ((hi >> 16) == b && (hi >> 9) < k_hi) k_hi = hi >> 9;
  uint16_t const* L2 = v.l2 + m.l2_off;
  auto before2 = [&](uint64_t k) -> uint64_t {
    uint32_t const x = __ldg(L2 + k);
    return Value ? x : ((k - first) << 9) - x;
  };
  uint64_t const k =
      coop_last_true(g, k_lo, max(k_lo, k_hi), [&](uint64_t x) { return before2(x) < rem; });
  return coop_select_in_words<Value>(g, v.words + m.word_off + k * kL2Words,
                                     static_cast<uint32_t>(kL2Words),
                                     static_cast<uint32_t>(rem - before2(k)),
                                     k * kL2Bits, m.bits);
}

/* ---- group levels ----------------------------------------------------- */

__device__ __forceinline__ void quad_words(uint4 a, uint4 b, uint64_t q[4]) {
  q[0] = (uint64_t(a.y) << 32) | a.x;
  q[1] = (uint64_t(a.w) << 32) | a.z;
  q[2] = (uint64_t(b.y) << 32) | b.x;
  q[3] = (uint64_t(b.w) << 32) | b.z;
}

/* Quad lane-match mask: the lower bit of every 2-bit lane of q equal to d. */
__device__ __forceinline__ uint64_t quad_match(uint64_t q, uint32_t d) {
  uint64_t const e = ~(q ^ (0x5555555555555555ull * d));
  return e & (e >> 1) & 0x5555555555555555ull;
}

constexpr uint64_t kOctPlane = (1ull << 42) - 1;

/* Octal: bit t set where digit t of the block equals d. */
__device__ __forceinline__ uint64_t oct_match(uint64_t const q[4], uint32_t d) {
  return (d & 4 ? q[1] : ~q[1]) & (d & 2 ? q[2] : ~q[2]) & (d & 1 ? q[3] : ~q[3]) &
         kOctPlane;
}

/* Digit-d count among the first t digits of a block. */
template <int W>
__device__ __forceinline__ uint32_t group_count(uint64_t const q[4], uint32_t d,
                                                uint32_t t) {
  if constexpr (W == 2) {
    uint32_t c = 0;
#pragma unroll
    for (uint32_t w = 1; w < 4; ++w) {
      uint32_t const lo = 32 * (w - 1);  // first digit of word w
      uint64_t const mask = t >= lo + 32 ? ~0ull
                            : t > lo     ? (1ull << (2 * (t - lo))) - 1
                                         : 0ull;
      c += __popcll(quad_match(q[w], d) & mask);
    }
    return c;
  } else {
    return __popcll(oct_match(q, d) & ((1ull << t) - 1));  // t <= 42
  }
}

template <int W>
__device__ __forceinline__ uint32_t group_digit(uint64_t const q[4], uint32_t t) {
  if constexpr (W == 2) {
    uint64_t const w = t < 32 ? q[1] : t < 64 ? q[2] : q[3];
    return static_cast<uint32_t>(w >> (2 * (t & 31))) & 3u;
  } else {
    return (static_cast<uint32_t>(q[1] >> t) & 1u) << 2 |
           (static_cast<uint32_t>(q[2] >> t) & 1u) << 1 |
           (static_cast<uint32_t>(q[3] >> t) & 1u);
  }
}

/* Digit-d count before the block from its header and superblock entry. */
template <int W>
__device__ __forceinline__ uint64_t group_before(uint64_t const q[4], uint64_t sbv,
                                                 uint32_t d, uint64_t blk) {
  constexpr uint32_t kD = GroupShape<W>::kDigits, kSb = GroupShape<W>::kSbBlocks;
  uint32_t const in_sb = static_cast<uint32_t>(blk % kSb) * kD;
  uint64_t const q0 = q[0];
  uint32_t const h0 = static_cast<uint32_t>(q0) & 0xFFFFu;
  uint32_t const h1 = static_cast<uint32_t>(q0 >> 16) & 0xFFFFu;
  uint32_t const h2 = static_cast<uint32_t>(q0 >> 32) & 0xFFFFu;
  uint32_t h;
  if constexpr (W == 2) {
    h = d == 0 ? h0 : d == 1 ? h1 : d == 2 ? h2 : in_sb - h0 - h1 - h2;
  } else {
    uint32_t const h3 = static_cast<uint32_t>(q0 >> 48);
    uint32_t const h4 = static_cast<uint32_t>(q[1] >> 42) & 0xFFFFu;
    uint32_t const h5 = static_cast<uint32_t>(q[2] >> 42) & 0xFFFFu;
    uint32_t const h6 = static_cast<uint32_t>(q[3] >> 42) & 0xFFFFu;
    uint32_t const lo = d & 2 ? (d & 1 ? h3 : h2) : (d & 1 ? h1 : h0);
    uint32_t const hi = d & 2 ? (d & 1 ? in_sb - h0 - h1 - h2 - h3 - h4 - h5 - h6 : h6)
                              : (d & 1 ? h5 : h4);
    h = d & 4 ? hi : lo;
  }
  return sbv + h;
}

/* Superblock entry of digit d from the entries loaded ahead of the block
 * (so that the table read does not wait for the digit). */
template <int W>
__device__ __forceinline__ uint64_t sb_pick(uint4 const e[1u << (W - 1)], uint32_t d) {
  uint4 u;
  if constexpr (W == 2) {
    u = d & 2 ? e[1] : e[0];
  } else {
    u = d & 4 ? (d & 2 ? e[3] : e[2]) : (d & 2 ? e[1] : e[0]);
  }
  return d & 1 ? (uint64_t(u.w) << 32 | u.z) : (uint64_t(u.y) << 32 | u.x);
}

/* Digit at position p < n of group level ql and its occurrences before p. */
template <int W>
__device__ __forceinline__ uint32_t group_access(const GroupView& v,
                                                 GroupLevel const& ql, uint64_t p,
                                                 uint64_t* before) {
  constexpr uint32_t kD = GroupShape<W>::kDigits, kSb = GroupShape<W>::kSbBlocks;
  constexpr uint32_t kE = 1u << (W - 1);  // uint4 per superblock entry
  uint64_t const blk = p / kD;
  uint32_t const t = static_cast<uint32_t>(p - blk * kD);
  uint4 const* bp = v.blocks + (ql.blk_off + blk) * 2;
  uint4 const* sp =
      reinterpret_cast<uint4 const*>(v.sb + ql.sb_off + (blk / kSb) * (1u << W));
  uint4 e[kE];
#pragma unroll
  for (uint32_t k = 0; k < kE; ++k) e[k] = __ldg(sp + k);  // L2 hits, in parallel
  uint4 const a = __ldg(bp), b = __ldg(bp + 1);
  uint64_t q[4];
  quad_words(a, b, q);
  uint32_t const d = group_digit<W>(q, t);
  *before = group_before<W>(q, sb_pick<W>(e, d), d, blk) + group_count<W>(q, d, t);
  return d;
}

/* Occurrences of digit d in [0, p) of group level ql, p <= n. */
template <int W>
__device__ __forceinline__ uint64_t group_rank(const GroupView& v,
                                               GroupLevel const& ql, uint64_t p,
                                               uint32_t d) {
  constexpr uint32_t kD = GroupShape<W>::kDigits, kSb = GroupShape<W>::kSbBlocks;
  uint64_t const blk = p / kD;
  uint32_t const t = static_cast<uint32_t>(p - blk * kD);
  uint4 const* bp = v.blocks + (ql.blk_off + blk) * 2;
  uint4 const a = __ldg(bp), b = __ldg(bp + 1);
  uint64_t const sbv = __ldg(v.sb + ql.sb_off + (blk / kSb) * (1u << W) + d);
  uint64_t q[4];
  quad_words(a, b, q);
  return group_before<W>(q, sbv, d, blk) + group_count<W>(q, d, t);
}

/* Position (in the block) of the r-th digit d, 1 <= r <= its count there;
 * kD when absent (not reached for valid structures). */
template <int W>
__device__ __forceinline__ uint32_t group_select_in(uint64_t const q[4],
                                                    uint32_t d, uint32_t r) {
  if constexpr (W == 2) {
    uint32_t pos = GroupShape<W>::kDigits;
    bool found = false;
#pragma unroll
    for (uint32_t w = 1; w < 4; ++w) {
      uint64_t const m = quad_match(q[w], d);
      uint32_t const c = __popcll(m);
      if (!found) {
        if (r <= c) {
          uint32_t const lo32 = static_cast<uint32_t>(m);
          uint32_t const cl = __popc(lo32);
          uint32_t const bit =
              r <= cl ? select_in_word(lo32, r)
                      : 32 + select_in_word(static_cast<uint32_t>(m >> 32), r - cl);
          pos = 32 * (w - 1) + bit / 2;
          found = true;
        } else {
          r -= c;
        }
      }
    }
    return pos;
  } else {
    uint64_t const m = oct_match(q, d);
    if (r > static_cast<uint32_t>(__popcll(m))) return GroupShape<W>::kDigits;
    uint32_t const lo32 = static_cast<uint32_t>(m);
    uint32_t const cl = __popc(lo32);
    return r <= cl ? select_in_word(lo32, r)
                   : 32 + select_in_word(static_cast<uint32_t>(m >> 32), r - cl);
  }
}

/* Position of the k-th (1-based, k <= total[d]) digit d of group level ql:
 * dense samples bracket its block (without them the superblock table does),
 * brackets wider than 16 blocks are narrowed by binary search, then the
 * search starts at the block the sample rank interpolates to and moves one
 * block at a time (throughput follows the sectors read). */
template <int W>
__device__ __forceinline__ uint64_t group_select(const GroupView& v,
                                                 GroupLevel const& ql,
                                                 uint32_t d, uint64_t k) {
  constexpr uint32_t kD = GroupShape<W>::kDigits, kSb = GroupShape<W>::kSbBlocks;
  constexpr uint32_t kS = 1u << W;  // superblock-table words per superblock
  uint64_t const nblk = ql.num_blocks;
  if (k == 0 || k > ql.total[d]) return nblk * kD;  // invalid structure
  uint64_t const* sb = v.sb + ql.sb_off + d;
  uint4 const* blocks = v.blocks + ql.blk_off * 2;
  uint64_t lo, hi, est;
  if (v.ds && ql.sel_shift) {
    uint32_t const sh = ql.sel_shift;
    uint32_t const* S = v.ds + ql.ds_off[d];
    uint64_t const j = (k - 1) >> sh;
    lo = min(uint64_t(__ldg(S + j)), nblk - 1);
    hi = ((j + 1) << sh) < ql.total[d] ? __ldg(S + j + 1) : nblk - 1;
    hi = min(max(hi, lo), nblk - 1);
    est = lo + (((hi - lo) * ((k - 1) - (j << sh))) >> sh);
  } else {  // superblock whose count before it is below k
    uint64_t a = 0, z = (nblk - 1) / kSb;
    while (a < z) {
      uint64_t const mid = (a + z + 1) >> 1;
      if (__ldg(sb + mid * kS) < k) a = mid; else z = mid - 1;
    }
    lo = a * kSb;
    hi = min(lo + kSb - 1, nblk - 1);
    est = lo;
  }
  auto before = [&](uint64_t blk) -> uint64_t {
    uint64_t h[4];
    quad_words(__ldg(blocks + blk * 2), __ldg(blocks + blk * 2 + 1), h);
    return group_before<W>(h, __ldg(sb + (blk / kSb) * kS), d, blk);
  };
  while (hi - lo > 16) {  // wide brackets only (rare digits)
    uint64_t const mid = (lo + hi + 1) >> 1;
    if (before(mid) < k) lo = mid; else hi = mid - 1;
    est = lo;
  }
  uint64_t blk = min(max(est, lo), hi);
  uint64_t q[4];
  uint64_t bt = 0;
  for (uint32_t guard = 0; guard < 24; ++guard) {
    uint4 const a0 = __ldg(blocks + blk * 2), a1 = __ldg(blocks + blk * 2 + 1);
    quad_words(a0, a1, q);
    bt = group_before<W>(q, __ldg(sb + (blk / kSb) * kS), d, blk);
    if (bt >= k && blk > lo) {  // it lies before this block
      hi = blk - 1;
      --blk;
      continue;
    }
    if (blk < hi && bt + group_count<W>(q, d, kD) < k) {  // after it
      lo = blk + 1;
      ++blk;
      continue;
    }
    break;
  }
  uint32_t const pos = group_select_in<W>(q, d, static_cast<uint32_t>(k - bt));
  if (pos >= kD) return nblk * kD;  // not reached for valid structures
  return blk * kD + pos;
}

/* ---- tree walks ------------------------------------------------------- */

/* Index into node_ranks of the node starting at symbol cs on level l >= 1
 * (getNodePosAtLevel, wavelet_tree.cuh:2241-2268, plus the per-level base
 * the reference accumulates in ranks_start). */
__device__ __forceinline__ uint64_t node_index(const TreeView& t,
                                               uint64_t const* node_base,
                                               uint64_t cs, uint32_t l) {
  uint64_t pos;
  if (l == 1) {
    pos = 0;
  } else if (t.is_pow2) {
    pos = (cs >> (t.levels - l)) - 1;
  } else {
    uint64_t num_prev = 0, node_lens = 1, remaining = t.sigma, sym = cs;
    for (int i = int(l) - 1; i >= 0; --i) {
      uint64_t const sub = prev_pow2_u64(remaining);
      node_lens = sub >> i;
      if (sym <= sub) break;
      remaining -= sub;
      num_prev += sub / node_lens;
      sym -= sub;
    }
    pos = sym / node_lens + num_prev - 1;
  }
  return node_base[l] + pos;
}

__device__ __forceinline__ uint64_t occurrences(const TreeView& t,
                                                uint64_t const* counts,
                                                uint64_t c) {
  return (c + 1 == t.sigma ? t.n : counts[c + 1]) - counts[c];
}

/* The three walks over group levels (power-of-two alphabets): the same
 * descent as the binary walks below, w binary levels per step; binary levels
 * past the groups (at most one) are walked as in the binary code. */
__device__ __forceinline__ uint64_t group_node_rank(const TreeView& t,
                                                   GroupLevel const& ql,
                                                   uint64_t g, uint32_t d) {
  return __ldg(t.groups.node_ranks + ql.nr_off + (g << ql.width) + d);
}

__device__ __forceinline__ uint64_t wt_access_groups(const TreeView& t,
                                                   ArrayMeta const* meta,
                                                   uint64_t const* counts,
                                                   uint64_t idx) {
  uint32_t const L = t.levels;
  uint64_t cs = 0;
  for (uint32_t j = 0; j < t.groups.num; ++j) {
    GroupLevel const& ql = t.groups.levels[j];
    uint32_t const w = ql.width;
    uint32_t const sh = L - ql.start;  // log2 of the symbols under a node
    uint64_t before;
    uint32_t const d = w == 3 ? group_access<3>(t.groups, ql, counts[cs] + idx, &before)
                              : group_access<2>(t.groups, ql, counts[cs] + idx, &before);
    if (j + 1 < t.groups.num || t.groups.covered < L)
      idx = before - group_node_rank(t, ql, cs >> sh, d);
    cs += uint64_t(d) << (sh - w);
  }
  if (t.groups.covered < L) {  // last binary level: its bit alone
    if (rs_bit(t.rs, meta[L - 1], counts[cs] + idx)) cs += 1;
  }
  return cs;
}

__device__ __forceinline__ uint64_t wt_rank_groups(const TreeView& t,
                                                 ArrayMeta const* meta,
                                                 uint64_t const* counts,
                                                 uint64_t const* ranks,
                                                 uint64_t const* node_base,
                                                 uint64_t c, uint64_t i) {
  uint32_t const L = t.levels;
  uint64_t cs = 0, res = i;
  for (uint32_t j = 0; j < t.groups.num; ++j) {
    GroupLevel const& ql = t.groups.levels[j];
    uint32_t const w = ql.width;
    uint32_t const sh = L - ql.start;
    uint32_t const d = static_cast<uint32_t>(c >> (sh - w)) & ((1u << w) - 1u);
    uint64_t const p = counts[cs] + res;
    res = (w == 3 ? group_rank<3>(t.groups, ql, p, d) : group_rank<2>(t.groups, ql, p, d)) -
          group_node_rank(t, ql, cs >> sh, d);
    cs += uint64_t(d) << (sh - w);
  }
  if (t.groups.covered < L) {
    ArrayMeta const& m = meta[L - 1];
    uint64_t const start = cs ? ranks[node_index(t, node_base, cs, L - 1)] : 0;
    uint64_t const p = counts[cs] + res;
    uint64_t const r0 = p - rs_rank1<false>(t.rs, m, p, nullptr);
    if (c & 1) res -= r0 - start; else res = r0 - start;
  }
  return res;
}

__device__ __forceinline__ uint64_t wt_select_groups(const TreeView& t,
                                                   ArrayMeta const* meta,
                                                   uint64_t const* counts,
                                                   uint64_t const* ranks,
                                                   uint64_t const* node_base,
                                                   uint64_t c, uint64_t k) {
  uint32_t const L = t.levels;
  uint64_t res = k;  // 1-based occurrence inside the current node
  if (t.groups.covered < L) {
    ArrayMeta const& m = meta[L - 1];
    uint64_t const cs = c & ~uint64_t(1);
    uint64_t const z = cs ? ranks[node_index(t, node_base, cs, L - 1)] : 0;
    if (c & 1)
      res = rs_select<1>(t.rs, m, (cs ? counts[cs] - z : 0) + res) + 1;
    else
      res = rs_select<0>(t.rs, m, z + res) + 1;
    if (res > m.bits) return t.n;
    res -= counts[cs];
  }
  for (int j = int(t.groups.num) - 1; j >= 0; --j) {
    GroupLevel const& ql = t.groups.levels[j];
    uint32_t const w = ql.width;
    uint32_t const sh = L - ql.start;
    uint64_t const g = c >> sh;
    uint32_t const d = static_cast<uint32_t>(c >> (sh - w)) & ((1u << w) - 1u);
    uint64_t const kk = group_node_rank(t, ql, g, d) + res;
    uint64_t const pos = w == 3 ? group_select<3>(t.groups, ql, d, kk)
                                : group_select<2>(t.groups, ql, d, kk);
    res = pos + 1 - counts[g << sh];
  }
  return res - 1;
}

/* Minimal symbol at text position idx < n (deviceAccess,
 * wavelet_tree.cuh:1815-1877). */
__device__ __forceinline__ uint64_t wt_access(const TreeView& t,
                                              ArrayMeta const* meta,
                                              uint64_t const* counts,
                                              uint64_t const* ranks,
                                              uint64_t const* node_base,
                                              uint64_t idx) {
  if (t.groups.num) return wt_access_groups(t, meta, counts, idx);
  uint64_t cs = 0, ce = t.sigma - 1;
  for (uint32_t l = 0; l < t.levels; ++l) {
    ArrayMeta const& m = meta[l];
    uint64_t const cc = counts[cs];
    if (ce - cs < 2) {
      if (ce - cs > 0 && rs_bit(t.rs, m, cc + idx)) cs++;
      break;
    }
    uint64_t const start = cs ? ranks[node_index(t, node_base, cs, l)] : 0;
    uint64_t const p = cc + idx;
    bool b;
    uint64_t const r0 = p - rs_rank1<true>(t.rs, m, p, &b);
    uint64_t const diff = prev_pow2_u64(ce - cs + 1);
    if (!b) {
      idx = r0 - start;
      ce = cs + diff - 1;
    } else {
      idx -= r0 - start;
      cs += diff;
    }
  }
  return cs;
}

/* Occurrences of minimal symbol c in [0, i), i <= n (deviceRank,
 * wavelet_tree.cuh:1896-1956; zero-count shortcut :481-486). */
__device__ __forceinline__ uint64_t wt_rank(const TreeView& t,
                                            ArrayMeta const* meta,
                                            uint64_t const* counts,
                                            uint64_t const* ranks,
                                            uint64_t const* node_base,
                                            uint64_t c, uint64_t i) {
  if (occurrences(t, counts, c) == 0) return 0;
  if (t.groups.num) return wt_rank_groups(t, meta, counts, ranks, node_base, c, i);
  uint64_t cs = 0, ce = t.sigma - 1, res = i;
  for (uint32_t l = 0; l < t.levels; ++l) {
    if (ce == cs) break;
    ArrayMeta const& m = meta[l];
    uint64_t const cc = counts[cs];
    uint64_t const start = cs ? ranks[node_index(t, node_base, cs, l)] : 0;
    uint64_t const p = cc + res;
    uint64_t const r0 = p - rs_rank1<false>(t.rs, m, p, nullptr);
    uint64_t const split = cs + prev_pow2_u64(ce - cs + 1);
    if (c < split) {
      res = r0 - start;
      ce = split - 1;
    } else {
      res -= r0 - start;
      cs = split;
    }
  }
  return res;
}

/* Position of the k-th (1-based) occurrence of minimal symbol c, or n when
 * there are fewer (deviceSelect :2007-2079, getPrevCharStart :1970-1992,
 * k > count check :532-536). */
__device__ __forceinline__ uint64_t wt_select(const TreeView& t,
                                              ArrayMeta const* meta,
                                              uint64_t const* counts,
                                              uint64_t const* ranks,
                                              uint64_t const* node_base,
                                              uint64_t c, uint64_t k) {
  if (k == 0 || k > occurrences(t, counts, c)) return t.n;
  if (t.groups.num) return wt_select_groups(t, meta, counts, ranks, node_base, c, k);
  uint32_t const L = t.levels;
  uint64_t len = L, code = c;
  if (!t.is_pow2 && c >= t.codes_start) {
    len = t.code_len[c - t.codes_start];
    code = t.code_bits[c - t.codes_start];
  }
  uint64_t res = k, cs = c;
  for (int l = int(len) - 1; l >= 0; --l) {
    ArrayMeta const& m = meta[l];
    uint64_t start;
    if ((code >> (L - 1 - l)) & 1u) {
      if (t.is_pow2) {
        uint64_t const node_lens = uint64_t(1) << (L - l);
        cs &= ~(node_lens - 1);
      } else {
        uint64_t const top = (L - l >= 64) ? 0 : (code >> (L - l));
        if (__popcll(top) == l) {
          uint64_t ns = 0;
          for (int j = 0; j < l; ++j) ns += prev_pow2_u64(t.sigma - ns);
          cs = ns;
        } else {
          cs -= uint64_t(1) << (len - 1 - l);
        }
      }
      start = cs ? counts[cs] - ranks[node_index(t, node_base, cs, l)] : 0;
      res = rs_select<1>(t.rs, m, start + res) + 1;
    } else {
      start = cs ? ranks[node_index(t, node_base, cs, l)] : 0;
      res = rs_select<0>(t.rs, m, start + res) + 1;
    }
    if (uint64_t(l) == len - 1 && res > m.bits) return t.n;
    res -= counts[cs];
  }
  return res - 1;
}

/* lower_bound of s in the sorted device alphabet (the reference's host-side
 * query remap, wavelet_tree.cuh:1425-1436).  Returns sigma if s is above
 * the last symbol. */
template <class T>
__device__ __forceinline__ uint64_t to_minimal(const TreeView& t, T s) {
  if (t.is_min) return static_cast<uint64_t>(s) < t.sigma ? s : t.sigma;
  T const* a = static_cast<T const*>(t.alphabet);
  uint64_t lo = 0, hi = t.sigma;
  while (lo < hi) {
    uint64_t const mid = (lo + hi) >> 1;
    if (__ldg(a + mid) < s) lo = mid + 1; else hi = mid;
  }
  return lo;
}

template <class T>
__device__ __forceinline__ T from_minimal(const TreeView& t, uint64_t c) {
  if (t.is_min) return static_cast<T>(c);
  return __ldg(static_cast<T const*>(t.alphabet) + c);
}

}  // namespace detail
}  // namespace ecl
