/*
 * CPU oracle for the GB300 wavelet-tree path — TEST INFRASTRUCTURE ONLY.
 *
 * Restates, on the CPU, the data structure built by mfranzreb/ECL_wavelet
 * (paths are inside that project) and answers queries two ways:
 *   - by walking the restated structure the way the reference's device code
 *     does (checks every level bit, count table, sample and node rank);
 *   - by plain scan of the stored text (the definition of the answers).
 * Nothing in the product links or loads this file; tests/, smoke() and the
 * CPU-baseline leg of bench.py use it as the checker.
 */
#include "ewt_oracle.h"

#include <omp.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

namespace {

constexpr uint64_t kL1Bits = 65536;  // RSConfig::L1_BIT_SIZE  rank_select.cuh:49
constexpr uint64_t kL2Bits = 512;    // RSConfig::L2_BIT_SIZE  rank_select.cuh:44
constexpr uint64_t kL2PerL1 = 128;   // RSConfig::NUM_L2_PER_L1 rank_select.cuh:47
constexpr uint64_t kSampleRate = 4096;  // RSConfig::SELECT_SAMPLE_RATE :58

// utils.cuh:107-114 isPowTwo (0 counts as a power of two there too).
inline bool is_pow2(uint64_t n) { return (n & (n - 1)) == 0; }

// utils.cuh:123-146 getPrevPowTwo: n/2 for powers of two, else the largest
// power of two below n.
inline uint64_t prev_pow2(uint64_t n) {
  if (n == 0) return 0;
  if (is_pow2(n)) return n >> 1;
  return uint64_t(1) << (63 - __builtin_clzll(n));
}

// utils.cuh:201-232 ceilLog2.
inline uint32_t ceil_log2(uint64_t n) {
  uint32_t hi = 63 - __builtin_clzll(n);
  return is_pow2(n) ? hi : hi + 1;
}

inline bool get_bit(uint32_t i, uint64_t c) { return (c >> i) & 1; }

struct Code {
  uint64_t len;
  uint64_t code;
};

// wavelet_tree.cuh:2100-2159 createMinimalCodes, restated step by step.
// Returns the codes of the last `total` symbols of 0..sigma-1.
std::vector<Code> minimal_codes(uint64_t sigma) {
  if (is_pow2(sigma)) return {};
  uint64_t total_num_codes = 0;
  std::vector<Code> codes(sigma);
  uint32_t const total_bits = ceil_log2(sigma);
  for (uint64_t i = 0; i < sigma; ++i) codes[i] = {total_bits, i};
  uint32_t start_bit = 0;
  uint64_t start_i = 0;
  uint32_t code_len = total_bits;
  uint64_t num_codes = sigma;
  do {
    for (uint32_t i = code_len - 1; i > 0; --i) {
      uint64_t p = uint64_t(1) << i;
      if (num_codes <= p) break;
      num_codes -= p;
      start_i += p;
      start_bit++;
    }
    if (code_len == total_bits) total_num_codes = num_codes;
    if (num_codes == 1) {
      code_len = 1;
      codes[sigma - 1].len = start_bit;
      codes[sigma - 1].code = ((uint64_t(1) << start_bit) - 1)
                              << (total_bits - start_bit);
    } else {
      code_len = ceil_log2(num_codes);
      for (uint64_t i = sigma - num_codes; i < sigma; i++) {
        uint64_t code = i - start_i;
        code <<= (total_bits - start_bit - code_len);
        code += (~((uint64_t(1) << (total_bits - start_bit)) - 1)) &
                codes[i].code;
        codes[i].code = code;
        codes[i].len = start_bit + code_len;
      }
    }
  } while (code_len > 1);
  codes.erase(codes.begin(), codes.begin() + (sigma - total_num_codes));
  return codes;
}

struct NodeInfo {
  uint64_t start;
  uint64_t level;
};

// wavelet_tree.cuh:2501-2532 getNodeInfos over the minimal alphabet.
std::vector<NodeInfo> node_infos(uint64_t sigma, std::vector<Code> const& codes) {
  uint32_t const L = ceil_log2(sigma);
  std::vector<Code> ac(sigma);
  uint64_t const cs = sigma - codes.size();
  for (uint64_t i = 0; i < sigma; ++i)
    ac[i] = i < cs ? Code{L, i} : codes[i - cs];
  std::vector<NodeInfo> out;
  for (uint32_t l = 1; l < L; ++l)
    for (uint64_t i = 1; i < sigma; ++i)
      if (ac[i].len > l && !get_bit(L - l - 1, ac[i].code) &&
          get_bit(L - l - 1, ac[i - 1].code))
        out.push_back({i, l});
  return out;
}

// wavelet_tree.cuh:2241-2268 getNodePosAtLevel (both alphabet shapes).
uint64_t node_pos(uint64_t sigma, uint32_t L, uint64_t symbol, uint32_t level) {
  if (level == 1) return 0;
  uint64_t num_prev = 0, node_lens = 1;
  if (is_pow2(sigma)) {
    node_lens = uint64_t(1) << (L - level);
  } else {
    uint64_t remaining = sigma;
    for (int i = int(level) - 1; i >= 0; --i) {
      uint64_t const sub = prev_pow2(remaining);
      node_lens = sub >> i;
      if (symbol <= sub) break;
      remaining -= sub;
      num_prev += sub / node_lens;
      symbol -= sub;
    }
  }
  return symbol / node_lens + num_prev - 1;
}

// One packed bit array plus its RankSelect support, as built by
// BitArray (bit_array.cu:40-100) and RankSelect (rank_select.cu:50-304).
struct BitRS {
  uint64_t bits = 0;
  std::vector<uint32_t> words;  // ceil(bits/32), bits >= `bits` are zero
  std::vector<uint64_t> l1;     // ones before each 65,536-bit block
  std::vector<uint16_t> l2;     // ones since the L1 block start, per 512 bits
  std::vector<uint64_t> s0, s1; // position of the (k+1)*4096-th zero / one
  uint64_t ones = 0;
  uint64_t num_last_l2 = 0;

  bool bit(uint64_t i) const { return (words[i >> 5] >> (i & 31)) & 1; }

  // rank_select.cu:50-120 (block counts), :412-552 (L2 scan, L1 totals,
  // masked tail), :580-591 (total ones), :554-578 (samples).
  void build() {
    uint64_t const nw = (bits + 31) / 32;
    words.resize(nw);
    if (bits % 32) words[nw - 1] &= (uint32_t(1) << (bits % 32)) - 1;
    uint64_t const num_l1 = (bits + kL1Bits - 1) / kL1Bits;
    num_last_l2 = ((bits % kL1Bits) + kL2Bits - 1) / kL2Bits;
    if (num_last_l2 == 0) num_last_l2 = kL2PerL1;
    uint64_t const num_l2 = (num_l1 - 1) * kL2PerL1 + num_last_l2;
    l1.assign(num_l1, 0);
    l2.assign(num_l2, 0);
    std::vector<uint64_t> block_ones(num_l2, 0);
#pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < int64_t(num_l2); ++b) {
      uint64_t c = 0;
      uint64_t const w0 = uint64_t(b) * 16;
      uint64_t const w1 = std::min<uint64_t>(w0 + 16, nw);
      for (uint64_t w = w0; w < w1; ++w) c += __builtin_popcount(words[w]);
      block_ones[b] = c;
    }
    uint64_t cum = 0;
    for (uint64_t b = 0; b < num_l2; ++b) {
      if (b % kL2PerL1 == 0) {
        l1[b / kL2PerL1] = cum;
      }
      l2[b] = uint16_t(cum - l1[b / kL2PerL1]);
      cum += block_ones[b];
    }
    ones = cum;
    uint64_t const zeros = bits - ones;
    s1.assign(ones / kSampleRate, 0);
    s0.assign(zeros / kSampleRate, 0);
    // Sample k holds the position of the (k+1)*4096-th one (zero).
    uint64_t c1 = 0, c0 = 0;
    for (uint64_t i = 0; i < bits; ++i) {
      if (bit(i)) {
        if (++c1 % kSampleRate == 0) s1[c1 / kSampleRate - 1] = i;
      } else {
        if (++c0 % kSampleRate == 0) s0[c0 / kSampleRate - 1] = i;
      }
    }
  }

  // rank_select.cuh:125-208 rank: number of `value` bits in [0, pos).
  uint64_t rank1(uint64_t pos) const {
    if (pos == 0) return 0;
    if (pos == bits) return ones;
    uint64_t const b1 = pos / kL1Bits, b2 = pos / kL2Bits;
    uint64_t r = l1[b1] + l2[b2];
    uint64_t const w_end = pos / 32;
    for (uint64_t w = b2 * 16; w < w_end; ++w) r += __builtin_popcount(words[w]);
    if (pos % 32)
      r += __builtin_popcount(words[w_end] & ((uint32_t(1) << (pos % 32)) - 1));
    return r;
  }
  uint64_t rank(uint64_t pos, int value) const {
    uint64_t const r = rank1(pos);
    return value ? r : pos - r;
  }

  // rank_select.cuh:224-523 select: position of the i-th (1-based) `value`
  // bit, or `bits` when there are fewer.  Sample bracket, then the last L1
  // block and L2 block holding fewer than i values, then a word scan.
  uint64_t select(uint64_t i, int value) const {
    uint64_t const total = value ? ones : bits - ones;
    if (i == 0 || i > total) return bits;
    auto const& smp = value ? s1 : s0;
    uint64_t const q = i / kSampleRate;
    uint64_t lo_pos = q > 0 ? smp[q - 1] : 0;
    uint64_t hi_pos = (q + 1) * kSampleRate <= total ? smp[q] : bits - 1;
    auto before_l1 = [&](uint64_t b) {
      return value ? l1[b] : b * kL1Bits - l1[b];
    };
    uint64_t b = lo_pos / kL1Bits;
    uint64_t const b_hi = hi_pos / kL1Bits;
    while (b + 1 <= b_hi && before_l1(b + 1) < i) ++b;
    uint64_t rem = i - before_l1(b);
    uint64_t const first_l2 = b * kL2PerL1;
    uint64_t const last_l2 =
        std::min<uint64_t>(first_l2 + kL2PerL1, l2.size());
    auto before_l2 = [&](uint64_t k) -> uint64_t {
      return value ? l2[k] : (k - first_l2) * kL2Bits - l2[k];
    };
    uint64_t k = first_l2;
    while (k + 1 < last_l2 && before_l2(k + 1) < rem) ++k;
    rem -= before_l2(k);
    uint64_t const nw = words.size();
    for (uint64_t w = k * 16; w < nw; ++w) {
      uint32_t x = value ? words[w] : ~words[w];
      uint64_t const c = __builtin_popcount(x);
      if (c >= rem) {
        for (uint32_t t = 0; t < 32; ++t)
          if ((x >> t) & 1)
            if (--rem == 0) return w * 32 + t;
      }
      rem -= c;
    }
    return bits;
  }
};

struct Tree {
  uint64_t n = 0, sigma = 0;
  uint32_t L = 0, elem_size = 0;
  bool is_min = false, pow2 = false;
  std::vector<uint64_t> text;      // original symbols
  std::vector<uint64_t> alphabet;  // sorted
  std::vector<Code> codes;
  uint64_t codes_start = 0;
  std::vector<uint64_t> counts;    // exclusive prefix C[c]
  std::vector<uint64_t> occ;       // plain occurrence counts
  std::vector<NodeInfo> nodes;
  std::vector<uint64_t> nodes_at_level;  // d_num_nodes_at_level_ (size L-1)
  uint64_t nodes_until_last = 0;
  std::vector<uint64_t> node_base;  // sum of node starts on levels < l
  std::vector<uint64_t> ranks;      // d_ranks_
  std::vector<BitRS> levels;
  // plain-scan index: positions of each minimal symbol
  std::vector<uint64_t> pos_start;  // = counts
  std::vector<uint64_t> positions;

  uint64_t nodes_of(uint32_t l) const {
    if (pow2) return (uint64_t(1) << l) - 1;
    return l < nodes_at_level.size() ? nodes_at_level[l] : 0;
  }
  // wavelet_tree.cuh:1425-1436 host remap of a query symbol: lower_bound
  // into the sorted alphabet.  Returns sigma if the symbol is above all.
  uint64_t to_min(uint64_t s) const {
    if (is_min) return s < sigma ? s : sigma;
    return std::lower_bound(alphabet.begin(), alphabet.end(), s) -
           alphabet.begin();
  }
  uint64_t total(uint64_t c) const {  // getTotalAppearances :2207-2215
    return occ[c];
  }
  Code code_of(uint64_t c) const {
    if (!pow2 && c >= codes_start) return codes[c - codes_start];
    return {L, c};
  }

  // wavelet_tree.cuh:1815-1877 deviceAccess.
  uint64_t access(uint64_t index) const {
    uint64_t cs = 0, ce = sigma - 1, rs = 0;
    for (uint32_t l = 0; l < L; ++l) {
      uint64_t const cc = counts[cs];
      if (ce - cs < 2) {
        if (ce - cs > 0 && levels[l].bit(cc + index)) cs++;
        break;
      }
      uint64_t const start =
          cs == 0 ? 0 : ranks[rs + node_pos(sigma, L, cs, l)];
      uint64_t const p = cc + index;
      uint64_t const r0 = levels[l].rank(p, 0);
      bool const b = levels[l].bit(p);
      uint64_t const diff = prev_pow2(ce - cs + 1);
      if (!b) {
        index = r0 - start;
        ce = cs + diff - 1;
      } else {
        index -= r0 - start;
        cs += diff;
      }
      rs += nodes_of(l);
    }
    return cs;
  }

  // wavelet_tree.cuh:1896-1956 deviceRank (+ zero-count shortcut :481-486).
  uint64_t rank(uint64_t c, uint64_t index) const {
    if (total(c) == 0) return 0;
    uint64_t cs = 0, ce = sigma - 1, rs = 0, result = index;
    for (uint32_t l = 0; l < L; ++l) {
      if (ce == cs) break;
      uint64_t const cc = counts[cs];
      uint64_t const start =
          cs == 0 ? 0 : ranks[rs + node_pos(sigma, L, cs, l)];
      uint64_t const p = levels[l].rank(cc + result, 0);
      uint64_t const split = cs + prev_pow2(ce - cs + 1);
      if (c < split) {
        result = p - start;
        ce = split - 1;
      } else {
        result -= p - start;
        cs = split;
      }
      rs += nodes_of(l);
    }
    return result;
  }

  // wavelet_tree.cuh:1970-1992 getPrevCharStart.
  uint64_t prev_char_start(uint64_t cs, bool rightmost, uint32_t level,
                           uint32_t code_len) const {
    if (pow2) {
      uint64_t const node_lens = uint64_t(1) << (L - level);
      return cs & ~(node_lens - 1);
    }
    if (rightmost) {
      uint64_t ns = 0;
      for (uint32_t l = 0; l < level; ++l) ns += prev_pow2(sigma - ns);
      return ns;
    }
    return cs - (uint64_t(1) << (code_len - 1 - level));
  }

  // wavelet_tree.cuh:2007-2079 deviceSelect (+ k > count check :532-536).
  uint64_t select(uint64_t c, uint64_t k) const {
    if (k > total(c)) return n;
    Code const code = code_of(c);
    uint64_t result = k, cs = c;
    for (int l = int(code.len) - 1; l >= 0; --l) {
      uint64_t const rs = node_base[l];
      uint64_t start;
      if (get_bit(L - 1 - l, code.code)) {
        bool const rightmost =
            __builtin_popcountll(L - l >= 64 ? 0 : code.code >> (L - l)) == l;
        cs = prev_char_start(cs, rightmost, l, code.len);
        start = cs == 0 ? 0 : counts[cs] - ranks[rs + node_pos(sigma, L, cs, l)];
        result = levels[l].select(start + result, 1) + 1;
      } else {
        start = cs == 0 ? 0 : ranks[rs + node_pos(sigma, L, cs, l)];
        result = levels[l].select(start + result, 0) + 1;
      }
      if (uint64_t(l) == code.len - 1 && result > levels[l].bits) return n;
      result -= counts[cs];
    }
    return result - 1;
  }
};

template <class T>
void load_text(const void* data, uint64_t n, std::vector<uint64_t>& out) {
  const T* p = static_cast<const T*>(data);
  out.resize(n);
  for (uint64_t i = 0; i < n; ++i) out[i] = p[i];
}

// Alphabet shape of a tree whose sorted alphabet is set: sigma, levels,
// codes, node starts, nodes per level (wavelet_tree.cuh:618-724).
int setup_shape(Tree& t) {
  t.sigma = t.alphabet.size();
  if (t.sigma < 2) return EWT_ERR_ALPHABET;  // utils.cuh:80 kMinAlphabetSize
  t.L = ceil_log2(t.sigma);
  t.pow2 = is_pow2(t.sigma);
  t.is_min = true;
  for (uint64_t i = 0; i < t.sigma; ++i)
    if (t.alphabet[i] != i) t.is_min = false;
  // :618-638 codes and node starts over the minimal alphabet.
  t.codes = minimal_codes(t.sigma);
  t.codes_start = t.sigma - t.codes.size();
  t.nodes = node_infos(t.sigma, t.codes);
  // :703-724 nodes per level (counted the reference's way) and the number
  // of node starts above the last level.
  // Entry L-1 (never read by the reference) holds the last level's count.
  t.nodes_at_level.assign(t.L, 0);
  if (!t.pow2) {
    uint64_t counter = 0;
    for (uint64_t i = 0; i < t.nodes.size(); ++i) {
      if (i > 0 && t.nodes[i].level > t.nodes[i - 1].level) {
        t.nodes_at_level[t.nodes[i].level - 1] = counter;
        counter = 0;
      }
      counter++;
    }
    if (!t.nodes.empty() && t.nodes.back().level == t.L - 1)
      t.nodes_at_level[t.L - 1] = counter;
    t.nodes_until_last = 0;
    for (uint32_t l = 0; l + 1 < t.L; ++l)
      t.nodes_until_last += t.nodes_at_level[l];
  } else {
    t.nodes_until_last =
        t.nodes.size() - ((uint64_t(1) << (t.L - 1)) - 1);
  }
  t.node_base.assign(t.L + 1, 0);
  for (uint32_t l = 1; l <= t.L; ++l)
    t.node_base[l] = t.node_base[l - 1] + t.nodes_of(l - 1);
  return EWT_OK;
}

// wavelet_tree.cuh:776-790 level sizes: n minus the occurrences of the
// symbols whose code ended above level l.
std::vector<uint64_t> level_sizes(Tree const& t) {
  uint64_t const n = t.n;
  std::vector<uint64_t> level_bits(t.L, n);
  if (!t.codes.empty()) {
    uint64_t const min_len = t.codes.back().len;
    for (uint64_t i = t.L - 1; i >= min_len; --i) {
      for (int64_t j = int64_t(t.sigma - t.codes_start) - 1; j >= 0; --j) {
        if (i >= t.codes[j].len)
          level_bits[i] -= t.occ[t.codes_start + j];
        else
          break;
      }
      if (i == 0) break;
    }
  }
  return level_bits;
}

int build_tree(Tree& t, const void* data, uint64_t n, int es,
               const uint64_t* alphabet, uint64_t sigma) {
  if (!data || n == 0) return EWT_ERR_INVALID_ARGUMENT;
  t.n = n;
  t.elem_size = es;
  switch (es) {
    case 1: load_text<uint8_t>(data, n, t.text); break;
    case 2: load_text<uint16_t>(data, n, t.text); break;
    case 4: load_text<uint32_t>(data, n, t.text); break;
    case 8: load_text<uint64_t>(data, n, t.text); break;
    default: return EWT_ERR_INVALID_ARGUMENT;
  }
  // wavelet_tree.cuh:590-614 alphabet detection when none is given.
  if (sigma == 0) {
    t.alphabet = t.text;
    std::sort(t.alphabet.begin(), t.alphabet.end());
    t.alphabet.erase(std::unique(t.alphabet.begin(), t.alphabet.end()),
                     t.alphabet.end());
  } else {
    t.alphabet.assign(alphabet, alphabet + sigma);
    for (uint64_t i = 1; i < sigma; ++i)
      if (t.alphabet[i] <= t.alphabet[i - 1]) return EWT_ERR_ALPHABET;
  }
  if (int st = setup_shape(t); st != EWT_OK) return st;
  // Minimal symbols and histogram (computeGlobalHistogramKernel :170-227).
  std::vector<uint64_t> sym(n);
  for (uint64_t i = 0; i < n; ++i) {
    uint64_t const m = t.to_min(t.text[i]);
    if (m >= t.sigma) return EWT_ERR_ALPHABET;
    sym[i] = m;
  }
  t.occ.assign(t.sigma, 0);
  for (uint64_t i = 0; i < n; ++i) t.occ[sym[i]]++;
  t.counts.assign(t.sigma, 0);
  for (uint64_t c = 1; c < t.sigma; ++c)
    t.counts[c] = t.counts[c - 1] + t.occ[c - 1];
  std::vector<uint64_t> const level_bits = level_sizes(t);
  // :806-818 level l order = text stably sorted on the top l code bits;
  // level l stores bit L-1-l of the first level_bits[l] codes.
  std::vector<uint64_t> cur(n), nxt(n);
  for (uint64_t i = 0; i < n; ++i) cur[i] = t.code_of(sym[i]).code;
  t.levels.resize(t.L);
  for (uint32_t l = 0; l < t.L; ++l) {
    BitRS& b = t.levels[l];
    b.bits = level_bits[l];
    b.words.assign((b.bits + 31) / 32, 0);
    uint32_t const sh = t.L - 1 - l;
    for (uint64_t i = 0; i < b.bits; ++i)
      if ((cur[i] >> sh) & 1) b.words[i >> 5] |= uint32_t(1) << (i & 31);
    b.build();
    if (l + 1 == t.L) break;
    // Stable partition of each equal-prefix run by bit `sh`.
    uint64_t i = 0;
    while (i < n) {
      uint64_t const pref = cur[i] >> (sh + 1);
      uint64_t j = i;
      while (j < n && (cur[j] >> (sh + 1)) == pref) ++j;
      uint64_t w = i;
      for (uint64_t k = i; k < j; ++k)
        if (!((cur[k] >> sh) & 1)) nxt[w++] = cur[k];
      for (uint64_t k = i; k < j; ++k)
        if ((cur[k] >> sh) & 1) nxt[w++] = cur[k];
      i = j;
    }
    cur.swap(nxt);
  }
  // :332-352 precomputeRanksKernel: rank0 at each node start.
  t.ranks.resize(t.nodes.size());
  for (uint64_t i = 0; i < t.nodes.size(); ++i)
    t.ranks[i] = t.levels[t.nodes[i].level].rank(t.counts[t.nodes[i].start], 0);
  // plain-scan position lists
  t.positions.resize(n);
  std::vector<uint64_t> fill(t.counts);
  for (uint64_t i = 0; i < n; ++i) t.positions[fill[sym[i]]++] = i;
  return EWT_OK;
}

template <class V>
int put(const std::vector<V>& v, void* buf, uint64_t cap, uint64_t* size) {
  uint64_t const bytes = v.size() * sizeof(V);
  if (size) *size = bytes;
  if (!buf) return EWT_OK;
  if (cap < bytes) return EWT_ERR_INVALID_ARGUMENT;
  if (bytes) std::memcpy(buf, v.data(), bytes);
  return EWT_OK;
}

int export_bitrs(const BitRS& b, int comp, void* buf, uint64_t cap,
                 uint64_t* size) {
  switch (comp) {
    case EWT_EXP_LEVEL_WORDS: return put(b.words, buf, cap, size);
    case EWT_EXP_L1: return put(b.l1, buf, cap, size);
    case EWT_EXP_L2: return put(b.l2, buf, cap, size);
    case EWT_EXP_SAMPLES0: return put(b.s0, buf, cap, size);
    case EWT_EXP_SAMPLES1: return put(b.s1, buf, cap, size);
  }
  return EWT_ERR_INVALID_ARGUMENT;
}

struct RSSet {
  std::vector<BitRS> arrays;
};

// ---- multithreaded build -------------------------------------------------
// The same structure as build_tree, built on all host cores for texts of
// billions of symbols: the CPU baseline of the benchmark and the independent
// full-size checker of the GPU build.  The level order is kept as narrow
// codes (the code type C holds L bits); each level is one parallel stable
// partition, one parallel bit packing and a RankSelect built from per-block
// popcounts (rank_select.cu:50-304, 412-591).  The text itself is not kept:
// the plain-scan calls of a tree built this way are refused; full-size
// plain-scan answers come from ewto_scan_batch over the caller's text.

inline uint64_t shr(uint64_t x, uint32_t s) { return s >= 64 ? 0 : x >> s; }

// Ranges [r*n/parts, (r+1)*n/parts).
inline uint64_t part_begin(uint64_t n, uint64_t parts, uint64_t r) {
  return static_cast<uint64_t>((static_cast<unsigned __int128>(n) * r) / parts);
}

// RankSelect of one packed array (words already hold the bits), in
// parallel: L2 block popcounts, a two-phase scan over whole L1 blocks, and
// the select samples found by one walk over each L1 block's words.
void build_rs_mt(BitRS& b, int nt) {
  uint64_t const bits = b.bits;
  uint64_t const nw = (bits + 31) / 32;
  if (bits % 32) b.words[nw - 1] &= (uint32_t(1) << (bits % 32)) - 1;
  uint64_t const num_l1 = (bits + kL1Bits - 1) / kL1Bits;
  b.num_last_l2 = ((bits % kL1Bits) + kL2Bits - 1) / kL2Bits;
  if (b.num_last_l2 == 0) b.num_last_l2 = kL2PerL1;
  uint64_t const num_l2 = (num_l1 - 1) * kL2PerL1 + b.num_last_l2;
  b.l1.assign(num_l1, 0);
  b.l2.assign(num_l2, 0);
  // ones per L1 block
  std::vector<uint64_t> l1_ones(num_l1, 0);
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int64_t B = 0; B < int64_t(num_l1); ++B) {
    uint64_t const w1 = std::min<uint64_t>((uint64_t(B) + 1) * (kL1Bits / 32), nw);
    uint64_t const k0 = uint64_t(B) * kL2PerL1;
    uint64_t const k1 = std::min<uint64_t>(k0 + kL2PerL1, num_l2);
    uint64_t run = 0;
    for (uint64_t k = k0; k < k1; ++k) {
      b.l2[k] = static_cast<uint16_t>(run);
      uint64_t const a = k * 16, e = std::min<uint64_t>(a + 16, w1);
      for (uint64_t w = a; w < e; ++w) run += __builtin_popcount(b.words[w]);
    }
    l1_ones[B] = run;
  }
  uint64_t cum = 0;
  for (uint64_t B = 0; B < num_l1; ++B) {
    b.l1[B] = cum;
    cum += l1_ones[B];
  }
  b.ones = cum;
  uint64_t const zeros = bits - b.ones;
  b.s1.assign(b.ones / kSampleRate, 0);
  b.s0.assign(zeros / kSampleRate, 0);
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt)
  for (int64_t B = 0; B < int64_t(num_l1); ++B) {
    uint64_t const pos0 = uint64_t(B) * kL1Bits;
    uint64_t const blk_bits = std::min<uint64_t>(kL1Bits, bits - pos0);
    uint64_t c1 = b.l1[B], c0 = pos0 - b.l1[B];
    uint64_t const e1 = c1 + l1_ones[B], e0 = c0 + (blk_bits - l1_ones[B]);
    // next thresholds: the (k+1)*4096-th one / zero
    uint64_t t1 = (c1 / kSampleRate + 1) * kSampleRate;
    uint64_t t0 = (c0 / kSampleRate + 1) * kSampleRate;
    if (t1 > e1 && t0 > e0) continue;
    uint64_t const w0 = pos0 / 32;
    uint64_t const w1 = (pos0 + blk_bits + 31) / 32;
    for (uint64_t w = w0; w < w1 && (t1 <= e1 || t0 <= e0); ++w) {
      uint32_t const x = b.words[w];
      uint32_t const valid = std::min<uint64_t>(32, bits - w * 32);
      uint32_t const o = __builtin_popcount(x);
      uint32_t const z = valid - o;
      while (t1 <= c1 + o) {  // the sample's one lies in this word
        uint32_t need = uint32_t(t1 - c1), y = x;
        for (uint32_t r = 1; r < need; ++r) y &= y - 1;
        b.s1[t1 / kSampleRate - 1] = w * 32 + __builtin_ctz(y);
        t1 += kSampleRate;
      }
      while (t0 <= c0 + z) {
        uint32_t need = uint32_t(t0 - c0), y = ~x;
        if (valid < 32) y &= (uint32_t(1) << valid) - 1;
        for (uint32_t r = 1; r < need; ++r) y &= y - 1;
        b.s0[t0 / kSampleRate - 1] = w * 32 + __builtin_ctz(y);
        t0 += kSampleRate;
      }
      c1 += o;
      c0 += z;
    }
  }
}

// Zeros of bit `sh` among the first x codes of the level order, from the
// level's bits (positions past the level size hold codes that ended above
// this level; their bit is 0).
inline uint64_t zeros_before(BitRS const& b, uint64_t x) {
  if (x <= b.bits) return x - b.rank1(x);
  return (b.bits - b.ones) + (x - b.bits);
}

// Level l+1 order from level l's: inside every node (equal top-l code
// bits, contiguous), zeros of bit sh keep their order in front of the ones
// (wavelet_tree.cuh:806-818).  Destinations come from zero counts: a node
// [s, e) sends its j-th code to s + (zeros before j in the node) or, for a
// one, to s + (zeros in the node) + (ones before j in the node).
template <class C>
void partition_mt(std::vector<C> const& cur, std::vector<C>& nxt, BitRS const& b,
                  uint32_t sh, int nt) {
  uint64_t const n = cur.size();
  uint32_t const psh = sh + 1;
  auto prefix = [&](uint64_t i) { return shr(cur[i], psh); };
  uint64_t const parts = uint64_t(nt) * 8;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
  for (int64_t r = 0; r < int64_t(parts); ++r) {
    uint64_t i = part_begin(n, parts, r);
    uint64_t const end = part_begin(n, parts, r + 1);
    if (i >= end) continue;
    uint64_t z = zeros_before(b, i);
    while (i < end) {
      uint64_t const p = prefix(i);
      // node bounds by binary search (the order is sorted by prefix)
      uint64_t lo = 0, hi = i;
      while (lo < hi) {
        uint64_t const mid = lo + (hi - lo) / 2;
        if (prefix(mid) < p) lo = mid + 1; else hi = mid;
      }
      uint64_t const s = lo;
      lo = i + 1;
      hi = n;
      while (lo < hi) {
        uint64_t const mid = lo + (hi - lo) / 2;
        if (prefix(mid) <= p) lo = mid + 1; else hi = mid;
      }
      uint64_t const e = lo;
      uint64_t const zs = zeros_before(b, s);
      uint64_t const nz = zeros_before(b, e) - zs;
      uint64_t const stop = std::min(e, end);
      uint64_t const zero_base = s - zs, one_base = nz + zs;  // branch-free
      for (uint64_t j = i; j < stop; ++j) {
        C const c = cur[j];
        uint64_t const bit = (c >> sh) & 1;
        uint64_t const d0 = zero_base + z, d1 = one_base + j - z;
        nxt[bit ? d1 : d0] = c;
        z += bit ^ 1;
      }
      i = stop;
    }
  }
}

// Bit sh of 32 consecutive codes, LSB first.  One- and two-byte codes are
// gathered eight or four at a time by a multiply: the masked bits sit 8
// (16) apart and the constant's terms move bit j of the word to bit 56 + j
// (48 + j) without two terms meeting.
template <class C>
inline uint32_t pack32(C const* p, uint32_t sh, uint64_t cnt) {
  uint32_t x = 0;
  if (sizeof(C) <= 2 && cnt == 32) {
    for (int g = 0; g < 4; ++g) {
      uint64_t v[2];
      std::memcpy(v, p + g * 8, 8 * sizeof(C) > 16 ? 16 : 8 * sizeof(C));
      if (sizeof(C) == 1) {
        uint64_t const m = (v[0] >> sh) & 0x0101010101010101ull;
        x |= uint32_t((m * 0x0102040810204080ull) >> 56) << (8 * g);
      } else {
        for (int h = 0; h < 2; ++h) {
          uint64_t const m = (v[h] >> sh) & 0x0001000100010001ull;
          uint64_t const k = (uint64_t(1) << 3) | (uint64_t(1) << 18) |
                             (uint64_t(1) << 33) | (uint64_t(1) << 48);
          x |= uint32_t((m * k) >> 48 & 0xF) << (8 * g + 4 * h);
        }
      }
    }
    return x;
  }
  for (uint64_t j = 0; j < cnt; ++j) x |= uint32_t((p[j] >> sh) & 1) << j;
  return x;
}

template <class C>
int build_levels_mt(Tree& t, std::vector<C>& cur, int nt) {
  uint64_t const n = t.n;
  std::vector<uint64_t> const level_bits = level_sizes(t);
  std::vector<C> nxt;
  if (t.L > 1) nxt.resize(n);
  t.levels.resize(t.L);
  for (uint32_t l = 0; l < t.L; ++l) {
    BitRS& b = t.levels[l];
    b.bits = level_bits[l];
    uint64_t const nw = (b.bits + 31) / 32;
    b.words.resize(nw);
    uint32_t const sh = t.L - 1 - l;
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t w = 0; w < int64_t(nw); ++w) {
      uint64_t const i0 = uint64_t(w) * 32;
      b.words[w] = pack32(cur.data() + i0, sh, std::min<uint64_t>(32, b.bits - i0));
    }
  build_rs_mt(b, nt);
    if (l + 1 == t.L) break;
    partition_mt(cur, nxt, b, sh, nt);
    cur.swap(nxt);
  }
  // :332-352 rank0 at each node start
  t.ranks.resize(t.nodes.size());
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int64_t i = 0; i < int64_t(t.nodes.size()); ++i)
    t.ranks[i] = t.levels[t.nodes[i].level].rank(t.counts[t.nodes[i].start], 0);
  return EWT_OK;
}

// Minimal symbol of a raw value (sigma when not in the alphabet).
template <class T>
struct MinMap {
  std::vector<uint32_t> lut;  // 1- and 2-byte symbols
  Tree const* t;
  explicit MinMap(Tree const& tree) : t(&tree) {
    if (sizeof(T) <= 2) {
      lut.assign(size_t(1) << (8 * sizeof(T)), uint32_t(tree.sigma));
      for (uint64_t i = 0; i < tree.sigma; ++i) lut[tree.alphabet[i]] = uint32_t(i);
    }
  }
  uint64_t operator()(T v) const {
    if (sizeof(T) <= 2) return lut[v];
    return t->to_min(v);
  }
};

template <class T, class C>
int build_text_mt(Tree& t, T const* text, int nt) {
  uint64_t const n = t.n;
  MinMap<T> const mm(t);
  // code of every minimal symbol
  std::vector<C> code(t.sigma);
  for (uint64_t c = 0; c < t.sigma; ++c) code[c] = static_cast<C>(t.code_of(c).code);
  std::vector<C> cur(n);
  uint64_t const parts = uint64_t(nt);
  std::vector<std::vector<uint64_t>> hist(parts);
  int bad = 0;
#pragma omp parallel for schedule(static) num_threads(nt) reduction(| : bad)
  for (int64_t r = 0; r < int64_t(parts); ++r) {
    auto& h = hist[r];
    h.assign(t.sigma, 0);
    uint64_t const a = part_begin(n, parts, r), e = part_begin(n, parts, r + 1);
    for (uint64_t i = a; i < e; ++i) {
      uint64_t const m = mm(text[i]);
      if (m >= t.sigma) {
        bad = 1;
        break;
      }
      h[m]++;
      cur[i] = code[m];
    }
  }
  if (bad) return EWT_ERR_ALPHABET;
  t.occ.assign(t.sigma, 0);
  for (auto const& h : hist)
    for (uint64_t c = 0; c < t.sigma; ++c) t.occ[c] += h[c];
  t.counts.assign(t.sigma, 0);
  for (uint64_t c = 1; c < t.sigma; ++c)
    t.counts[c] = t.counts[c - 1] + t.occ[c - 1];
  return build_levels_mt(t, cur, nt);
}

template <class T>
int build_tree_mt_typed(Tree& t, T const* text, uint64_t n,
                        const uint64_t* alphabet, uint64_t sigma, int nt) {
  if (sigma == 0) {  // detection (wavelet_tree.cuh:590-614)
    if (sizeof(T) <= 2) {
      std::vector<uint8_t> seen(size_t(1) << (8 * sizeof(T)), 0);
      uint64_t const parts = uint64_t(nt);
      std::vector<std::vector<uint8_t>> loc(parts);
#pragma omp parallel for schedule(static) num_threads(nt)
      for (int64_t r = 0; r < int64_t(parts); ++r) {
        loc[r].assign(seen.size(), 0);
        uint64_t const a = part_begin(n, parts, r), e = part_begin(n, parts, r + 1);
        for (uint64_t i = a; i < e; ++i) loc[r][text[i]] = 1;
      }
      for (auto const& v : loc)
        for (size_t i = 0; i < seen.size(); ++i) seen[i] |= v[i];
      for (size_t i = 0; i < seen.size(); ++i)
        if (seen[i]) t.alphabet.push_back(i);
    } else {
      std::vector<T> tmp(text, text + n);
      std::sort(tmp.begin(), tmp.end());
      tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
      t.alphabet.assign(tmp.begin(), tmp.end());
    }
  } else {
    t.alphabet.assign(alphabet, alphabet + sigma);
    for (uint64_t i = 1; i < sigma; ++i)
      if (t.alphabet[i] <= t.alphabet[i - 1]) return EWT_ERR_ALPHABET;
  }
  if (int st = setup_shape(t); st != EWT_OK) return st;
  if (t.L <= 8) return build_text_mt<T, uint8_t>(t, text, nt);
  if (t.L <= 16) return build_text_mt<T, uint16_t>(t, text, nt);
  if (t.L <= 32) return build_text_mt<T, uint32_t>(t, text, nt);
  return build_text_mt<T, uint64_t>(t, text, nt);
}

// Plain-scan answers of a mixed batch straight from a 1- or 2-byte text,
// in O(n + m log m): per-chunk symbol counts, then one walk of every chunk
// answering the rank queries whose position and the select queries whose
// k-th occurrence fall in it.  Symbols >= sigma are invalid.
template <class T>
int scan_batch(T const* text, uint64_t n, uint64_t sigma, uint8_t const* types,
               uint64_t const* idx, uint64_t const* sym, uint64_t m,
               uint64_t* out, int nt) {
  size_t const V = size_t(1) << (8 * sizeof(T));
  if (sigma > V) sigma = V;
  uint64_t const parts = uint64_t(nt) * 2;
  std::vector<uint64_t> before((parts + 1) * V, 0);  // [part][v]
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int64_t r = 0; r < int64_t(parts); ++r) {
    uint64_t* h = &before[(r + 1) * V];
    uint64_t const a = part_begin(n, parts, r), e = part_begin(n, parts, r + 1);
    for (uint64_t i = a; i < e; ++i) h[text[i]]++;
  }
  for (uint64_t r = 1; r <= parts; ++r)
    for (size_t v = 0; v < V; ++v) before[r * V + v] += before[(r - 1) * V + v];
  uint64_t const* total = &before[parts * V];
  int bad = 0;
  struct Q {
    uint64_t key;  // position (rank) or k (select)
    uint64_t sym;
    uint64_t q;
  };
  std::vector<std::vector<Q>> rq(parts), sq(parts);
  for (uint64_t q = 0; q < m; ++q) {
    uint8_t const ty = types[q];
    if (ty == EWT_Q_ACCESS) {
      out[q] = idx[q] < n ? text[idx[q]] : 0;
      continue;
    }
    if (ty > EWT_Q_SELECT || sym[q] >= sigma ||
        (ty == EWT_Q_RANK ? idx[q] > n : idx[q] == 0)) {
      out[q] = UINT64_MAX;
      bad = 1;
      continue;
    }
    uint64_t const c = sym[q];
    if (ty == EWT_Q_RANK) {
      if (idx[q] == n) {
        out[q] = total[c];
        continue;
      }
      uint64_t lo = 0, hi = parts - 1;  // the part holding position idx
      while (lo < hi) {
        uint64_t const mid = (lo + hi + 1) / 2;
        if (part_begin(n, parts, mid) <= idx[q]) lo = mid; else hi = mid - 1;
      }
      rq[lo].push_back({idx[q], c, q});
    } else {
      uint64_t const k = idx[q];
      if (k > total[c]) {
        out[q] = n;
        continue;
      }
      uint64_t r = 0;  // the part holding the k-th occurrence
      while (before[(r + 1) * V + c] < k) ++r;
      sq[r].push_back({k, c, q});
    }
  }
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
  for (int64_t r = 0; r < int64_t(parts); ++r) {
    auto& R = rq[r];
    auto& S = sq[r];
    if (R.empty() && S.empty()) continue;
    std::sort(R.begin(), R.end(), [](Q const& x, Q const& y) { return x.key < y.key; });
    std::sort(S.begin(), S.end(), [](Q const& x, Q const& y) {
      return x.sym != y.sym ? x.sym < y.sym : x.key < y.key;
    });
    std::vector<uint64_t> run(before.begin() + r * V, before.begin() + (r + 1) * V);
    std::vector<uint64_t> ptr(V, 0), pend(V, 0);
    for (uint64_t j = 0; j < S.size(); ++j) {
      if (j == 0 || S[j].sym != S[j - 1].sym) ptr[S[j].sym] = j;
      pend[S[j].sym] = j + 1;
    }
    uint64_t const a = part_begin(n, parts, r), e = part_begin(n, parts, r + 1);
    uint64_t ri = 0;
    for (uint64_t i = a; i < e; ++i) {
      while (ri < R.size() && R[ri].key == i) {
        out[R[ri].q] = run[R[ri].sym];
        ++ri;
      }
      T const v = text[i];
      uint64_t const cnt = ++run[v];
      while (ptr[v] < pend[v] && S[ptr[v]].key == cnt) {
        out[S[ptr[v]].q] = i;
        ++ptr[v];
      }
    }
  }
  return bad ? EWT_ERR_QUERY : EWT_OK;
}

}  // namespace

extern "C" {

int ewto_build(const void* data, uint64_t n, int elem_size,
               const uint64_t* alphabet, uint64_t sigma, void** out) {
  if (!out) return EWT_ERR_INVALID_ARGUMENT;
  auto* t = new Tree();
  int const st = build_tree(*t, data, n, elem_size, alphabet, sigma);
  if (st != EWT_OK) {
    delete t;
    *out = nullptr;
    return st;
  }
  *out = t;
  return EWT_OK;
}

void ewto_free(void* h) { delete static_cast<Tree*>(h); }

int ewto_build_mt(const void* data, uint64_t n, int elem_size,
                  const uint64_t* alphabet, uint64_t sigma, int nthreads,
                  void** out) {
  if (!out || !data || n == 0) return EWT_ERR_INVALID_ARGUMENT;
  int const nt = nthreads > 0 ? nthreads : omp_get_max_threads();
  auto* t = new Tree();
  t->n = n;
  t->elem_size = elem_size;
  int st;
  switch (elem_size) {
    case 1: st = build_tree_mt_typed(*t, static_cast<const uint8_t*>(data), n, alphabet, sigma, nt); break;
    case 2: st = build_tree_mt_typed(*t, static_cast<const uint16_t*>(data), n, alphabet, sigma, nt); break;
    case 4: st = build_tree_mt_typed(*t, static_cast<const uint32_t*>(data), n, alphabet, sigma, nt); break;
    case 8: st = build_tree_mt_typed(*t, static_cast<const uint64_t*>(data), n, alphabet, sigma, nt); break;
    default: st = EWT_ERR_INVALID_ARGUMENT;
  }
  if (st != EWT_OK) {
    delete t;
    *out = nullptr;
    return st;
  }
  *out = t;
  return EWT_OK;
}

int ewto_scan_batch(const void* text, uint64_t n, int elem_size,
                    uint64_t sigma, const uint8_t* types, const uint64_t* idx,
                    const uint64_t* sym, uint64_t m, uint64_t* out,
                    int nthreads) {
  if (!text || !types || !idx || !sym || !out) return EWT_ERR_INVALID_ARGUMENT;
  int const nt = nthreads > 0 ? nthreads : omp_get_max_threads();
  if (elem_size == 1)
    return scan_batch(static_cast<const uint8_t*>(text), n, sigma, types, idx, sym, m, out, nt);
  if (elem_size == 2)
    return scan_batch(static_cast<const uint16_t*>(text), n, sigma, types, idx, sym, m, out, nt);
  return EWT_ERR_UNSUPPORTED;
}

int ewto_info(void* h, ewt_info* info) {
  auto* t = static_cast<Tree*>(h);
  if (!t || !info) return EWT_ERR_INVALID_ARGUMENT;
  std::memset(info, 0, sizeof(*info));
  info->n = t->n;
  info->sigma = t->sigma;
  info->num_ranks = t->nodes.size();
  info->codes_start = t->codes_start;
  info->num_codes = t->codes.size();
  info->num_nodes_until_last_level = t->nodes_until_last;
  info->levels = t->L;
  info->elem_size = t->elem_size;
  info->is_min_alphabet = t->is_min;
  info->is_pow2 = t->pow2;
  return EWT_OK;
}

int ewto_export(void* h, int comp, int level, void* buf, uint64_t cap,
                uint64_t* size) {
  auto* t = static_cast<Tree*>(h);
  if (!t) return EWT_ERR_INVALID_ARGUMENT;
  std::vector<uint64_t> v;
  switch (comp) {
    case EWT_EXP_COUNTS: return put(t->counts, buf, cap, size);
    case EWT_EXP_ALPHABET: return put(t->alphabet, buf, cap, size);
    case EWT_EXP_NODE_RANKS: return put(t->ranks, buf, cap, size);
    case EWT_EXP_TOTAL_ONES:
      for (auto& b : t->levels) v.push_back(b.ones);
      return put(v, buf, cap, size);
    case EWT_EXP_LEVEL_SIZES:
      for (auto& b : t->levels) v.push_back(b.bits);
      return put(v, buf, cap, size);
    case EWT_EXP_NUM_LAST_L2:
      for (auto& b : t->levels) v.push_back(b.num_last_l2);
      return put(v, buf, cap, size);
    case EWT_EXP_NODES_AT_LEVEL:
      for (uint32_t l = 0; l < t->L; ++l) v.push_back(t->nodes_of(l));
      return put(v, buf, cap, size);
    case EWT_EXP_NODE_INFOS:
      for (auto& nd : t->nodes) {
        v.push_back(nd.start);
        v.push_back(nd.level);
      }
      return put(v, buf, cap, size);
    case EWT_EXP_CODES:
      for (auto& c : t->codes) {
        v.push_back(c.len);
        v.push_back(c.code);
      }
      return put(v, buf, cap, size);
  }
  if (level < 0 || uint32_t(level) >= t->L) return EWT_ERR_INVALID_ARGUMENT;
  return export_bitrs(t->levels[level], comp, buf, cap, size);
}

static int nthreads_or_max(int nt) {
  return nt > 0 ? nt : omp_get_max_threads();
}

int ewto_access(void* h, const uint64_t* idx, uint64_t m, uint64_t* out,
                int nthreads) {
  auto* t = static_cast<Tree*>(h);
  if (!t) return EWT_ERR_INVALID_ARGUMENT;
#pragma omp parallel for schedule(static) num_threads(nthreads_or_max(nthreads))
  for (int64_t i = 0; i < int64_t(m); ++i) {
    out[i] = idx[i] < t->n ? t->alphabet[t->access(idx[i])] : 0;
  }
  return EWT_OK;
}

int ewto_rank(void* h, const uint64_t* idx, const uint64_t* sym, uint64_t m,
              uint64_t* out, int nthreads) {
  auto* t = static_cast<Tree*>(h);
  if (!t) return EWT_ERR_INVALID_ARGUMENT;
  int bad = 0;
#pragma omp parallel for schedule(static) num_threads(nthreads_or_max(nthreads)) reduction(| : bad)
  for (int64_t i = 0; i < int64_t(m); ++i) {
    uint64_t const c = t->to_min(sym[i]);
    if (c >= t->sigma || idx[i] > t->n) {
      out[i] = UINT64_MAX;
      bad = 1;
      continue;
    }
    out[i] = t->rank(c, idx[i]);
  }
  return bad ? EWT_ERR_QUERY : EWT_OK;
}

int ewto_select(void* h, const uint64_t* k, const uint64_t* sym, uint64_t m,
                uint64_t* out, int nthreads) {
  auto* t = static_cast<Tree*>(h);
  if (!t) return EWT_ERR_INVALID_ARGUMENT;
  int bad = 0;
#pragma omp parallel for schedule(static) num_threads(nthreads_or_max(nthreads)) reduction(| : bad)
  for (int64_t i = 0; i < int64_t(m); ++i) {
    uint64_t const c = t->to_min(sym[i]);
    if (c >= t->sigma || k[i] == 0) {
      out[i] = UINT64_MAX;
      bad = 1;
      continue;
    }
    out[i] = t->select(c, k[i]);
  }
  return bad ? EWT_ERR_QUERY : EWT_OK;
}

int ewto_mixed(void* h, const uint8_t* types, const uint64_t* idx,
               const uint64_t* sym, uint64_t m, uint64_t* out, int nthreads) {
  auto* t = static_cast<Tree*>(h);
  if (!t) return EWT_ERR_INVALID_ARGUMENT;
  int bad = 0;
#pragma omp parallel for schedule(static) num_threads(nthreads_or_max(nthreads)) reduction(| : bad)
  for (int64_t i = 0; i < int64_t(m); ++i) {
    if (types[i] == EWT_Q_ACCESS) {
      out[i] = idx[i] < t->n ? t->alphabet[t->access(idx[i])] : 0;
      continue;
    }
    uint64_t const c = t->to_min(sym[i]);
    if (types[i] == EWT_Q_RANK) {
      if (c >= t->sigma || idx[i] > t->n) {
        out[i] = UINT64_MAX;
        bad = 1;
      } else {
        out[i] = t->rank(c, idx[i]);
      }
    } else if (types[i] == EWT_Q_SELECT) {
      if (c >= t->sigma || idx[i] == 0) {
        out[i] = UINT64_MAX;
        bad = 1;
      } else {
        out[i] = t->select(c, idx[i]);
      }
    } else {
      out[i] = UINT64_MAX;
      bad = 1;
    }
  }
  return bad ? EWT_ERR_QUERY : EWT_OK;
}

int ewto_scan_access(void* h, const uint64_t* idx, uint64_t m, uint64_t* out) {
  auto* t = static_cast<Tree*>(h);
  if (!t) return EWT_ERR_INVALID_ARGUMENT;
  if (t->text.size() != t->n) return EWT_ERR_UNSUPPORTED;  // built by ewto_build_mt
  for (uint64_t i = 0; i < m; ++i) out[i] = idx[i] < t->n ? t->text[idx[i]] : 0;
  return EWT_OK;
}

int ewto_scan_rank(void* h, const uint64_t* idx, const uint64_t* sym,
                   uint64_t m, uint64_t* out) {
  auto* t = static_cast<Tree*>(h);
  if (!t) return EWT_ERR_INVALID_ARGUMENT;
  if (t->text.size() != t->n) return EWT_ERR_UNSUPPORTED;  // built by ewto_build_mt
  int st = EWT_OK;
  for (uint64_t i = 0; i < m; ++i) {
    uint64_t const c = t->to_min(sym[i]);
    if (c >= t->sigma || idx[i] > t->n) {
      out[i] = UINT64_MAX;
      st = EWT_ERR_QUERY;
      continue;
    }
    auto b = t->positions.begin() + t->counts[c];
    auto e = b + t->occ[c];
    out[i] = std::lower_bound(b, e, idx[i]) - b;
  }
  return st;
}

int ewto_scan_select(void* h, const uint64_t* k, const uint64_t* sym,
                     uint64_t m, uint64_t* out) {
  auto* t = static_cast<Tree*>(h);
  if (!t) return EWT_ERR_INVALID_ARGUMENT;
  if (t->text.size() != t->n) return EWT_ERR_UNSUPPORTED;  // built by ewto_build_mt
  int st = EWT_OK;
  for (uint64_t i = 0; i < m; ++i) {
    uint64_t const c = t->to_min(sym[i]);
    if (c >= t->sigma || k[i] == 0) {
      out[i] = UINT64_MAX;
      st = EWT_ERR_QUERY;
      continue;
    }
    out[i] = k[i] <= t->occ[c] ? t->positions[t->counts[c] + k[i] - 1] : t->n;
  }
  return st;
}

int ewto_rs_build(const uint32_t* words, const uint64_t* bits,
                  uint32_t num_arrays, void** out) {
  if (!out || !bits || num_arrays == 0) return EWT_ERR_INVALID_ARGUMENT;
  auto* s = new RSSet();
  s->arrays.resize(num_arrays);
  uint64_t off = 0;
  for (uint32_t a = 0; a < num_arrays; ++a) {
    if (bits[a] == 0) {
      delete s;
      return EWT_ERR_INVALID_ARGUMENT;
    }
    BitRS& b = s->arrays[a];
    b.bits = bits[a];
    uint64_t const nw = (bits[a] + 31) / 32;
    b.words.assign(words + off, words + off + nw);
    off += nw;
    b.build();
  }
  *out = s;
  return EWT_OK;
}

void ewto_rs_free(void* h) { delete static_cast<RSSet*>(h); }

int ewto_rs_export(void* h, int comp, int array, void* buf, uint64_t cap,
                   uint64_t* size) {
  auto* s = static_cast<RSSet*>(h);
  if (!s) return EWT_ERR_INVALID_ARGUMENT;
  std::vector<uint64_t> v;
  switch (comp) {
    case EWT_EXP_TOTAL_ONES:
      for (auto& b : s->arrays) v.push_back(b.ones);
      return put(v, buf, cap, size);
    case EWT_EXP_LEVEL_SIZES:
      for (auto& b : s->arrays) v.push_back(b.bits);
      return put(v, buf, cap, size);
    case EWT_EXP_NUM_LAST_L2:
      for (auto& b : s->arrays) v.push_back(b.num_last_l2);
      return put(v, buf, cap, size);
  }
  if (array < 0 || size_t(array) >= s->arrays.size())
    return EWT_ERR_INVALID_ARGUMENT;
  return export_bitrs(s->arrays[array], comp, buf, cap, size);
}

uint64_t ewto_rs_rank(void* h, int array, uint64_t pos, int value) {
  auto* s = static_cast<RSSet*>(h);
  return s->arrays[array].rank(pos, value);
}

uint64_t ewto_rs_select(void* h, int array, uint64_t i, int value) {
  auto* s = static_cast<RSSet*>(h);
  return s->arrays[array].select(i, value);
}

// Batches of binary rank / select on all host threads (the CPU popcount
// baseline of the standalone RankSelect; one query per loop iteration).
void ewto_rs_rank_batch(void* h, int array, const uint64_t* pos, uint64_t m,
                        int value, uint64_t* out, int nthreads) {
  auto& b = static_cast<RSSet*>(h)->arrays[array];
#pragma omp parallel for schedule(static) num_threads(nthreads_or_max(nthreads))
  for (int64_t i = 0; i < static_cast<int64_t>(m); ++i) out[i] = b.rank(pos[i], value);
}

void ewto_rs_select_batch(void* h, int array, const uint64_t* idx, uint64_t m,
                          int value, uint64_t* out, int nthreads) {
  auto& b = static_cast<RSSet*>(h)->arrays[array];
#pragma omp parallel for schedule(static) num_threads(nthreads_or_max(nthreads))
  for (int64_t i = 0; i < static_cast<int64_t>(m); ++i) out[i] = b.select(idx[i], value);
}

int ewto_minimal_codes(uint64_t sigma, uint64_t* lens, uint64_t* codes,
                       uint64_t cap, uint64_t* count) {
  if (sigma < 2) return EWT_ERR_INVALID_ARGUMENT;
  auto c = minimal_codes(sigma);
  if (count) *count = c.size();
  for (uint64_t i = 0; i < c.size() && i < cap; ++i) {
    lens[i] = c[i].len;
    codes[i] = c[i].code;
  }
  return EWT_OK;
}

int ewto_node_infos(uint64_t sigma, uint64_t* starts, uint64_t* levels,
                    uint64_t cap, uint64_t* count) {
  if (sigma < 2) return EWT_ERR_INVALID_ARGUMENT;
  auto nd = node_infos(sigma, minimal_codes(sigma));
  if (count) *count = nd.size();
  for (uint64_t i = 0; i < nd.size() && i < cap; ++i) {
    starts[i] = nd[i].start;
    levels[i] = nd[i].level;
  }
  return EWT_OK;
}

uint64_t ewto_node_pos(uint64_t sigma, uint64_t symbol, uint32_t level) {
  return node_pos(sigma, ceil_log2(sigma), symbol, level);
}

uint64_t ewto_prev_pow2(uint64_t n) { return prev_pow2(n); }
uint32_t ewto_ceil_log2(uint64_t n) { return ceil_log2(n); }
int ewto_max_threads(void) { return omp_get_max_threads(); }

}  // extern "C"
