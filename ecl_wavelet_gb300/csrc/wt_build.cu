// Wavelet-tree construction on the GPU.
//
// Pipeline (one GPU, one stream, no host round trip between levels):
//   1. alphabet: given, or detected (presence bitmap kernel for 1/2-byte
//      symbols, host sort for wider ones) — wavelet_tree.cuh:590-614;
//   2. shape on the host: minimal codes for non-power-of-two alphabets
//      (:2100-2159), node starts (:2501-2532), nodes per level (:703-724),
//      and the list of (start, split, end) symbol ranges of every node;
//   3. a non-minimal alphabet is remapped to 0..sigma-1 (:170-227); a
//      non-power-of-two alphabet also gets a histogram (its short codes
//      make level sizes depend on symbol counts, :776-790);
//   4. level 0 bits are packed from the text; then for every level l:
//      RankSelect counts of level l; the node kernel computes rank0 at every
//      node start of level l (precomputeRanksKernel, :332-352) and from it
//      the count table C at each node's split point (zeros of a node =
//      rank0(end) - rank0(start)), so no histogram pass is needed for
//      power-of-two alphabets; the split kernel stably partitions every
//      node of level l by its bit (the level l+1 order; the reference
//      re-sorts the text on the top l+1 code bits, :806-818) and writes the
//      bits of level l+1 directly;
//   5. select samples of all levels.
// The split kernel has a fast path for tiles that lie inside one node of a
// power-of-two alphabet: warp ballots rank the tile's zeros and ones, both
// go to two contiguous runs, and the next level's bits of each run are
// compacted with warp OR-reductions into shared memory and stored as whole
// words (only a run's two edge words use atomicOr).  Other tiles take a
// general path that stages (destination, symbol) pairs in shared memory.
// No kernel waits on another CTA.
#include <algorithm>
#include <cstring>
#include <string>

#include "internal.cuh"

namespace ewt {

using ecl::detail::prev_pow2_u64;

namespace {

inline bool h_is_pow2(uint64_t n) { return (n & (n - 1)) == 0; }
inline uint64_t h_prev_pow2(uint64_t n) {
  if (n == 0) return 0;
  if (h_is_pow2(n)) return n >> 1;
  return uint64_t(1) << (63 - __builtin_clzll(n));
}
inline uint32_t h_ceil_log2(uint64_t n) {
  uint32_t const hi = 63 - __builtin_clzll(n);
  return h_is_pow2(n) ? hi : hi + 1;
}

// Shortened codes of the last symbols when sigma is not a power of two;
// same construction as createMinimalCodes (wavelet_tree.cuh:2100-2159).
std::vector<CodeH> make_codes(uint64_t sigma) {
  if (h_is_pow2(sigma)) return {};
  uint32_t const bits = h_ceil_log2(sigma);
  std::vector<CodeH> c(sigma);
  for (uint64_t i = 0; i < sigma; ++i) c[i] = {bits, i};
  uint32_t start_bit = 0, code_len = bits;
  uint64_t start_i = 0, left = sigma, kept = 0;
  do {
    for (uint32_t i = code_len - 1; i > 0; --i) {
      uint64_t const p = uint64_t(1) << i;
      if (left <= p) break;
      left -= p;
      start_i += p;
      ++start_bit;
    }
    if (code_len == bits) kept = left;
    if (left == 1) {
      code_len = 1;
      c[sigma - 1] = {start_bit, ((uint64_t(1) << start_bit) - 1)
                                     << (bits - start_bit)};
    } else {
      code_len = h_ceil_log2(left);
      uint64_t const high_mask = ~((uint64_t(1) << (bits - start_bit)) - 1);
      for (uint64_t i = sigma - left; i < sigma; ++i) {
        uint64_t code = (i - start_i) << (bits - start_bit - code_len);
        code += high_mask & c[i].code;
        c[i] = {start_bit + code_len, code};
      }
    }
  } while (code_len > 1);
  return std::vector<CodeH>(c.end() - kept, c.end());
}

// Node starts per level (getNodeInfos, wavelet_tree.cuh:2501-2532).
std::vector<NodeInfoH> make_nodes(uint64_t sigma,
                                  std::vector<CodeH> const& codes) {
  uint32_t const L = h_ceil_log2(sigma);
  uint64_t const cs = sigma - codes.size();
  auto code_of = [&](uint64_t i) {
    return i < cs ? CodeH{L, i} : codes[i - cs];
  };
  std::vector<NodeInfoH> out;
  for (uint32_t l = 1; l < L; ++l) {
    uint32_t const sh = L - l - 1;
    CodeH prev = code_of(0);
    for (uint64_t i = 1; i < sigma; ++i) {
      CodeH const cur = code_of(i);
      if (cur.len > l && !((cur.code >> sh) & 1) && ((prev.code >> sh) & 1))
        out.push_back({i, l});
      prev = cur;
    }
  }
  return out;
}

// Every node with at least two symbols, level by level, in symbol order:
// [start, end) splits at start + prevPow2(end - start), the descent of
// deviceAccess (wavelet_tree.cuh:1854-1868).
struct LevelNode {
  uint64_t cs, split, end;
};

std::vector<std::vector<LevelNode>> make_level_nodes(uint64_t sigma,
                                                     uint32_t L) {
  std::vector<std::vector<LevelNode>> lv(L);
  std::vector<std::pair<uint64_t, uint64_t>> cur{{0, sigma}}, nxt;
  for (uint32_t l = 0; l < L; ++l) {
    nxt.clear();
    for (auto [a, e] : cur) {
      if (e - a < 2) continue;
      uint64_t const s = a + h_prev_pow2(e - a);
      lv[l].push_back({a, s, e});
      nxt.push_back({a, s});
      nxt.push_back({s, e});
    }
    cur.swap(nxt);
  }
  return lv;
}

// --------------------------------------------------------------------------
// Alphabet detection for 1- and 2-byte symbols: presence bitmap.
template <class T>
__global__ void presence_kernel(T const* __restrict__ text, uint64_t n,
                                uint32_t* __restrict__ bitmap) {
  constexpr uint32_t kWords = (sizeof(T) == 1 ? 256u : 65536u) / 32u;
  __shared__ uint32_t sm[kWords];
  for (uint32_t i = threadIdx.x; i < kWords; i += blockDim.x) sm[i] = 0;
  __syncthreads();
  uint64_t const stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n;
       i += stride) {
    uint32_t const c = text[i];
    uint32_t const bit = 1u << (c & 31);
    if (!(sm[c >> 5] & bit)) atomicOr(&sm[c >> 5], bit);
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < kWords; i += blockDim.x)
    if (sm[i]) atomicOr(&bitmap[i], sm[i]);
}

// Alphabet detection for 4- and 8-byte symbols: a device hash set of the
// distinct symbols (open addressing, linear probing, 64-bit slots).  An
// empty slot holds kEmptySlot; for 8-byte texts the one symbol equal to it is
// recorded in a flag instead.  A symbol is looked up with a plain load first
// (most symbols repeat) and inserted with atomicCAS only when missing; warp
// peers holding the same symbol insert once.  A probe that runs around the
// whole table reports overflow and the host retries with a larger table.
constexpr uint64_t kEmptySlot = ~uint64_t(0);

__device__ __forceinline__ uint64_t slot_hash(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  return x;
}

template <class T>
__global__ void __launch_bounds__(256)
distinct_kernel(T const* __restrict__ text, uint64_t n,
                unsigned long long* __restrict__ table, uint64_t cap_mask,
                unsigned long long* __restrict__ count,
                uint32_t* __restrict__ flags) {  // [0] overflow, [1] max symbol seen
  uint64_t const stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n;
       i += stride) {
    uint64_t const key = static_cast<uint64_t>(text[i]);
    uint32_t const peers = __match_any_sync(__activemask(), key);
    if ((threadIdx.x & 31) != __ffs(peers) - 1) continue;  // one per value
    if (key == kEmptySlot) {
      flags[1] = 1;
      continue;
    }
    uint64_t h = slot_hash(key) & cap_mask;
    for (uint64_t probe = 0;; ++probe) {
      if (probe > cap_mask) {
        flags[0] = 1;
        break;
      }
      uint64_t const cur = table[h];
      if (cur == key) break;
      if (cur == kEmptySlot) {
        unsigned long long const prev =
            atomicCAS(&table[h], static_cast<unsigned long long>(kEmptySlot),
                      static_cast<unsigned long long>(key));
        if (prev == kEmptySlot) {
          atomicAdd(count, 1ull);
          break;
        }
        if (prev == key) break;
      }
      h = (h + 1) & cap_mask;
    }
  }
}

// Sorted distinct symbols of a device-resident 4- or 8-byte text.
template <class T>
std::vector<uint64_t> detect_alphabet_wide(T const* d_text, uint64_t n,
                                           cudaStream_t st) {
  uint64_t cap = 1ull << 16;
  uint32_t const blocks = static_cast<uint32_t>(
      std::min<uint64_t>(ceil_div(n, 256), uint64_t(sm_count()) * 8));
  for (;;) {
    DevBuf table(cap * 8), cnt(8), flags(8);
    EWT_CUDA(cudaMemsetAsync(table.get(), 0xFF, cap * 8, st));
    EWT_CUDA(cudaMemsetAsync(cnt.get(), 0, 8, st));
    EWT_CUDA(cudaMemsetAsync(flags.get(), 0, 8, st));
    distinct_kernel<T><<<blocks, 256, 0, st>>>(
        d_text, n, table.as<unsigned long long>(), cap - 1,
        cnt.as<unsigned long long>(), flags.as<uint32_t>());
    EWT_LAUNCHED();
    uint64_t count = 0;
    uint32_t fl[2] = {0, 0};
    EWT_CUDA(cudaMemcpyAsync(&count, cnt.get(), 8, cudaMemcpyDeviceToHost, st));
    EWT_CUDA(cudaMemcpyAsync(fl, flags.get(), 8, cudaMemcpyDeviceToHost, st));
    EWT_CUDA(cudaStreamSynchronize(st));
    if (!fl[0] && count * 2 <= cap) {
      std::vector<uint64_t> h(cap);
      EWT_CUDA(cudaMemcpyAsync(h.data(), table.get(), cap * 8,
                               cudaMemcpyDeviceToHost, st));
      EWT_CUDA(cudaStreamSynchronize(st));
      std::vector<uint64_t> out;
      out.reserve(count + 1);
      for (uint64_t v : h)
        if (v != kEmptySlot) out.push_back(v);
      if (fl[1]) out.push_back(kEmptySlot);
      std::sort(out.begin(), out.end());
      return out;
    }
    // table too small: at least four times the symbols seen so far
    uint64_t want = std::max(cap * 2, count * 4);
    cap = 1;
    while (cap < want) cap <<= 1;
  }
}

// Text -> minimal symbols (lower_bound in the sorted alphabet).
template <class T>
__global__ void __launch_bounds__(256)
remap_kernel(T const* __restrict__ text, uint64_t n,
             T const* __restrict__ alphabet, uint64_t sigma,
             T* __restrict__ cur, uint32_t* __restrict__ err) {
  uint64_t const stride = uint64_t(gridDim.x) * blockDim.x;
  uint32_t bad = 0;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n;
       i += stride) {
    T const x = text[i];
    uint64_t lo = 0, hi = sigma;
    while (lo < hi) {
      uint64_t const mid = (lo + hi) >> 1;
      if (alphabet[mid] < x) lo = mid + 1; else hi = mid;
    }
    if (lo >= sigma) {
      bad = 1;
      lo = 0;
    }
    cur[i] = static_cast<T>(lo);
  }
  if (bad) atomicOr(err, 1u);
}

// Histogram of minimal symbols (non-power-of-two alphabets only).
template <class T>
__global__ void __launch_bounds__(256)
hist_kernel(T const* __restrict__ text, uint64_t n, uint64_t sigma,
            unsigned long long* __restrict__ occ, uint32_t smem_bins) {
  extern __shared__ uint32_t hist[];
  bool const use_smem = smem_bins != 0;
  if (use_smem) {
    for (uint32_t i = threadIdx.x; i < smem_bins; i += blockDim.x) hist[i] = 0;
    __syncthreads();
  }
  uint64_t const stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n;
       i += stride) {
    uint64_t const c = text[i];
    if (c >= sigma) continue;
    if (use_smem) atomicAdd(&hist[c], 1u);
    else atomicAdd(&occ[c], 1ull);
  }
  if (use_smem) {
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < smem_bins; i += blockDim.x)
      if (hist[i]) atomicAdd(&occ[i], static_cast<unsigned long long>(hist[i]));
  }
}

// --------------------------------------------------------------------------
// Node of minimal symbol c on level l: [cs, ce] and its split point.
struct NodeRange {
  uint64_t cs, ce, split;
};

template <bool Pow2>
__device__ __forceinline__ NodeRange node_of(uint64_t c, uint32_t l,
                                             uint32_t L, uint64_t sigma) {
  NodeRange r;
  if (Pow2) {
    uint32_t const w = L - l;  // node width is 2^w symbols
    uint64_t const mask = (w >= 64) ? ~uint64_t(0) : ((uint64_t(1) << w) - 1);
    r.cs = c & ~mask;
    r.ce = r.cs + mask;
    r.split = r.cs + (uint64_t(1) << (w - 1));
  } else {
    uint64_t cs = 0, ce = sigma - 1;
    for (uint32_t k = 0; k < l; ++k) {
      uint64_t const s = cs + prev_pow2_u64(ce - cs + 1);
      if (c < s) ce = s - 1; else cs = s;
    }
    r.cs = cs;
    r.ce = ce;
    r.split = cs + prev_pow2_u64(ce - cs + 1);
  }
  return r;
}

template <bool Pow2>
__device__ __forceinline__ bool level_bit(uint64_t c, uint32_t l, uint32_t L,
                                          uint64_t sigma) {
  if (Pow2) return (c >> (L - 1 - l)) & 1;
  return c >= node_of<false>(c, l, L, sigma).split;
}

// Level 0 bits: each thread writes fill_words<T>() output words (words
// blockIdx.x * 256 * fill_words + threadIdx.x + 256 * j), with all their
// symbol loads (128 bytes) issued before any is used.  Check = validate
// symbols of a minimal alphabet (c < sigma).
template <class T>
__host__ __device__ constexpr uint32_t fill_words() {
  return sizeof(T) == 1 ? 4u : (sizeof(T) == 2 ? 2u : 1u);
}

template <class T, bool Pow2, bool Check>
__global__ void __launch_bounds__(256)
fill0_kernel(T const* __restrict__ src, uint64_t size0, uint32_t L,
             uint64_t sigma, uint32_t* __restrict__ out,
             uint32_t* __restrict__ err) {
  constexpr uint32_t kFillWords = fill_words<T>();
  constexpr int kVec = 32 * sizeof(T) / 16;
  uint64_t const base = uint64_t(blockIdx.x) * 256 * kFillWords + threadIdx.x;
  uint4 buf[kFillWords][kVec];
#pragma unroll
  for (uint32_t j = 0; j < kFillWords; ++j) {
    uint64_t const p0 = (base + 256 * j) * 32;
    if (p0 + 32 <= size0) {
      uint4 const* s = reinterpret_cast<uint4 const*>(src + p0);
#pragma unroll
      for (int q = 0; q < kVec; ++q) buf[j][q] = __ldg(s + q);
    }
  }
  bool bad = false;
#pragma unroll
  for (uint32_t j = 0; j < kFillWords; ++j) {
    uint64_t const w = base + 256 * j;
    uint64_t const p0 = w * 32;
    if (p0 >= size0) break;
    uint32_t word = 0;
    if (p0 + 32 <= size0) {
      if constexpr (Pow2 && sizeof(T) <= 2) {
        // SWAR: bit L-1 of four bytes (two 16-bit symbols) per operation;
        // a symbol is >= sigma = 2^L iff it has a bit at or above L.
        uint32_t const* w32 = reinterpret_cast<uint32_t const*>(buf[j]);
        uint32_t const b = L - 1;
        uint32_t const hi = sizeof(T) == 1
                                ? 0x01010101u * ((0xFFu << L) & 0xFFu)
                                : 0x00010001u * ((0xFFFFu << L) & 0xFFFFu);
#pragma unroll
        for (int i = 0; i < 8 * int(sizeof(T)); ++i) {
          if (Check) bad |= (w32[i] & hi) != 0;
          if constexpr (sizeof(T) == 1) {
            uint32_t const t = (w32[i] >> b) & 0x01010101u;
            word |= (((t * 0x00204081u) >> 21) & 0xFu) << (4 * i);
          } else {
            uint32_t const t = (w32[i] >> b) & 0x00010001u;
            word |= ((t | (t >> 15)) & 3u) << (2 * i);
          }
        }
      } else {
        T const* e = reinterpret_cast<T const*>(buf[j]);
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          uint64_t const c = e[i];
          if (Check) bad |= c >= sigma;
          word |= uint32_t(level_bit<Pow2>(c, 0, L, sigma)) << i;
        }
      }
    } else {
      for (uint32_t i = 0; p0 + i < size0; ++i) {
        uint64_t const c = src[p0 + i];
        if (Check) bad |= c >= sigma;
        word |= uint32_t(level_bit<Pow2>(c, 0, L, sigma)) << i;
      }
    }
    out[w] = word;
  }
  if (Check && bad) atomicOr(err, 1u);
}

// For every node of level l with >= 2 symbols: rank0 at its start (stored
// as the node-start rank of the reference) and the count table at its
// split point, C[split] = C[start] + rank0(C[end]) - rank0(C[start]).
__global__ void __launch_bounds__(128)
level_nodes_kernel(TreeView t, LevelNode const* __restrict__ nodes,
                   uint64_t count, uint32_t l, uint64_t* __restrict__ counts,
                   uint64_t* __restrict__ ranks, uint32_t* __restrict__ err) {
  uint64_t const i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= count) return;
  LevelNode const nd = nodes[i];
  ArrayMeta const m = t.rs.meta[l];
  uint64_t const ps = counts[nd.cs];
  uint64_t const pe = counts[nd.end];
  uint64_t const r_start =
      nd.cs ? ps - ecl::detail::rs_rank1<false>(t.rs, m, ps, nullptr) : 0;
  uint64_t const r_end = pe - ecl::detail::rs_rank1<false>(t.rs, m, pe, nullptr);
  counts[nd.split] = ps + (r_end - r_start);
  if (nd.cs) {
    uint64_t const ni = ecl::detail::node_index(t, t.node_base, nd.cs, l);
    if (ni < t.num_ranks) ranks[ni] = r_start;
    else atomicOr(err, 2u);
  }
}

}  // namespace
}  // namespace ewt

#include "split.cuh"
#include "passes.cuh"

namespace ewt {
namespace {

// Levels 1 .. L-1 of a power-of-two alphabet by multi-level passes (see
// passes.cuh); level 0 is already written (or, with an ingested text,
// written by the first pass).
template <class T>
void run_passes(ewt_tree& t, T const* sym, uint64_t n, uint32_t* err,
                cudaStream_t st, T const* ingest_src = nullptr,
                bool ingest_copy = false, bool group_order = false) {
  uint32_t* const words = t.rs.words.as<uint32_t>();
  uint64_t const w1 = t.rs.meta[1].word_off;
  EWT_CUDA(cudaMemsetAsync(words + w1, 0, (t.rs.total_words - w1) * 4, st));
  std::vector<uint64_t> off(t.L), bits(t.L);
  for (uint32_t l = 0; l < t.L; ++l) {
    off[l] = t.rs.meta[l].word_off;
    bits[l] = t.rs.meta[l].bits;
  }
  // With octal group levels at 0 and 3 and at most four levels after level
  // 3, the first pass covers levels 1-3 and hands its level-3 order to the
  // group build, which reads octal level 3 straight from those symbols
  // instead of routing levels 4 and 5 into level-3 order.
  uint32_t first_k = 0;
  DevBuf* keep = nullptr;
  t.groups.order.reset();
  t.groups.order_level = 0;
  if (group_order) {
    std::vector<uint32_t> const w = group_widths(t.L);
    if (w.size() >= 2 && w[0] == 3 && w[1] == 3 && t.L >= 5 && t.L - 4 <= kPMaxK) {
      first_k = 3;
      keep = &t.groups.order;
    }
  }
  run_pass_pipeline<T>(sym, n, t.L, 0, words, off.data(), bits.data(),
                       t.counts_d.as<uint64_t>(), err, st, ingest_src,
                       ingest_copy, first_k, keep);
  if (keep && t.groups.order.get()) t.groups.order_level = 3;
}

thread_local bool t_texts_synced = false;
thread_local bool t_batch_member = false;

// Whether a host text goes straight to the first pass's ingest kernel
// (kernels read the host text: a Grace host's pageable memory, or pinned
// memory): 1- and 2-byte symbols, a given minimal power-of-two alphabet of at
// least four symbols, a 16-byte aligned text.
// A given alphabet 0 .. sigma-1 with sigma a power of two >= 4 (1- and
// 2-byte symbols): the texts whose first pass can read them directly.
template <class T>
bool minimal_pow2_alphabet(const void* alphabet, uint64_t sigma) {
  if constexpr (sizeof(T) > 2) {
    return false;
  } else {
    if (sigma < 4 || (sigma & (sigma - 1)) || !alphabet) return false;
    T const* a = static_cast<T const*>(alphabet);
    for (uint64_t i = 0; i < sigma; ++i)
      if (uint64_t(a[i]) != i) return false;
    return true;
  }
}

template <class T>
bool host_ingest(const void* data, uint64_t n, const void* alphabet, uint64_t sigma) {
  if constexpr (sizeof(T) > 2) {
    return false;
  } else {
    if (!minimal_pow2_alphabet<T>(alphabet, sigma) || n == 0 ||
        reinterpret_cast<uintptr_t>(data) % 16)
      return false;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    int pageable = 0;
    cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev);
    cudaPointerAttributes pa{};
    bool const pinned = cudaPointerGetAttributes(&pa, data) == cudaSuccess &&
                        pa.type == cudaMemoryTypeHost;
    (void)cudaGetLastError();
    return pageable || pinned;
  }
}

template <class T>
void build_typed(ewt_tree& t, const void* data, uint64_t n,
                 const void* alphabet, uint64_t sigma, cudaStream_t st) {
  // ---- text on the device
  DevBuf text_owned;
  T const* d_text;
  T const* ingest = nullptr;  // text read by the first pass's ingest kernel
  bool ingest_copy = false;   // ... a host text, copied by it
  bool const on_device = is_device_pointer(data);
  // The text may still be in flight on the caller's streams; the build runs
  // on its own stream, so order it after all prior device work (once per
  // batch when a batch of builds already did).
  if (on_device && !texts_synchronized()) EWT_CUDA(cudaDeviceSynchronize());
  if (on_device && reinterpret_cast<uintptr_t>(data) % 16 == 0) {
    d_text = static_cast<T const*>(data);
  } else if (on_device) {
    // The kernels read the text with 16-byte vector loads.
    text_owned.alloc(n * sizeof(T));
    EWT_CUDA(cudaMemcpyAsync(text_owned.get(), data, n * sizeof(T),
                             cudaMemcpyDeviceToDevice, st));
    d_text = text_owned.as<T>();
  } else if (host_ingest<T>(data, n, alphabet, sigma)) {
    // read by the first pass's ingest kernel (see run_passes)
    text_owned.alloc(n * sizeof(T) + 64);
    d_text = text_owned.as<T>();
    ingest = static_cast<T const*>(data);
    ingest_copy = true;
  } else {
    text_owned.alloc(n * sizeof(T));
    PhaseTimer pt(EWT_PHASE_H2D, st);
    EWT_CUDA(cudaMemcpyAsync(text_owned.get(), data, n * sizeof(T),
                             cudaMemcpyHostToDevice, st));
    d_text = text_owned.as<T>();
  }
  // ---- alphabet
  t.alphabet.clear();
  if (sigma == 0) {
    if (sizeof(T) <= 2) {
      constexpr uint32_t kWords = (sizeof(T) == 1 ? 256u : 65536u) / 32u;
      DevBuf bm(kWords * 4);
      EWT_CUDA(cudaMemsetAsync(bm.get(), 0, kWords * 4, st));
      uint32_t const blocks =
          static_cast<uint32_t>(std::min<uint64_t>(ceil_div(n, 256),
                                                   uint64_t(sm_count()) * 8));
      presence_kernel<T><<<blocks, 256, 0, st>>>(d_text, n, bm.as<uint32_t>());
      EWT_LAUNCHED();
      std::vector<uint32_t> h(kWords);
      EWT_CUDA(cudaMemcpyAsync(h.data(), bm.get(), kWords * 4,
                               cudaMemcpyDeviceToHost, st));
      EWT_CUDA(cudaStreamSynchronize(st));
      for (uint64_t v = 0; v < kWords * 32ull; ++v)
        if ((h[v >> 5] >> (v & 31)) & 1) t.alphabet.push_back(v);
    } else {
      t.alphabet = detect_alphabet_wide<T>(d_text, n, st);
    }
  } else {
    T const* a = static_cast<T const*>(alphabet);
    EWT_REQUIRE(a != nullptr, EWT_ERR_INVALID_ARGUMENT, "alphabet is null");
    t.alphabet.assign(a, a + sigma);
    for (uint64_t i = 1; i < sigma; ++i)
      EWT_REQUIRE(t.alphabet[i] > t.alphabet[i - 1], EWT_ERR_ALPHABET,
                  "alphabet must be sorted and free of duplicates");
  }
  t.sigma = t.alphabet.size();
  EWT_REQUIRE(t.sigma >= 2, EWT_ERR_ALPHABET,
              "alphabet must hold at least two symbols");
  sigma = t.sigma;
  t.L = h_ceil_log2(sigma);
  t.pow2 = h_is_pow2(sigma);
  t.is_min = true;
  for (uint64_t i = 0; i < sigma; ++i)
    if (t.alphabet[i] != i) { t.is_min = false; break; }
  // ---- shape
  set_tree_shape(t);
  uint32_t const L = t.L;
  auto const level_nodes = make_level_nodes(sigma, L);

  // ---- device tables
  t.err_d.alloc(kTreeErrBytes);
  EWT_CUDA(cudaMemsetAsync(t.err_d.get(), 0, kTreeErrBytes, st));
  uint32_t* err_build = t.err_d.as<uint32_t>() + 1;
  uint32_t const grid_stream =
      static_cast<uint32_t>(std::min<uint64_t>(ceil_div(n, 256),
                                               uint64_t(sm_count()) * 8));
  DevBuf cur_buf;  // minimal symbols when the alphabet is not 0..sigma-1
  T const* sym = d_text;
  if (!t.is_min) {
    std::vector<T> a(t.alphabet.begin(), t.alphabet.end());
    t.alphabet_d.alloc(sigma * sizeof(T));
    EWT_CUDA(cudaMemcpyAsync(t.alphabet_d.get(), a.data(), sigma * sizeof(T),
                             cudaMemcpyHostToDevice, st));
    cur_buf.alloc(n * sizeof(T));
    PhaseTimer pt(EWT_PHASE_HIST, st);
    remap_kernel<T><<<grid_stream, 256, 0, st>>>(
        d_text, n, t.alphabet_d.as<T>(), sigma, cur_buf.as<T>(), err_build);
    EWT_LAUNCHED();
    sym = cur_buf.as<T>();
  }
  // Count table: exact histogram for non-power-of-two alphabets (their level
  // sizes need it); otherwise only C[0] = 0 and C[sigma] = n, the rest is
  // derived level by level.
  t.counts_d.alloc((sigma + 1) * 8);
  t.level_bits.assign(L, n);
  if (!t.pow2) {
    DevBuf occ_d(sigma * 8);
    EWT_CUDA(cudaMemsetAsync(occ_d.get(), 0, sigma * 8, st));
    uint32_t const smem_bins = sigma <= 8192 ? static_cast<uint32_t>(sigma) : 0;
    {
      PhaseTimer pt(EWT_PHASE_HIST, st);
      hist_kernel<T><<<grid_stream, 256, smem_bins * 4, st>>>(
          sym, n, sigma, occ_d.as<unsigned long long>(), smem_bins);
      EWT_LAUNCHED();
    }
    t.occ.assign(sigma, 0);
    EWT_CUDA(cudaMemcpyAsync(t.occ.data(), occ_d.get(), sigma * 8,
                             cudaMemcpyDeviceToHost, st));
    EWT_CUDA(cudaStreamSynchronize(st));
    // Level sizes (wavelet_tree.cuh:776-790): drop symbols whose code ended.
    for (uint32_t l = 0; l < L; ++l)
      for (size_t j = 0; j < t.codes.size(); ++j)
        if (t.codes[j].len <= l) t.level_bits[l] -= t.occ[t.codes_start + j];
    std::vector<uint64_t> c(sigma + 1, 0);
    for (uint64_t i = 1; i <= sigma; ++i) c[i] = c[i - 1] + t.occ[i - 1];
    EWT_CUDA(cudaMemcpyAsync(t.counts_d.get(), c.data(), (sigma + 1) * 8,
                             cudaMemcpyHostToDevice, st));
  } else {
    uint64_t const ends[2] = {0, n};
    EWT_CUDA(cudaMemcpyAsync(t.counts_d.get(), &ends[0], 8,
                             cudaMemcpyHostToDevice, st));
    EWT_CUDA(cudaMemcpyAsync(t.counts_d.as<uint64_t>() + sigma, &ends[1], 8,
                             cudaMemcpyHostToDevice, st));
    EWT_CUDA(cudaStreamSynchronize(st));  // `ends` leaves scope
  }
  for (uint32_t l = 0; l < L; ++l)
    EWT_REQUIRE(t.level_bits[l] > 0, EWT_ERR_UNSUPPORTED,
                "empty level: every symbol with a code this long is absent");

  t.rs.layout(t.level_bits);
  t.ranks_d.alloc(std::max<size_t>(t.nodes.size(), 1) * 8);
  t.node_base_d.alloc((L + 1) * 8);
  EWT_CUDA(cudaMemcpyAsync(t.node_base_d.get(), t.node_base.data(), (L + 1) * 8,
                           cudaMemcpyHostToDevice, st));
  t.nodes_at_level_d.alloc(L * 8);
  EWT_CUDA(cudaMemcpyAsync(t.nodes_at_level_d.get(), t.nodes_at_level.data(),
                           L * 8, cudaMemcpyHostToDevice, st));
  size_t const nc = std::max<size_t>(t.codes.size(), 1);
  std::vector<uint64_t> cl(nc, 0), cb(nc, 0);
  for (size_t i = 0; i < t.codes.size(); ++i) {
    cl[i] = t.codes[i].len;
    cb[i] = t.codes[i].code;
  }
  t.code_len_d.alloc(nc * 8);
  t.code_bits_d.alloc(nc * 8);
  EWT_CUDA(cudaMemcpyAsync(t.code_len_d.get(), cl.data(), nc * 8,
                           cudaMemcpyHostToDevice, st));
  EWT_CUDA(cudaMemcpyAsync(t.code_bits_d.get(), cb.data(), nc * 8,
                           cudaMemcpyHostToDevice, st));
  std::vector<LevelNode> flat;
  std::vector<uint64_t> lv_off(L + 1, 0);
  for (uint32_t l = 0; l < L; ++l) {
    flat.insert(flat.end(), level_nodes[l].begin(), level_nodes[l].end());
    lv_off[l + 1] = flat.size();
  }
  DevBuf lnodes_d(std::max<size_t>(flat.size(), 1) * sizeof(LevelNode));
  EWT_CUDA(cudaMemcpyAsync(lnodes_d.get(), flat.data(),
                           flat.size() * sizeof(LevelNode),
                           cudaMemcpyHostToDevice, st));
  EWT_CUDA(cudaStreamSynchronize(st));  // host vectors above leave scope

  t.n = n;
  fill_tree_view(t);
  TreeView& v = t.view;

  // ---- level 0 bits (with an ingested host text: written by the first pass)
  uint32_t* const words = t.rs.words.as<uint32_t>();
  t.groups.level0_built = false;
  // Group query levels for power-of-two alphabets -- except for the short
  // texts of a batch build: the group build's launch latency would be most
  // of their build time; they get rank blocks on every level instead.
  bool const want_groups =
      groups_eligible(t) && !(t_batch_member && n < kBatchGroupMinSymbols);
  if (!ingest && want_groups && octal_text_eligible(t, sizeof(T))) {
    // level 0 is the octal level 0's top bit plane: both in one read
    build_octal_level0(t, sym, sizeof(T), words + t.rs.meta[0].word_off, t.is_min,
                       err_build, st);
  } else if (!ingest) {
    PhaseTimer pt(EWT_PHASE_FILL, st);
    uint64_t const w0 = ceil_div(t.level_bits[0], 32);
    uint32_t const blocks =
        static_cast<uint32_t>(ceil_div(w0, uint64_t(256) * fill_words<T>()));
    auto k = t.pow2 ? (t.is_min ? fill0_kernel<T, true, true>
                                : fill0_kernel<T, true, false>)
                    : (t.is_min ? fill0_kernel<T, false, true>
                                : fill0_kernel<T, false, false>);
    k<<<blocks, 256, 0, st>>>(sym, t.level_bits[0], L, sigma,
                              words + t.rs.meta[0].word_off, err_build);
    EWT_LAUNCHED();
  }
  // ---- levels
  bool by_passes = false;
  if constexpr (sizeof(T) <= 2) {
    if (t.pow2 && L >= 2) {
      run_passes<T>(t, sym, n, err_build, st, ingest, ingest_copy, want_groups);
      by_passes = true;
    }
  }
  if (by_passes) {
    // All levels' bits came from the multi-level passes; now their counts
    // and the node-start ranks (the count table is complete).
    build_rs_counts(t.rs, 0, L, st);
    for (uint32_t l = 0; l < L; ++l) {
      uint64_t const ncount = lv_off[l + 1] - lv_off[l];
      if (ncount == 0) continue;
      PhaseTimer pt(EWT_PHASE_NODE_RANKS, st);
      level_nodes_kernel<<<static_cast<uint32_t>(ceil_div(ncount, 128)), 128,
                           0, st>>>(v, lnodes_d.as<LevelNode>() + lv_off[l],
                                    ncount, l, t.counts_d.as<uint64_t>(),
                                    t.ranks_d.as<uint64_t>(), err_build);
      EWT_LAUNCHED();
    }
  } else {
    DevBuf ping, pong;
    if (L > 2) ping.alloc(n * sizeof(T));
    if (L > 3) pong.alloc(n * sizeof(T));
    T* bufs[2] = {ping.as<T>(), pong.as<T>()};
    // tiles the fast split leaves to the general one, and their count
    DevBuf slow_tiles((ceil_div(n, kSplitTile) + 1) * 4);
    T const* src = sym;
    for (uint32_t l = 0; l < L; ++l) {
      build_rs_counts(t.rs, l, l + 1, st);
      uint64_t const ncount = lv_off[l + 1] - lv_off[l];
      if (ncount > 0) {
        PhaseTimer pt(EWT_PHASE_NODE_RANKS, st);
        level_nodes_kernel<<<static_cast<uint32_t>(ceil_div(ncount, 128)), 128,
                             0, st>>>(v, lnodes_d.as<LevelNode>() + lv_off[l],
                                      ncount, l, t.counts_d.as<uint64_t>(),
                                      t.ranks_d.as<uint64_t>(), err_build);
        EWT_LAUNCHED();
      }
      if (l + 1 < L) {
        ArrayMeta const& mn = t.rs.meta[l + 1];
        EWT_CUDA(cudaMemsetAsync(words + mn.word_off, 0,
                                 ceil_div(mn.bits, 32) * 4, st));
        bool const write_order = l + 2 < L;
        T* dst = write_order ? bufs[l & 1] : nullptr;
        PhaseTimer pt(EWT_PHASE_SPLIT, st);
        if (t.pow2)
          launch_split<T, true>(write_order, src, dst, n, t.level_bits[l],
                                mn.bits, l, v, words + mn.word_off,
                                slow_tiles.as<uint32_t>(), err_build, st);
        else
          launch_split<T, false>(write_order, src, dst, n, t.level_bits[l],
                                 mn.bits, l, v, words + mn.word_off,
                                 slow_tiles.as<uint32_t>(), err_build, st);
        src = dst;
      }
    }
  }
  build_rs_samples(t.rs, st);
  // binary levels that group levels cover get no rank blocks
  t.rs.skip_blocks.assign(L, 0);
  if (want_groups) {
    uint32_t covered = 0;
    for (uint32_t w : group_widths(L)) covered += w;
    for (uint32_t l = 0; l < covered; ++l) t.rs.skip_blocks[l] = 1;
  }
  build_rank_blocks(t.rs, st);
  v.rs = t.rs.view();
  v.groups = ecl::detail::GroupView{};
  uint32_t build_err = 0;
  EWT_CUDA(cudaMemcpyAsync(&build_err, err_build, 4, cudaMemcpyDeviceToHost,
                           st));
  std::vector<uint64_t> c(sigma + 1);
  EWT_CUDA(cudaMemcpyAsync(c.data(), t.counts_d.get(), (sigma + 1) * 8,
                           cudaMemcpyDeviceToHost, st));
  EWT_CUDA(cudaStreamSynchronize(st));
  EWT_REQUIRE(!(build_err & 1), EWT_ERR_ALPHABET,
              "the text holds a symbol above the alphabet's last symbol");
  EWT_REQUIRE(build_err == 0, EWT_ERR_CUDA,
              "internal consistency check failed while building levels (kind " +
                  std::to_string(build_err) + ")");
  t.counts.assign(c.begin(), c.begin() + sigma);
  t.occ.resize(sigma);
  for (uint64_t i = 0; i < sigma; ++i) t.occ[i] = c[i + 1] - c[i];
  if (want_groups) build_groups(t, c, sym, sizeof(T), st);
  v.groups = t.groups.view();
}

}  // namespace

void set_texts_synchronized(bool v) { t_texts_synced = v; }
bool texts_synchronized() { return t_texts_synced; }
void set_batch_member(bool v) { t_batch_member = v; }

void fill_tree_view(ewt_tree& t) {
  TreeView& v = t.view;
  v.rs = t.rs.view();
  v.counts = t.counts_d.as<uint64_t>();
  v.node_ranks = t.ranks_d.as<uint64_t>();
  v.node_base = t.node_base_d.as<uint64_t>();
  v.nodes_at_level = t.nodes_at_level_d.as<uint64_t>();
  v.code_len = t.code_len_d.as<uint64_t>();
  v.code_bits = t.code_bits_d.as<uint64_t>();
  v.alphabet = t.is_min ? nullptr : t.alphabet_d.get();
  v.n = t.n;
  v.sigma = t.sigma;
  v.codes_start = t.codes_start;
  v.num_ranks = t.nodes.size();
  v.num_nodes_until_last_level = t.nodes_until_last;
  v.levels = t.L;
  v.elem_size = t.elem_size;
  v.is_pow2 = t.pow2;
  v.is_min = t.is_min;
  v.groups = t.groups.view();
}

void build_tree(ewt_tree& t, const void* data, uint64_t n, int elem_size,
                const void* alphabet, uint64_t sigma, cudaStream_t stream) {
  EWT_REQUIRE(data != nullptr && n > 0, EWT_ERR_INVALID_ARGUMENT,
              "text must be non-empty");
  t.elem_size = static_cast<uint32_t>(elem_size);
  switch (elem_size) {
    case 1: build_typed<uint8_t>(t, data, n, alphabet, sigma, stream); break;
    case 2: build_typed<uint16_t>(t, data, n, alphabet, sigma, stream); break;
    case 4: build_typed<uint32_t>(t, data, n, alphabet, sigma, stream); break;
    case 8: build_typed<uint64_t>(t, data, n, alphabet, sigma, stream); break;
    default:
      throw Error(EWT_ERR_INVALID_ARGUMENT, "elem_size must be 1, 2, 4 or 8");
  }
}

void minimal_codes(uint64_t sigma, std::vector<uint64_t>& lens,
                   std::vector<uint64_t>& codes) {
  lens.clear();
  codes.clear();
  for (CodeH const& c : make_codes(sigma)) {
    lens.push_back(c.len);
    codes.push_back(c.code);
  }
}

uint64_t build_bytes_bound(uint64_t n, uint32_t elem_size, uint64_t sigma) {
  uint64_t const L = sigma < 2 ? 1 : h_ceil_log2(sigma);
  uint64_t const text = n * elem_size;
  // resident: level bits, L1/L2/samples, and the query side (group levels
  // or rank blocks, and dense select samples: below 2.5 times the level
  // bits -- octal blocks add 61 % and their samples 33 %)
  uint64_t const level_bits = L * (ceil_div(n, 32) + 64) * 4;
  uint64_t const support = L * (n / 8192 * 8 + n / 256 + n / 512 + 256);
  uint64_t const query = 5 * level_bits / 2;
  // count table, node ranks and node bases (per symbol and level)
  uint64_t const shape = (sigma + 1) * 8 * 4 + L * 64;
  // transient: a copy of a host text, two level orders of the widest
  // minimal symbol, chunk tables and scratch
  uint64_t const order = n * std::max<uint32_t>(elem_size, L > 16 ? 4 : (L > 8 ? 2 : 1));
  uint64_t const transient = text + 2 * order + n / 64 + (64ull << 20);
  return level_bits + support + query + shape + transient;
}

void set_tree_shape(ewt_tree& t) {
  uint64_t const sigma = t.sigma;
  t.codes = make_codes(sigma);
  t.codes_start = sigma - t.codes.size();
  t.nodes = make_nodes(sigma, t.codes);
  uint32_t const L = t.L;
  t.nodes_at_level.assign(L, 0);
  if (t.pow2) {
    for (uint32_t l = 0; l < L; ++l) t.nodes_at_level[l] = (uint64_t(1) << l) - 1;
  } else {
    // Counted as wavelet_tree.cuh:703-724 does (entry l-1 receives the
    // count of the level that just ended); the last level is counted too.
    uint64_t counter = 0;
    for (size_t i = 0; i < t.nodes.size(); ++i) {
      if (i > 0 && t.nodes[i].level > t.nodes[i - 1].level) {
        t.nodes_at_level[t.nodes[i].level - 1] = counter;
        counter = 0;
      }
      counter++;
    }
    if (!t.nodes.empty() && t.nodes.back().level == L - 1)
      t.nodes_at_level[L - 1] = counter;
  }
  t.node_base.assign(L + 1, 0);
  for (uint32_t l = 1; l <= L; ++l)
    t.node_base[l] = t.node_base[l - 1] + t.nodes_at_level[l - 1];
  EWT_REQUIRE(t.node_base[L] == t.nodes.size(), EWT_ERR_UNSUPPORTED,
              "inconsistent node bookkeeping for this alphabet size");
  t.nodes_until_last = L >= 1 ? t.node_base[L - 1] : 0;
}

}  // namespace ewt
