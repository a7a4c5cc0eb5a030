// Wavelet-tree construction on the GPU.
//
// Pipeline (one GPU, one stream; host code orchestrates):
//   1. alphabet: given, or detected (presence bitmap kernel for 1/2-byte
//      symbols, host sort for wider ones) — wavelet_tree.cuh:590-614;
//   2. shape on the host: minimal codes for non-power-of-two alphabets
//      (:2100-2159), node starts (:2501-2532), nodes per level (:703-724);
//   3. histogram kernel: occurrences per minimal symbol, and for a
//      non-minimal alphabet the remapped text (:170-227, :2295-2413);
//   4. for every level l: fill kernel packs the level's bits (bit L-1-l of
//      each symbol, in level order) into words; RankSelect counts of the
//      level; rank0 at the level's node starts (:332-352); then the split
//      kernel stably partitions every node of level l by its bit, which
//      yields the level l+1 order (the reference re-sorts the whole text on
//      the top l+1 code bits with cub::DeviceRadixSort, :806-818);
//   5. select samples of all levels.
// Level order is carried as minimal symbols; the node of symbol c at level l
// is found arithmetically for power-of-two alphabets and by the reference's
// prevPow2 descent otherwise.  No kernel waits on another CTA.
#include <algorithm>
#include <cstring>

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

// --------------------------------------------------------------------------
// Histogram (+ remap to minimal symbols when the alphabet is not 0..s-1).
template <class T, bool IsMin>
__global__ void __launch_bounds__(256)
hist_kernel(T const* __restrict__ text, uint64_t n,
            T const* __restrict__ alphabet, uint64_t sigma,
            T* __restrict__ cur, unsigned long long* __restrict__ occ,
            uint32_t* __restrict__ err, uint32_t smem_bins) {
  extern __shared__ uint32_t hist[];  // smem_bins counters, or none
  bool const use_smem = smem_bins != 0;
  if (use_smem) {
    for (uint32_t i = threadIdx.x; i < smem_bins; i += blockDim.x) hist[i] = 0;
    __syncthreads();
  }
  uint64_t const stride = uint64_t(gridDim.x) * blockDim.x;
  uint32_t bad = 0;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n;
       i += stride) {
    T const x = text[i];
    uint64_t c;
    if (IsMin) {
      c = x;
    } else {
      uint64_t lo = 0, hi = sigma;
      while (lo < hi) {
        uint64_t const mid = (lo + hi) >> 1;
        if (alphabet[mid] < x) lo = mid + 1; else hi = mid;
      }
      c = lo;
    }
    if (c >= sigma) {
      bad = 1;
      c = 0;
    }
    if (!IsMin) cur[i] = static_cast<T>(c);
    if (use_smem) {
      // Aggregate equal symbols of the warp into one shared atomic.
      uint32_t const peers = __match_any_sync(__activemask(), uint32_t(c));
      uint32_t const lane = threadIdx.x & 31;
      if ((__ffs(peers) - 1) == int(lane))
        atomicAdd(&hist[c], __popc(peers));
    } else {
      atomicAdd(&occ[c], 1ull);
    }
  }
  if (bad) atomicOr(err, 1u);
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

// One thread per output word of level l: bit (c >= split) of 32 symbols.
template <class T, bool Pow2>
__global__ void __launch_bounds__(256)
fill_level_kernel(T const* __restrict__ src, uint64_t size_l, uint32_t l,
                  uint32_t L, uint64_t sigma, uint32_t* __restrict__ out) {
  uint64_t const w = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  uint64_t const p0 = w * 32;
  if (p0 >= size_l) return;
  uint32_t word = 0;
  if (p0 + 32 <= size_l) {
    constexpr int kVec = 32 * sizeof(T) / 16;
    uint4 buf[kVec];
    uint4 const* s = reinterpret_cast<uint4 const*>(src + p0);
#pragma unroll
    for (int q = 0; q < kVec; ++q) buf[q] = __ldg(s + q);
    T const* e = reinterpret_cast<T const*>(buf);
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      uint64_t const c = e[j];
      bool b;
      if (Pow2) b = (c >> (L - 1 - l)) & 1;
      else b = c >= node_of<false>(c, l, L, sigma).split;
      word |= uint32_t(b) << j;
    }
  } else {
    for (uint32_t j = 0; p0 + j < size_l; ++j) {
      uint64_t const c = src[p0 + j];
      bool b;
      if (Pow2) b = (c >> (L - 1 - l)) & 1;
      else b = c >= node_of<false>(c, l, L, sigma).split;
      word |= uint32_t(b) << j;
    }
  }
  out[w] = word;
}

// rank0 at each node start of level l (precomputeRanksKernel :332-352).
__global__ void node_ranks_kernel(TreeView t, uint64_t const* __restrict__ starts,
                                  uint64_t first, uint64_t count, uint32_t l,
                                  uint64_t* __restrict__ ranks) {
  uint64_t const i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= count) return;
  ArrayMeta const m = t.rs.meta[l];
  uint64_t const pos = t.counts[starts[first + i]];
  ranks[first + i] =
      pos - ecl::detail::rs_rank1<false>(t.rs, m, pos, nullptr);
}

constexpr uint32_t kSplitThreads = 256;
constexpr uint32_t kSplitItems = 16;
constexpr uint32_t kSplitTile = kSplitThreads * kSplitItems;

// Stable partition of every node of level l by the level's bit: the symbol
// at level position p (node [cs,ce], split s, zeros before p in the level Z)
// moves to C[cs] + (Z - Zn) if c < s, else to C[s] + (p - C[cs]) - (Z - Zn),
// where Zn = rank0 at the node start.  Positions >= size_l (symbols whose
// code already ended) keep their place.  The tile stages (value, dest) in
// shared memory in destination-run order so the global writes coalesce.
template <class T, bool Pow2>
__global__ void __launch_bounds__(kSplitThreads)
split_level_kernel(T const* __restrict__ src, T* __restrict__ dst, uint64_t n,
                   uint64_t size_l, uint32_t l, TreeView t,
                   uint32_t* __restrict__ err) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t* dests = reinterpret_cast<uint64_t*>(smem);
  T* vals = reinterpret_cast<T*>(smem + kSplitTile * sizeof(uint64_t));
  __shared__ uint32_t warp_z[kSplitThreads / 32];

  uint64_t const tile_start = blockIdx.x * uint64_t(kSplitTile);
  uint64_t const tile_end = min(tile_start + kSplitTile, n);
  uint32_t const tid = threadIdx.x;
  ArrayMeta const m = t.rs.meta[l];
  uint64_t const* counts = t.counts;
  uint32_t const L = t.levels;

  // Zeros of level l before the tile start (tile starts are 512-aligned).
  uint64_t z_tile;
  if (tile_start < size_l)
    z_tile = tile_start - (t.rs.l1[m.l1_off + (tile_start >> 16)] +
                           t.rs.l2[m.l2_off + (tile_start >> 9)]);
  else
    z_tile = m.bits - m.ones;

  // Load this thread's 16 consecutive symbols.
  uint64_t const p0 = tile_start + uint64_t(tid) * kSplitItems;
  T item[kSplitItems];
  if (p0 + kSplitItems <= n) {
    constexpr int kVec = kSplitItems * sizeof(T) / 16;
    uint4 buf[kVec];
    uint4 const* s = reinterpret_cast<uint4 const*>(src + p0);
#pragma unroll
    for (int q = 0; q < kVec; ++q) buf[q] = __ldg(s + q);
    T const* e = reinterpret_cast<T const*>(buf);
#pragma unroll
    for (int j = 0; j < int(kSplitItems); ++j) item[j] = e[j];
  } else {
#pragma unroll
    for (int j = 0; j < int(kSplitItems); ++j)
      item[j] = (p0 + j < n) ? src[p0 + j] : T(0);
  }
  uint32_t bits = 0, part = 0;
#pragma unroll
  for (int j = 0; j < int(kSplitItems); ++j) {
    uint64_t const p = p0 + j;
    if (p < size_l) {
      part |= 1u << j;
      uint64_t const c = item[j];
      bool b;
      if (Pow2) b = (c >> (L - 1 - l)) & 1;
      else b = c >= node_of<false>(c, l, L, t.sigma).split;
      bits |= uint32_t(b) << j;
    }
  }
  uint32_t const zcnt = __popc(part & ~bits);
  // CTA exclusive scan of zero counts.
  uint32_t inc = zcnt;
  uint32_t const lane = tid & 31, wid = tid >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t const y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) warp_z[wid] = inc;
  __syncthreads();
  uint32_t wbase = 0, tile_zeros = 0;
#pragma unroll
  for (uint32_t w = 0; w < kSplitThreads / 32; ++w) {
    uint32_t const v = warp_z[w];
    if (w < wid) wbase += v;
    tile_zeros += v;
  }
  uint64_t zp = z_tile + wbase + inc - zcnt;

#pragma unroll
  for (int j = 0; j < int(kSplitItems); ++j) {
    uint64_t const p = p0 + j;
    if (p >= tile_end) break;
    uint64_t slot, dest;
    if ((part >> j) & 1) {
      uint64_t const c = item[j];
      bool const b = (bits >> j) & 1;
      NodeRange const nr = node_of<Pow2>(c, l, L, t.sigma);
      uint64_t const ca = counts[nr.cs];
      uint64_t const cm = counts[nr.split];
      uint64_t const cend = (nr.ce + 1 >= t.sigma) ? t.n : counts[nr.ce + 1];
      uint64_t zn = 0;
      if (nr.cs != 0) {
        uint64_t const ni = ecl::detail::node_index(t, t.node_base, nr.cs, l);
        if (ni < t.num_ranks) zn = t.node_ranks[ni];
        else {
          atomicOr(err, 2u);
          atomicMin(err + 1, blockIdx.x);
        }
      }
      uint64_t const f = max(ca, tile_start);
      uint64_t const zf = ca > tile_start ? zn : z_tile;
      uint64_t const ze =
          cend <= tile_end ? zn + (cm - ca) : z_tile + tile_zeros;
      uint64_t const zb = zp - zf;
      slot = (f - tile_start) + (b ? (ze - zf) + (p - f - zb) : zb);
      dest = b ? cm + (p - ca) - (zp - zn) : ca + (zp - zn);
      if (!b) ++zp;
    } else {
      slot = p - tile_start;
      dest = p;
    }
    // Consistency guard: a slot or destination outside the tile / text
    // means corrupt bookkeeping; record it instead of writing out of range.
    if (slot >= kSplitTile || dest >= n) {
      atomicOr(err, slot >= kSplitTile ? 4u : 8u);
      atomicMin(err + 1, blockIdx.x);
      continue;
    }
    dests[slot] = dest;
    vals[slot] = item[j];
  }
  __syncthreads();
  uint32_t const cnt = static_cast<uint32_t>(tile_end - tile_start);
  for (uint32_t s = tid; s < cnt; s += kSplitThreads) {
    uint64_t const d = dests[s];
    if (d < n) dst[d] = vals[s];
  }
}

template <class T>
void build_typed(ewt_tree& t, const void* data, uint64_t n,
                 const void* alphabet, uint64_t sigma, cudaStream_t st) {
  int const dev = t.device;
  (void)dev;
  // ---- text on the device
  DevBuf text_owned;
  T const* d_text;
  bool const on_device = is_device_pointer(data);
  // The text may still be in flight on the caller's streams; the build runs
  // on its own stream, so order it after all prior device work.
  if (on_device) EWT_CUDA(cudaDeviceSynchronize());
  if (on_device && reinterpret_cast<uintptr_t>(data) % 16 == 0) {
    d_text = static_cast<T const*>(data);
  } else if (on_device) {
    // The kernels read the text with 16-byte vector loads.
    text_owned.alloc(n * sizeof(T));
    EWT_CUDA(cudaMemcpyAsync(text_owned.get(), data, n * sizeof(T),
                             cudaMemcpyDeviceToDevice, st));
    d_text = text_owned.as<T>();
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
      std::vector<T> host(n);
      EWT_CUDA(cudaMemcpyAsync(host.data(), d_text, n * sizeof(T),
                               cudaMemcpyDeviceToHost, st));
      EWT_CUDA(cudaStreamSynchronize(st));
      std::sort(host.begin(), host.end());
      host.erase(std::unique(host.begin(), host.end()), host.end());
      t.alphabet.assign(host.begin(), host.end());
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
  for (size_t i = 0; i < t.nodes.size(); ++i) {
    uint64_t const l = t.nodes[i].level;
    EWT_REQUIRE(i >= t.node_base[l] && i < t.node_base[l + 1],
                EWT_ERR_UNSUPPORTED, "node starts not grouped by level");
  }
  t.nodes_until_last = L >= 1 ? t.node_base[L - 1] : 0;

  // ---- device tables
  t.err_d.alloc(16);
  EWT_CUDA(cudaMemsetAsync(t.err_d.get(), 0, 16, st));
  EWT_CUDA(cudaMemsetAsync(t.err_d.as<uint32_t>() + 2, 0xFF, 4, st));
  DevBuf cur_buf;  // remapped text when the alphabet is not 0..sigma-1
  if (!t.is_min) {
    std::vector<T> a(t.alphabet.begin(), t.alphabet.end());
    t.alphabet_d.alloc(sigma * sizeof(T));
    EWT_CUDA(cudaMemcpyAsync(t.alphabet_d.get(), a.data(), sigma * sizeof(T),
                             cudaMemcpyHostToDevice, st));
    EWT_CUDA(cudaStreamSynchronize(st));
    cur_buf.alloc(n * sizeof(T));
  }
  DevBuf occ_d(sigma * 8);
  EWT_CUDA(cudaMemsetAsync(occ_d.get(), 0, sigma * 8, st));
  {
    uint32_t const smem_bins = sigma <= 8192 ? static_cast<uint32_t>(sigma) : 0;
    uint32_t const blocks = static_cast<uint32_t>(
        std::min<uint64_t>(ceil_div(n, 256), uint64_t(sm_count()) * 8));
    auto k = t.is_min ? hist_kernel<T, true> : hist_kernel<T, false>;
    size_t const smem = smem_bins * 4;
    if (smem > 48 * 1024)
      EWT_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(smem)));
    PhaseTimer pt(EWT_PHASE_HIST, st);
    k<<<blocks, 256, smem, st>>>(d_text, n, t.alphabet_d.as<T>(), sigma,
                                 cur_buf.as<T>(),
                                 occ_d.as<unsigned long long>(),
                                 t.err_d.as<uint32_t>(), smem_bins);
    EWT_LAUNCHED();
  }
  t.occ.assign(sigma, 0);
  uint32_t err = 0;
  EWT_CUDA(cudaMemcpyAsync(t.occ.data(), occ_d.get(), sigma * 8,
                           cudaMemcpyDeviceToHost, st));
  EWT_CUDA(cudaMemcpyAsync(&err, t.err_d.get(), 4, cudaMemcpyDeviceToHost, st));
  EWT_CUDA(cudaStreamSynchronize(st));
  EWT_REQUIRE(err == 0, EWT_ERR_ALPHABET,
              "the text holds a symbol above the alphabet's last symbol");
  t.counts.assign(sigma, 0);
  for (uint64_t c = 1; c < sigma; ++c) t.counts[c] = t.counts[c - 1] + t.occ[c - 1];
  // Level sizes (wavelet_tree.cuh:776-790): drop symbols whose code ended.
  t.level_bits.assign(L, n);
  for (uint32_t l = 0; l < L; ++l)
    for (size_t j = 0; j < t.codes.size(); ++j)
      if (t.codes[j].len <= l) t.level_bits[l] -= t.occ[t.codes_start + j];
  for (uint32_t l = 0; l < L; ++l)
    EWT_REQUIRE(t.level_bits[l] > 0, EWT_ERR_UNSUPPORTED,
                "empty level: every symbol with a code this long is absent");

  t.rs.layout(t.level_bits);
  t.counts_d.alloc(sigma * 8);
  EWT_CUDA(cudaMemcpyAsync(t.counts_d.get(), t.counts.data(), sigma * 8,
                           cudaMemcpyHostToDevice, st));
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
  std::vector<uint64_t> starts(std::max<size_t>(t.nodes.size(), 1), 0);
  for (size_t i = 0; i < t.nodes.size(); ++i) starts[i] = t.nodes[i].start;
  DevBuf starts_d(starts.size() * 8);
  EWT_CUDA(cudaMemcpyAsync(starts_d.get(), starts.data(), starts.size() * 8,
                           cudaMemcpyHostToDevice, st));

  t.n = n;
  TreeView& v = t.view;
  v.rs = t.rs.view();
  v.counts = t.counts_d.as<uint64_t>();
  v.node_ranks = t.ranks_d.as<uint64_t>();
  v.node_base = t.node_base_d.as<uint64_t>();
  v.nodes_at_level = t.nodes_at_level_d.as<uint64_t>();
  v.code_len = t.code_len_d.as<uint64_t>();
  v.code_bits = t.code_bits_d.as<uint64_t>();
  v.alphabet = t.is_min ? nullptr : t.alphabet_d.get();
  v.n = n;
  v.sigma = sigma;
  v.codes_start = t.codes_start;
  v.num_ranks = t.nodes.size();
  v.num_nodes_until_last_level = t.nodes_until_last;
  v.levels = L;
  v.elem_size = sizeof(T);
  v.is_pow2 = t.pow2;
  v.is_min = t.is_min;

  // ---- levels
  T const* src = t.is_min ? d_text : cur_buf.as<T>();
  DevBuf ping, pong;
  if (L > 1) ping.alloc(n * sizeof(T));
  if (L > 2) pong.alloc(n * sizeof(T));
  T* bufs[2] = {ping.as<T>(), pong.as<T>()};
  size_t const split_smem = kSplitTile * (sizeof(uint64_t) + sizeof(T));
  auto split_k = t.pow2 ? split_level_kernel<T, true> : split_level_kernel<T, false>;
  EWT_CUDA(cudaFuncSetAttribute(split_k,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(split_smem)));
  auto fill_k = t.pow2 ? fill_level_kernel<T, true> : fill_level_kernel<T, false>;
  for (uint32_t l = 0; l < L; ++l) {
    uint64_t const size_l = t.level_bits[l];
    uint64_t const words = ceil_div(size_l, 32);
    {
    PhaseTimer pt(EWT_PHASE_FILL, st);
    fill_k<<<static_cast<uint32_t>(ceil_div(words, 256)), 256, 0, st>>>(
        src, size_l, l, L, sigma,
        t.rs.words.as<uint32_t>() + t.rs.meta[l].word_off);
    EWT_LAUNCHED();
    }
    build_rs_counts(t.rs, l, l + 1, st);
    uint64_t const nfirst = t.node_base[l], ncount = t.node_base[l + 1] - nfirst;
    if (ncount > 0) {
      PhaseTimer pt(EWT_PHASE_NODE_RANKS, st);
      node_ranks_kernel<<<static_cast<uint32_t>(ceil_div(ncount, 128)), 128, 0,
                          st>>>(v, starts_d.as<uint64_t>(), nfirst, ncount, l,
                                t.ranks_d.as<uint64_t>());
      EWT_LAUNCHED();
    }
    if (l + 1 < L) {
      T* dst = bufs[l & 1];
      PhaseTimer pt(EWT_PHASE_SPLIT, st);
      split_k<<<static_cast<uint32_t>(ceil_div(n, kSplitTile)), kSplitThreads,
                split_smem, st>>>(src, dst, n, size_l, l, v,
                                  t.err_d.as<uint32_t>() + 1);
      EWT_LAUNCHED();
      src = dst;
      uint32_t build_err[2] = {0, 0};
      EWT_CUDA(cudaMemcpyAsync(build_err, t.err_d.as<uint32_t>() + 1, 8,
                               cudaMemcpyDeviceToHost, st));
      EWT_CUDA(cudaStreamSynchronize(st));
      EWT_REQUIRE(build_err[0] == 0, EWT_ERR_CUDA,
                  "internal consistency check failed while partitioning "
                  "level " + std::to_string(l) + " (kind " +
                      std::to_string(build_err[0]) + ", first tile " +
                      std::to_string(build_err[1]) + ")");
    }
  }
  build_rs_samples(t.rs, st);
  v.rs = t.rs.view();
  EWT_CUDA(cudaStreamSynchronize(st));
}

}  // namespace

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

}  // namespace ewt
