// Multi-level passes of the wavelet-tree build (power-of-two alphabets,
// 1- and 2-byte symbols).
//
// For a power-of-two alphabet (sigma = 2^L) the level-j order is the text
// stably sorted by the top j bits of every symbol, and a symbol's position
// in it is C[prefix] + (symbols with the same j-bit prefix before it).  A
// pass covers levels a+1 .. b (k = b - a <= 4) in one read of the level-a
// order X_a (the text for a = 0):
//
//   1. chunk table: every level-a node [C[N << (L-a)], C[(N+1) << (L-a)])
//      is cut into chunks of kPChunk symbols (chunks never cross a node);
//   2. digit counts: per chunk, how many symbols carry each k-bit digit
//      (the bits a .. b-1 from the top);
//   3. per-node scan of those counts: digit counts before every chunk inside
//      its node, and the count table C at every class start of levels
//      a+1 .. b (node start + counts of the smaller digits);
//   4. the pass kernel: each CTA walks its chunks tile by tile (8192 one-
//      or 4096 two-byte symbols, bulk-copied into shared memory),
//      partitions the tile
//      k times in shared memory -- level a+r+1 order = stable partition of
//      every class of level a+r by the level's bit, with destinations from a
//      CTA scan of zero counts -- and after each partition writes the tile's
//      runs of level a+r+1 bits to their places (C + running class count);
//      the level-b order goes out the same way when another pass follows.
//
// The reference re-sorts the whole text with a radix sort per level and
// fills each level from it (wavelet_tree.cuh:806-818, 2422-2493); the bits
// written here are identical: both are bit (L-1-j) of the level-j order.
// Edge words shared by two runs are combined with atomicOr into levels that
// are zeroed beforehand; all global writes are bounds-checked.
#pragma once

#include <type_traits>
#include <vector>

#include "bulk_copy.cuh"

namespace ewt {
namespace {

constexpr uint32_t kPThreads = 256;
constexpr uint32_t kPWarps = kPThreads / 32;
constexpr uint32_t kPChunk = 65536;               // symbols per chunk
constexpr uint32_t kPMaxK = 4;                     // levels per pass
constexpr uint32_t kPMaxDigits = 1u << kPMaxK;
constexpr uint32_t kPMaxStartLevel = 12;           // <= 4096 nodes per pass
// Bulk-copy stages per CTA: one, so that six CTAs fit an SM (their
// staggered tiles hide each other's copies; measured faster than two stages
// at five CTAs per SM).
constexpr uint32_t kPStages = 1;

struct PassArgs {
  uint64_t n;
  uint32_t L, a, k, nodes;  // nodes = 2^a
  uint32_t* words;
  uint64_t word_off[kPMaxK + 1];  // index r: level a + r (r = 1..k)
  uint64_t nwords[kPMaxK + 1];
  uint64_t* counts;        // count table C, sigma + 1 entries
  uint32_t* chunk_first;   // per node: first chunk; [nodes] = chunk count
  uint32_t* chunk_tot;     // [chunk][kPMaxDigits]
  uint64_t* chunk_pre;     // [chunk][kPMaxDigits]
  uint64_t* node_tot;      // [node][kPMaxDigits]
  uint32_t* err;
};

struct ChunkInfo {
  uint64_t start;
  uint32_t len, node;
};


// Chunk c -> its node and symbol range (chunk_first is non-decreasing; the
// node is the last one whose first chunk is <= c).
__device__ __forceinline__ ChunkInfo locate_chunk(PassArgs const& p,
                                                  uint32_t c) {
  uint32_t lo = 0, hi = p.nodes - 1;
  while (lo < hi) {
    uint32_t const mid = (lo + hi + 1) >> 1;
    if (p.chunk_first[mid] <= c) lo = mid; else hi = mid - 1;
  }
  uint32_t const sh = p.L - p.a;
  uint64_t const s = p.counts[uint64_t(lo) << sh];
  uint64_t const e = p.counts[uint64_t(lo + 1) << sh];
  ChunkInfo ci;
  ci.node = lo;
  ci.start = s + uint64_t(c - p.chunk_first[lo]) * kPChunk;
  ci.len = ci.start < e ? static_cast<uint32_t>(min(uint64_t(kPChunk), e - ci.start))
                        : 0u;
  return ci;
}

// 1. Chunks per node and their exclusive prefix (one CTA of 1024 threads,
//    at most 4096 nodes).
__global__ void __launch_bounds__(1024)
chunk_table_kernel(PassArgs p) {
  __shared__ uint32_t warp_sum[32];
  uint32_t const tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  uint32_t const per = (p.nodes + 1023) / 1024;  // <= 4
  uint32_t const sh = p.L - p.a;
  uint32_t nc[4] = {0, 0, 0, 0};
  uint32_t local = 0;
  for (uint32_t j = 0; j < per; ++j) {
    uint32_t const N = tid * per + j;
    if (N < p.nodes) {
      uint64_t const len = p.counts[uint64_t(N + 1) << sh] -
                           p.counts[uint64_t(N) << sh];
      nc[j] = static_cast<uint32_t>((len + kPChunk - 1) / kPChunk);
      local += nc[j];
    }
  }
  uint32_t inc = local;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t const y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) warp_sum[wid] = inc;
  __syncthreads();
  uint32_t base = 0;
  for (uint32_t w = 0; w < wid; ++w) base += warp_sum[w];
  uint32_t run = base + inc - local;
  for (uint32_t j = 0; j < per; ++j) {
    uint32_t const N = tid * per + j;
    if (N < p.nodes) p.chunk_first[N] = run;
    run += nc[j];
  }
  if (tid == 1023) p.chunk_first[p.nodes] = run;
}

// Digit of a symbol within the pass: the k bits below its level-a prefix.
template <class T>
__device__ __forceinline__ uint32_t pass_digit(T s, uint32_t shift,
                                               uint32_t mask) {
  return (static_cast<uint32_t>(s) >> shift) & mask;
}

// 2. Digit counts per chunk.  Private per-thread counters in shared memory
//    (conflict-free: counter d of thread t at d * 256 + t) bumped by shared
//    reductions, two sets, reduced at the end of every chunk.
template <class T>
__global__ void __launch_bounds__(kPThreads)
digit_count_kernel(T const* __restrict__ x, PassArgs p) {
  __shared__ uint32_t cnt_a[kPMaxDigits * kPThreads];
  __shared__ uint32_t cnt_b[kPMaxDigits * kPThreads];
  __shared__ uint32_t tot[kPMaxDigits];
  __shared__ ChunkInfo ck;
  uint32_t const tid = threadIdx.x;
  uint32_t const digits = 1u << p.k;
  uint32_t const dshift = p.L - p.a - p.k, dmask = digits - 1;
  uint32_t const total = p.chunk_first[p.nodes];
  for (uint32_t c = blockIdx.x; c < total; c += gridDim.x) {
    if (tid == 0) ck = locate_chunk(p, c);
    if (tid < kPMaxDigits) tot[tid] = 0;
    for (uint32_t d = 0; d < digits; ++d) {
      cnt_a[d * kPThreads + tid] = 0;
      cnt_b[d * kPThreads + tid] = 0;
    }
    __syncthreads();
    uint64_t const s = ck.start, e = s + ck.len;
    // 16-byte aligned body with vector loads, scalar head and tail.
    uint64_t const b0 = min(e, (s * sizeof(T) + 15) / 16 * 16 / sizeof(T));
    uint64_t const b1 = max(b0, e * sizeof(T) / 16 * 16 / sizeof(T));
    for (uint64_t i = s + tid; i < b0; i += kPThreads)
      ++cnt_a[pass_digit<T>(x[i], dshift, dmask) * kPThreads + tid];
    for (uint64_t i = b1 + tid; i < e; i += kPThreads)
      ++cnt_b[pass_digit<T>(x[i], dshift, dmask) * kPThreads + tid];
    uint4 const* v = reinterpret_cast<uint4 const*>(x + b0);
    uint64_t const nv = (b1 - b0) * sizeof(T) / 16;
    // Counter d of this thread sits at byte d * 1024 + 4 * tid of each set;
    // the digits of four bytes (two 16-bit symbols) come out of one SWAR
    // shift-and-mask, each then costs one multiply-add for its address.
    uint32_t const base_a = smem_u32(cnt_a) + 4 * tid;
    uint32_t const base_b = smem_u32(cnt_b) + 4 * tid;
    uint32_t const lanes_mask =
        sizeof(T) == 1 ? 0x01010101u * dmask : 0x00010001u * dmask;
    // fire-and-forget shared-memory increments: no read-modify-write
    // chain between consecutive symbols
    auto bump = [](uint32_t addr) {
      asm volatile("red.shared.add.u32 [%0], 1;" ::"r"(addr) : "memory");
    };
    // four 16-byte loads in flight per thread, then their symbols
    for (uint64_t i = tid; i < nv; i += 4 * kPThreads) {
      uint4 q[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        uint64_t const at = i + uint64_t(u) * kPThreads;
        q[u] = at < nv ? v[at] : make_uint4(0, 0, 0, 0);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (i + uint64_t(u) * kPThreads >= nv) break;
        uint32_t const w[4] = {q[u].x, q[u].y, q[u].z, q[u].w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          uint32_t const dw = (w[j] >> dshift) & lanes_mask;
#pragma unroll
          for (int h = 0; h < int(4 / sizeof(T)); ++h) {
            uint32_t const d =
                (dw >> (8 * sizeof(T) * h)) & (sizeof(T) == 1 ? 0xFFu : 0xFFFFu);
            bump(((h & 1) ? base_b : base_a) + d * (kPThreads * 4));
          }
        }
      }
    }
    __syncthreads();
    for (uint32_t d = 0; d < digits; ++d) {
      uint32_t v2 = cnt_a[d * kPThreads + tid] + cnt_b[d * kPThreads + tid];
      for (int o = 16; o > 0; o >>= 1) v2 += __shfl_down_sync(0xffffffffu, v2, o);
      if ((tid & 31) == 0) atomicAdd(&tot[d], v2);
    }
    __syncthreads();
    if (tid < kPMaxDigits)
      p.chunk_tot[uint64_t(c) * kPMaxDigits + tid] = tid < digits ? tot[tid] : 0u;
    __syncthreads();
  }
}

// 2'. The first pass's read of the text (a = 0: one node, chunks of kPChunk
//     symbols from the text start): each CTA takes whole chunks, writes
//     level 0 (the top bit of every symbol) and counts the pass's digits per
//     chunk, and for a host text (dev != null) also copies the chunk into
//     device memory -- the level-0 fill, the first digit count and the copy
//     in one read of the text.  Symbols at or above 2^L set bit 0 of err.
template <class T>
__global__ void __launch_bounds__(kPThreads)
ingest_kernel(T const* __restrict__ host, T* __restrict__ dev,
              uint32_t* __restrict__ level0, PassArgs p) {
  __shared__ uint32_t cnt[kPMaxDigits * kPThreads];
  __shared__ uint32_t tot[kPMaxDigits];
  constexpr uint32_t kSym = 32;  // symbols per thread step: one level-0 word
  constexpr uint32_t kVec = kSym * sizeof(T) / 16;
  uint32_t const tid = threadIdx.x;
  uint32_t const digits = 1u << p.k;
  uint32_t const dshift = p.L - p.k, dmask = digits - 1;
  uint32_t const total = p.chunk_first[p.nodes];
  // bits at or above L in every symbol lane of a 32-bit word
  uint32_t const hi_lanes = sizeof(T) == 1
                                ? ((0xFFu << p.L) & 0xFFu) * 0x01010101u
                                : ((0xFFFFu << p.L) & 0xFFFFu) * 0x00010001u;
  uint32_t bad = 0;
  for (uint32_t c = blockIdx.x; c < total; c += gridDim.x) {
    if (tid < kPMaxDigits) tot[tid] = 0;
    for (uint32_t d = 0; d < digits; ++d) cnt[d * kPThreads + tid] = 0;
    __syncthreads();
    uint64_t const s = uint64_t(c) * kPChunk;
    uint64_t const e = min(p.n, s + kPChunk);
    for (uint64_t u = s / kSym + tid; u * kSym < e; u += kPThreads) {
      uint64_t const p0 = u * kSym;
      uint32_t const valid = static_cast<uint32_t>(min(uint64_t(kSym), e - p0));
      uint32_t w[kSym * sizeof(T) / 4];
      if (valid == kSym) {
        uint4 const* src = reinterpret_cast<uint4 const*>(host + p0);
        uint4* dst = reinterpret_cast<uint4*>(dev + p0);
#pragma unroll
        for (uint32_t i = 0; i < kVec; ++i) {
          uint4 const x = src[i];
          if (dev) dst[i] = x;
          w[4 * i] = x.x;
          w[4 * i + 1] = x.y;
          w[4 * i + 2] = x.z;
          w[4 * i + 3] = x.w;
        }
      } else {
#pragma unroll
        for (uint32_t i = 0; i < kSym * sizeof(T) / 4; ++i) w[i] = 0;
        for (uint32_t i = 0; i < valid; ++i) {
          T const v = host[p0 + i];
          if (dev) dev[p0 + i] = v;
          w[(i * sizeof(T)) >> 2] |= uint32_t(v) << (8 * ((i * sizeof(T)) & 3));
        }
      }
      uint32_t bits = 0, over = 0;
      uint32_t const top = p.L - 1;
#pragma unroll
      for (uint32_t i = 0; i < kSym * sizeof(T) / 4; ++i) {
        if constexpr (sizeof(T) == 1) {
          uint32_t const t1 = (w[i] >> top) & 0x01010101u;
          bits |= (((t1 * 0x00204081u) >> 21) & 0xFu) << (4 * i);
        } else {
          uint32_t const t1 = (w[i] >> top) & 0x00010001u;
          bits |= ((t1 | (t1 >> 15)) & 3u) << (2 * i);
        }
        over |= w[i] & hi_lanes;
        // digits of the first pass: the top k bits
#pragma unroll
        for (uint32_t h = 0; h < 4 / sizeof(T); ++h) {
          uint32_t const sym = (w[i] >> (8 * sizeof(T) * h)) & (sizeof(T) == 1 ? 0xFFu : 0xFFFFu);
          if (i * (4 / sizeof(T)) + h < valid)
            asm volatile("red.shared.add.u32 [%0], 1;" ::"r"(smem_u32(
                             &cnt[((sym >> dshift) & dmask) * kPThreads + tid]))
                         : "memory");
        }
      }
      bad |= over;
      level0[u] = bits;  // bits past the text end are zero
    }
    __syncthreads();
    for (uint32_t d = 0; d < digits; ++d) {
      uint32_t v2 = cnt[d * kPThreads + tid];
      for (int o = 16; o > 0; o >>= 1) v2 += __shfl_down_sync(0xffffffffu, v2, o);
      if ((tid & 31) == 0) atomicAdd(&tot[d], v2);
    }
    __syncthreads();
    if (tid < kPMaxDigits)
      p.chunk_tot[uint64_t(c) * kPMaxDigits + tid] = tid < digits ? tot[tid] : 0u;
    __syncthreads();
  }
  if (bad) atomicOr(p.err, 1u);
}

// 3. One CTA of 1024 threads per (level-a node, digit): exclusive counts of
//    the digit before each chunk of the node (8 consecutive chunks per
//    thread and step, block scan), and the node's total of the digit.
constexpr uint32_t kScanThreads = 1024;
constexpr uint32_t kScanPer = 8;

__global__ void __launch_bounds__(kScanThreads)
pass_scan_kernel(PassArgs p) {
  __shared__ uint32_t warp_sum[32];
  __shared__ uint32_t step_total;
  uint32_t const tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  uint32_t const N = blockIdx.x >> p.k, d = blockIdx.x & ((1u << p.k) - 1);
  uint32_t const c0 = p.chunk_first[N], c1 = p.chunk_first[N + 1];
  uint64_t carry = 0;
  for (uint32_t base = c0; base < c1; base += kScanThreads * kScanPer) {
    uint32_t v[kScanPer], s = 0;
#pragma unroll
    for (uint32_t j = 0; j < kScanPer; ++j) {
      uint32_t const c = base + tid * kScanPer + j;
      v[j] = c < c1 ? p.chunk_tot[uint64_t(c) * kPMaxDigits + d] : 0u;
      s += v[j];
    }
    uint32_t inc = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t const y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= static_cast<uint32_t>(o)) inc += y;
    }
    if (lane == 31) warp_sum[wid] = inc;
    __syncthreads();
    if (wid == 0) {
      uint32_t const x = warp_sum[lane];
      uint32_t y = x;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t const t = __shfl_up_sync(0xffffffffu, y, o);
        if (lane >= static_cast<uint32_t>(o)) y += t;
      }
      warp_sum[lane] = y - x;
      if (lane == 31) step_total = y;
    }
    __syncthreads();
    uint64_t ex = carry + warp_sum[wid] + (inc - s);
#pragma unroll
    for (uint32_t j = 0; j < kScanPer; ++j) {
      uint32_t const c = base + tid * kScanPer + j;
      if (c < c1) p.chunk_pre[uint64_t(c) * kPMaxDigits + d] = ex;
      ex += v[j];
    }
    carry += step_total;
    __syncthreads();  // warp_sum and step_total are rewritten next step
  }
  if (tid == 0) p.node_tot[uint64_t(N) * kPMaxDigits + d] = carry;
}

// C at the start of every digit class of every level-a node: the node start
// plus the totals of the smaller digits.
__global__ void __launch_bounds__(256)
pass_counts_kernel(PassArgs p) {
  uint32_t const N = blockIdx.x * blockDim.x + threadIdx.x;
  if (N >= p.nodes) return;
  uint32_t const digits = 1u << p.k;
  uint32_t const sh = p.L - p.a - p.k;
  uint64_t pos = p.counts[uint64_t(N) << (p.L - p.a)];
  for (uint32_t d = 0; d + 1 < digits; ++d) {
    pos += p.node_tot[uint64_t(N) * kPMaxDigits + d];
    p.counts[((uint64_t(N) << p.k) | (d + 1)) << sh] = pos;
  }
}

// ---- pass kernel helpers ---------------------------------------------------

// Tile shape per symbol size: 32 one-byte or 16 two-byte symbols per thread.
template <class T>
struct PassShape {
  static constexpr uint32_t kItems = sizeof(T) == 1 ? 32 : 16;
  static constexpr uint32_t kTile = kPThreads * kItems;
  static constexpr uint32_t kWords = kItems * sizeof(T) / 4;
};

template <class T>
__host__ __device__ constexpr uint32_t pass_stage_bytes() {
  return PassShape<T>::kTile * sizeof(T) + 32;
}
template <class T>
__host__ __device__ constexpr uint32_t pass_sbuf_elems() {
  return PassShape<T>::kTile + 32;
}
template <class T>
__host__ __device__ constexpr size_t pass_smem_bytes() {
  return size_t(kPStages) * pass_stage_bytes<T>() +
         2 * size_t(pass_sbuf_elems<T>()) * sizeof(T);
}

// A thread's symbols as bytes in 32-bit words.
template <class T>
struct SymW {
  uint32_t w[PassShape<T>::kWords];
  __device__ __forceinline__ uint32_t get(int i) const {
    if constexpr (sizeof(T) == 1) return (w[i >> 2] >> (8 * (i & 3))) & 0xFFu;
    else return (w[i >> 1] >> (16 * (i & 1))) & 0xFFFFu;
  }
};

// Bit `b` of each of the thread's symbols as a mask (SWAR: one multiply
// gathers the bit of four bytes).
template <class T>
__device__ __forceinline__ uint32_t sym_bits(SymW<T> const& s, uint32_t b) {
  uint32_t m = 0;
  if constexpr (sizeof(T) == 1) {
#pragma unroll
    for (int i = 0; i < int(PassShape<T>::kWords); ++i) {
      uint32_t const t = (s.w[i] >> b) & 0x01010101u;
      m |= (((t * 0x00204081u) >> 21) & 0xFu) << (4 * i);
    }
  } else {
#pragma unroll
    for (int i = 0; i < int(PassShape<T>::kWords); ++i) {
      uint32_t const t = (s.w[i] >> b) & 0x00010001u;
      m |= ((t | (t >> 15)) & 3u) << (2 * i);
    }
  }
  return m;
}

// Store of one symbol at a 32-bit shared-memory address.
template <class T>
__device__ __forceinline__ void st_shared(uint32_t addr, uint32_t v) {
  if constexpr (sizeof(T) == 1)
    asm volatile("st.shared.u8 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
  else
    asm volatile("st.shared.u16 [%0], %1;" ::"r"(addr), "h"(static_cast<uint16_t>(v))
                 : "memory");
}

// 4. The pass kernel.  Persistent: CTA b takes chunks b, b + G, ...; tiles
//    of a chunk in order (running class counts carry from tile to tile).
template <class T, bool WriteOrder, uint32_t K>
__global__ void __launch_bounds__(kPThreads, 6)
pass_kernel(T const* __restrict__ src, T* __restrict__ dst, PassArgs p) {
  using Shape = PassShape<T>;
  constexpr uint32_t kItems = Shape::kItems;
  constexpr uint32_t kTile = Shape::kTile;
  constexpr uint32_t kStage = pass_stage_bytes<T>();
  constexpr uint32_t kSElems = pass_sbuf_elems<T>();
  constexpr uint32_t kVE = 16 / sizeof(T);  // symbols per 16-byte unit
  constexpr uint32_t kFull = kItems == 32 ? ~0u : (1u << kItems) - 1u;
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned char* const ring = smem;
  T* const S0 = reinterpret_cast<T*>(smem + kPStages * kStage);
  T* const S1 = S0 + kSElems;
  __shared__ __align__(8) uint64_t bars[kPStages];
  __shared__ __align__(16) uint32_t bitbuf[2][kPThreads + 1];
  __shared__ uint32_t incl_s[kPThreads], zmask_s[kPThreads];
  __shared__ uint32_t warp_tot[kPWarps];
  __shared__ uint16_t cls[kPMaxK + 1][kPMaxDigits + 1];
  __shared__ uint16_t T0s[kPMaxDigits / 2], T1s[kPMaxDigits / 2];  // class table
  __shared__ uint32_t warp_pre[kPWarps + 1];  // zeros before each warp
  __shared__ uint64_t Cb[kPMaxK + 1][kPMaxDigits];
  __shared__ uint64_t run[kPMaxK + 1][kPMaxDigits];
  __shared__ uint64_t gpos[kPMaxDigits];             // level-b run starts
  // global bit of a class run's tile position 0 (its first bit's global
  // position minus its start in the tile)
  __shared__ uint64_t gpb[kPMaxK + 1][kPMaxDigits];
  __shared__ ChunkInfo ck;
  __shared__ uint32_t fix_n[2];  // threads whose symbols span a class boundary
  __shared__ uint16_t fix_list[kPThreads];

  uint32_t const tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  uint32_t const L = p.L, a = p.a;
  constexpr uint32_t k = K;  // levels of this pass (p.k)
  uint32_t const total_chunks = p.chunk_first[p.nodes];
  if (tid < 2) fix_n[tid] = 0;
  uint32_t const G = gridDim.x;

  // ---- producer state (thread 0): the tile sequence of this CTA
  uint32_t pc = blockIdx.x, pt = 0;
  uint64_t pstart = 0;
  uint32_t plen = 0;
  auto p_fix = [&]() {  // skip to a chunk with symbols
    while (pc < total_chunks) {
      ChunkInfo const ci = locate_chunk(p, pc);
      if (ci.len) { pstart = ci.start; plen = ci.len; return; }
      pc += G;
    }
  };
  auto issue = [&](uint32_t stage) {  // load (pc, pt) into `stage`, advance
    uint64_t const ts = pstart + uint64_t(pt) * kTile;
    uint32_t const tc = min(kTile, plen - pt * kTile);
    uint64_t const b0 = ts * sizeof(T) / 16 * 16;
    uint64_t const b1 = (ts + tc) * sizeof(T) / 16 * 16;
    uint32_t const bytes = static_cast<uint32_t>(b1 > b0 ? b1 - b0 : 0);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                     smem_u32(&bars[stage])),
                 "r"(bytes)
                 : "memory");
    if (bytes)
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
          "[%0], [%1], %2, [%3];" ::"r"(smem_u32(ring + stage * kStage)),
          "l"(reinterpret_cast<unsigned char const*>(src) + b0), "r"(bytes),
          "r"(smem_u32(&bars[stage]))
          : "memory");
    if (++pt * kTile >= plen) {
      pt = 0;
      pc += G;
      p_fix();
    }
  };

  if (tid == 0) {
    for (uint32_t s = 0; s < kPStages; ++s) mbar_init(&bars[s], 1);
    fence_async_shared();
    p_fix();
    for (uint32_t s = 0; s < kPStages && pc < total_chunks; ++s) issue(s);
  }
  __syncthreads();

  uint64_t q = 0;  // tiles consumed by this CTA
  for (uint32_t c = blockIdx.x; c < total_chunks; c += G) {
    if (tid == 0) ck = locate_chunk(p, c);
    __syncthreads();
    ChunkInfo const ci = ck;
    __syncthreads();  // ck is rewritten for the next chunk
    if (ci.len == 0) continue;  // never produced by the chunk table
    // class bases and running counts of this chunk
    for (uint32_t r = 1; r <= k; ++r) {
      if (tid < (1u << r)) {
        uint32_t const sh = L - a - r;
        Cb[r][tid] = p.counts[((uint64_t(ci.node) << r) | tid) << sh];
        uint64_t s = 0;
        uint32_t const per = 1u << (k - r);
        for (uint32_t d = tid * per; d < (tid + 1) * per; ++d)
          s += p.chunk_pre[uint64_t(c) * kPMaxDigits + d];
        run[r][tid] = s;
      }
    }
    uint32_t const tiles = (ci.len + kTile - 1) / kTile;
    for (uint32_t ti = 0; ti < tiles; ++ti, ++q) {
      uint32_t const stage = static_cast<uint32_t>(q % kPStages);
      uint64_t const ts = ci.start + uint64_t(ti) * kTile;
      uint32_t const tcnt = min(kTile, ci.len - ti * kTile);
      uint64_t const b0 = ts * sizeof(T) / 16 * 16;
      uint64_t const b1 = (ts + tcnt) * sizeof(T) / 16 * 16;
      if (!mbar_wait(&bars[stage], static_cast<uint32_t>((q / kPStages) & 1)))
        atomicOr(p.err, 16u);
      if (tid == 0) {
        cls[0][0] = 0;
        cls[0][1] = static_cast<uint16_t>(tcnt);
      }
      uint32_t const p0 = tid * kItems;
      uint32_t const nvalid = p0 >= tcnt ? 0u : min(kItems, tcnt - p0);
      uint32_t const vmask = nvalid >= 32 ? ~0u : (1u << nvalid) - 1u;
      T* Sc = nullptr;  // level a+r order in shared memory (r >= 1)
#pragma unroll
      for (uint32_t r = 0; r <= k; ++r) {
        T* const Sn = (r & 1) ? S1 : S0;
        // -- a. the thread's symbols of the level a+r order
        SymW<T> e;
        if (r == 0) {
          unsigned char const* rb = ring + stage * kStage;
          uint64_t const g0 = (ts + p0) * sizeof(T);
          if (nvalid == kItems && g0 + kItems * sizeof(T) <= b1) {
            uint32_t const o = static_cast<uint32_t>(g0 - b0);
            uint32_t const* w32 = reinterpret_cast<uint32_t const*>(rb + (o & ~3u));
            uint32_t const sh = (o & 3u) * 8;
#pragma unroll
            for (int i = 0; i < int(Shape::kWords); ++i)
              e.w[i] = __funnelshift_r(w32[i], w32[i + 1], sh);
          } else {
#pragma unroll
            for (int i = 0; i < int(Shape::kWords); ++i) e.w[i] = 0;
#pragma unroll
            for (uint32_t i = 0; i < kItems; ++i) {
              if (i < nvalid) {
                uint64_t const g = ts + p0 + i;
                uint32_t const v =
                    g * sizeof(T) < b1
                        ? reinterpret_cast<T const*>(rb)[g - b0 / sizeof(T)]
                        : src[g];
                e.w[(i * sizeof(T)) >> 2] |= v << (8 * ((i * sizeof(T)) & 3));
              }
            }
          }
        } else {
          uint4 const* v = reinterpret_cast<uint4 const*>(Sc + p0);
#pragma unroll
          for (int i = 0; i < int(Shape::kWords / 4); ++i) {
            uint4 const x = v[i];
            e.w[4 * i] = x.x;
            e.w[4 * i + 1] = x.y;
            e.w[4 * i + 2] = x.z;
            e.w[4 * i + 3] = x.w;
          }
        }
        uint32_t const bits = sym_bits<T>(e, L - 1 - a - r) & vmask;
        if (r >= 1) {
          if constexpr (kItems == 32) bitbuf[r & 1][tid] = bits;
          else reinterpret_cast<uint16_t*>(bitbuf[r & 1])[tid] = static_cast<uint16_t>(bits);
        }
        uint32_t z = 0, inc = 0;
        // Threads whose symbols span a class boundary (levels >= a+1) are
        // listed and their symbols partitioned afterwards, one listed thread
        // per warp and one symbol per lane, so that the main partition runs
        // the one-class loop without divergence.
        uint32_t const cshift = L - a - r;  // class = bits above the level bit
        uint32_t const cmask = (1u << r) - 1u;
        uint32_t const c_first = (e.get(0) >> cshift) & cmask;
        bool const one_class =
            nvalid == kItems && c_first == ((e.get(kItems - 1) >> cshift) & cmask);
        bool const to_fix = r < k && nvalid == kItems && !one_class;
        if (to_fix)
          fix_list[atomicAdd(&fix_n[r & 1], 1u)] = static_cast<uint16_t>(tid);
        if (r < k) {
          z = __popc(vmask & ~bits);
          inc = z;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            uint32_t const y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= static_cast<uint32_t>(o)) inc += y;
          }
          incl_s[tid] = inc;
          zmask_s[tid] = vmask & ~bits;
          if (lane == 31) warp_tot[wid] = inc;
        }
        __syncthreads();  // A: symbols read, masks and warp totals ready
        if (tid == 0) fix_n[(r + 1) & 1] = 0;  // last read at level r - 1
        if (r == 0 && tid == 0) {
          // the copy stage is free again: start the CTA's next tile
          fence_async_shared();
          if (pc < total_chunks) issue(stage);
        }
        // -- b. level a+r bits out (level a's came from the previous pass),
        //    32 tile positions per writer: a unit inside one class run is
        //    a 32-bit window of the run's global bits, so it fills one whole
        //    output word (its low bits from the unit before) and ORs its
        //    high bits into the next word only where the next unit is not
        //    inside the run too; words shared with another run or tile are
        //    ORed.  Units across a class boundary or the tile end OR each
        //    class's piece.
        if (r >= 1) {
          constexpr uint32_t kTPU = 32 / kItems;  // threads per unit
          uint32_t* const out = p.words + p.word_off[r];
          uint64_t const nw = p.nwords[r];
          uint32_t const* bb = bitbuf[r & 1];
          if (tid % kTPU == 0 && p0 < tcnt) {
            uint32_t const u = tid / kTPU;
            uint32_t const ce = cls[r][c_first + 1];
            uint32_t const w = bb[u];
            if (p0 + 32 <= ce) {
              uint64_t const g = gpb[r][c_first] + p0;
              uint32_t const s = static_cast<uint32_t>(g) & 31u;
              uint64_t const q = g >> 5;
              bool const spill = s && p0 + 64 > ce;
              if (q >= nw || (spill && q + 1 >= nw)) {
                atomicOr(p.err, 8u);
              } else if (s == 0) {
                out[q] = w;
              } else {
                if (p0 >= cls[r][c_first] + s)
                  out[q] = (w << s) | (bb[u - 1] >> (32 - s));
                else
                  atomicOr(out + q, w << s);
                if (spill) atomicOr(out + q + 1, w >> (32 - s));
              }
            } else {
              uint32_t const end = min(p0 + 32, tcnt);
              for (uint32_t x = p0, cc = c_first; x < end; ++cc) {
                uint32_t const xe = min(end, static_cast<uint32_t>(cls[r][cc + 1]));
                if (xe > x) {
                  uint32_t const len = xe - x;
                  uint32_t const v = (w >> (x - p0)) & (len >= 32 ? ~0u : (1u << len) - 1u);
                  uint64_t const g = gpb[r][cc] + x;
                  uint32_t const s = static_cast<uint32_t>(g) & 31u;
                  uint64_t const q = g >> 5;
                  uint32_t const hi = s ? v >> (32 - s) : 0u;
                  if (q >= nw || (hi && q + 1 >= nw)) {
                    atomicOr(p.err, 8u);
                  } else {
                    if (v) atomicOr(out + q, v << s);
                    if (hi) atomicOr(out + q + 1, hi);
                  }
                }
                x = xe;
              }
            }
          }
        }
        if (r == k) {
          // -- level-b order out: warp w writes class runs w, w + 8, ... in
          //    16-byte units (a run's edge units symbol by symbol)
          if (WriteOrder) {
            uint32_t const runs = 1u << k;
            uint32_t const* s32 = reinterpret_cast<uint32_t const*>(Sc);
            for (uint32_t cc = wid; cc < runs; cc += kPWarps) {
              uint32_t const cs = cls[k][cc], len = cls[k][cc + 1] - cs;
              if (len == 0) continue;
              uint64_t const gp = gpos[cc];
              uint64_t const ge = gp + len;
              if (ge > p.n) {
                if (lane == 0) atomicOr(p.err, 8u);
                continue;
              }
              // head [gp, hb) and tail [tb, ge): at most kVE - 1 symbols each,
              // one per lane; whole 16-byte units in between
              uint64_t const hb = min((gp + kVE - 1) / kVE * kVE, ge);
              uint64_t const tb = max(ge / kVE * kVE, hb);
              {
                uint64_t const g = lane < kVE ? gp + lane : tb + (lane - kVE);
                bool const ok = lane < kVE ? g < hb : (lane < 2 * kVE && g < ge);
                if (ok) dst[g] = Sc[cs + static_cast<uint32_t>(g - gp)];
              }
              uint32_t const nu = static_cast<uint32_t>((tb - hb) / kVE);
              for (uint32_t du = lane; du < nu; du += 32) {
                uint64_t const v0 = hb + uint64_t(du) * kVE;
                uint32_t const sb = (cs + static_cast<uint32_t>(v0 - gp)) * sizeof(T);
                uint32_t const* qq = s32 + (sb >> 2);
                uint32_t const sh = (sb & 3u) * 8;
                uint4 o;
                o.x = __funnelshift_r(qq[0], qq[1], sh);
                o.y = __funnelshift_r(qq[1], qq[2], sh);
                o.z = __funnelshift_r(qq[2], qq[3], sh);
                o.w = __funnelshift_r(qq[3], qq[4], sh);
                *reinterpret_cast<uint4*>(dst + v0) = o;
              }
            }
          }
          __syncthreads();  // everything of this tile is out
          for (uint32_t rr = 1; rr <= k; ++rr)
            if (tid < (1u << rr))
              run[rr][tid] += cls[rr][tid + 1] - cls[rr][tid];
          break;
        }
        // -- c. class table of level a+r (warp 0, lane j = class j): where
        //    its zeros and ones go; the child classes of level a+r+1 (lane
        //    c = class c) and the global placement of their runs.
        if (wid == 0) {
          uint32_t const wt = lane < kPWarps ? warp_tot[lane] : 0u;
          uint32_t wp = wt;
#pragma unroll
          for (int o = 1; o <= 8; o <<= 1) {
            uint32_t const y = __shfl_up_sync(0xffffffffu, wp, o);
            if (lane >= static_cast<uint32_t>(o)) wp += y;
          }
          wp -= wt;  // zeros before warp `lane` (lane 8: all)
          if (lane <= kPWarps) warp_pre[lane] = wp;
          auto z_at = [&](uint32_t qq) -> uint32_t {
            uint32_t const t = qq / kItems, i = qq % kItems;
            uint32_t const base = __shfl_sync(0xffffffffu, wp, min(t >> 5, kPWarps));
            if (t >= kPThreads) return base;
            uint32_t zz = base;
            if (t & 31) zz += incl_s[t - 1];
            return zz + __popc(zmask_s[t] & ((1u << i) - 1u));
          };
          bool const own = lane < (1u << r);
          uint32_t const cs = own ? cls[r][lane] : 0u;
          uint32_t const ce = own ? cls[r][lane + 1] : 0u;
          uint32_t const zs = z_at(cs), ze = z_at(ce);
          if (own) {
            T0s[lane] = static_cast<uint16_t>(cs - zs);
            T1s[lane] = static_cast<uint16_t>(ze);
          }
          uint32_t const par = lane >> 1;
          uint32_t const pcs = __shfl_sync(0xffffffffu, cs, par);
          uint32_t const pce = __shfl_sync(0xffffffffu, ce, par);
          uint32_t const pzs = __shfl_sync(0xffffffffu, zs, par);
          uint32_t const pze = __shfl_sync(0xffffffffu, ze, par);
          uint32_t const mid = pcs + (pze - pzs);
          uint32_t const nch = 2u << r;
          uint32_t const ccs = (lane & 1) ? mid : pcs;
          uint32_t const cce = (lane & 1) ? pce : mid;
          uint64_t const gp = lane < nch ? Cb[r + 1][lane] + run[r + 1][lane] : 0u;
          if (lane < nch) {
            cls[r + 1][lane] = static_cast<uint16_t>(ccs);
            if (lane == nch - 1) cls[r + 1][nch] = static_cast<uint16_t>(cce);
            gpb[r + 1][lane] = gp - ccs;
            if (r + 1 == k) gpos[lane] = gp;
          }
        }
        __syncthreads();  // C: tables ready
        // -- d. partition into the level a+r+1 order
        {
          uint32_t const sbase = smem_u32(Sn);
          uint32_t const zt = warp_pre[wid] + inc - z;
          if (one_class) {
            // zeros and ones each go to a contiguous stretch
            uint32_t az = sbase + (T0s[c_first] + zt) * sizeof(T);
            uint32_t ao = sbase + (T1s[c_first] + p0 - zt) * sizeof(T);
#pragma unroll
            for (int i = 0; i < int(kItems); ++i) {
              if ((bits >> i) & 1u) {
                st_shared<T>(ao, e.get(i));
                ao += sizeof(T);
              } else {
                st_shared<T>(az, e.get(i));
                az += sizeof(T);
              }
            }
          } else if (!to_fix) {
            // a tile's last, partial thread: per-symbol class lookup
            uint32_t zc = zt;
#pragma unroll
            for (int i = 0; i < int(kItems); ++i) {
              if (static_cast<uint32_t>(i) < nvalid) {
                uint32_t const sv = e.get(i);
                uint32_t const cc = (sv >> cshift) & cmask;
                uint32_t const b = (bits >> i) & 1u;
                uint32_t const d = b ? T1s[cc] + (p0 + i - zc) : T0s[cc] + zc;
                st_shared<T>(sbase + (d & (kTile - 1)) * sizeof(T), sv);
                zc += b ^ 1u;
              }
            }
          }
          // listed threads: warp w takes list entries w, w + 8, ...; lane i
          // places symbol i of the listed thread.
          uint32_t const nfix = fix_n[r & 1];
          for (uint32_t j = wid; j < nfix; j += kPWarps) {
            uint32_t const t = fix_list[j];
            if (lane < kItems) {
              uint32_t const q = t * kItems + lane;
              uint32_t const zm = zmask_s[t];
              uint32_t const zc = warp_pre[t >> 5] + ((t & 31) ? incl_s[t - 1] : 0u) +
                                  __popc(zm & ((1u << lane) - 1u));
              uint32_t const sv = Sc[q];
              uint32_t const cc = (sv >> cshift) & cmask;
              uint32_t const d = ((zm >> lane) & 1u) ? T0s[cc] + zc : T1s[cc] + (q - zc);
              st_shared<T>(sbase + (d & (kTile - 1)) * sizeof(T), sv);
            }
          }
        }
        __syncthreads();  // D: level a+r+1 order complete
        Sc = Sn;
      }
    }
  }
}

// The pass pipeline: levels a0+1 .. L-1 of a power-of-two alphabet of 2^L
// symbols from the level-a0 order `sym` of n symbols (the text when a0 = 0),
// level l written at words + word_off[l] (nbits[l] bits, zeroed
// beforehand), with the count table `counts` holding the start of every
// level-a0 node.  The L-1-a0 levels go in ceil((L-1-a0)/4) passes of
// near-equal size.  With ingest_src (a0 = 0 only) the first pass reads that
// text instead: it writes level 0 and, when ingest_copy, copies the text to
// `sym`.  A batch of texts runs as one tree whose top a0 levels are the text
// number (the concatenated texts are its level-a0 order).
// With `first_k` the first pass covers levels a0+1 .. a0+first_k and the
// rest follow in passes of near-equal size; with `keep_first_order` (two
// passes) the level order the first pass wrote is handed to the caller.
template <class T>
void run_pass_pipeline(T const* sym, uint64_t n, uint32_t L, uint32_t a0,
                       uint32_t* words, uint64_t const* word_off,
                       uint64_t const* nbits, uint64_t* counts, uint32_t* err,
                       cudaStream_t st, T const* ingest_src = nullptr,
                       bool ingest_copy = false, uint32_t first_k = 0,
                       DevBuf* keep_first_order = nullptr) {
  uint32_t const levels = L - 1 - a0;
  if (levels == 0) return;
  // the pass sizes
  std::vector<uint32_t> ks;
  uint32_t rest = levels;
  if (first_k) {
    EWT_REQUIRE(first_k <= kPMaxK && first_k < levels, EWT_ERR_UNSUPPORTED,
                "first pass out of range");
    ks.push_back(first_k);
    rest -= first_k;
  }
  uint32_t const nr = (rest + kPMaxK - 1) / kPMaxK;
  for (uint32_t i = 0; i < nr; ++i) ks.push_back(rest / nr + (i < rest % nr ? 1u : 0u));
  uint32_t const np = static_cast<uint32_t>(ks.size());
  // chunks of a pass starting at level a: at most n / kPChunk + 2^a (one
  // partial chunk per level-a node); tables sized for the deepest start
  uint32_t a_last = a0;
  for (uint32_t i = 0, a = a0; i < np; ++i) {
    a_last = a;
    a += ks[i];
  }
  auto chunks_at = [&](uint32_t a) {
    return n / kPChunk + (uint64_t(1) << a) + 2;
  };
  uint64_t const max_chunks = chunks_at(a_last);
  DevBuf chunk_first(((uint64_t(1) << kPMaxStartLevel) + 1) * 4);
  DevBuf chunk_tot(max_chunks * kPMaxDigits * 4);
  DevBuf chunk_pre(max_chunks * kPMaxDigits * 8);
  DevBuf node_tot(((uint64_t(1) << kPMaxStartLevel) + 1) * kPMaxDigits * 8);
  DevBuf order[2];
  uint32_t const sms = static_cast<uint32_t>(sm_count());
  T const* cur = sym;
  uint32_t a = a0;
  for (uint32_t i = 0; i < np; ++i) {
    uint32_t const k = ks[i];
    uint32_t const b = a + k;
    bool const write_order = b < L - 1;
    EWT_REQUIRE(a <= kPMaxStartLevel && k >= 1 && k <= kPMaxK,
                EWT_ERR_UNSUPPORTED, "pass plan out of range");
    PassArgs pa{};
    pa.n = n;
    pa.L = L;
    pa.a = a;
    pa.k = k;
    pa.nodes = 1u << a;
    pa.words = words;
    for (uint32_t r = 1; r <= k; ++r) {
      pa.word_off[r] = word_off[a + r];
      pa.nwords[r] = ceil_div(nbits[a + r], 32);
    }
    pa.counts = counts;
    pa.chunk_first = chunk_first.as<uint32_t>();
    pa.chunk_tot = chunk_tot.as<uint32_t>();
    pa.chunk_pre = chunk_pre.as<uint64_t>();
    pa.node_tot = node_tot.as<uint64_t>();
    pa.err = err;
    T* next = nullptr;
    if (write_order) {
      DevBuf& ob = order[i & 1];
      if (!ob.get()) ob.alloc(n * sizeof(T) + 64);
      next = ob.as<T>();
    }
    // grids follow the pass's chunk count, so a small text's launches leave
    // the GPU to other streams' work
    uint64_t const pass_chunks = chunks_at(a);
    uint32_t const grid = static_cast<uint32_t>(
        std::min<uint64_t>(pass_chunks, uint64_t(sms) * 6));
    {
      PhaseTimer pt(EWT_PHASE_HIST, st);
      chunk_table_kernel<<<1, 1024, 0, st>>>(pa);
      EWT_LAUNCHED();
      if (i == 0 && ingest_src) {
        // level 0 and the first digit counts in one read of the text (and,
        // for a host text, its copy to the device)
        PhaseTimer pt2(ingest_copy ? EWT_PHASE_H2D : EWT_PHASE_FILL, st);
        ingest_kernel<T><<<static_cast<uint32_t>(std::min<uint64_t>(
                               pass_chunks, uint64_t(sms) * 6)),
                           kPThreads, 0, st>>>(ingest_src,
                                               ingest_copy ? const_cast<T*>(cur) : nullptr,
                                               words + word_off[0], pa);
      } else {
        digit_count_kernel<T><<<static_cast<uint32_t>(std::min<uint64_t>(
                                    pass_chunks, uint64_t(sms) * 6)),
                                kPThreads, 0, st>>>(cur, pa);
      }
      EWT_LAUNCHED();
      pass_scan_kernel<<<pa.nodes << k, kScanThreads, 0, st>>>(pa);
      EWT_LAUNCHED();
      pass_counts_kernel<<<(pa.nodes + 255) / 256, 256, 0, st>>>(pa);
      EWT_LAUNCHED();
    }
    {
      PhaseTimer pt(EWT_PHASE_SPLIT, st);
      auto pick = [&](auto kk) {
        constexpr uint32_t K = decltype(kk)::value;
        return write_order ? pass_kernel<T, true, K> : pass_kernel<T, false, K>;
      };
      auto kern = k == 1   ? pick(std::integral_constant<uint32_t, 1>{})
                  : k == 2 ? pick(std::integral_constant<uint32_t, 2>{})
                  : k == 3 ? pick(std::integral_constant<uint32_t, 3>{})
                           : pick(std::integral_constant<uint32_t, 4>{});
      size_t const smem = pass_smem_bytes<T>();
      set_smem_limit(kern, static_cast<int>(smem));
      kern<<<grid, kPThreads, smem, st>>>(cur, next, pa);
      EWT_LAUNCHED();
    }
    cur = next;
    a = b;
  }
  if (keep_first_order && np == 2) *keep_first_order = std::move(order[0]);
}

}  // namespace
}  // namespace ewt
