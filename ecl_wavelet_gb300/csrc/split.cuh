// Split kernels of the wavelet-tree level pipeline: the stable partition
// of every node of level l by the level's bit, which produces the level
// l+1 order and that level's bits.  Included by wt_build.cu after the node
// helpers (node_of, level_bit) and views these kernels use.
#pragma once

#include "bulk_copy.cuh"

namespace ewt {
namespace {

constexpr uint32_t kSplitThreads = 256;
constexpr uint32_t kSplitWarps = kSplitThreads / 32;
constexpr uint32_t kSplitItems = 16;
constexpr uint32_t kSplitTile = kSplitThreads * kSplitItems;
constexpr uint32_t kRunWords = kSplitTile / 32;

// Stores `len` bits (buffer bits 0..len-1) at global bit position `pos`;
// whole words inside the run are plain stores, the run's partial first and
// last words are atomicOr'ed (neighbouring runs share them; the level's
// words are zeroed before the launch).
__device__ __forceinline__ void store_run(uint32_t* __restrict__ out,
                                          uint64_t out_words, uint64_t pos,
                                          uint32_t len, uint32_t const* buf) {
  if (len == 0) return;
  uint32_t const sh = static_cast<uint32_t>(pos & 31);
  uint64_t const w0 = pos >> 5;
  uint32_t const nw = (sh + len + 31) >> 5;
  if (w0 + nw > out_words) return;  // corrupt position: never write past
  for (uint32_t k = threadIdx.x; k < nw; k += kSplitThreads) {
    uint32_t const hi = k < kRunWords ? buf[k] : 0u;
    uint32_t const lo = k > 0 ? buf[k - 1] : 0u;
    uint32_t const word = sh ? ((hi << sh) | (lo >> (32 - sh))) : hi;
    bool const partial = (k == 0 && sh != 0) ||
                         (k == nw - 1 && ((sh + len) & 31) != 0);
    if (partial) {
      if (word) atomicOr(out + w0 + k, word);
    } else {
      out[w0 + k] = word;
    }
  }
}

// Stable partition of every node of level l by the level's bit.  A symbol
// at level position p in node [cs, ce] (split s, zeros before p in the level
// Z, rank0 at the node start Zn) moves to C[cs] + (Z - Zn) if its bit is 0
// and to C[s] + (p - C[cs]) - (Z - Zn) otherwise.  Positions >= size_l
// (symbols whose code already ended) keep their place.  The bits of level
// l+1 of the moved symbols are written into `next` (zeroed beforehand);
// the new order is written only when WriteOrder.
template <class T, bool Pow2, bool WriteOrder>
__global__ void __launch_bounds__(kSplitThreads, 3)
split_kernel(T const* __restrict__ src, T* __restrict__ dst, uint64_t n,
             uint64_t size_l, uint64_t size_next, uint32_t l, TreeView t,
             uint32_t* __restrict__ next, uint32_t const* __restrict__ list,
             uint32_t const* __restrict__ list_len,
             uint32_t* __restrict__ err) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint32_t warp_z[kSplitWarps];
  // Work items: every tile, or (after the fast kernel) the tiles it listed
  // plus the text's last tile when that one is partial.
  uint64_t const tiles = (n + kSplitTile - 1) / kSplitTile;
  uint64_t const listed = list ? *list_len : 0;
  uint64_t const items = list ? listed + (n % kSplitTile ? 1 : 0) : tiles;
  for (uint64_t wi = blockIdx.x; wi < items; wi += gridDim.x) {
  uint64_t const tile = !list ? wi : (wi < listed ? list[wi] : tiles - 1);
  uint64_t const tile_start = tile * uint64_t(kSplitTile);
  uint64_t const tile_end = min(tile_start + kSplitTile, n);
  uint32_t const cnt = static_cast<uint32_t>(tile_end - tile_start);
  uint32_t const tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
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

  // ---- general path -------------------------------------------------------
  uint64_t* dests = reinterpret_cast<uint64_t*>(smem);
  T* vals = reinterpret_cast<T*>(smem + kSplitTile * sizeof(uint64_t));
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
      bits |= uint32_t(level_bit<Pow2>(item[j], l, L, t.sigma)) << j;
    }
  }
  uint32_t const zcnt = __popc(part & ~bits);
  uint32_t inc = zcnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t const y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) warp_z[wid] = inc;
  __syncthreads();
  uint32_t wbase = 0, tile_zeros = 0;
#pragma unroll
  for (uint32_t w = 0; w < kSplitWarps; ++w) {
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
        else atomicOr(err, 2u);
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
    if (slot >= kSplitTile || dest >= n) {
      atomicOr(err, slot >= kSplitTile ? 4u : 8u);
      continue;
    }
    if (dest < size_next && level_bit<Pow2>(item[j], l + 1, L, t.sigma))
      atomicOr(next + (dest >> 5), 1u << (dest & 31));
    if (WriteOrder) {
      dests[slot] = dest;
      vals[slot] = item[j];
    }
  }
  if (WriteOrder) {
    __syncthreads();
    for (uint32_t s = tid; s < cnt; s += kSplitThreads) {
      uint64_t const d = dests[s];
      if (d < n) dst[d] = vals[s];
    }
  }
  __syncthreads();  // shared memory is reused by the next item
  }
}

// Copies `len` staged symbols (shared memory, 32-byte aligned) to
// dst[pos, pos + len).  Bytes move as 4-byte words: a few head and tail
// bytes singly, the body with funnel shifts from two staged words.
template <class T>
__device__ __forceinline__ void copy_run(T* __restrict__ dst, uint64_t n,
                                         uint64_t pos, uint32_t len,
                                         T const* src) {
  if (len == 0 || pos + len > n) return;  // corrupt position: never write past
  uint32_t const tid = threadIdx.x;
  if constexpr (sizeof(T) == 1) {
    uint32_t const head = min(len, static_cast<uint32_t>((4 - (pos & 3)) & 3));
    if (tid < head) dst[pos + tid] = src[tid];
    uint32_t const body = (len - head) >> 2;
    uint32_t const* s32 = reinterpret_cast<uint32_t const*>(src);
    uint32_t* d32 = reinterpret_cast<uint32_t*>(dst + pos + head);
    uint32_t const shift = head * 8;
    for (uint32_t i = tid; i < body; i += kSplitThreads) {
      uint32_t const lo = s32[i], hi = s32[i + 1];
      d32[i] = head ? __funnelshift_r(lo, hi, shift) : lo;
    }
    uint32_t const tail = (len - head) & 3;
    uint32_t const t0 = head + 4 * body;
    if (tid < tail) dst[pos + t0 + tid] = src[t0 + tid];
  } else {
    for (uint32_t i = tid; i < len; i += kSplitThreads) dst[pos + i] = src[i];
  }
}

template <class T>
__host__ __device__ constexpr uint32_t split_stages() {
  return sizeof(T) <= 2 ? 4 : (sizeof(T) == 4 ? 3 : 2);
}

// Bytes of the output staging area: the zero run at offset 0, the one run
// at the next 32-element boundary, plus slack for the funnel reads.
template <class T>
__host__ __device__ constexpr uint32_t split_stage_bytes() {
  return (kSplitTile + 64) * sizeof(T);
}

// Packs bit `b` of 32 consecutive symbols starting at element 32*k of a
// staged run into one word (bit i = symbol i).
template <class T>
__device__ __forceinline__ uint32_t pack_bits32(T const* run, uint32_t b) {
  uint32_t w = 0;
  if constexpr (sizeof(T) == 1) {
    uint4 const* q = reinterpret_cast<uint4 const*>(run);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      uint4 const v = q[h];
      uint32_t const x[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        // bit b of each byte -> bits 0, 8, 16, 24; the multiply gathers
        // them into bits 21..24 without carries.
        uint32_t const t = (x[i] >> b) & 0x01010101u;
        w |= (((t * 0x00204081u) >> 21) & 0xFu) << (16 * h + 4 * i);
      }
    }
  } else {
#pragma unroll
    for (int i = 0; i < 32; ++i)
      w |= uint32_t((uint64_t(run[i]) >> b) & 1u) << i;
  }
  return w;
}

// Persistent fast path of the split for power-of-two alphabets.
//
// Every CTA walks the full tiles blockIdx.x, blockIdx.x + gridDim.x, ...; a
// ring of split_stages<T>() shared-memory buffers is filled by bulk copies
// (cp.async.bulk, completion on an mbarrier) issued kStages tiles ahead; the
// tile-start zero count is fetched one tile ahead and the node's
// (C[start], C[split], rank0 at start) is cached while consecutive tiles
// stay in one node.  Per tile:
//   1. each thread takes 16 consecutive symbols (blocked), checks that they
//      share the node prefix, and packs their level bits (SWAR for bytes);
//   2. one CTA scan of the per-thread zero counts;
//   3. symbols are staged in output order: the tile's zeros, then (from the
//      next 32-symbol boundary) its ones;
//   4. the staged runs go to the new order with funnel-shifted word stores
//      and their level l+1 bits are packed from the staged symbols and
//      written as whole words (atomicOr only on a run's two edge words).
// A tile whose symbols span two nodes is appended to `slow_list` for the
// general kernel.
template <class T, bool WriteOrder>
__global__ void __launch_bounds__(kSplitThreads, 3)
split_fast_kernel(T const* __restrict__ src, T* __restrict__ dst, uint64_t n,
                  uint32_t l, TreeView t, uint32_t* __restrict__ next,
                  uint64_t next_words, uint32_t* __restrict__ slow_list,
                  uint32_t* __restrict__ slow_len, uint32_t* __restrict__ err) {
  constexpr uint32_t kStages = split_stages<T>();
  constexpr uint32_t kTileBytes = kSplitTile * sizeof(T);
  constexpr uint32_t kStageBytes = split_stage_bytes<T>();
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char* ring = smem;
  T* stage = reinterpret_cast<T*>(smem + kStages * kTileBytes);
  __shared__ __align__(8) uint64_t bars[kStages];
  __shared__ uint32_t warp_z[kSplitWarps];
  __shared__ uint32_t zwords[kRunWords + 2], owords[kRunWords + 2];
  __shared__ uint64_t node_s[3];  // C[start], C[split], rank0 at start
  __shared__ uint64_t z_s;

  uint32_t const tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  ArrayMeta const m = t.rs.meta[l];
  uint32_t const L = t.levels;
  uint32_t const sh = L - 1 - l;
  uint64_t const full = n / kSplitTile;
  uint64_t const G = gridDim.x;
  uint64_t const mine =
      blockIdx.x < full ? (full - blockIdx.x + G - 1) / G : 0;

  auto z_at = [&](uint64_t pos) -> uint64_t {
    return pos - (t.rs.l1[m.l1_off + (pos >> 16)] +
                  t.rs.l2[m.l2_off + (pos >> 9)]);
  };
  if (tid == 0) {
    for (uint32_t s = 0; s < kStages; ++s) mbar_init(&bars[s], 1);
    fence_async_shared();
  }
  __syncthreads();
  uint64_t z_next = 0, key_cached = ~uint64_t(0);
  if (tid == 0) {
    for (uint64_t s = 0; s < kStages && s < mine; ++s)
      bulk_load(ring + s * kTileBytes, src + (blockIdx.x + s * G) * kSplitTile,
                kTileBytes, &bars[s]);
    if (mine) z_next = z_at(blockIdx.x * uint64_t(kSplitTile));
  }
  for (uint64_t k = 0; k < mine; ++k) {
    uint64_t const tile = blockIdx.x + k * G;
    uint64_t const tile_start = tile * kSplitTile;
    uint32_t const s = static_cast<uint32_t>(k % kStages);
    T const* buf = reinterpret_cast<T const*>(ring + s * kTileBytes);
    // A copy that never lands is reported; every global write below is
    // bounds-checked, so a stale buffer cannot write out of range.
    if (!mbar_wait(&bars[s], static_cast<uint32_t>((k / kStages) & 1)))
      atomicOr(err, 16u);
    uint64_t const key = uint64_t(buf[0]) >> (sh + 1);
    if (tid == 0) {
      z_s = z_next;
      if (k + 1 < mine) z_next = z_at((tile + G) * kSplitTile);
      if (key != key_cached) {
        key_cached = key;
        uint64_t const cs = key << (sh + 1);
        uint64_t zn = 0;
        if (cs) {
          uint64_t const ni = ecl::detail::node_index(t, t.node_base, cs, l);
          if (ni < t.num_ranks) zn = t.node_ranks[ni];
          else atomicOr(err, 2u);
        }
        node_s[0] = t.counts[cs];
        node_s[1] = t.counts[cs + (uint64_t(1) << sh)];
        node_s[2] = zn;
      }
    }
    // 1. 16 consecutive symbols per thread
    T e[kSplitItems];
    {
      constexpr int kVec = kSplitItems * sizeof(T) / 16;
      uint4 v[kVec];
      uint4 const* q = reinterpret_cast<uint4 const*>(buf) + tid * kVec;
#pragma unroll
      for (int i = 0; i < kVec; ++i) v[i] = q[i];
      T const* p = reinterpret_cast<T const*>(v);
#pragma unroll
      for (int i = 0; i < int(kSplitItems); ++i) e[i] = p[i];
    }
    uint32_t bits = 0;
    bool same = true;
    if constexpr (sizeof(T) == 1) {
      uint32_t const* w = reinterpret_cast<uint32_t const*>(e);
      uint32_t const pre_mask = 0x01010101u * (0xFFu >> (sh + 1));
      uint32_t const pre_key = 0x01010101u * static_cast<uint32_t>(key);
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        same &= ((w[i] >> (sh + 1)) & pre_mask) == pre_key;
        uint32_t const tb = (w[i] >> sh) & 0x01010101u;
        bits |= (((tb * 0x00204081u) >> 21) & 0xFu) << (4 * i);
      }
    } else {
#pragma unroll
      for (int i = 0; i < int(kSplitItems); ++i) {
        same &= (uint64_t(e[i]) >> (sh + 1)) == key;
        bits |= uint32_t((uint64_t(e[i]) >> sh) & 1u) << i;
      }
    }
    uint32_t const z = kSplitItems - __popc(bits);
    // 2. CTA exclusive scan of the zero counts
    uint32_t inc = z;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t const y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    if (lane == 31) warp_z[wid] = inc;
    bool const fast = __syncthreads_and(same);
    if (fast) {
      uint32_t zx = inc - z, tile_zeros = 0;
#pragma unroll
      for (uint32_t w = 0; w < kSplitWarps; ++w) {
        uint32_t const v = warp_z[w];
        if (w < wid) zx += v;
        tile_zeros += v;
      }
      uint32_t const ones_base = (tile_zeros + 31) & ~31u;
      uint32_t ox = tid * kSplitItems - zx;
      // 3. stage in output order
#pragma unroll
      for (int i = 0; i < int(kSplitItems); ++i) {
        bool const b = (bits >> i) & 1;
        stage[b ? ones_base + ox : zx] = e[i];
        ox += b;
        zx += !b;
      }
      uint64_t const z_tile = z_s, ca = node_s[0], cm = node_s[1],
                     zn = node_s[2];
      uint64_t const d0 = ca + (z_tile - zn);
      uint64_t const d1 = cm + (tile_start - ca) - (z_tile - zn);
      __syncthreads();
      // 4. runs out: next-level words, then the symbols
      uint32_t const nz = tile_zeros, no = kSplitTile - tile_zeros;
      uint32_t const wz = (nz + 31) >> 5, wo = (no + 31) >> 5;
      for (uint32_t i = tid; i < wz + wo; i += kSplitThreads) {
        bool const zero_run = i < wz;
        uint32_t const wi = zero_run ? i : i - wz;
        uint32_t const len = zero_run ? nz : no;
        uint32_t word =
            pack_bits32<T>(stage + (zero_run ? 0 : ones_base) + 32 * wi, sh - 1);
        uint32_t const valid = len - 32 * wi;
        if (valid < 32) word &= (1u << valid) - 1u;
        (zero_run ? zwords : owords)[wi] = word;
      }
      if (tid == 0) {
        zwords[wz] = 0;
        owords[wo] = 0;
      }
      if (WriteOrder) {
        copy_run<T>(dst, n, d0, nz, stage);
        copy_run<T>(dst, n, d1, no, stage + ones_base);
      }
      __syncthreads();
      store_run(next, next_words, d0, nz, zwords);
      store_run(next, next_words, d1, no, owords);
    } else if (tid == 0) {
      slow_list[atomicAdd(slow_len, 1u)] = static_cast<uint32_t>(tile);
    }
    __syncthreads();  // stage, words and ring stage s are free again
    if (tid == 0 && k + kStages < mine) {
      fence_async_shared();
      bulk_load(ring + s * kTileBytes, src + (tile + kStages * G) * kSplitTile,
                kTileBytes, &bars[s]);
    }
  }
}

template <class T, bool Pow2>
void launch_split(bool write_order, T const* src, T* dst, uint64_t n,
                  uint64_t size_l, uint64_t size_next, uint32_t l,
                  TreeView const& v, uint32_t* next, uint32_t* slow_list,
                  uint32_t* err, cudaStream_t st) {
  uint64_t const tiles = ceil_div(n, kSplitTile);
  // The fast kernel covers full tiles of a power-of-two alphabet (all of
  // them participate: size_l == n); the general kernel finishes the rest.
  bool const use_fast = Pow2 && size_l == n && n >= kSplitTile;
  uint32_t* slow_len = slow_list + tiles;
  if (use_fast) {
    EWT_CUDA(cudaMemsetAsync(slow_len, 0, 4, st));
    size_t const ring = size_t(split_stages<T>()) * kSplitTile * sizeof(T) +
                        split_stage_bytes<T>();
    auto fk = write_order ? split_fast_kernel<T, true>
                          : split_fast_kernel<T, false>;
    EWT_CUDA(cudaFuncSetAttribute(
        fk, cudaFuncAttributeMaxDynamicSharedMemorySize,
        static_cast<int>(ring)));
    uint32_t const grid = static_cast<uint32_t>(
        std::min<uint64_t>(n / kSplitTile, uint64_t(sm_count()) * 3));
    fk<<<grid, kSplitThreads, ring, st>>>(src, dst, n, l, v, next,
                                          ceil_div(size_next, 32), slow_list,
                                          slow_len, err);
    EWT_LAUNCHED();
  }
  size_t const smem = kSplitTile * (sizeof(uint64_t) + sizeof(T));
  auto k = write_order ? split_kernel<T, Pow2, true>
                       : split_kernel<T, Pow2, false>;
  EWT_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(smem)));
  uint32_t const grid = static_cast<uint32_t>(
      std::min<uint64_t>(tiles, uint64_t(sm_count()) * 3));
  k<<<grid, kSplitThreads, smem, st>>>(src, dst, n, size_l, size_next, l, v,
                                       next, use_fast ? slow_list : nullptr,
                                       use_fast ? slow_len : nullptr, err);
  EWT_LAUNCHED();
}

}  // namespace
}  // namespace ewt
