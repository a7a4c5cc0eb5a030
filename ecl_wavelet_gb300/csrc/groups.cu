// Group query levels of power-of-two trees: runs of w = 2 (quad) or 3
// (octal) consecutive binary levels l .. l+w-1 become one level of w-bit
// digits in level-l order, so a query resolves w binary levels per
// dependent DRAM access.  The plan covers all L levels: as many octal
// groups as fit, then one or two quad groups (L = 8: 3 + 3 + 2).  No
// reference counterpart; the binary levels and their RankSelect stay the
// source of truth for exports.
//
// A level-l node's zeros go, in order, to its left child on level l+1 and
// its ones to its right child, so the bits of level l+1 under a run of
// positions inside one node are two runs of level l+1, merged by the bits of
// level l ("routing" level l+1 into level-l order).
// Quad group at l:
//   1. quad_sb_count_kernel (thread per 512-block superblock): its digit
//      counts from six ranks per node segment (no per-position work);
//   2. group_scan_*: counts before every superblock (chunked scan);
//   3. quad_level_kernel (persistent, two superblocks per 1024-thread CTA,
//      one thread per 96-digit block): digits from the two runs, eight at a
//      time through a 64K-entry table in shared memory, block headers from
//      a scan, blocks and dense select samples written; the superblock's
//      totals are checked against pass 1.
// Octal group at l = 0 of 1- and 2-byte symbols: octal_text_kernel takes the
// digits straight from the (minimal) symbols; the same kernel builds octal
// level 3 from the level-3 order when the first pass kept it (trees of 6 or
// 8 levels: passes of 3 + 3 or 3 + 4 levels, see run_passes).  Other octal
// groups at l:
//   1. merge_plane_kernel: level l+2 routed into level-(l+1) order (a plane
//      of n bits);
//   2. octal_level_kernel (same shape, one thread per 42-digit block): the
//      digit's middle and low bits route level l+1 and that plane into
//      level-l order; blocks store the three bit planes; headers from a
//      scan; per-superblock counts written;
//   3. group_scan_*, then group_samples_kernel (dense samples; the level's
//      digit totals checked against the count table).
// Node ranks (digit counts before every node) and digit totals come from
// the count table on the host.
#include <algorithm>
#include <vector>

#include "internal.cuh"

namespace ewt {

using ecl::detail::GroupShape;
using ecl::detail::kQuadDigits;
using ecl::detail::kQuadSbBlocks;
using ecl::detail::kQuadSbDigits;
using ecl::detail::GroupLevel;
using ecl::detail::GroupView;

constexpr uint32_t kOctDigits = GroupShape<3>::kDigits;
constexpr uint32_t kOctSbBlocks = GroupShape<3>::kSbBlocks;
constexpr uint64_t kOctSbDigits = uint64_t(kOctDigits) * kOctSbBlocks;
constexpr uint64_t kMergeSbPos = 512 * 64;  // positions per merge-kernel superblock

namespace {

constexpr uint32_t kScanChunk = 4096;   // superblock entries per scan CTA

// Bits 2k of the result take bit k of x (k < 16).
__device__ __forceinline__ uint32_t spread16(uint32_t x) {
  x &= 0xFFFFu;
  x = (x | (x << 8)) & 0x00FF00FFu;
  x = (x | (x << 4)) & 0x0F0F0F0Fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}

// 32 bits of a level starting at bit q (words past `limit` read as 0).
__device__ __forceinline__ uint32_t bits_at(uint32_t const* __restrict__ w,
                                            uint64_t limit, uint64_t q) {
  uint64_t const i = q >> 5;
  uint32_t const s = static_cast<uint32_t>(q & 31);
  uint32_t const a = i < limit ? w[i] : 0u;
  uint32_t const b = s && i + 1 < limit ? w[i + 1] : 0u;
  return __funnelshift_r(a, b, s);
}

// 32 bits of a level starting at bit q, for q below the level's end (the
// word array has slack behind its last array).
__device__ __forceinline__ uint32_t bits_fast(uint32_t const* __restrict__ w,
                                              uint64_t q) {
  uint64_t const i = q >> 5;
  return __funnelshift_r(w[i], w[i + 1], static_cast<uint32_t>(q) & 31u);
}

// Geometry of one level-2j node as the digit kernels need it.
struct QuadNode {
  uint64_t start, end;   // positions on level 2j
  uint64_t zeros;        // zeros of the node on level 2j (left child size)
  uint64_t ones_before;  // ones of level 2j before the node
};

__device__ __forceinline__ uint64_t node_of(uint64_t const* C, uint32_t sh,
                                            uint64_t nodes, uint64_t p) {
  uint64_t a = 0, z = nodes - 1;  // the last node starting at or before p
  while (a < z) {
    uint64_t const mid = (a + z + 1) >> 1;
    if (C[mid << sh] <= p) a = mid; else z = mid - 1;
  }
  return a;
}

__device__ __forceinline__ QuadNode quad_node(TreeView const& v, uint32_t l,
                                              uint32_t sh, uint64_t nodes,
                                              uint64_t g) {
  uint64_t const* C = v.counts;
  QuadNode q;
  q.start = C[g << sh];
  q.end = g + 1 < nodes ? C[(g + 1) << sh] : v.n;
  q.zeros = C[(2 * g + 1) << (sh - 1)] - q.start;
  uint64_t const z0 =
      g ? v.node_ranks[ecl::detail::node_index(v, v.node_base, g << sh, l)] : 0;
  q.ones_before = q.start - z0;
  return q;
}

// What a superblock's CTA needs up front: the node holding its first
// position, the ones of level 2j before that position, and whether the
// whole superblock lies in that node.
struct SbStart {
  QuadNode node;
  uint64_t rank1;
  uint64_t uniform;
};

// Quad pass 1: digit counts of every superblock (thread per superblock).
__global__ void __launch_bounds__(128)
quad_sb_count_kernel(TreeView v, uint32_t l, uint64_t nsb,
                     uint64_t* __restrict__ sb, SbStart* __restrict__ info) {
  uint64_t const s = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (s > nsb) return;
  uint64_t c[4] = {0, 0, 0, 0};
  uint64_t const n = v.n;
  uint64_t a = s * kQuadSbDigits;
  uint64_t const e = min(n, a + kQuadSbDigits);
  if (s < nsb && a >= e) info[s] = SbStart{QuadNode{0, n, 0, 0}, 0, 1};
  if (s < nsb && a < e) {
    uint32_t const sh = v.levels - l;
    uint64_t const nodes = uint64_t(1) << l;
    ArrayMeta const mh = v.rs.meta[l], ml = v.rs.meta[l + 1];
    uint64_t g = node_of(v.counts, sh, nodes, a);
    uint64_t r1a = ecl::detail::rs_rank1<false>(v.rs, mh, a, nullptr);
    {
      QuadNode const nd = quad_node(v, l, sh, nodes, g);
      info[s] = SbStart{nd, r1a, e <= nd.end ? 1u : 0u};
    }
    while (a < e && g < nodes) {
      QuadNode const nd = quad_node(v, l, sh, nodes, g);
      uint64_t const b = min(e, nd.end);
      if (b > a) {
        uint64_t const r1b = ecl::detail::rs_rank1<false>(v.rs, mh, b, nullptr);
        uint64_t const o = r1b - r1a, z = (b - a) - o;
        uint64_t const ob = r1a - nd.ones_before;  // node ones before a
        uint64_t const q0 = nd.start + (a - nd.start) - ob;
        uint64_t const q1 = nd.start + nd.zeros + ob;
        uint64_t const l0 = ecl::detail::rs_rank1<false>(v.rs, ml, q0 + z, nullptr) -
                            ecl::detail::rs_rank1<false>(v.rs, ml, q0, nullptr);
        uint64_t const l1 = ecl::detail::rs_rank1<false>(v.rs, ml, q1 + o, nullptr) -
                            ecl::detail::rs_rank1<false>(v.rs, ml, q1, nullptr);
        c[0] += z - l0;
        c[1] += l0;
        c[2] += o - l1;
        c[3] += l1;
        a = b;
        r1a = r1b;
      }
      ++g;
    }
  }
  for (uint32_t d = 0; d < 4; ++d) sb[s * 4 + d] = c[d];  // entry nsb: zeros
}

// Block-wide exclusive scan of a uint64 (blockDim.x a multiple of 32, at
// most 1024); *total receives the sum.
__device__ __forceinline__ uint64_t cta_exclusive_scan(uint64_t x, uint64_t* total) {
  __shared__ uint64_t warp_sums[32];
  uint32_t const lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint64_t inc = x;
#pragma unroll
  for (uint32_t o = 1; o < 32; o <<= 1) {
    uint64_t const y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) warp_sums[wid] = inc;
  __syncthreads();
  uint32_t const nwarps = blockDim.x >> 5;
  if (wid == 0) {
    uint64_t t = lane < nwarps ? warp_sums[lane] : 0;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
      uint64_t const y = __shfl_up_sync(0xFFFFFFFFu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < nwarps) warp_sums[lane] = t;  // inclusive over warps
  }
  __syncthreads();
  uint64_t const before = wid ? warp_sums[wid - 1] : 0;
  *total = warp_sums[nwarps - 1];
  __syncthreads();
  return before + inc - x;
}

// Scan 1: per chunk of kScanChunk superblock entries (S digits each), the
// S sums.
template <uint32_t S>
__global__ void __launch_bounds__(256)
group_scan_partial_kernel(uint64_t const* __restrict__ sb, uint64_t count,
                          uint64_t* __restrict__ chunk) {
  uint64_t const first = uint64_t(blockIdx.x) * kScanChunk;
  uint64_t c[S];
#pragma unroll
  for (uint32_t d = 0; d < S; ++d) c[d] = 0;
  for (uint64_t i = first + threadIdx.x; i < min(count, first + kScanChunk);
       i += blockDim.x)
#pragma unroll
    for (uint32_t d = 0; d < S; ++d) c[d] += sb[i * S + d];
#pragma unroll
  for (uint32_t d = 0; d < S; ++d) {
    uint64_t tot = 0;
    cta_exclusive_scan(c[d], &tot);
    if (threadIdx.x == 0) chunk[blockIdx.x * S + d] = tot;
  }
}

// Scan 2: exclusive prefix of the chunk sums (one thread per digit).
template <uint32_t S>
__global__ void group_scan_chunks_kernel(uint64_t* __restrict__ chunk,
                                         uint64_t chunks) {
  uint32_t const d = threadIdx.x;
  if (d >= S) return;
  uint64_t run = 0;
  for (uint64_t i = 0; i < chunks; ++i) {
    uint64_t const x = chunk[i * S + d];
    chunk[i * S + d] = run;
    run += x;
  }
}

// Scan 3: exclusive prefix of every entry, in place (1024 threads; two
// digits packed per 64-bit scan: every entry is below 2^16, a round's sums
// below 2^32).
template <uint32_t S>
__global__ void __launch_bounds__(1024)
group_scan_apply_kernel(uint64_t* __restrict__ sb, uint64_t count,
                        uint64_t const* __restrict__ chunk) {
  uint64_t const first = uint64_t(blockIdx.x) * kScanChunk;
  uint64_t const end = min(count, first + kScanChunk);
  uint64_t carry[S];
  for (uint32_t d = 0; d < S; ++d) carry[d] = chunk ? chunk[blockIdx.x * S + d] : 0;
  for (uint64_t base = first; base < end; base += blockDim.x) {
    uint64_t const i = base + threadIdx.x;
    bool const in = i < end;
#pragma unroll
    for (uint32_t k = 0; k < S / 2; ++k) {
      uint4 const a = in ? reinterpret_cast<uint4 const*>(sb + i * S)[k]
                         : make_uint4(0, 0, 0, 0);
      uint64_t tot = 0;
      uint64_t const e = cta_exclusive_scan(uint64_t(a.x) | (uint64_t(a.z) << 32), &tot);
      if (in) {
        sb[i * S + 2 * k] = carry[2 * k] + (e & 0xFFFFFFFFu);
        sb[i * S + 2 * k + 1] = carry[2 * k + 1] + (e >> 32);
      }
      carry[2 * k] += tot & 0xFFFFFFFFu;
      carry[2 * k + 1] += tot >> 32;
    }
  }
}

// Counts before every superblock of one level's table (nsb + 1 entries of
// S digits, the last one zero before and the totals after).
template <uint32_t S>
void scan_superblocks(uint64_t* sb, uint64_t entries, DevBuf& chunk, cudaStream_t st) {
  uint64_t const chunks = ceil_div(entries, kScanChunk);
  if (chunks > 1) {
    group_scan_partial_kernel<S><<<static_cast<uint32_t>(chunks), 256, 0, st>>>(
        sb, entries, chunk.as<uint64_t>());
    EWT_LAUNCHED();
    group_scan_chunks_kernel<S><<<1, 32, 0, st>>>(chunk.as<uint64_t>(), chunks);
    EWT_LAUNCHED();
  }
  group_scan_apply_kernel<S><<<static_cast<uint32_t>(chunks), 1024, 0, st>>>(
      sb, entries, chunks > 1 ? chunk.as<uint64_t>() : nullptr);
  EWT_LAUNCHED();
}

// Dense samples of one block: entry k of digit d names the block holding
// its (k * R + 1)-th occurrence, R = 2^sel_shift <= 2^16; before/c =
// occurrences before / in it (S = 2^width digits).  The first multiple of R
// at or after `before` is before + ((R - before) mod R): an entry lies in the
// block iff that offset is below c (32-bit test; 64-bit work only then).
template <uint32_t S>
__device__ __forceinline__ void put_group_samples(uint32_t* __restrict__ ds,
                                                  GroupLevel const& ql, uint64_t blk,
                                                  uint64_t const before[S],
                                                  uint32_t const c[S]) {
  uint32_t const sh = ql.sel_shift;
  uint32_t const rm = (1u << sh) - 1u;
#pragma unroll
  for (uint32_t d = 0; d < S; ++d) {
    uint32_t const off = (0u - static_cast<uint32_t>(before[d])) & rm;
    if (off >= c[d]) continue;  // the common case: no entry here
    uint32_t* S_ = ds + ql.ds_off[d];
    uint64_t k = (before[d] + off) >> sh;
    for (uint32_t o = off; o < c[d]; o += rm + 1, ++k) S_[k] = static_cast<uint32_t>(blk);
  }
}

// 8 digits from one byte of high bits hb and the next low bits: the table
// entry (hb << 8 | v) holds digit k = (hb bit k) * 2 + low bit k at bits
// 2k..2k+1, where v carries the next z = 8 - popc(hb) bits of the left run
// followed by the next popc(hb) bits of the right run.
void make_digit_lut(std::vector<uint16_t>& lut) {
  lut.assign(65536, 0);
  for (uint32_t hb = 0; hb < 256; ++hb) {
    uint32_t const o = static_cast<uint32_t>(__builtin_popcount(hb)), z = 8 - o;
    for (uint32_t v = 0; v < 256; ++v) {
      uint32_t r0 = v & ((1u << z) - 1u), r1 = v >> z, out = 0;
      for (uint32_t k = 0; k < 8; ++k) {
        uint32_t const hi = hb >> k & 1u;
        uint32_t lo;
        if (hi) { lo = r1 & 1u; r1 >>= 1; } else { lo = r0 & 1u; r0 >>= 1; }
        out |= ((hi << 1) | lo) << (2 * k);
      }
      lut[(hb << 8) | v] = static_cast<uint16_t>(out);
    }
  }
}

// 32 positions (high bits h, valid) -> 64 digit bits; r0 / r1 the next
// bits of the left / right run.
__device__ __forceinline__ void digits_fast(uint16_t const* lut, uint32_t h,
                                            uint32_t r0, uint32_t r1,
                                            uint32_t& dlo, uint32_t& dhi) {
  uint32_t d[4];
#pragma unroll
  for (uint32_t i = 0; i < 4; ++i) {
    uint32_t const hb = (h >> (8 * i)) & 0xFFu;
    uint32_t const o = __popc(hb), z = 8 - o;
    uint32_t const v = (r0 & ((1u << z) - 1u)) | ((r1 & ((1u << o) - 1u)) << z);
    r0 >>= z;
    r1 >>= o;
    d[i] = lut[(hb << 8) | v];
  }
  dlo = d[0] | (d[1] << 16);
  dhi = d[2] | (d[3] << 16);
}

// Exclusive scan over the 512 threads of one half of a 1024-thread CTA
// (each half works on its own superblocks and synchronises on its own named
// barrier, 1 or 2, so the halves overlap); *total = the half's sum.
__device__ __forceinline__ uint32_t group_exclusive_scan32(uint32_t x, uint32_t* total) {
  __shared__ uint32_t ws32[2][17];
  uint32_t const lane = threadIdx.x & 31, wid = (threadIdx.x >> 5) & 15;
  uint32_t const g = threadIdx.x >> 9;
  uint32_t* const ws = ws32[g];
  uint32_t inc = x;
#pragma unroll
  for (uint32_t o = 1; o < 32; o <<= 1) {
    uint32_t const y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) ws[wid] = inc;
  asm volatile("bar.sync %0, 512;" ::"r"(g + 1) : "memory");
  if (wid == 0) {
    uint32_t t = lane < 16 ? ws[lane] : 0u;
#pragma unroll
    for (uint32_t o = 1; o < 16; o <<= 1) {
      uint32_t const y = __shfl_up_sync(0xFFFFFFFFu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < 16) ws[lane] = t;  // inclusive over the half's warps
  }
  asm volatile("bar.sync %0, 512;" ::"r"(g + 1) : "memory");
  uint32_t const before = wid ? ws[wid - 1] : 0u;
  *total = ws[15];
  asm volatile("bar.sync %0, 512;" ::"r"(g + 1) : "memory");
  return before + inc - x;
}

// Pass 3: persistent CTAs of 1024 threads; each 512-thread half walks its
// own superblocks (one thread per 96-digit block), the digit table shared
// in shared memory.
__global__ void __launch_bounds__(1024, 1)
quad_level_kernel(TreeView v, uint32_t l, GroupLevel ql,
                  uint32_t const* __restrict__ hi_w, uint64_t hi_words,
                  uint32_t const* __restrict__ lo_w, uint64_t lo_limit,
                  uint16_t const* __restrict__ lut_g,
                  uint4* __restrict__ blocks, uint64_t const* __restrict__ sb,
                  SbStart const* __restrict__ info, uint64_t nsb,
                  uint32_t* __restrict__ ds, uint32_t* __restrict__ err) {
  extern __shared__ __align__(16) uint16_t lut[];
  {
    uint4 const* src = reinterpret_cast<uint4 const*>(lut_g);
    uint4* dst = reinterpret_cast<uint4*>(lut);
    for (uint32_t i = threadIdx.x; i < 65536 * 2 / 16; i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  uint64_t const n = v.n;
  uint32_t const sh = v.levels - l;
  uint64_t const nodes = uint64_t(1) << l;
  uint32_t const t = threadIdx.x & (kQuadSbBlocks - 1);  // block inside its superblock
  // half h of CTA b takes superblocks 2b + h, 2b + h + 2G, ...
  uint64_t const first = uint64_t(blockIdx.x) * 2 + (threadIdx.x >> 9);
  for (uint64_t sbi = first; sbi < nsb; sbi += uint64_t(gridDim.x) * 2) {
    SbStart const st = info[sbi];
    uint64_t const blk = sbi * kQuadSbBlocks + t;
    bool const mine = blk < ql.num_blocks;
    uint64_t const p = blk * kQuadDigits;
    uint32_t h[3], vm[3];
    uint32_t ones = 0;
#pragma unroll
    for (uint32_t k = 0; k < 3; ++k) {
      uint64_t const w = blk * 3 + k;
      uint64_t const p0 = p + 32 * k;
      uint32_t const valid =
          mine && p0 < n ? static_cast<uint32_t>(min(uint64_t(32), n - p0)) : 0u;
      vm[k] = valid == 32 ? ~0u : (1u << valid) - 1u;
      h[k] = valid && w < hi_words ? hi_w[w] & vm[k] : 0u;
      ones += __popc(h[k]);
    }
    uint32_t tot = 0;
    // ones of level l in the superblock before this block (= its digits 2
    // and 3 before it)
    uint32_t const h23 = group_exclusive_scan32(ones, &tot);
    uint64_t r1 = st.rank1 + h23;  // ones before p
    uint32_t dw[6] = {0, 0, 0, 0, 0, 0};
    uint64_t const right = st.node.start + st.node.zeros;  // right child start
#pragma unroll
    for (uint32_t k = 0; k < 3; ++k) {
      uint64_t const p0 = p + 32 * k;
      if (vm[k]) {
        if (st.uniform) {
          uint64_t const ob = r1 - st.node.ones_before;  // node ones before p0
          digits_fast(lut, h[k], bits_fast(lo_w, p0 - ob), bits_fast(lo_w, right + ob),
                      dw[2 * k], dw[2 * k + 1]);
          if (vm[k] != ~0u) {  // positions past n: digit 0
            dw[2 * k] &= spread16(vm[k]) * 3u;
            dw[2 * k + 1] &= spread16(vm[k] >> 16) * 3u;
          }
        } else {  // the word may cross node boundaries: bit by bit per node
          uint32_t low = 0;
          uint64_t pos = p0;
          uint64_t const pend = min(n, p0 + 32);
          uint32_t guard = 0;
          while (pos < pend && guard++ < 32) {
            QuadNode const nd =
                quad_node(v, l, sh, nodes, node_of(v.counts, sh, nodes, pos));
            if (nd.end <= pos) break;  // inconsistent table (reported below)
            uint64_t const se = min(pend, nd.end);
            uint32_t const k0 = static_cast<uint32_t>(pos - p0);
            uint32_t const k1 = static_cast<uint32_t>(se - p0);
            uint64_t const ob = r1 + __popc(h[k] & ((1u << k0) - 1u)) - nd.ones_before;
            uint32_t a0 = bits_at(lo_w, lo_limit, pos - ob);
            uint32_t a1 = bits_at(lo_w, lo_limit, nd.start + nd.zeros + ob);
            for (uint32_t q = k0; q < k1; ++q) {
              uint32_t bit;
              if (h[k] >> q & 1u) { bit = a1 & 1u; a1 >>= 1; } else { bit = a0 & 1u; a0 >>= 1; }
              low |= bit << q;
            }
            pos = se;
          }
          if (pos < pend) atomicOr(err, 1u);
          dw[2 * k] = spread16(low) | (spread16(h[k]) << 1);
          dw[2 * k + 1] = spread16(low >> 16) | (spread16(h[k] >> 16) << 1);
        }
      }
      r1 += __popc(h[k]);
    }
    uint32_t c1 = 0, c3 = 0;  // digits 1 and 3 of the block
#pragma unroll
    for (uint32_t k = 0; k < 6; ++k) {
      uint32_t const lo = dw[k] & 0x55555555u, hi = (dw[k] >> 1) & 0x55555555u;
      c3 += __popc(lo & hi);
      c1 += __popc(lo & ~hi);
    }
    uint32_t tot13 = 0;
    uint32_t const h13 = group_exclusive_scan32(c1 | (c3 << 16), &tot13);  // each < 2^16
    uint64_t const* sbe = sb + sbi * 4;
    uint32_t const in_sb = t * kQuadDigits;  // positions before the block
    uint32_t const h1 = h13 & 0xFFFFu, h3 = h13 >> 16;
    uint32_t const h0 = in_sb - h23 - h1, h2 = h23 - h3;
    if (t == 0) {  // the pass-1 counts must agree
      uint64_t const first = sbi * kQuadSbDigits;
      uint32_t const all = first < n ? static_cast<uint32_t>(min(kQuadSbDigits, n - first)) : 0u;
      uint32_t const t1 = tot13 & 0xFFFFu, t3 = tot13 >> 16;
      if (sbe[5] - sbe[1] != t1 || sbe[7] - sbe[3] != t3 ||
          sbe[6] - sbe[2] != tot - t3 || sbe[4] - sbe[0] != all - tot - t1)
        atomicOr(err, 2u);
    }
    if (!mine) continue;
    uint4* out = blocks + blk * 2;
    out[0] = make_uint4(h0 | (h1 << 16), h2, dw[0], dw[1]);
    out[1] = make_uint4(dw[2], dw[3], dw[4], dw[5]);
    if (ds && ql.sel_shift) {
      uint32_t const vb = static_cast<uint32_t>(min(uint64_t(kQuadDigits), n - p));
      uint32_t const c[4] = {vb - ones - c1, c1, ones - c3, c3};
      uint64_t const before[4] = {sbe[0] + h0, sbe[1] + h1, sbe[2] + h2, sbe[3] + h3};
      put_group_samples<4>(ds, ql, blk, before, c);
    }
  }
}

// Bits q .. q+63 of a bit array with slack behind its end.
__device__ __forceinline__ uint64_t bits64(uint32_t const* __restrict__ w, uint64_t q) {
  return uint64_t(bits_fast(w, q)) | (uint64_t(bits_fast(w, q + 32)) << 32);
}

// Routes two runs into level-l order, eight positions per table lookup:
// position k takes the next bit of run a1 if bit k of h is set, else the
// next bit of run a0.  Table entry (hb << 8 | v) holds the 8 routed bits for
// high byte hb, v = the next 8 - popc(hb) bits of a0 then popc(hb) of a1.
template <uint32_t kChunks>
__device__ __forceinline__ uint64_t route_runs(uint8_t const* lut, uint64_t h,
                                               uint64_t a0, uint64_t a1) {
  uint64_t out = 0;
#pragma unroll
  for (uint32_t i = 0; i < kChunks; ++i) {
    uint32_t const hb = static_cast<uint32_t>(h >> (8 * i)) & 0xFFu;
    uint32_t const o = __popc(hb), z = 8 - o;
    uint32_t const v = (static_cast<uint32_t>(a0) & ((1u << z) - 1u)) |
                       ((static_cast<uint32_t>(a1) & ((1u << o) - 1u)) << z);
    a0 >>= z;
    a1 >>= o;
    out |= uint64_t(lut[(hb << 8) | v]) << (8 * i);
  }
  return out;
}

// Low 32 bits of (hi:lo) >> s, s < 64.
__device__ __forceinline__ uint32_t window32(uint32_t lo, uint32_t hi, uint32_t s) {
  return s < 32 ? __funnelshift_r(lo, hi, s) : hi >> (s - 32);
}

// route_runs for two planes under the same high bits (the octal digit's
// middle and low bits): one byte of h, its popcount and masks per chunk
// serve both, the runs are read through 32-bit windows.
template <uint32_t kChunks>
__device__ __forceinline__ void route_two(uint8_t const* lut, uint64_t h, uint64_t a0,
                                          uint64_t a1, uint64_t b0, uint64_t b1,
                                          uint64_t& ra, uint64_t& rb) {
  uint32_t const a0l = static_cast<uint32_t>(a0), a0h = static_cast<uint32_t>(a0 >> 32);
  uint32_t const a1l = static_cast<uint32_t>(a1), a1h = static_cast<uint32_t>(a1 >> 32);
  uint32_t const b0l = static_cast<uint32_t>(b0), b0h = static_cast<uint32_t>(b0 >> 32);
  uint32_t const b1l = static_cast<uint32_t>(b1), b1h = static_cast<uint32_t>(b1 >> 32);
  uint32_t Z = 0, O = 0;
  uint32_t oa[2] = {0, 0}, ob[2] = {0, 0};
#pragma unroll
  for (uint32_t i = 0; i < kChunks; ++i) {
    uint32_t const hb = (static_cast<uint32_t>(h >> (8 * i))) & 0xFFu;
    uint32_t const o = __popc(hb), z = 8 - o;
    uint32_t const mz = (1u << z) - 1u, mo = (1u << o) - 1u;
    uint32_t const va = (window32(a0l, a0h, Z) & mz) | ((window32(a1l, a1h, O) & mo) << z);
    uint32_t const vb = (window32(b0l, b0h, Z) & mz) | ((window32(b1l, b1h, O) & mo) << z);
    oa[i >> 2] |= uint32_t(lut[(hb << 8) | va]) << (8 * (i & 3));
    ob[i >> 2] |= uint32_t(lut[(hb << 8) | vb]) << (8 * (i & 3));
    Z += z;
    O += o;
  }
  ra = uint64_t(oa[0]) | (uint64_t(oa[1]) << 32);
  rb = uint64_t(ob[0]) | (uint64_t(ob[1]) << 32);
}

void make_route_lut(std::vector<uint8_t>& lut) {
  lut.assign(65536, 0);
  for (uint32_t hb = 0; hb < 256; ++hb) {
    uint32_t const o = static_cast<uint32_t>(__builtin_popcount(hb)), z = 8 - o;
    for (uint32_t v = 0; v < 256; ++v) {
      uint32_t r0 = v & ((1u << z) - 1u), r1 = v >> z, out = 0;
      for (uint32_t k = 0; k < 8; ++k) {
        uint32_t bit;
        if (hb >> k & 1u) { bit = r1 & 1u; r1 >>= 1; } else { bit = r0 & 1u; r0 >>= 1; }
        out |= bit << k;
      }
      lut[(hb << 8) | v] = static_cast<uint8_t>(out);
    }
  }
}

// Routed plane bits of positions [p0, pend) of level l (pend - p0 <= 32)
// whose node may change inside: bit q = the plane's bit at the child
// position of p0 + q.  h = their level-l bits, r1 = ones of level l before p0.
__device__ uint32_t route_slow(TreeView const& v, uint32_t l, uint32_t sh,
                               uint64_t nodes, uint32_t h, uint64_t r1, uint64_t p0,
                               uint64_t pend, uint32_t const* __restrict__ plane,
                               uint64_t limit, uint32_t* __restrict__ err) {
  uint32_t out = 0;
  uint64_t pos = p0;
  uint32_t guard = 0;
  while (pos < pend && guard++ < 32) {
    QuadNode const nd = quad_node(v, l, sh, nodes, node_of(v.counts, sh, nodes, pos));
    if (nd.end <= pos) break;  // inconsistent table (reported below)
    uint64_t const se = min(pend, nd.end);
    uint32_t const k0 = static_cast<uint32_t>(pos - p0);
    uint32_t const k1 = static_cast<uint32_t>(se - p0);
    uint64_t const ob = r1 + __popc(h & ((1u << k0) - 1u)) - nd.ones_before;
    uint32_t a0 = bits_at(plane, limit, pos - ob);
    uint32_t a1 = bits_at(plane, limit, nd.start + nd.zeros + ob);
    for (uint32_t q = k0; q < k1; ++q) {
      uint32_t bit;
      if (h >> q & 1u) { bit = a1 & 1u; a1 >>= 1; } else { bit = a0 & 1u; a0 >>= 1; }
      out |= bit << q;
    }
    pos = se;
  }
  if (pos < pend) atomicOr(err, 1u);
  return out;
}

// Node, ones before and uniformity of every superblock of sb_pos positions
// of level l (thread per superblock).
__global__ void __launch_bounds__(128)
sb_info_kernel(TreeView v, uint32_t l, uint64_t sb_pos, uint64_t nsb,
               SbStart* __restrict__ info) {
  uint64_t const s = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (s >= nsb) return;
  uint64_t const n = v.n;
  uint64_t const a = s * sb_pos, e = min(n, a + sb_pos);
  if (a >= e) {
    info[s] = SbStart{QuadNode{0, n, 0, 0}, 0, 1};
    return;
  }
  uint32_t const sh = v.levels - l;
  uint64_t const nodes = uint64_t(1) << l;
  QuadNode const nd = quad_node(v, l, sh, nodes, node_of(v.counts, sh, nodes, a));
  uint64_t const r1 = ecl::detail::rs_rank1<false>(v.rs, v.rs.meta[l], a, nullptr);
  info[s] = SbStart{nd, r1, e <= nd.end ? 1u : 0u};
}

__device__ __forceinline__ void load_lut8(uint8_t* lut, uint8_t const* lut_g) {
  uint4 const* src = reinterpret_cast<uint4 const*>(lut_g);
  uint4* dst = reinterpret_cast<uint4*>(lut);
  for (uint32_t i = threadIdx.x; i < 65536 / 16; i += blockDim.x) dst[i] = src[i];
  __syncthreads();
}

// Level l+1's bits routed into level-l order: persistent CTAs of 1024
// threads, each 512-thread half on its own superblocks, one thread per 64
// positions (2 output words).
__global__ void __launch_bounds__(1024, 1)
merge_plane_kernel(TreeView v, uint32_t l, uint32_t const* __restrict__ hi_w,
                   uint32_t const* __restrict__ lo_w, uint64_t lo_limit,
                   uint8_t const* __restrict__ lut_g, SbStart const* __restrict__ info,
                   uint64_t nsb, uint32_t* __restrict__ out, uint32_t* __restrict__ err) {
  extern __shared__ __align__(16) uint8_t lut8[];
  load_lut8(lut8, lut_g);
  uint64_t const n = v.n;
  uint32_t const sh = v.levels - l;
  uint64_t const nodes = uint64_t(1) << l;
  uint32_t const t = threadIdx.x & 511;
  uint64_t const first = uint64_t(blockIdx.x) * 2 + (threadIdx.x >> 9);
  for (uint64_t sbi = first; sbi < nsb; sbi += uint64_t(gridDim.x) * 2) {
    SbStart const st = info[sbi];
    uint64_t const p = (sbi * 512 + t) * 64;
    uint32_t const valid = p < n ? static_cast<uint32_t>(min(uint64_t(64), n - p)) : 0u;
    uint64_t const vm = valid == 64 ? ~0ull : (1ull << valid) - 1;
    uint64_t const wi = p >> 5;
    uint64_t const h =
        valid ? (uint64_t(hi_w[wi]) | (uint64_t(hi_w[wi + 1]) << 32)) & vm : 0ull;
    uint32_t tot = 0;
    uint64_t const r1 = st.rank1 + group_exclusive_scan32(__popcll(h), &tot);
    if (!valid) continue;
    uint64_t m;
    if (st.uniform) {
      uint64_t const ob = r1 - st.node.ones_before;  // node ones before p
      m = route_runs<8>(lut8, h, bits64(lo_w, p - ob),
                        bits64(lo_w, st.node.start + st.node.zeros + ob));
    } else {
      uint64_t const e0 = min(n, p + 32);
      m = route_slow(v, l, sh, nodes, static_cast<uint32_t>(h), r1, p, e0, lo_w,
                     lo_limit, err);
      if (valid > 32)
        m |= uint64_t(route_slow(v, l, sh, nodes, static_cast<uint32_t>(h >> 32),
                                 r1 + __popc(static_cast<uint32_t>(h)), p + 32,
                                 min(n, p + 64), lo_w, lo_limit, err))
             << 32;
    }
    m &= vm;
    out[wi] = static_cast<uint32_t>(m);
    out[wi + 1] = static_cast<uint32_t>(m >> 32);
  }
}

// Exclusive scan of four uint32 over one 512-thread half (as
// group_exclusive_scan32, one set of barriers).
__device__ __forceinline__ uint4 group_exclusive_scan4(uint4 x, uint4* total) {
  __shared__ uint4 ws4[2][16];
  uint32_t const lane = threadIdx.x & 31, wid = (threadIdx.x >> 5) & 15;
  uint32_t const g = threadIdx.x >> 9;
  uint4* const ws = ws4[g];
  uint4 inc = x;
#pragma unroll
  for (uint32_t o = 1; o < 32; o <<= 1) {
    uint32_t const a = __shfl_up_sync(0xFFFFFFFFu, inc.x, o);
    uint32_t const b = __shfl_up_sync(0xFFFFFFFFu, inc.y, o);
    uint32_t const c = __shfl_up_sync(0xFFFFFFFFu, inc.z, o);
    uint32_t const d = __shfl_up_sync(0xFFFFFFFFu, inc.w, o);
    if (lane >= o) { inc.x += a; inc.y += b; inc.z += c; inc.w += d; }
  }
  if (lane == 31) ws[wid] = inc;
  asm volatile("bar.sync %0, 512;" ::"r"(g + 1) : "memory");
  if (wid == 0) {
    uint4 t = lane < 16 ? ws[lane] : make_uint4(0, 0, 0, 0);
#pragma unroll
    for (uint32_t o = 1; o < 16; o <<= 1) {
      uint32_t const a = __shfl_up_sync(0xFFFFFFFFu, t.x, o);
      uint32_t const b = __shfl_up_sync(0xFFFFFFFFu, t.y, o);
      uint32_t const c = __shfl_up_sync(0xFFFFFFFFu, t.z, o);
      uint32_t const d = __shfl_up_sync(0xFFFFFFFFu, t.w, o);
      if (lane >= o) { t.x += a; t.y += b; t.z += c; t.w += d; }
    }
    if (lane < 16) ws[lane] = t;
  }
  asm volatile("bar.sync %0, 512;" ::"r"(g + 1) : "memory");
  uint4 const before = wid ? ws[wid - 1] : make_uint4(0, 0, 0, 0);
  *total = ws[15];
  asm volatile("bar.sync %0, 512;" ::"r"(g + 1) : "memory");
  return make_uint4(before.x + inc.x - x.x, before.y + inc.y - x.y,
                    before.z + inc.z - x.z, before.w + inc.w - x.w);
}

// Octal level at l: one thread per 42-digit block, each 512-thread half on
// its own superblocks.  Digit = (level l bit, level l+1 routed, plane routed)
// with the plane = level l+2 in level-(l+1) order.  Writes the blocks and the
// superblock's digit counts (scanned afterwards).
__global__ void __launch_bounds__(1024, 1)
octal_level_kernel(TreeView v, uint32_t l, uint32_t const* __restrict__ hi_w,
                   uint32_t const* __restrict__ mid_w, uint64_t mid_limit,
                   uint32_t const* __restrict__ low_w, uint64_t low_limit,
                   uint8_t const* __restrict__ lut_g, SbStart const* __restrict__ info,
                   uint64_t nsb, uint64_t num_blocks, uint4* __restrict__ blocks,
                   uint64_t* __restrict__ sb, uint32_t* __restrict__ err) {
  extern __shared__ __align__(16) uint8_t lut8[];
  load_lut8(lut8, lut_g);
  uint64_t const n = v.n;
  uint32_t const sh = v.levels - l;
  uint64_t const nodes = uint64_t(1) << l;
  uint32_t const t = threadIdx.x & (kOctSbBlocks - 1);
  uint64_t const first = uint64_t(blockIdx.x) * 2 + (threadIdx.x >> 9);
  for (uint64_t sbi = first; sbi < nsb; sbi += uint64_t(gridDim.x) * 2) {
    SbStart const st = info[sbi];
    uint64_t const blk = sbi * kOctSbBlocks + t;
    bool const mine = blk < num_blocks;
    uint64_t const p = blk * kOctDigits;
    uint32_t const valid =
        mine && p < n ? static_cast<uint32_t>(min(uint64_t(kOctDigits), n - p)) : 0u;
    uint64_t const vm = (1ull << valid) - 1;  // valid <= 42
    uint64_t const H = valid ? bits64(hi_w, p) & vm : 0ull;
    uint32_t tot = 0;
    uint64_t const r1 = st.rank1 + group_exclusive_scan32(__popcll(H), &tot);
    uint64_t M = 0, B = 0;
    if (valid) {
      if (st.uniform) {
        uint64_t const ob = r1 - st.node.ones_before;
        uint64_t const q0 = p - ob, q1 = st.node.start + st.node.zeros + ob;
        route_two<6>(lut8, H, bits64(mid_w, q0), bits64(mid_w, q1), bits64(low_w, q0),
                     bits64(low_w, q1), M, B);
        M &= vm;
        B &= vm;
      } else {
        uint64_t const end = p + valid;
#pragma unroll
        for (uint32_t k = 0; k < 2; ++k) {
          uint64_t const p0 = p + 32 * k;
          if (p0 >= end) break;
          uint64_t const pe = min(end, p0 + 32);
          uint32_t const hk = static_cast<uint32_t>(H >> (32 * k));
          uint64_t const rk = r1 + (k ? __popc(static_cast<uint32_t>(H)) : 0u);
          M |= uint64_t(route_slow(v, l, sh, nodes, hk, rk, p0, pe, mid_w, mid_limit, err))
               << (32 * k);
          B |= uint64_t(route_slow(v, l, sh, nodes, hk, rk, p0, pe, low_w, low_limit, err))
               << (32 * k);
        }
      }
    }
    uint32_t c[8];
#pragma unroll
    for (uint32_t d = 0; d < 8; ++d)
      c[d] = __popcll((d & 4 ? H : ~H) & (d & 2 ? M : ~M) & (d & 1 ? B : ~B) & vm);
    uint4 tot4;
    // every count below 2^16 (21,504 digits per superblock): two per word
    uint4 const e = group_exclusive_scan4(
        make_uint4(c[0] | (c[1] << 16), c[2] | (c[3] << 16), c[4] | (c[5] << 16),
                   c[6] | (c[7] << 16)),
        &tot4);
    if (t == 0) {
      uint64_t* o = sb + sbi * 8;
      uint32_t const w4[4] = {tot4.x, tot4.y, tot4.z, tot4.w};
#pragma unroll
      for (uint32_t d = 0; d < 8; ++d) o[d] = (w4[d >> 1] >> (16 * (d & 1))) & 0xFFFFu;
    }
    if (!mine) continue;
    // planes H, M, B in words 1..3, counts of digits 4..6 above them
    uint64_t const w1 = H | (uint64_t(e.z & 0xFFFFu) << 42);
    uint64_t const w2 = M | (uint64_t(e.z >> 16) << 42);
    uint64_t const w3 = B | (uint64_t(e.w & 0xFFFFu) << 42);
    uint4* out = blocks + blk * 2;
    out[0] = make_uint4(e.x, e.y, static_cast<uint32_t>(w1), static_cast<uint32_t>(w1 >> 32));
    out[1] = make_uint4(static_cast<uint32_t>(w2), static_cast<uint32_t>(w2 >> 32),
                        static_cast<uint32_t>(w3), static_cast<uint32_t>(w3 >> 32));
  }
}

// An octal group level of a tree of 1- or 2-byte minimal symbols straight
// from the symbols in that level's order (digit = bits sb0+2 .. sb0; no
// routing): level 0 from the text, a later level from the level order a
// pass wrote.  One CTA of 512 threads per superblock, three per SM (more
// loads in flight than persistent CTAs walking superblocks): it first turns
// the superblock's symbols (16-byte loads) into three bit planes in shared
// memory, then each thread takes its block's 42 bits of each.
template <class T>
__global__ void __launch_bounds__(512, 3)
octal_text_kernel(T const* __restrict__ sym, uint64_t n, uint32_t sb0, uint64_t nsb,
                  uint64_t num_blocks, uint4* __restrict__ blocks,
                  uint64_t* __restrict__ sb, uint32_t* __restrict__ level0,
                  uint32_t check_hi, uint32_t* __restrict__ err) {
  constexpr uint32_t kV = 16 / sizeof(T);           // symbols per 16-byte load
  constexpr uint32_t kLoads = uint32_t(kOctSbDigits) / kV;
  constexpr uint32_t kWords = uint32_t(kOctSbDigits) / 32 + 4;
  __shared__ uint32_t planes[1][3][kWords];
  uint32_t const half = 0;
  uint32_t const t = threadIdx.x;
  constexpr uint32_t kPer = (kLoads + kOctSbBlocks - 1) / kOctSbBlocks;  // loads / thread
  auto load = [&](uint64_t sbi, uint4 (&x)[kPer]) {
    uint64_t const base = sbi * kOctSbDigits;
#pragma unroll
    for (uint32_t j = 0; j < kPer; ++j) {
      uint32_t const u = t + j * kOctSbBlocks;
      uint64_t const pos = base + uint64_t(u) * kV;
      x[j] = make_uint4(0, 0, 0, 0);
      if (sbi >= nsb || u >= kLoads) continue;
      if (pos + kV <= n) {
        x[j] = __ldg(reinterpret_cast<uint4 const*>(sym + pos));
      } else if (pos < n) {
        T e[kV];
        for (uint32_t i = 0; i < kV; ++i) e[i] = pos + i < n ? sym[pos + i] : T(0);
        x[j] = *reinterpret_cast<uint4 const*>(e);
      }
    }
  };
  bool bad = false;
  for (uint64_t sbi = blockIdx.x; sbi < nsb; sbi += gridDim.x) {
    uint4 cx[kPer];
    load(sbi, cx);
#pragma unroll
    for (uint32_t j = 0; j < kPer; ++j) {
      uint32_t const u = t + j * kOctSbBlocks;
      if (u >= kLoads) continue;
      uint32_t const w[4] = {cx[j].x, cx[j].y, cx[j].z, cx[j].w};
      // a minimal symbol of 2^L is below it: no bit at or above L
      bad |= ((w[0] | w[1] | w[2] | w[3]) & check_hi) != 0;
#pragma unroll
      for (uint32_t b = 0; b < 3; ++b) {  // plane b: bit sb0 + 2 - b
        uint32_t const sh = sb0 + 2 - b;
        uint32_t f = 0;
#pragma unroll
        for (uint32_t k = 0; k < 4; ++k) {
          if constexpr (sizeof(T) == 1) {
            uint32_t const m = (w[k] >> sh) & 0x01010101u;
            f |= (((m * 0x00204081u) >> 21) & 0xFu) << (4 * k);
          } else {
            uint32_t const m = (w[k] >> sh) & 0x00010001u;
            f |= ((m | (m >> 15)) & 3u) << (2 * k);
          }
        }
        if constexpr (sizeof(T) == 1)
          reinterpret_cast<uint16_t*>(planes[half][b])[u] = static_cast<uint16_t>(f);
        else
          reinterpret_cast<uint8_t*>(planes[half][b])[u] = static_cast<uint8_t>(f);
      }
    }
    asm volatile("bar.sync %0, 512;" ::"r"(half + 1) : "memory");
    if (level0) {  // plane 0 is level 0's bits: 672 whole words per superblock
      uint64_t const w0 = sbi * (kOctSbDigits / 32), words = (n + 31) / 32;
      for (uint32_t w = t; w < kOctSbDigits / 32; w += kOctSbBlocks)
        if (w0 + w < words) level0[w0 + w] = planes[half][0][w];
    }
    uint64_t const blk = sbi * kOctSbBlocks + t;
    bool const mine = blk < num_blocks;
    uint64_t const p = blk * kOctDigits;
    uint32_t const valid =
        mine && p < n ? static_cast<uint32_t>(min(uint64_t(kOctDigits), n - p)) : 0u;
    uint64_t const vm = (1ull << valid) - 1;
    uint32_t const o = t * kOctDigits, wi = o >> 5, s = o & 31;
    uint64_t pl[3];
#pragma unroll
    for (uint32_t b = 0; b < 3; ++b) {
      uint32_t const* P = planes[half][b];
      pl[b] = (uint64_t(__funnelshift_r(P[wi], P[wi + 1], s)) |
               (uint64_t(__funnelshift_r(P[wi + 1], P[wi + 2], s)) << 32)) & vm;
    }
    uint64_t const H = pl[0], M = pl[1], B = pl[2];
    uint32_t c[8];
#pragma unroll
    for (uint32_t d = 0; d < 8; ++d)
      c[d] = __popcll((d & 4 ? H : ~H) & (d & 2 ? M : ~M) & (d & 1 ? B : ~B) & vm);
    uint4 tot4;
    uint4 const e = group_exclusive_scan4(
        make_uint4(c[0] | (c[1] << 16), c[2] | (c[3] << 16), c[4] | (c[5] << 16),
                   c[6] | (c[7] << 16)),
        &tot4);  // its barriers also end this superblock's plane reads
    if (t == 0) {
      uint64_t* out = sb + sbi * 8;
      uint32_t const w4[4] = {tot4.x, tot4.y, tot4.z, tot4.w};
#pragma unroll
      for (uint32_t d = 0; d < 8; ++d) out[d] = (w4[d >> 1] >> (16 * (d & 1))) & 0xFFFFu;
    }
    if (!mine) continue;
    uint64_t const w1 = H | (uint64_t(e.z & 0xFFFFu) << 42);
    uint64_t const w2 = M | (uint64_t(e.z >> 16) << 42);
    uint64_t const w3 = B | (uint64_t(e.w & 0xFFFFu) << 42);
    uint4* out = blocks + blk * 2;
    out[0] = make_uint4(e.x, e.y, static_cast<uint32_t>(w1), static_cast<uint32_t>(w1 >> 32));
    out[1] = make_uint4(static_cast<uint32_t>(w2), static_cast<uint32_t>(w2 >> 32),
                        static_cast<uint32_t>(w3), static_cast<uint32_t>(w3 >> 32));
  }
  if (bad) atomicOr(err, 1u);
}

// Dense samples of one group level from its finished blocks and scanned
// superblock table; block 0 also checks the level's digit totals.
template <int W>
__global__ void __launch_bounds__(256)
group_samples_kernel(uint4 const* __restrict__ blocks, uint64_t const* __restrict__ sb,
                     uint64_t n, GroupLevel ql, uint32_t* __restrict__ ds,
                     uint32_t* __restrict__ err) {
  constexpr uint32_t S = 1u << W;
  constexpr uint32_t kD = GroupShape<W>::kDigits, kSb = GroupShape<W>::kSbBlocks;
  uint64_t const b = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (b == 0 && err) {
    uint64_t const* tot = sb + (ql.num_blocks + kSb - 1) / kSb * S;
    for (uint32_t d = 0; d < S; ++d)
      if (tot[d] != ql.total[d]) atomicOr(err, 4u);
  }
  if (!ds || ql.sel_shift == 0 || b >= ql.num_blocks) return;
  uint4 const x = blocks[b * 2], y = blocks[b * 2 + 1];
  uint64_t q[4];
  ecl::detail::quad_words(x, y, q);
  uint64_t const first = b * kD;
  uint32_t const valid = first < n ? static_cast<uint32_t>(min(uint64_t(kD), n - first)) : 0u;
  uint4 const* sb4 = reinterpret_cast<uint4 const*>(sb + (b / kSb) * S);
  uint64_t sbv[S];
#pragma unroll
  for (uint32_t k = 0; k < S / 2; ++k) {
    uint4 const e = sb4[k];
    sbv[2 * k] = uint64_t(e.y) << 32 | e.x;
    sbv[2 * k + 1] = uint64_t(e.w) << 32 | e.z;
  }
  uint64_t before[S];
  uint32_t c[S];
  if constexpr (W == 3) {  // headers parsed once, counts from the planes
    uint64_t const vm = (1ull << valid) - 1;
    uint64_t const H = q[1] & vm, M = q[2] & vm, B = q[3] & vm;
    uint32_t h[8];
    h[0] = static_cast<uint32_t>(q[0]) & 0xFFFFu;
    h[1] = static_cast<uint32_t>(q[0] >> 16) & 0xFFFFu;
    h[2] = static_cast<uint32_t>(q[0] >> 32) & 0xFFFFu;
    h[3] = static_cast<uint32_t>(q[0] >> 48);
    h[4] = static_cast<uint32_t>(q[1] >> 42) & 0xFFFFu;
    h[5] = static_cast<uint32_t>(q[2] >> 42) & 0xFFFFu;
    h[6] = static_cast<uint32_t>(q[3] >> 42) & 0xFFFFu;
    h[7] = static_cast<uint32_t>(b % kSb) * kD - h[0] - h[1] - h[2] - h[3] - h[4] -
           h[5] - h[6];
#pragma unroll
    for (uint32_t d = 0; d < S; ++d) {
      c[d] = __popcll((d & 4 ? H : ~H) & (d & 2 ? M : ~M) & (d & 1 ? B : ~B) & vm);
      before[d] = sbv[d] + h[d];
    }
  } else {
#pragma unroll
    for (uint32_t d = 0; d < S; ++d) {
      c[d] = ecl::detail::group_count<W>(q, d, valid);
      before[d] = ecl::detail::group_before<W>(q, sbv[d], d, b);
    }
  }
  put_group_samples<S>(ds, ql, b, before, c);
}

// Sample shift of a group level for the tree-wide rate 2^shift: octal
// digits are about half as frequent and blocks hold 42 instead of 96, and
// the interpolated block is off by more blocks at equal bracket width, so
// octal levels sample 8 times as densely.
uint32_t level_shift(uint32_t width, uint32_t shift) {
  if (shift == 0) return 0;
  return width == 3 ? std::max<uint32_t>(shift, 7) - 3 : shift;
}

// Lays out the dense samples of every group level at rate 2^shift.
void layout_group_samples(GroupStore& qs, uint32_t shift) {
  qs.ds.reset();
  qs.sel_shift = shift;
  uint64_t total = 0;
  for (auto& ql : qs.levels) {
    ql.sel_shift = level_shift(ql.width, shift);
    for (uint32_t d = 0; d < 8; ++d) ql.ds_off[d] = 0;
    if (!ql.sel_shift) continue;
    for (uint32_t d = 0; d < (1u << ql.width); ++d) {
      ql.ds_off[d] = total;
      total += ceil_div(ql.total[d], uint64_t(1) << ql.sel_shift);
    }
  }
  if (shift) qs.ds.alloc(std::max<uint64_t>(total, 1) * 4);
}

void run_group_samples(GroupStore& qs, uint64_t n, uint32_t* err, cudaStream_t st) {
  if (!qs.ds.get()) return;
  for (auto const& ql : qs.levels) {
    uint32_t* const ds = qs.ds.get() ? qs.ds.as<uint32_t>() : nullptr;
    uint32_t const grid = static_cast<uint32_t>(ceil_div(ql.num_blocks, 256));
    uint4 const* const blocks = qs.blocks.as<uint4>() + ql.blk_off * 2;
    uint64_t const* const sb = qs.sb.as<uint64_t>() + ql.sb_off;
    if (ql.width == 3)
      group_samples_kernel<3><<<grid, 256, 0, st>>>(blocks, sb, n, ql, ds, err);
    else
      group_samples_kernel<2><<<grid, 256, 0, st>>>(blocks, sb, n, ql, ds, err);
    EWT_LAUNCHED();
  }
}

void upload_levels(GroupStore& qs, cudaStream_t st) {
  qs.levels_d.alloc(std::max<size_t>(qs.levels.size(), 1) * sizeof(GroupLevel));
  if (!qs.levels.empty())
    EWT_CUDA(cudaMemcpyAsync(qs.levels_d.get(), qs.levels.data(),
                             qs.levels.size() * sizeof(GroupLevel),
                             cudaMemcpyHostToDevice, st));
}

}  // namespace

std::vector<uint32_t> group_widths(uint32_t L) {
  std::vector<uint32_t> w;
  if (L < 2) return w;
  uint32_t const quads = L % 3 == 0 ? 0 : L % 3 == 2 ? 1 : 2;
  for (uint32_t i = 0; i < (L - 2 * quads) / 3; ++i) w.push_back(3);
  for (uint32_t i = 0; i < quads; ++i) w.push_back(2);
  return w;
}

GroupView GroupStore::view() const {
  GroupView v{};
  if (levels.empty() || !blocks.get()) return v;
  v.blocks = blocks.as<uint4>();
  v.sb = sb.as<uint64_t>();
  v.ds = sel_shift && ds.get() ? ds.as<uint32_t>() : nullptr;
  v.node_ranks = node_ranks.as<uint64_t>();
  v.levels = levels_d.as<GroupLevel>();
  v.num = static_cast<uint32_t>(levels.size());
  uint32_t covered = 0;
  for (auto const& ql : levels) covered += ql.width;
  v.covered = covered;
  return v;
}

bool groups_eligible(ewt_tree const& t) { return t.pow2 && t.L >= 2 && t.n >= 1; }

namespace {

// Block, superblock-table and level layout of a tree's group levels (needs n
// and L only); allocates the blocks and tables.
void layout_groups(ewt_tree& t) {
  GroupStore& qs = t.groups;
  uint64_t const n = t.n;
  std::vector<uint32_t> const widths = group_widths(t.L);
  uint64_t blk = 0, sbw = 0;
  qs.levels.assign(widths.size(), GroupLevel{});
  uint32_t l = 0;
  for (size_t j = 0; j < widths.size(); ++j) {
    uint32_t const w = widths[j];
    GroupLevel& ql = qs.levels[j];
    ql.width = w;
    ql.start = l;
    uint32_t const kD = w == 3 ? kOctDigits : kQuadDigits;
    uint32_t const kSb = w == 3 ? kOctSbBlocks : kQuadSbBlocks;
    ql.num_blocks = n / kD + 1;
    ql.blk_off = blk;
    ql.sb_off = sbw;
    blk += ql.num_blocks;
    sbw += (ceil_div(ql.num_blocks, uint64_t(kSb)) + 1) << w;  // + the totals entry
    l += w;
  }
  qs.blocks.alloc(blk * 32);
  qs.sb.alloc(sbw * 8);
}

void launch_octal_text(ewt_tree& t, void const* sym, uint32_t elem_size,
                       uint32_t* level0, bool check, uint32_t* err, cudaStream_t st,
                       size_t gi = 0) {
  GroupStore& qs = t.groups;
  GroupLevel const& ql = qs.levels[gi];
  uint32_t const sb0 = t.L - 3 - ql.start;  // bit of the digit's lowest plane
  uint64_t const n = t.n;
  uint64_t const nsb = ceil_div(ql.num_blocks, uint64_t(kOctSbBlocks));
  uint64_t* const sb = qs.sb.as<uint64_t>() + ql.sb_off;
  uint4* const blocks = qs.blocks.as<uint4>() + ql.blk_off * 2;
  uint32_t const grid = static_cast<uint32_t>(nsb);  // one CTA per superblock
  uint32_t const lanes = elem_size == 1 ? 0x01010101u : 0x00010001u;
  uint32_t const all = elem_size == 1 ? 0xFFu : 0xFFFFu;
  uint32_t const check_hi = check ? lanes * ((all << t.L) & all) : 0u;
  EWT_CUDA(cudaMemsetAsync(sb + nsb * 8, 0, 64, st));  // the totals entry
  if (elem_size == 1)
    octal_text_kernel<uint8_t><<<grid, kOctSbBlocks, 0, st>>>(
        static_cast<uint8_t const*>(sym), n, sb0, nsb, ql.num_blocks, blocks, sb, level0,
        check_hi, err);
  else
    octal_text_kernel<uint16_t><<<grid, kOctSbBlocks, 0, st>>>(
        static_cast<uint16_t const*>(sym), n, sb0, nsb, ql.num_blocks, blocks, sb, level0,
        check_hi, err);
  EWT_LAUNCHED();
}

}  // namespace

bool octal_text_eligible(ewt_tree const& t, uint32_t elem_size) {
  return groups_eligible(t) && elem_size <= 2 && group_widths(t.L).front() == 3;
}

// The routing and digit tables in device memory, uploaded once per device
// (every later build on it reads the same copy; held until exit).
template <class V>
V const* lut_on_device(std::vector<V> const& host, V* (&cache)[64]) {
  static std::mutex mu;
  int dev = 0;
  EWT_CUDA(cudaGetDevice(&dev));
  EWT_REQUIRE(dev >= 0 && dev < 64, EWT_ERR_INVALID_ARGUMENT,
              "device index out of range");
  std::lock_guard<std::mutex> lk(mu);
  if (!cache[dev]) {
    V* p = nullptr;
    EWT_CUDA(cudaMalloc(&p, host.size() * sizeof(V)));
    EWT_CUDA(cudaMemcpy(p, host.data(), host.size() * sizeof(V),
                        cudaMemcpyHostToDevice));
    cache[dev] = p;
  }
  return cache[dev];
}

uint8_t const* route_lut_on_device() {
  static std::vector<uint8_t> const lut8 = [] {
    std::vector<uint8_t> v;
    make_route_lut(v);
    return v;
  }();
  static uint8_t* cache[64] = {};
  return lut_on_device(lut8, cache);
}

uint16_t const* digit_lut_on_device() {
  static std::vector<uint16_t> const lut = [] {
    std::vector<uint16_t> v;
    make_digit_lut(v);
    return v;
  }();
  static uint16_t* cache[64] = {};
  return lut_on_device(lut, cache);
}

void build_octal_level0(ewt_tree& t, void const* sym, uint32_t elem_size,
                        uint32_t* level0, bool check, uint32_t* err, cudaStream_t st) {
  t.groups.level0_built = false;
  EWT_REQUIRE(octal_text_eligible(t, elem_size), EWT_ERR_CUDA, "octal level 0 not eligible");
  PhaseTimer pt(EWT_PHASE_FILL, st);
  layout_groups(t);
  launch_octal_text(t, sym, elem_size, level0, check, err, st);
  t.groups.level0_built = true;
}

void build_groups(ewt_tree& t, std::vector<uint64_t> const& C, void const* sym,
                uint32_t elem_size, cudaStream_t st) {
  GroupStore& qs = t.groups;
  bool const early = qs.level0_built;  // octal level 0 written with level 0
  qs.level0_built = false;
  if (!early) {
    qs.levels.clear();
    qs.blocks.reset();
  }
  if (!groups_eligible(t)) return;
  PhaseTimer pt(EWT_PHASE_QUAD, st);
  uint32_t const L = t.L;
  uint64_t const n = t.n;
  EWT_REQUIRE(C.size() == t.sigma + 1 && C[t.sigma] == n, EWT_ERR_CUDA,
              "count table inconsistent");
  if (!early) layout_groups(t);
  // host: digit totals, node ranks
  std::vector<uint64_t> nr;
  uint64_t max_info = 0;
  bool any_octal = false;
  for (auto& ql : qs.levels) {
    uint32_t const w = ql.width, S = 1u << w, l = ql.start;
    uint32_t const kSb = w == 3 ? kOctSbBlocks : kQuadSbBlocks;
    ql.nr_off = nr.size();
    max_info = std::max(max_info, ceil_div(ql.num_blocks, uint64_t(kSb)));
    bool const from_symbols = (l == 0 && (early || (sym && elem_size <= 2))) ||
                              (l > 0 && l == qs.order_level && qs.order.get());
    if (w == 3 && !from_symbols) {  // routed through a merged plane
      any_octal = true;
      max_info = std::max(max_info, ceil_div(n, kMergeSbPos));
    }
    uint32_t const sh = L - l;  // symbols under a level-l node: 2^sh
    uint64_t const nodes = uint64_t(1) << l;
    uint64_t run[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (uint64_t g = 0; g < nodes; ++g)
      for (uint32_t d = 0; d < S; ++d) {
        nr.push_back(run[d]);
        uint64_t const pre = (g << w) | d;  // prefix of l + w bits
        run[d] += C[(pre + 1) << (sh - w)] - C[pre << (sh - w)];
      }
    for (uint32_t d = 0; d < S; ++d) ql.total[d] = run[d];
  }
  std::vector<uint32_t> widths;
  for (auto const& ql : qs.levels) widths.push_back(ql.width);
  qs.node_ranks.alloc(nr.size() * 8);
  EWT_CUDA(cudaMemcpyAsync(qs.node_ranks.get(), nr.data(), nr.size() * 8,
                           cudaMemcpyHostToDevice, st));
  layout_group_samples(qs, qs.sel_shift);
  upload_levels(qs, st);
  DevBuf plane, err_d(4);
  EWT_CUDA(cudaMemsetAsync(err_d.get(), 0, 4, st));
  uint64_t plane_words = 0;
  uint8_t const* lut8_d = nullptr;
  uint16_t const* lut_d = nullptr;
  if (any_octal) {
    lut8_d = route_lut_on_device();
    plane_words = ceil_div(n, 64) * 2 + 16;  // slack for the 64-bit reads
    plane.alloc(plane_words * 4);
    set_smem_limit(merge_plane_kernel, 65536);
    set_smem_limit(octal_level_kernel, 65536);
  }
  if (widths.back() == 2) {
    lut_d = digit_lut_on_device();
    set_smem_limit(quad_level_kernel, 65536 * 2);
  }
  DevBuf chunk(ceil_div(max_info + 1, kScanChunk) * 8 * 8);
  DevBuf info(std::max<uint64_t>(max_info, 1) * sizeof(SbStart));
  TreeView const& v = t.view;
  uint32_t* const words = t.rs.words.as<uint32_t>();
  uint64_t const total_words = t.rs.total_words;
  uint32_t const sms = static_cast<uint32_t>(sm_count());
  for (size_t gi = 0; gi < qs.levels.size(); ++gi) {
    GroupLevel const& ql = qs.levels[gi];
    uint32_t const lv = ql.start;
    ArrayMeta const& m0 = t.rs.meta[lv];
    ArrayMeta const& m1 = t.rs.meta[lv + 1];
    uint64_t* const sb = qs.sb.as<uint64_t>() + ql.sb_off;
    uint4* const blocks = qs.blocks.as<uint4>() + ql.blk_off * 2;
    if (ql.width == 2) {
      uint64_t const nsb = ceil_div(ql.num_blocks, uint64_t(kQuadSbBlocks));
      quad_sb_count_kernel<<<static_cast<uint32_t>(ceil_div(nsb + 1, 128)), 128, 0, st>>>(
          v, lv, nsb, sb, info.as<SbStart>());
      EWT_LAUNCHED();
      scan_superblocks<4>(sb, nsb + 1, chunk, st);
      uint32_t const grid =
          static_cast<uint32_t>(std::min<uint64_t>(ceil_div(nsb, 2), uint64_t(sms)));
      quad_level_kernel<<<grid, 1024, 65536 * 2, st>>>(
          v, lv, ql, words + m0.word_off, ceil_div(n, 32), words + m1.word_off,
          total_words - m1.word_off, lut_d, blocks, sb,
          info.as<SbStart>(), nsb, qs.ds.get() ? qs.ds.as<uint32_t>() : nullptr,
          err_d.as<uint32_t>());
      EWT_LAUNCHED();
      continue;
    }
    uint64_t const nsb = ceil_div(ql.num_blocks, uint64_t(kOctSbBlocks));
    uint32_t const grid_o =
        static_cast<uint32_t>(std::min<uint64_t>(ceil_div(nsb, 2), uint64_t(sms)));
    if (lv == 0 && (early || (sym && elem_size <= 2))) {  // from the symbols
      if (!early) launch_octal_text(t, sym, elem_size, nullptr, false, nullptr, st);
      scan_superblocks<8>(sb, nsb + 1, chunk, st);
      continue;
    }
    if (lv == qs.order_level && qs.order.get()) {  // from the level-lv order
      launch_octal_text(t, qs.order.get(), elem_size, nullptr, false, nullptr, st, gi);
      scan_superblocks<8>(sb, nsb + 1, chunk, st);
      continue;
    }
    // octal: level lv+2 routed into level-(lv+1) order first
    ArrayMeta const& m2 = t.rs.meta[lv + 2];
    uint64_t const nsb_m = ceil_div(n, kMergeSbPos);
    sb_info_kernel<<<static_cast<uint32_t>(ceil_div(nsb_m, 128)), 128, 0, st>>>(
        v, lv + 1, kMergeSbPos, nsb_m, info.as<SbStart>());
    EWT_LAUNCHED();
    merge_plane_kernel<<<static_cast<uint32_t>(
                             std::min<uint64_t>(ceil_div(nsb_m, 2), uint64_t(sms))),
                         1024, 65536, st>>>(
        v, lv + 1, words + m1.word_off, words + m2.word_off, total_words - m2.word_off,
        lut8_d, info.as<SbStart>(), nsb_m, plane.as<uint32_t>(),
        err_d.as<uint32_t>());
    EWT_LAUNCHED();
    sb_info_kernel<<<static_cast<uint32_t>(ceil_div(nsb, 128)), 128, 0, st>>>(
        v, lv, kOctSbDigits, nsb, info.as<SbStart>());
    EWT_LAUNCHED();
    EWT_CUDA(cudaMemsetAsync(sb + nsb * 8, 0, 64, st));  // the totals entry
    octal_level_kernel<<<grid_o, 1024, 65536, st>>>(
        v, lv, words + m0.word_off, words + m1.word_off, total_words - m1.word_off,
        plane.as<uint32_t>(), plane_words, lut8_d, info.as<SbStart>(), nsb,
        ql.num_blocks, blocks, sb, err_d.as<uint32_t>());
    EWT_LAUNCHED();
    scan_superblocks<8>(sb, nsb + 1, chunk, st);
  }
  // octal samples (quad levels wrote theirs) and every level's totals check
  for (auto const& ql : qs.levels) {
    uint32_t* const ds = ql.width == 3 && qs.ds.get() ? qs.ds.as<uint32_t>() : nullptr;
    uint32_t const grid =
        ds ? static_cast<uint32_t>(ceil_div(ql.num_blocks, 256)) : 1u;
    uint4 const* const blocks = qs.blocks.as<uint4>() + ql.blk_off * 2;
    uint64_t const* const sb = qs.sb.as<uint64_t>() + ql.sb_off;
    if (ql.width == 3)
      group_samples_kernel<3><<<grid, 256, 0, st>>>(blocks, sb, n, ql, ds,
                                                    err_d.as<uint32_t>());
    else
      group_samples_kernel<2><<<grid, 256, 0, st>>>(blocks, sb, n, ql, ds,
                                                    err_d.as<uint32_t>());
    EWT_LAUNCHED();
  }
  uint32_t bad = 0;
  EWT_CUDA(cudaMemcpyAsync(&bad, err_d.get(), 4, cudaMemcpyDeviceToHost, st));
  EWT_CUDA(cudaStreamSynchronize(st));
  qs.order.reset();
  qs.order_level = 0;
  EWT_REQUIRE(bad == 0, EWT_ERR_CUDA,
              "internal consistency check failed (group levels, kind " +
                  std::to_string(bad) + ")");
}

void set_select_rate(ewt_tree& t, uint32_t shift, cudaStream_t st) {
  build_dense_samples(t.rs, shift, st);
  build_group_samples(t, shift, st);
  t.view.rs = t.rs.view();
  t.view.groups = t.groups.view();
}

void build_group_samples(ewt_tree& t, uint32_t shift, cudaStream_t st) {
  GroupStore& qs = t.groups;
  if (qs.levels.empty()) return;
  EWT_CUDA(cudaStreamSynchronize(st));  // no query may read the old samples
  layout_group_samples(qs, shift);
  upload_levels(qs, st);
  run_group_samples(qs, t.n, nullptr, st);
  EWT_CUDA(cudaStreamSynchronize(st));
}

}  // namespace ewt
