// Quad (4-ary) query levels of power-of-two trees: every pair of binary
// levels (2j, 2j+1) becomes one level of 2-bit digits in level-2j order, so
// a query resolves two binary levels per dependent DRAM access.  No
// reference counterpart; the binary levels and their RankSelect stay the
// source of truth for exports and are walked for an odd last level.
//
// A level-2j node's zeros go, in order, to its left child on level 2j+1 and
// its ones to its right child, so the low bits of a run of positions inside
// one node are two runs of level 2j+1, merged by the high bits.  Per quad
// level:
//   1. quad_sb_count_kernel (thread per 512-block superblock): its digit
//      counts from six ranks per node segment (no per-position work);
//   2. quad_scan_*: counts before every superblock (chunked scan);
//   3. quad_level_kernel (persistent, two superblocks per 1024-thread CTA,
//      one thread per 96-digit block): digits from the two runs, eight at a
//      time through a 64K-entry table in shared memory, block headers from
//      a scan, blocks and dense select samples written; the superblock's
//      totals are checked against pass 1.
// Node ranks (digit counts before every node) and digit totals come from
// the count table on the host.
#include <algorithm>
#include <vector>

#include "internal.cuh"

namespace ewt {

using ecl::detail::kQuadDigits;
using ecl::detail::kQuadSbBlocks;
using ecl::detail::kQuadSbDigits;
using ecl::detail::QuadLevel;
using ecl::detail::QuadView;

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

// Pass 1: digit counts of every superblock (thread per superblock).
__global__ void __launch_bounds__(128)
quad_sb_count_kernel(TreeView v, uint32_t j, uint64_t nsb,
                     uint64_t* __restrict__ sb, SbStart* __restrict__ info) {
  uint64_t const s = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (s > nsb) return;
  uint64_t c[4] = {0, 0, 0, 0};
  uint64_t const n = v.n;
  uint64_t a = s * kQuadSbDigits;
  uint64_t const e = min(n, a + kQuadSbDigits);
  if (s < nsb && a >= e) info[s] = SbStart{QuadNode{0, n, 0, 0}, 0, 1};
  if (s < nsb && a < e) {
    uint32_t const l = 2 * j, sh = v.levels - l;
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

// Pass 2a: per chunk of kScanChunk superblock entries, the four sums.
__global__ void __launch_bounds__(256)
quad_scan_partial_kernel(uint64_t const* __restrict__ sb, uint64_t count,
                         uint64_t* __restrict__ chunk) {
  uint64_t const first = uint64_t(blockIdx.x) * kScanChunk;
  uint64_t c[4] = {0, 0, 0, 0};
  for (uint64_t i = first + threadIdx.x; i < min(count, first + kScanChunk);
       i += blockDim.x)
    for (uint32_t d = 0; d < 4; ++d) c[d] += sb[i * 4 + d];
  for (uint32_t d = 0; d < 4; ++d) {
    uint64_t tot = 0;
    cta_exclusive_scan(c[d], &tot);
    if (threadIdx.x == 0) chunk[blockIdx.x * 4 + d] = tot;
  }
}

// Pass 2b: exclusive prefix of the chunk sums (one thread per digit).
__global__ void quad_scan_chunks_kernel(uint64_t* __restrict__ chunk,
                                        uint64_t chunks) {
  uint32_t const d = threadIdx.x;
  if (d >= 4) return;
  uint64_t run = 0;
  for (uint64_t i = 0; i < chunks; ++i) {
    uint64_t const x = chunk[i * 4 + d];
    chunk[i * 4 + d] = run;
    run += x;
  }
}

// Pass 2c: exclusive prefix of every entry, in place (1024 threads; two
// digits packed per 64-bit scan: a round's sums stay below 2^32).
__global__ void __launch_bounds__(1024)
quad_scan_apply_kernel(uint64_t* __restrict__ sb, uint64_t count,
                       uint64_t const* __restrict__ chunk) {
  uint64_t const first = uint64_t(blockIdx.x) * kScanChunk;
  uint64_t const end = min(count, first + kScanChunk);
  uint64_t carry[4];
  for (uint32_t d = 0; d < 4; ++d) carry[d] = chunk ? chunk[blockIdx.x * 4 + d] : 0;
  for (uint64_t base = first; base < end; base += blockDim.x) {
    uint64_t const i = base + threadIdx.x;
    bool const in = i < end;
    uint4 const a = in ? reinterpret_cast<uint4 const*>(sb)[i * 2] : make_uint4(0, 0, 0, 0);
    uint4 const b = in ? reinterpret_cast<uint4 const*>(sb)[i * 2 + 1] : make_uint4(0, 0, 0, 0);
    // per entry each digit count is below 2^16 (49,152 digits per superblock)
    uint64_t tot01 = 0, tot23 = 0;
    uint64_t const e01 = cta_exclusive_scan(uint64_t(a.x) | (uint64_t(a.z) << 32), &tot01);
    uint64_t const e23 = cta_exclusive_scan(uint64_t(b.x) | (uint64_t(b.z) << 32), &tot23);
    if (in) {
      uint64_t* o = sb + i * 4;
      o[0] = carry[0] + (e01 & 0xFFFFFFFFu);
      o[1] = carry[1] + (e01 >> 32);
      o[2] = carry[2] + (e23 & 0xFFFFFFFFu);
      o[3] = carry[3] + (e23 >> 32);
    }
    carry[0] += tot01 & 0xFFFFFFFFu;
    carry[1] += tot01 >> 32;
    carry[2] += tot23 & 0xFFFFFFFFu;
    carry[3] += tot23 >> 32;
  }
}

// Dense samples of one block: entry k of digit d names the block holding
// its (k * 2^sh + 1)-th occurrence; before/c = occurrences before / in it.
__device__ __forceinline__ void put_quad_samples(uint32_t* __restrict__ ds,
                                                 QuadLevel const& ql, uint32_t sh,
                                                 uint64_t blk,
                                                 uint64_t const before[4],
                                                 uint32_t const c[4]) {
  uint64_t const R = uint64_t(1) << sh;
#pragma unroll
  for (uint32_t d = 0; d < 4; ++d) {
    if (c[d] == 0) continue;
    // entries fit in 32 bits (at most n / 32 of them)
    uint32_t const entries = static_cast<uint32_t>((ql.total[d] + R - 1) >> sh);
    uint32_t const last =
        min(static_cast<uint32_t>((before[d] + c[d] - 1) >> sh), entries - 1);
    uint32_t* S = ds + ql.ds_off[d];
    for (uint32_t k = static_cast<uint32_t>((before[d] + R - 1) >> sh); k <= last; ++k)
      S[k] = static_cast<uint32_t>(blk);
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
quad_level_kernel(TreeView v, uint32_t j, QuadLevel ql,
                  uint32_t const* __restrict__ hi_w, uint64_t hi_words,
                  uint32_t const* __restrict__ lo_w, uint64_t lo_limit,
                  uint16_t const* __restrict__ lut_g,
                  uint4* __restrict__ blocks, uint64_t const* __restrict__ sb,
                  SbStart const* __restrict__ info, uint64_t nsb,
                  uint32_t* __restrict__ ds, uint32_t sel_shift,
                  uint32_t* __restrict__ err) {
  extern __shared__ __align__(16) uint16_t lut[];
  {
    uint4 const* src = reinterpret_cast<uint4 const*>(lut_g);
    uint4* dst = reinterpret_cast<uint4*>(lut);
    for (uint32_t i = threadIdx.x; i < 65536 * 2 / 16; i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  uint64_t const n = v.n;
  uint32_t const l = 2 * j, sh = v.levels - l;
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
    // ones of level 2j in the superblock before this block (= its digits 2
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
    if (ds) {
      uint32_t const vb = static_cast<uint32_t>(min(uint64_t(kQuadDigits), n - p));
      uint32_t const c[4] = {vb - ones - c1, c1, ones - c3, c3};
      uint64_t const before[4] = {sbe[0] + h0, sbe[1] + h1, sbe[2] + h2, sbe[3] + h3};
      put_quad_samples(ds, ql, sel_shift, blk, before, c);
    }
  }
}

// Dense samples of one quad level from its finished blocks (rate changes).
__global__ void __launch_bounds__(256)
quad_samples_kernel(uint4 const* __restrict__ blocks,
                    uint64_t const* __restrict__ sb, uint64_t n, QuadLevel ql,
                    uint32_t* __restrict__ ds, uint32_t sh) {
  uint64_t const b = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (b >= ql.num_blocks) return;
  uint4 const x = blocks[b * 2], y = blocks[b * 2 + 1];
  uint64_t q[4];
  ecl::detail::quad_words(x, y, q);
  uint64_t const first = b * kQuadDigits;
  uint32_t const valid =
      first < n ? static_cast<uint32_t>(min(uint64_t(kQuadDigits), n - first)) : 0u;
  uint64_t const* sbv = sb + (b / kQuadSbBlocks) * 4;
  uint64_t before[4];
  uint32_t c[4];
#pragma unroll
  for (uint32_t d = 0; d < 4; ++d) {
    c[d] = ecl::detail::quad_count(q, d, valid);
    before[d] = ecl::detail::quad_before(q[0], sbv[d], d, b);
  }
  put_quad_samples(ds, ql, sh, b, before, c);
}

// Lays out the dense samples of every quad level at rate 2^shift.
void layout_quad_samples(QuadStore& qs, uint32_t shift) {
  qs.ds.reset();
  qs.sel_shift = shift;
  if (shift == 0) return;
  uint64_t total = 0;
  for (auto& ql : qs.levels)
    for (uint32_t d = 0; d < 4; ++d) {
      ql.ds_off[d] = total;
      total += ceil_div(ql.total[d], uint64_t(1) << shift);
    }
  qs.ds.alloc(std::max<uint64_t>(total, 1) * 4);
}

void run_quad_samples(QuadStore& qs, uint64_t n, cudaStream_t st) {
  if (!qs.ds.get() || qs.sel_shift == 0) return;
  for (auto const& ql : qs.levels) {
    quad_samples_kernel<<<static_cast<uint32_t>(ceil_div(ql.num_blocks, 256)), 256, 0,
                          st>>>(qs.blocks.as<uint4>() + ql.blk_off * 2,
                                qs.sb.as<uint64_t>() + ql.sb_off * 4, n, ql,
                                qs.ds.as<uint32_t>(), qs.sel_shift);
    EWT_LAUNCHED();
  }
}

void upload_levels(QuadStore& qs, cudaStream_t st) {
  qs.levels_d.alloc(std::max<size_t>(qs.levels.size(), 1) * sizeof(QuadLevel));
  if (!qs.levels.empty())
    EWT_CUDA(cudaMemcpyAsync(qs.levels_d.get(), qs.levels.data(),
                             qs.levels.size() * sizeof(QuadLevel),
                             cudaMemcpyHostToDevice, st));
}

}  // namespace

QuadView QuadStore::view() const {
  QuadView v{};
  if (levels.empty() || !blocks.get()) return v;
  v.blocks = blocks.as<uint4>();
  v.sb = sb.as<uint64_t>();
  v.ds = sel_shift && ds.get() ? ds.as<uint32_t>() : nullptr;
  v.node_ranks = node_ranks.as<uint64_t>();
  v.levels = levels_d.as<QuadLevel>();
  v.num = static_cast<uint32_t>(levels.size());
  v.sel_shift = v.ds ? sel_shift : 0;
  return v;
}

bool quad_eligible(ewt_tree const& t) { return t.pow2 && t.L >= 2 && t.n >= 1; }

void build_quad(ewt_tree& t, std::vector<uint64_t> const& C, cudaStream_t st) {
  QuadStore& qs = t.quad;
  qs.levels.clear();
  qs.blocks.reset();
  if (!quad_eligible(t)) return;
  PhaseTimer pt(EWT_PHASE_QUAD, st);
  uint32_t const L = t.L, QL = L / 2;
  uint64_t const n = t.n;
  EWT_REQUIRE(C.size() == t.sigma + 1 && C[t.sigma] == n, EWT_ERR_CUDA,
              "count table inconsistent");
  // host: layout, digit totals, node ranks
  std::vector<uint64_t> nr;
  uint64_t blk = 0, sbs = 0;
  qs.levels.resize(QL);
  for (uint32_t j = 0; j < QL; ++j) {
    QuadLevel& ql = qs.levels[j];
    ql = QuadLevel{};
    ql.num_blocks = n / kQuadDigits + 1;
    ql.blk_off = blk;
    ql.sb_off = sbs;
    ql.nr_off = nr.size();
    blk += ql.num_blocks;
    sbs += ceil_div(ql.num_blocks, kQuadSbBlocks) + 1;  // + the totals entry
    uint32_t const sh = L - 2 * j;  // symbols under a level-2j node: 2^sh
    uint64_t const nodes = uint64_t(1) << (2 * j);
    uint64_t run[4] = {0, 0, 0, 0};
    for (uint64_t g = 0; g < nodes; ++g)
      for (uint32_t d = 0; d < 4; ++d) {
        nr.push_back(run[d]);
        uint64_t const pre = (g << 2) | d;  // prefix of 2j + 2 bits
        run[d] += C[(pre + 1) << (sh - 2)] - C[pre << (sh - 2)];
      }
    for (uint32_t d = 0; d < 4; ++d) ql.total[d] = run[d];
  }
  qs.blocks.alloc(blk * 32);
  qs.sb.alloc(sbs * 32);
  qs.node_ranks.alloc(nr.size() * 8);
  EWT_CUDA(cudaMemcpyAsync(qs.node_ranks.get(), nr.data(), nr.size() * 8,
                           cudaMemcpyHostToDevice, st));
  layout_quad_samples(qs, qs.sel_shift);
  upload_levels(qs, st);
  static std::vector<uint16_t> const lut = [] {
    std::vector<uint16_t> v;
    make_digit_lut(v);
    return v;
  }();
  DevBuf lut_d(lut.size() * 2), err_d(4);
  EWT_CUDA(cudaMemcpyAsync(lut_d.get(), lut.data(), lut.size() * 2,
                           cudaMemcpyHostToDevice, st));
  EWT_CUDA(cudaMemsetAsync(err_d.get(), 0, 4, st));
  set_smem_limit(quad_level_kernel, 65536 * 2);
  uint64_t const max_nsb = ceil_div(n / kQuadDigits + 1, kQuadSbBlocks);
  DevBuf chunk(ceil_div(max_nsb + 1, kScanChunk) * 32);
  DevBuf info(max_nsb * sizeof(SbStart));
  TreeView const& v = t.view;
  uint32_t* const words = t.rs.words.as<uint32_t>();
  for (uint32_t j = 0; j < QL; ++j) {
    QuadLevel const& ql = qs.levels[j];
    ArrayMeta const& mh = t.rs.meta[2 * j];
    ArrayMeta const& ml = t.rs.meta[2 * j + 1];
    uint64_t const nsb = ceil_div(ql.num_blocks, kQuadSbBlocks);
    uint64_t* const sb = qs.sb.as<uint64_t>() + ql.sb_off * 4;
    quad_sb_count_kernel<<<static_cast<uint32_t>(ceil_div(nsb + 1, 128)), 128, 0, st>>>(
        v, j, nsb, sb, info.as<SbStart>());
    EWT_LAUNCHED();
    uint64_t const chunks = ceil_div(nsb + 1, kScanChunk);
    if (chunks > 1) {
      quad_scan_partial_kernel<<<static_cast<uint32_t>(chunks), 256, 0, st>>>(
          sb, nsb + 1, chunk.as<uint64_t>());
      EWT_LAUNCHED();
      quad_scan_chunks_kernel<<<1, 32, 0, st>>>(chunk.as<uint64_t>(), chunks);
      EWT_LAUNCHED();
    }
    quad_scan_apply_kernel<<<static_cast<uint32_t>(chunks), 1024, 0, st>>>(
        sb, nsb + 1, chunks > 1 ? chunk.as<uint64_t>() : nullptr);
    EWT_LAUNCHED();
    uint32_t const grid = static_cast<uint32_t>(
        std::min<uint64_t>(ceil_div(nsb, 2), uint64_t(sm_count())));
    quad_level_kernel<<<grid, 1024, 65536 * 2, st>>>(
        v, j, ql, words + mh.word_off, ceil_div(n, 32), words + ml.word_off,
        t.rs.total_words - ml.word_off, lut_d.as<uint16_t>(),
        qs.blocks.as<uint4>() + ql.blk_off * 2, sb, info.as<SbStart>(), nsb,
        qs.ds.get() ? qs.ds.as<uint32_t>() : nullptr, qs.sel_shift,
        err_d.as<uint32_t>());
    EWT_LAUNCHED();
  }
  uint32_t bad = 0;
  EWT_CUDA(cudaMemcpyAsync(&bad, err_d.get(), 4, cudaMemcpyDeviceToHost, st));
  EWT_CUDA(cudaStreamSynchronize(st));
  EWT_REQUIRE(bad == 0, EWT_ERR_CUDA,
              "internal consistency check failed (quad levels, kind " +
                  std::to_string(bad) + ")");
}

void set_select_rate(ewt_tree& t, uint32_t shift, cudaStream_t st) {
  build_dense_samples(t.rs, shift, st);
  build_quad_samples(t, shift, st);
  t.view.rs = t.rs.view();
  t.view.quad = t.quad.view();
}

void build_quad_samples(ewt_tree& t, uint32_t shift, cudaStream_t st) {
  QuadStore& qs = t.quad;
  if (qs.levels.empty()) return;
  EWT_CUDA(cudaStreamSynchronize(st));  // no query may read the old samples
  layout_quad_samples(qs, shift);
  upload_levels(qs, st);
  run_quad_samples(qs, t.n, st);
  EWT_CUDA(cudaStreamSynchronize(st));
}

}  // namespace ewt
