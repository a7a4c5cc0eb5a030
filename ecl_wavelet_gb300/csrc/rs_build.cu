// RankSelect construction for a group of packed bit arrays.
//
// Produces the reference's format (src/bitarray/rank_select.cu:50-304):
//   L2[k]  = ones in [start of k's L1 block, start of k)      (uint16)
//   L1[j]  = ones in [0, j * 65536)                           (uint64)
//   ones   = total ones
//   s1[k]  = position of the (k+1)*4096-th one, s0 likewise for zeros.
// Kernels: one CTA per 65,536-bit L1 block counts its 128 L2 blocks with
// 128-bit coalesced loads and a CTA scan; one CTA per array scans the L1
// block totals; one thread per 512-bit block emits the (at most one) one-
// and zero-sample that falls inside it.  No kernel waits on another CTA.
#include <algorithm>

#include "internal.cuh"

namespace ewt {

using ecl::detail::kL1Bits;
using ecl::detail::kL2Bits;
using ecl::detail::kL2PerL1;
using ecl::detail::kL2Words;
using ecl::detail::kSampleRate;

struct BlockJob {
  uint64_t word_off, bits, l2_off, l1_off, num_l1, num_last_l2;
};

void RSStore::layout(std::vector<uint64_t> const& bits) {
  meta.assign(bits.size(), ArrayMeta{});
  total_words = total_l1 = total_l2 = 0;
  for (size_t a = 0; a < bits.size(); ++a) {
    ArrayMeta& m = meta[a];
    m.bits = bits[a];
    uint64_t const w = ceil_div(bits[a], 32);
    m.word_off = total_words;
    total_words += ceil_div(w, 32) * 32;  // 128-byte padding per array
    m.num_l1 = std::max<uint64_t>(1, ceil_div(bits[a], kL1Bits));
    m.num_last_l2 = ceil_div(bits[a] % kL1Bits, kL2Bits);
    if (m.num_last_l2 == 0) m.num_last_l2 = kL2PerL1;
    m.l1_off = total_l1;
    m.l2_off = total_l2;
    total_l1 += m.num_l1;
    total_l2 += (m.num_l1 - 1) * kL2PerL1 + m.num_last_l2;
  }
  total_words += total_words % 2;
  // 16 words of slack: readers may fetch one word past an array's end
  words.alloc(total_words * 4 + 64);
  l1.alloc(total_l1 * 8);
  l2.alloc(total_l2 * 2);
  meta_d.alloc(meta.size() * sizeof(ArrayMeta));
  cudaStream_t const st = alloc_stream();
  EWT_CUDA(cudaMemcpyAsync(meta_d.get(), meta.data(),
                           meta.size() * sizeof(ArrayMeta),
                           cudaMemcpyHostToDevice, st));
  std::vector<BlockJob> jobs(meta.size());
  for (size_t a = 0; a < meta.size(); ++a)
    jobs[a] = {meta[a].word_off, meta[a].bits, meta[a].l2_off, meta[a].l1_off,
               meta[a].num_l1, meta[a].num_last_l2};
  jobs_d.alloc(jobs.size() * sizeof(BlockJob));
  EWT_CUDA(cudaMemcpyAsync(jobs_d.get(), jobs.data(),
                           jobs.size() * sizeof(BlockJob),
                           cudaMemcpyHostToDevice, st));
  // Zero the padding words behind every array (the arrays themselves are
  // written completely by their producer).
  for (auto const& m : meta) {
    uint64_t const w = ceil_div(m.bits, 32);
    uint64_t const padded = ceil_div(w, 32) * 32;
    if (padded > w)
      EWT_CUDA(cudaMemsetAsync(words.as<uint32_t>() + m.word_off + w, 0,
                               (padded - w) * 4, st));
  }
  if (total_words > 0 && total_words % 32)  // the even-rounding word
    EWT_CUDA(cudaMemsetAsync(words.as<uint32_t>() + total_words - 1, 0, 4, st));
}

RSView RSStore::view() const {
  RSView v{};
  v.words = words.as<uint32_t>();
  v.l1 = l1.as<uint64_t>();
  v.l2 = l2.as<uint16_t>();
  v.s0 = s0.as<uint64_t>();
  v.s1 = s1.as<uint64_t>();
  v.meta = meta_d.as<ArrayMeta>();
  v.rb = rb.get() ? rb.as<uint4>() : nullptr;
  if (v.rb && !meta.empty()) {  // the high-count table follows the blocks
    std::vector<uint64_t> start;
    uint64_t const blocks = rank_block_starts(meta, start);
    v.rbh = reinterpret_cast<uint64_t const*>(rb.as<unsigned char>() + blocks * 32);
  }
  if (v.rb && ds.get()) {
    v.ds = ds.as<uint32_t>();
    v.sel_shift = sel_shift;
  }
  v.num_arrays = static_cast<uint32_t>(meta.size());
  return v;
}

namespace {

// Finds the array owning global L1 block g among jobs[0..count).
__device__ __forceinline__ uint32_t find_job(BlockJob const* jobs,
                                             uint32_t count, uint64_t g) {
  uint32_t lo = 0, hi = count - 1;
  while (lo < hi) {
    uint32_t const mid = (lo + hi + 1) >> 1;
    if (jobs[mid].l1_off <= g) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// One CTA of 128 threads per L1 block; thread k owns L2 block k.
__global__ void __launch_bounds__(128)
rs_block_kernel(uint32_t const* __restrict__ words, BlockJob const* jobs,
                uint32_t num_jobs, uint64_t l1_base,
                uint16_t* __restrict__ l2, uint64_t* __restrict__ l1) {
  uint64_t const g = l1_base + blockIdx.x;
  uint32_t const j = find_job(jobs, num_jobs, g);
  BlockJob const job = jobs[j];
  uint64_t const b = g - job.l1_off;
  uint32_t const k = threadIdx.x;
  uint64_t const nblk = (b + 1 == job.num_l1) ? job.num_last_l2 : kL2PerL1;
  uint32_t cnt = 0;
  if (k < nblk) {
    uint64_t const kb = b * kL2PerL1 + k;  // L2 block inside the array
    uint64_t const bit0 = kb * kL2Bits;
    uint64_t const valid = min(job.bits - bit0, kL2Bits);
    uint4 const* p = reinterpret_cast<uint4 const*>(words + job.word_off +
                                                    kb * kL2Words);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      uint4 v = p[q];
      uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        uint32_t const lo = (q * 4 + t) * 32;
        uint32_t x = w[t];
        if (lo >= valid) x = 0;
        else if (valid - lo < 32) x &= (1u << (valid - lo)) - 1u;
        cnt += __popc(x);
      }
    }
  }
  // CTA exclusive scan of 128 counts.
  __shared__ uint32_t warp_tot[4];
  uint32_t const lane = k & 31, wid = k >> 5;
  uint32_t inc = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t const y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) warp_tot[wid] = inc;
  __syncthreads();
  uint32_t base = 0;
  for (uint32_t w = 0; w < wid; ++w) base += warp_tot[w];
  uint32_t const excl = base + inc - cnt;
  if (k < nblk) l2[job.l2_off + b * kL2PerL1 + k] = static_cast<uint16_t>(excl);
  if (k == 127) l1[job.l1_off + b] = base + inc;  // block total for now
}

// One CTA per array: in-place exclusive scan of the L1 block totals; the
// grand total goes straight into the array's device meta entry.
__global__ void __launch_bounds__(1024)
rs_l1_scan_kernel(BlockJob const* jobs, uint32_t first_array,
                  uint64_t* __restrict__ l1, ArrayMeta* __restrict__ meta) {
  BlockJob const job = jobs[blockIdx.x];
  uint64_t* p = l1 + job.l1_off;
  __shared__ uint64_t warp_tot[32];
  __shared__ uint64_t carry_s;
  uint32_t const t = threadIdx.x, lane = t & 31, wid = t >> 5;
  if (t == 0) carry_s = 0;
  __syncthreads();
  for (uint64_t base = 0; base < job.num_l1; base += blockDim.x) {
    uint64_t const i = base + t;
    uint64_t const v = i < job.num_l1 ? p[i] : 0;
    uint64_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint64_t const y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    if (lane == 31) warp_tot[wid] = inc;
    __syncthreads();
    uint64_t wb = 0;
    for (uint32_t w = 0; w < wid; ++w) wb += warp_tot[w];
    uint64_t const carry = carry_s;
    if (i < job.num_l1) p[i] = carry + wb + inc - v;
    __syncthreads();
    if (t == blockDim.x - 1) carry_s = carry + wb + inc;
    __syncthreads();
  }
  if (t == 0) meta[first_array + blockIdx.x].ones = carry_s;
}

struct SampleJob {
  uint64_t word_off, bits, l1_off, l2_off, num_l1, num_l2, ones, s0_off,
      s1_off;
};

__device__ __forceinline__ uint32_t find_sjob(SampleJob const* jobs,
                                              uint32_t count, uint64_t g) {
  uint32_t lo = 0, hi = count - 1;
  while (lo < hi) {
    uint32_t const mid = (lo + hi + 1) >> 1;
    if (jobs[mid].l2_off <= g) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Position inside the 512-bit block of the r-th (1-based) `value` bit.
__device__ __forceinline__ uint32_t select_in_block(uint32_t const* blk,
                                                    uint32_t r, int value) {
  for (uint32_t w = 0; w < kL2Words; ++w) {
    uint32_t const x = value ? blk[w] : ~blk[w];
    uint32_t const c = __popc(x);
    if (r <= c) return w * 32 + ecl::detail::select_in_word(x, r);
    r -= c;
  }
  return kL2Bits;  // not reached
}

// One thread per L2 block of every array.
__global__ void __launch_bounds__(256)
rs_samples_kernel(uint32_t const* __restrict__ words,
                  uint64_t const* __restrict__ l1,
                  uint16_t const* __restrict__ l2, SampleJob const* jobs,
                  uint32_t num_jobs, uint64_t total_l2,
                  uint64_t* __restrict__ s0, uint64_t* __restrict__ s1) {
  uint64_t const g = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (g >= total_l2) return;
  SampleJob const job = jobs[find_sjob(jobs, num_jobs, g)];
  uint64_t const k = g - job.l2_off;  // L2 block inside the array
  uint64_t const b = k / kL2PerL1;
  uint64_t const l1v = l1[job.l1_off + b];
  uint64_t const before1 = l1v + l2[g];
  uint64_t after1;
  if ((k + 1) % kL2PerL1 != 0 && k + 1 < job.num_l2)
    after1 = l1v + l2[g + 1];
  else if (b + 1 < job.num_l1)
    after1 = l1[job.l1_off + b + 1];
  else
    after1 = job.ones;
  uint64_t const bit0 = k * kL2Bits;
  uint64_t const nbits = min(job.bits - bit0, kL2Bits);
  uint64_t const before0 = bit0 - before1;
  uint64_t const after0 = bit0 + nbits - after1;
  uint32_t const* blk = words + job.word_off + k * kL2Words;
  uint64_t const t1 = (before1 / kSampleRate + 1) * kSampleRate;
  if (t1 <= after1)
    s1[job.s1_off + t1 / kSampleRate - 1] =
        bit0 + select_in_block(blk, static_cast<uint32_t>(t1 - before1), 1);
  uint64_t const t0 = (before0 / kSampleRate + 1) * kSampleRate;
  if (t0 <= after0)
    s0[job.s0_off + t0 / kSampleRate - 1] =
        bit0 + select_in_block(blk, static_cast<uint32_t>(t0 - before0), 0);
}

}  // namespace

void build_rs_counts(RSStore& rs, uint32_t first, uint32_t last,
                     cudaStream_t stream) {
  if (first >= last) return;
  uint32_t const count = last - first;
  BlockJob const* jobs = rs.jobs_d.as<BlockJob>() + first;
  PhaseTimer pt(EWT_PHASE_RS_COUNTS, stream);
  uint64_t const l1_first = rs.meta[first].l1_off;
  uint64_t const l1_end = rs.meta[last - 1].l1_off + rs.meta[last - 1].num_l1;
  for (uint64_t base = l1_first; base < l1_end; base += (1u << 30)) {
    uint64_t const nb = std::min<uint64_t>(l1_end - base, 1u << 30);
    rs_block_kernel<<<static_cast<uint32_t>(nb), 128, 0, stream>>>(
        rs.words.as<uint32_t>(), jobs, count, base, rs.l2.as<uint16_t>(),
        rs.l1.as<uint64_t>());
    EWT_LAUNCHED();
  }
  rs_l1_scan_kernel<<<count, 1024, 0, stream>>>(
      jobs, first, rs.l1.as<uint64_t>(), rs.meta_d.as<ArrayMeta>());
  EWT_LAUNCHED();
}

void build_rs_samples(RSStore& rs, cudaStream_t stream) {
  uint32_t const count = static_cast<uint32_t>(rs.meta.size());
  // Totals of ones were written on the device by the L1 scans.
  std::vector<ArrayMeta> dm(count);
  EWT_CUDA(cudaMemcpyAsync(dm.data(), rs.meta_d.get(), count * sizeof(ArrayMeta),
                           cudaMemcpyDeviceToHost, stream));
  EWT_CUDA(cudaStreamSynchronize(stream));
  for (uint32_t a = 0; a < count; ++a) rs.meta[a].ones = dm[a].ones;
  rs.total_s0 = rs.total_s1 = 0;
  for (auto& m : rs.meta) {
    m.s1_off = rs.total_s1;
    m.s0_off = rs.total_s0;
    rs.total_s1 += m.ones / kSampleRate;
    rs.total_s0 += (m.bits - m.ones) / kSampleRate;
  }
  rs.s0.alloc(rs.total_s0 * 8);
  rs.s1.alloc(rs.total_s1 * 8);
  EWT_CUDA(cudaMemcpyAsync(rs.meta_d.get(), rs.meta.data(),
                           count * sizeof(ArrayMeta), cudaMemcpyHostToDevice,
                           stream));
  if (rs.total_s0 + rs.total_s1 > 0) {
    std::vector<SampleJob> jobs(count);
    for (uint32_t a = 0; a < count; ++a) {
      ArrayMeta const& m = rs.meta[a];
      jobs[a] = {m.word_off, m.bits, m.l1_off, m.l2_off, m.num_l1,
                 (m.num_l1 - 1) * kL2PerL1 + m.num_last_l2, m.ones, m.s0_off,
                 m.s1_off};
    }
    DevBuf jobs_d(count * sizeof(SampleJob));
    EWT_CUDA(cudaMemcpyAsync(jobs_d.get(), jobs.data(),
                             count * sizeof(SampleJob), cudaMemcpyHostToDevice,
                             stream));
    uint64_t const total_l2 = rs.meta.back().l2_off +
                              (rs.meta.back().num_l1 - 1) * kL2PerL1 +
                              rs.meta.back().num_last_l2;
    uint64_t const blocks = ceil_div(total_l2, 256);
    PhaseTimer pt(EWT_PHASE_SAMPLES, stream);
    rs_samples_kernel<<<static_cast<uint32_t>(blocks), 256, 0, stream>>>(
        rs.words.as<uint32_t>(), rs.l1.as<uint64_t>(), rs.l2.as<uint16_t>(),
        jobs_d.as<SampleJob>(), count, total_l2, rs.s0.as<uint64_t>(),
        rs.s1.as<uint64_t>());
    EWT_LAUNCHED();
    EWT_CUDA(cudaStreamSynchronize(stream));
  } else {
    EWT_CUDA(cudaStreamSynchronize(stream));
  }
}

namespace {

using ecl::detail::kRankBlockBits;
using ecl::detail::kRankBlockWords;

__device__ __forceinline__ uint32_t owner_array(uint64_t const* start,
                                                uint32_t num_arrays, uint64_t g) {
  uint32_t lo = 0, hi = num_arrays - 1;
  while (lo < hi) {
    uint32_t const mid = (lo + hi + 1) >> 1;
    if (start[mid] <= g) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Dense samples that fall in rank block b of array m: entry j names the
// block holding the (j*R+1)-th zero / one, R = 2^sh.  ones = ones before the
// block, w = its words (bits past the array end are not counted).
__device__ __forceinline__ void put_dense_samples(uint32_t* __restrict__ ds,
                                                  ArrayMeta const& m, uint64_t b,
                                                  uint64_t ones,
                                                  uint32_t const* w, uint32_t sh) {
  uint64_t const pos = b * kRankBlockBits;
  uint32_t const valid = static_cast<uint32_t>(
      min(uint64_t(kRankBlockBits), m.bits - pos));
  uint32_t c1 = 0;
#pragma unroll
  for (uint32_t j = 0; j < kRankBlockWords; ++j) {
    uint32_t const lo = j * 32;
    uint32_t const mask = valid >= lo + 32 ? ~0u
                          : valid > lo     ? (1u << (valid - lo)) - 1u
                                           : 0u;
    c1 += __popc(w[j] & mask);
  }
  uint64_t const R = uint64_t(1) << sh;
  uint32_t const blk = static_cast<uint32_t>(b);
#pragma unroll
  for (int val = 0; val < 2; ++val) {
    uint64_t const before = val ? ones : pos - ones;
    uint32_t const c = val ? c1 : valid - c1;
    if (c == 0) continue;
    uint32_t* S = ds + (val ? m.ds1_off : m.ds0_off);
    uint64_t const entries = ((val ? m.ones : m.bits - m.ones) + R - 1) >> sh;
    uint64_t const last = min((before + c - 1) >> sh, entries - 1);
    for (uint64_t j = (before + R - 1) >> sh; j <= last && entries; ++j)
      S[j] = blk;
  }
}

// One thread per rank block (32-byte sector) of every array: the low word
// of the ones before the block (from the L1/L2 counts) and the block's 7
// words; the first block of every 2^24 also writes the full count to the
// high-count table, and with ds set the block's dense select samples.
__global__ void __launch_bounds__(256)
rank_blocks_kernel(RSView v, uint64_t const* __restrict__ line_start,
                   uint32_t num_arrays, uint64_t total_lines,
                   uint64_t total_words, uint4* __restrict__ out,
                   uint64_t* __restrict__ high, uint32_t* __restrict__ ds,
                   uint32_t sel_shift) {
  uint64_t const g = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (g >= total_lines) return;
  uint32_t const a = owner_array(line_start, num_arrays, g);
  ArrayMeta const m = v.meta[a];
  uint64_t const b = g - line_start[a];
  uint64_t const pos = b * kRankBlockBits;
  uint64_t const ones = ecl::detail::rs_rank1<false>(v, m, pos, nullptr);
  uint64_t const w0 = m.word_off + b * kRankBlockWords;
  uint32_t w[kRankBlockWords];
#pragma unroll
  for (uint32_t j = 0; j < kRankBlockWords; ++j)
    w[j] = w0 + j < total_words ? v.words[w0 + j] : 0u;
  uint4* line = out + g * 2;
  line[0] = make_uint4(static_cast<uint32_t>(ones), w[0], w[1], w[2]);
  line[1] = make_uint4(w[3], w[4], w[5], w[6]);
  if ((b & ((uint64_t(1) << ecl::detail::kRankHighShift) - 1)) == 0)
    high[m.rbh_off + (b >> ecl::detail::kRankHighShift)] = ones;
  if (ds) put_dense_samples(ds, m, b, ones, w, sel_shift);
}

// Dense select samples at a new rate from the finished rank blocks.
__global__ void __launch_bounds__(256)
dense_samples_kernel(RSView v, uint64_t const* __restrict__ line_start,
                     uint32_t num_arrays, uint64_t total_lines,
                     uint32_t* __restrict__ ds, uint32_t sel_shift) {
  uint64_t const g = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (g >= total_lines) return;
  uint32_t const a = owner_array(line_start, num_arrays, g);
  ArrayMeta const m = v.meta[a];
  uint64_t const b = g - line_start[a];
  uint4 const q0 = v.rb[g * 2], q1 = v.rb[g * 2 + 1];
  uint32_t const w[kRankBlockWords] = {q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
  uint64_t const ones = ecl::detail::rb_ones_before(v, m, b, q0.x);
  put_dense_samples(ds, m, b, ones, w, sel_shift);
}

// Lays out the dense samples of every array at rate 2^shift (offsets into
// the meta table) and allocates them; returns false for shift 0.
bool layout_dense(RSStore& rs, uint32_t shift) {
  rs.ds.reset();
  rs.sel_shift = shift;
  if (shift == 0) return false;
  uint64_t total = 0;
  for (auto& m : rs.meta) {
    if (m.rb_off == ecl::detail::kNoBlocks) {
      m.ds0_off = m.ds1_off = ecl::detail::kNoBlocks;
      continue;
    }
    m.ds1_off = total;
    total += ceil_div(m.ones, uint64_t(1) << shift);
    m.ds0_off = total;
    total += ceil_div(m.bits - m.ones, uint64_t(1) << shift);
  }
  rs.ds.alloc(std::max<uint64_t>(total, 1) * 4);
  return true;
}

}  // namespace

uint64_t rank_block_starts(std::vector<ArrayMeta> const& meta,
                           std::vector<uint64_t>& start) {
  start.assign(meta.size(), 0);
  uint64_t total = 0;
  for (size_t a = 0; a < meta.size(); ++a) {
    start[a] = total;
    if (meta[a].rb_off != ecl::detail::kNoBlocks)
      total += ceil_div(meta[a].bits, kRankBlockBits);
  }
  return total;
}

void build_rank_blocks(RSStore& rs, cudaStream_t stream) {
  uint32_t const count = static_cast<uint32_t>(rs.meta.size());
  std::vector<uint64_t> start(count);
  uint64_t total = 0, highs = 0;
  for (uint32_t a = 0; a < count; ++a) {
    start[a] = total;
    if (a < rs.skip_blocks.size() && rs.skip_blocks[a]) {
      rs.meta[a].rb_off = rs.meta[a].rbh_off = ecl::detail::kNoBlocks;
      continue;
    }
    rs.meta[a].rb_off = total;
    rs.meta[a].rbh_off = highs;
    uint64_t const blocks = ceil_div(rs.meta[a].bits, ecl::detail::kRankBlockBits);
    total += blocks;
    highs += ceil_div(std::max<uint64_t>(blocks, 1),
                      uint64_t(1) << ecl::detail::kRankHighShift);
  }
  // blocks, then the high-count table in the same allocation
  rs.rb.alloc(total * 32 + highs * 8);
  bool const dense = layout_dense(rs, rs.sel_shift);
  DevBuf start_d(count * 8);
  EWT_CUDA(cudaMemcpyAsync(start_d.get(), start.data(), count * 8,
                           cudaMemcpyHostToDevice, stream));
  EWT_CUDA(cudaMemcpyAsync(rs.meta_d.get(), rs.meta.data(),
                           count * sizeof(ArrayMeta), cudaMemcpyHostToDevice,
                           stream));
  RSView v = rs.view();
  v.rb = nullptr;  // headers come from the L1/L2 counts
  v.ds = nullptr;
  v.sel_shift = 0;
  if (total > 0) {
    PhaseTimer pt(EWT_PHASE_SAMPLES, stream);
    rank_blocks_kernel<<<static_cast<uint32_t>(ceil_div(total, 256)), 256, 0,
                         stream>>>(v, start_d.as<uint64_t>(), count, total,
                                   rs.total_words, rs.rb.as<uint4>(),
                                   reinterpret_cast<uint64_t*>(
                                       rs.rb.as<unsigned char>() + total * 32),
                                   dense ? rs.ds.as<uint32_t>() : nullptr,
                                   rs.sel_shift);
    EWT_LAUNCHED();
  }
  EWT_CUDA(cudaStreamSynchronize(stream));
}

void build_dense_samples(RSStore& rs, uint32_t shift, cudaStream_t stream) {
  EWT_REQUIRE(shift == 0 || (shift >= 5 && shift <= 16), EWT_ERR_INVALID_ARGUMENT,
              "dense select sample rate must be 2^5 .. 2^16");
  EWT_CUDA(cudaStreamSynchronize(stream));  // no query may read the old ones
  uint32_t const count = static_cast<uint32_t>(rs.meta.size());
  if (!layout_dense(rs, shift) || count == 0 || !rs.rb.get()) {
    rs.ds.reset();
    return;
  }
  std::vector<uint64_t> start;
  uint64_t const total = rank_block_starts(rs.meta, start);
  DevBuf start_d(count * 8);
  EWT_CUDA(cudaMemcpyAsync(start_d.get(), start.data(), count * 8,
                           cudaMemcpyHostToDevice, stream));
  EWT_CUDA(cudaMemcpyAsync(rs.meta_d.get(), rs.meta.data(),
                           count * sizeof(ArrayMeta), cudaMemcpyHostToDevice,
                           stream));
  if (total > 0) {
    dense_samples_kernel<<<static_cast<uint32_t>(ceil_div(total, 256)), 256, 0,
                           stream>>>(rs.view(), start_d.as<uint64_t>(), count,
                                     total, rs.ds.as<uint32_t>(), shift);
    EWT_LAUNCHED();
  }
  EWT_CUDA(cudaStreamSynchronize(stream));
}

uint64_t rs_bytes_bound(uint64_t bits, uint32_t arrays, bool with_support) {
  uint64_t const words = (ceil_div(ceil_div(bits, 32), 32) * 32 + 2) * 4;
  uint64_t const l1 = (ceil_div(bits, kL1Bits) + 1) * 8;
  uint64_t const l2 = (ceil_div(bits, kL2Bits) + 1) * 2;
  uint64_t per = words + l1 + l2 + sizeof(ArrayMeta) + 64;
  if (with_support) {
    uint64_t const samples = (bits / kSampleRate + 2) * 8;
    uint64_t const blocks = (ceil_div(bits, 224) + 1) * 32 + 8;
    uint64_t const dense = (bits / 32 + 2) * 4;  // densest rate (32)
    per += samples + blocks + dense;
  }
  return per * arrays + 64;
}

}  // namespace ewt
