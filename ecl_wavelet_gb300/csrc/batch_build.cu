// Batch builds of short texts as one segmented build (ewt_build_batch).
//
// ewt_build_batch hands its short texts (below kBatchGroupMinSymbols) with a
// given alphabet 0 .. sigma-1, sigma a power of two in [4, 4096], and 1- or
// 2-byte symbols to build_small_texts, grouped by alphabet size.  Built one
// by one, such texts cost a few hundred CUDA calls each (launches, pool
// allocations, small copies, synchronisations) for very little GPU work.
// Here a group of G texts is built as one tree whose top a0 = ceil(log2 G)
// levels are the text number: the concatenated texts are that tree's
// level-a0 order, its level a0 + j holds every text's level j side by side,
// and one run of the pass pipeline (passes.cuh) writes all of them.  One
// launch then cuts each of those levels into the texts' own arrays, laid out
// back to back in one shared RankSelect store; one launch of each RankSelect
// kernel (counts, select samples, rank blocks) covers every array of every
// text, one launch counts every text's symbols and one computes every
// node-start rank.
//
// Every text still gets its own tree with the exports and answers of a
// single build (same level bits, counts, samples and node ranks): its
// arrays are views into the shared store, which lives until the group's
// last tree is freed.  Their query side is rank blocks on every level (no
// group levels), and the dense select-sample rate of their shared store
// stays as built.
#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "internal.cuh"
#include "passes.cuh"

namespace ewt {
namespace {

using ecl::detail::ArrayMeta;
using ecl::detail::RSView;

// The shared store of one group: the texts' level arrays and their
// RankSelect support, plus one block of small per-tree tables.  Freed on its
// own stream when the last tree of the group lets go of it.
struct SharedStore {
  int device = 0;
  cudaStream_t stream = nullptr;
  RSStore rs;
  DevBuf tables;
  ~SharedStore() {
    DeviceGuard g(device);
    for (DevBuf* b : {&rs.words, &rs.l1, &rs.l2, &rs.s0, &rs.s1, &rs.meta_d,
                      &rs.jobs_d, &rs.rb, &rs.ds, &tables})
      b->reset();  // stream-ordered frees, then the stream goes
    if (stream) {
      cudaStreamSynchronize(stream);
      cudaStreamDestroy(stream);
    }
  }
};

// Level a0 of the group tree (every text's level 0): the top bit of each
// of the n concatenated symbols, 32 per word; symbols at or above 2^L set
// bit 0 of err.
template <class T>
__global__ void __launch_bounds__(256)
concat_level0_kernel(T const* __restrict__ x, uint64_t n, uint32_t L,
                     uint32_t* __restrict__ words, uint32_t* __restrict__ err) {
  uint64_t const nw = (n + 31) / 32;
  uint64_t const stride = uint64_t(gridDim.x) * blockDim.x;
  uint32_t bad = 0;
  for (uint64_t w = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; w < nw;
       w += stride) {
    uint64_t const p0 = w * 32;
    uint32_t const cnt = static_cast<uint32_t>(min(uint64_t(32), n - p0));
    uint32_t bits = 0;
    if (cnt == 32) {
      // 32 symbols: 32 * sizeof(T) bytes at a 32-byte aligned offset
      constexpr uint32_t kU = 32 * sizeof(T) / 16;
      uint4 const* v = reinterpret_cast<uint4 const*>(x + p0);
#pragma unroll
      for (uint32_t u = 0; u < kU; ++u) {
        uint4 const q = v[u];
        uint32_t const wd[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (uint32_t j = 0; j < 4; ++j) {
#pragma unroll
          for (uint32_t h = 0; h < 4 / sizeof(T); ++h) {
            uint32_t const s = (wd[j] >> (8 * sizeof(T) * h)) &
                               (sizeof(T) == 1 ? 0xFFu : 0xFFFFu);
            uint32_t const i = (u * 4 + j) * (4 / sizeof(T)) + h;
            bad |= s >> L;
            bits |= ((s >> (L - 1)) & 1u) << i;
          }
        }
      }
    } else {
      for (uint32_t i = 0; i < cnt; ++i) {
        uint32_t const s = x[p0 + i];
        bad |= s >> L;
        bits |= ((s >> (L - 1)) & 1u) << i;
      }
    }
    words[w] = bits;
  }
  if (bad) atomicOr(err, 1u);
}

// One text's level: `bits` bits from bit src_shift of word src_word of the
// group level go to word dst_word onwards of the shared store.  `first`:
// destination words of all earlier jobs.
struct SplitJob {
  uint64_t src_word, bits, dst_word, first;
  uint32_t src_shift, pad;
};

__global__ void __launch_bounds__(256)
split_levels_kernel(uint32_t const* __restrict__ src, uint32_t* __restrict__ dst,
                    SplitJob const* __restrict__ jobs, uint32_t njobs,
                    uint64_t total) {
  uint64_t const stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t f = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; f < total;
       f += stride) {
    uint32_t lo = 0, hi = njobs - 1;  // the last job with first <= f
    while (lo < hi) {
      uint32_t const mid = (lo + hi + 1) >> 1;
      if (jobs[mid].first <= f) lo = mid; else hi = mid - 1;
    }
    SplitJob const j = jobs[lo];
    uint64_t const w = f - j.first;
    uint32_t v = __funnelshift_r(src[j.src_word + w], src[j.src_word + w + 1],
                                 j.src_shift);
    uint64_t const left = j.bits - w * 32;  // bits of the job from word w on
    if (left < 32) v &= (1u << left) - 1u;
    dst[j.dst_word + w] = v;
  }
}

// Symbol counts of every text: a job is a stretch of at most 65536 symbols
// of one text, counted in shared memory (sigma bins) and added to
// occ[text * sigma + symbol].
struct HistJob {
  uint64_t start;
  uint32_t len, text;
};

template <class T>
__global__ void __launch_bounds__(256)
group_hist_kernel(T const* __restrict__ x, HistJob const* __restrict__ jobs,
                  uint32_t njobs, uint32_t sigma,
                  unsigned long long* __restrict__ occ) {
  extern __shared__ uint32_t h[];
  for (uint32_t jb = blockIdx.x; jb < njobs; jb += gridDim.x) {
    HistJob const j = jobs[jb];
    for (uint32_t s = threadIdx.x; s < sigma; s += blockDim.x) h[s] = 0;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < j.len; i += blockDim.x) {
      uint32_t const s = x[j.start + i];
      if (s < sigma) atomicAdd(&h[s], 1u);  // larger ones were reported
    }
    __syncthreads();
    for (uint32_t s = threadIdx.x; s < sigma; s += blockDim.x)
      if (h[s]) atomicAdd(&occ[uint64_t(j.text) * sigma + s], h[s]);
    __syncthreads();
  }
}

// rank0 at a node start (precomputeRanksKernel, wavelet_tree.cuh:332-352):
// out[i] = zeros of array `array` before position `pos`.
struct RankJob {
  uint64_t pos, out;
  uint32_t array, pad;
};

__global__ void __launch_bounds__(256)
node_rank_jobs_kernel(RSView v, RankJob const* __restrict__ jobs, uint64_t njobs,
                      uint64_t* __restrict__ out) {
  uint64_t const stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < njobs;
       i += stride) {
    RankJob const j = jobs[i];
    ArrayMeta const m = v.meta[j.array];
    out[j.out] = j.pos - ecl::detail::rs_rank1<false>(v, m, j.pos, nullptr);
  }
}

uint32_t log2_ceil(uint64_t g) {
  uint32_t a = 0;
  while ((uint64_t(1) << a) < g) ++a;
  return a;
}

// The start level of the pass pipeline's last pass for a group tree of
// levels a0 .. a0 + L - 1 (as run_pass_pipeline plans it).
uint32_t last_pass_start(uint32_t a0, uint32_t L) {
  uint32_t const levels = L - 1;
  if (levels == 0) return a0;
  uint32_t const np = (levels + kPMaxK - 1) / kPMaxK;
  uint32_t a = a0, last = a0;
  for (uint32_t i = 0; i < np; ++i) {
    last = a;
    a += levels / np + (i < levels % np ? 1u : 0u);
  }
  return last;
}

size_t round_up(size_t x) { return (x + 255) / 256 * 256; }

template <class T>
void build_group(void const* const* texts, uint64_t const* lengths,
                 std::vector<uint32_t> const& ids, uint32_t L, int gpu,
                 ewt_tree** out) {
  uint32_t const G = static_cast<uint32_t>(ids.size());
  uint64_t const sigma = uint64_t(1) << L;
  auto store = std::make_shared<SharedStore>();
  store->device = gpu;
  EWT_CUDA(cudaStreamCreateWithFlags(&store->stream, cudaStreamNonBlocking));
  cudaStream_t const st = store->stream;
  AllocStream as(st);
  uint32_t const sms = static_cast<uint32_t>(sm_count());
  // ---- the concatenated texts
  std::vector<uint64_t> off(G + 1, 0);
  for (uint32_t g = 0; g < G; ++g) off[g + 1] = off[g] + lengths[ids[g]];
  uint64_t const N = off[G];
  DevBuf x(N * sizeof(T) + 64);
  for (uint32_t g = 0; g < G; ++g)
    EWT_CUDA(cudaMemcpyAsync(x.as<T>() + off[g], texts[ids[g]],
                             lengths[ids[g]] * sizeof(T), cudaMemcpyDefault, st));
  // ---- the group tree: text number above the symbol, a0 + L levels
  uint32_t const a0 = log2_ceil(G);
  uint32_t const Lg = a0 + L;
  std::vector<uint64_t> c_host((uint64_t(1) << Lg) + 1, 0);
  for (uint64_t t = 0; t < (uint64_t(1) << a0); ++t)
    c_host[t << L] = t < G ? off[t] : N;
  c_host.back() = N;
  DevBuf c_d(c_host.size() * 8);
  EWT_CUDA(cudaMemcpyAsync(c_d.get(), c_host.data(), c_host.size() * 8,
                           cudaMemcpyHostToDevice, st));
  uint64_t const stride_w = ceil_div(N, 32) + 64;  // words per group level
  DevBuf lw(L * stride_w * 4);
  EWT_CUDA(cudaMemsetAsync(lw.get(), 0, L * stride_w * 4, st));
  DevBuf err(16);
  EWT_CUDA(cudaMemsetAsync(err.get(), 0, 16, st));
  uint32_t* const words = lw.as<uint32_t>();
  concat_level0_kernel<T><<<static_cast<uint32_t>(std::max<uint64_t>(
                                1, std::min<uint64_t>(ceil_div(ceil_div(N, 32), 256),
                                                      uint64_t(sms) * 8))),
                            256, 0, st>>>(x.as<T>(), N, L, words,
                                          err.as<uint32_t>());
  EWT_LAUNCHED();
  std::vector<uint64_t> woff(Lg, 0), wbits(Lg, 0);
  for (uint32_t j = 0; j < L; ++j) {
    woff[a0 + j] = j * stride_w;
    wbits[a0 + j] = N;
  }
  run_pass_pipeline<T>(x.as<T>(), N, Lg, a0, words, woff.data(), wbits.data(),
                       c_d.as<uint64_t>(), err.as<uint32_t>() + 1, st);
  // ---- every text's arrays in one store; cut the group levels into them
  std::vector<uint64_t> bits;
  bits.reserve(uint64_t(G) * L);
  for (uint32_t g = 0; g < G; ++g)
    for (uint32_t j = 0; j < L; ++j) bits.push_back(lengths[ids[g]]);
  RSStore& rs = store->rs;
  rs.layout(bits);
  std::vector<SplitJob> sj;
  sj.reserve(bits.size());
  uint64_t total_w = 0;
  for (uint32_t g = 0; g < G; ++g)
    for (uint32_t j = 0; j < L; ++j) {
      ArrayMeta const& m = rs.meta[g * L + j];
      SplitJob s{};
      s.src_word = j * stride_w + off[g] / 32;
      s.src_shift = static_cast<uint32_t>(off[g] % 32);
      s.bits = lengths[ids[g]];
      s.dst_word = m.word_off;
      s.first = total_w;
      total_w += ceil_div(s.bits, 32);
      sj.push_back(s);
    }
  DevBuf sj_d(sj.size() * sizeof(SplitJob));
  EWT_CUDA(cudaMemcpyAsync(sj_d.get(), sj.data(), sj.size() * sizeof(SplitJob),
                           cudaMemcpyHostToDevice, st));
  split_levels_kernel<<<static_cast<uint32_t>(std::max<uint64_t>(
                            1, std::min<uint64_t>(ceil_div(total_w, 256),
                                                  uint64_t(sms) * 8))),
                        256, 0, st>>>(words, rs.words.as<uint32_t>(),
                                      sj_d.as<SplitJob>(),
                                      static_cast<uint32_t>(sj.size()), total_w);
  EWT_LAUNCHED();
  uint32_t const arrays = G * L;
  build_rs_counts(rs, 0, arrays, st);
  build_rs_samples(rs, st);
  rs.skip_blocks.assign(arrays, 0);
  build_rank_blocks(rs, st);
  // ---- symbol counts of every text
  std::vector<HistJob> hj;
  for (uint32_t g = 0; g < G; ++g)
    for (uint64_t s0 = 0; s0 < lengths[ids[g]]; s0 += 65536)
      hj.push_back({off[g] + s0,
                    static_cast<uint32_t>(std::min<uint64_t>(65536, lengths[ids[g]] - s0)),
                    g});
  DevBuf hj_d(hj.size() * sizeof(HistJob));
  EWT_CUDA(cudaMemcpyAsync(hj_d.get(), hj.data(), hj.size() * sizeof(HistJob),
                           cudaMemcpyHostToDevice, st));
  DevBuf occ_d(uint64_t(G) * sigma * 8);
  EWT_CUDA(cudaMemsetAsync(occ_d.get(), 0, uint64_t(G) * sigma * 8, st));
  group_hist_kernel<T><<<static_cast<uint32_t>(std::min<uint64_t>(
                             hj.size(), uint64_t(sms) * 8)),
                         256, sigma * 4, st>>>(x.as<T>(), hj_d.as<HistJob>(),
                                               static_cast<uint32_t>(hj.size()),
                                               static_cast<uint32_t>(sigma),
                                               occ_d.as<unsigned long long>());
  EWT_LAUNCHED();
  std::vector<uint64_t> occ(uint64_t(G) * sigma);
  uint32_t errs[4] = {0, 0, 0, 0};
  EWT_CUDA(cudaMemcpyAsync(occ.data(), occ_d.get(), occ.size() * 8,
                           cudaMemcpyDeviceToHost, st));
  EWT_CUDA(cudaMemcpyAsync(errs, err.get(), 16, cudaMemcpyDeviceToHost, st));
  EWT_CUDA(cudaStreamSynchronize(st));
  EWT_REQUIRE(!(errs[0] & 1), EWT_ERR_ALPHABET,
              "a text holds a symbol above its alphabet's last symbol");
  EWT_REQUIRE(errs[1] == 0, EWT_ERR_CUDA,
              "internal consistency check failed while building levels (kind " +
                  std::to_string(errs[1]) + ")");
  // ---- per-tree shape, counts and small tables
  std::vector<std::unique_ptr<ewt_tree>> trees(G);
  struct Slot {
    size_t counts, ranks, node_base, nodes_at_level, code_len, code_bits, err;
  };
  std::vector<Slot> slots(G);
  size_t tb = 0;
  for (uint32_t g = 0; g < G; ++g) {
    auto t = std::make_unique<ewt_tree>();
    t->device = gpu;
    t->elem_size = sizeof(T);
    t->n = lengths[ids[g]];
    t->sigma = sigma;
    t->L = L;
    t->pow2 = true;
    t->is_min = true;
    t->alphabet.resize(sigma);
    for (uint64_t i = 0; i < sigma; ++i) t->alphabet[i] = i;
    set_tree_shape(*t);
    t->occ.assign(occ.begin() + uint64_t(g) * sigma,
                  occ.begin() + uint64_t(g + 1) * sigma);
    t->counts.assign(sigma, 0);
    for (uint64_t i = 1; i < sigma; ++i) t->counts[i] = t->counts[i - 1] + t->occ[i - 1];
    t->level_bits.assign(L, t->n);
    Slot& s = slots[g];
    s.counts = tb; tb += round_up((sigma + 1) * 8);
    s.ranks = tb; tb += round_up(std::max<size_t>(t->nodes.size(), 1) * 8);
    s.node_base = tb; tb += round_up((L + 1) * 8);
    s.nodes_at_level = tb; tb += round_up(L * 8);
    s.code_len = tb; tb += 256;
    s.code_bits = tb; tb += 256;
    s.err = tb; tb += round_up(kTreeErrBytes);
    trees[g] = std::move(t);
  }
  std::vector<unsigned char> host_tables(tb, 0);
  std::vector<RankJob> rj;
  for (uint32_t g = 0; g < G; ++g) {
    ewt_tree const& t = *trees[g];
    Slot const& s = slots[g];
    auto put = [&](size_t at, uint64_t const* v, size_t count) {
      std::memcpy(host_tables.data() + at, v, count * 8);
    };
    std::vector<uint64_t> c(t.counts);
    c.push_back(t.n);
    put(s.counts, c.data(), c.size());
    put(s.node_base, t.node_base.data(), t.node_base.size());
    put(s.nodes_at_level, t.nodes_at_level.data(), t.nodes_at_level.size());
    for (size_t i = 0; i < t.nodes.size(); ++i) {
      RankJob r{};
      r.pos = t.counts[t.nodes[i].start];
      r.out = s.ranks / 8 + i;
      r.array = static_cast<uint32_t>(g * L + t.nodes[i].level);
      rj.push_back(r);
    }
  }
  store->tables.alloc(tb);
  EWT_CUDA(cudaMemcpyAsync(store->tables.get(), host_tables.data(), tb,
                           cudaMemcpyHostToDevice, st));
  RSView const sv = rs.view();
  if (!rj.empty()) {
    DevBuf rj_d(rj.size() * sizeof(RankJob));
    EWT_CUDA(cudaMemcpyAsync(rj_d.get(), rj.data(), rj.size() * sizeof(RankJob),
                             cudaMemcpyHostToDevice, st));
    node_rank_jobs_kernel<<<static_cast<uint32_t>(std::max<uint64_t>(
                                1, std::min<uint64_t>(ceil_div(rj.size(), 256),
                                                      uint64_t(sms) * 8))),
                            256, 0, st>>>(sv, rj_d.as<RankJob>(), rj.size(),
                                          store->tables.as<uint64_t>());
    EWT_LAUNCHED();
  }
  EWT_CUDA(cudaStreamSynchronize(st));  // host vectors above leave scope
  // ---- the trees: views into the shared store
  unsigned char* const tab = store->tables.as<unsigned char>();
  for (uint32_t g = 0; g < G; ++g) {
    ewt_tree& t = *trees[g];
    Slot const& s = slots[g];
    RSStore& r = t.rs;
    r.meta.assign(rs.meta.begin() + uint64_t(g) * L, rs.meta.begin() + uint64_t(g + 1) * L);
    r.words.view(rs.words.get(), rs.words.bytes());
    r.l1.view(rs.l1.get(), rs.l1.bytes());
    r.l2.view(rs.l2.get(), rs.l2.bytes());
    if (rs.s0.get()) r.s0.view(rs.s0.get(), rs.s0.bytes());
    if (rs.s1.get()) r.s1.view(rs.s1.get(), rs.s1.bytes());
    if (rs.rb.get()) r.rb.view(rs.rb.get(), rs.rb.bytes());
    if (rs.ds.get()) r.ds.view(rs.ds.get(), rs.ds.bytes());
    r.meta_d.view(rs.meta_d.as<ArrayMeta>() + uint64_t(g) * L, L * sizeof(ArrayMeta));
    r.total_words = rs.total_words;
    r.total_l1 = rs.total_l1;
    r.total_l2 = rs.total_l2;
    r.total_s0 = rs.total_s0;
    r.total_s1 = rs.total_s1;
    r.sel_shift = rs.sel_shift;
    r.skip_blocks.assign(L, 0);
    t.counts_d.view(tab + s.counts, (t.sigma + 1) * 8);
    t.ranks_d.view(tab + s.ranks, std::max<size_t>(t.nodes.size(), 1) * 8);
    t.node_base_d.view(tab + s.node_base, (L + 1) * 8);
    t.nodes_at_level_d.view(tab + s.nodes_at_level, L * 8);
    t.code_len_d.view(tab + s.code_len, 8);
    t.code_bits_d.view(tab + s.code_bits, 8);
    t.err_d.view(tab + s.err, kTreeErrBytes);
    // this tree's share of the store: its arrays and their support
    uint64_t share = 0;
    for (ArrayMeta const& m : r.meta) {
      share += ceil_div(ceil_div(m.bits, 32), 32) * 128 + m.num_l1 * 8 +
               ((m.num_l1 - 1) * 128 + m.num_last_l2) * 2 +
               (m.bits / 4096 + 1) * 8 + ceil_div(m.bits, 224) * 32 +
               sizeof(ArrayMeta);
      if (rs.ds.get() && rs.sel_shift)
        share += (m.bits >> rs.sel_shift) * 4 + 8;
    }
    t.rs_share_bytes = share;
    t.shared_store = store;
    fill_tree_view(t);
    RSView tv = sv;  // the store's view, narrowed to this tree's arrays
    tv.meta = rs.meta_d.as<ArrayMeta>() + uint64_t(g) * L;
    tv.num_arrays = L;
    t.view.rs = tv;
  }
  for (uint32_t g = 0; g < G; ++g) {
    EWT_CUDA(cudaStreamCreateWithFlags(&trees[g]->stream, cudaStreamNonBlocking));
    out[ids[g]] = trees[g].release();
  }
}

}  // namespace

bool small_batch_eligible(uint64_t n, int elem_size, void const* alphabet,
                          uint64_t sigma) {
  if (n == 0 || n >= kBatchGroupMinSymbols || (elem_size != 1 && elem_size != 2))
    return false;
  if (sigma < 4 || sigma > 4096 || (sigma & (sigma - 1)) || !alphabet) return false;
  for (uint64_t i = 0; i < sigma; ++i) {
    uint64_t const a = elem_size == 1 ? static_cast<uint8_t const*>(alphabet)[i]
                                      : static_cast<uint16_t const*>(alphabet)[i];
    if (a != i) return false;
  }
  return true;
}

void build_small_texts(void const* const* texts, uint64_t const* lengths,
                       std::vector<uint32_t> const& ids, int elem_size,
                       uint32_t L, int gpu, ewt_tree** out) {
  DeviceGuard g(gpu);
  // groups of at most 2^(kPMaxStartLevel - start of the last pass) texts,
  // so that every pass of the group tree starts at a supported level
  uint32_t const span = last_pass_start(0, L);
  uint32_t const max_a0 = kPMaxStartLevel >= span ? kPMaxStartLevel - span : 0;
  size_t const per = size_t(1) << std::min<uint32_t>(max_a0, 16);
  for (size_t s0 = 0; s0 < ids.size(); s0 += per) {
    std::vector<uint32_t> part(ids.begin() + s0,
                               ids.begin() + std::min(ids.size(), s0 + per));
    if (elem_size == 1)
      build_group<uint8_t>(texts, lengths, part, L, gpu, out);
    else
      build_group<uint16_t>(texts, lengths, part, L, gpu, out);
  }
}

}  // namespace ewt
