// Batched access / rank / select kernels over a built tree, and binary
// rank / select over a standalone RankSelect.
//
// One thread answers one query (the reference's ThreadsPerQuery = 1,
// wavelet_tree.cuh:958-960).  Every CTA first stages the per-level array
// metadata and node bases in shared memory, plus the count table and the
// node-start ranks when they fit (the reference's ShmemOffsets / ShmemRanks
// / ShmemCounts variants, :373-544).  The grid is sized to keep every SM
// full and strides over the batch.  Invalid queries (select k == 0, rank
// index > n, a symbol above the alphabet) write UINT64_MAX and raise the
// tree's error word; access with index >= n writes 0.
#include <algorithm>

#include "internal.cuh"

namespace ewt {

using namespace ecl::detail;

template <class T>
struct alignas(8) QueryRec {
  uint64_t index;
  T symbol;
};
static_assert(sizeof(QueryRec<uint8_t>) == 16, "RankSelectQuery layout");
static_assert(sizeof(QueryRec<uint64_t>) == 16, "RankSelectQuery layout");

enum Kind { kAccess = 0, kRank = 1, kSelect = 2, kMixed = 3 };

constexpr uint32_t kQueryThreads = 256;     // default threads per CTA
constexpr uint32_t kMaxQueryThreads = 256;  // largest the autotuner tries
// Staging budget per CTA: small enough that 8 CTAs (2048 threads) fit on an
// SM's 228 KB of shared memory.
constexpr uint64_t kStageLimitBytes = 24 * 1024;

struct StagePlan {
  uint32_t stage_counts, stage_ranks;
  size_t bytes;
};

inline StagePlan plan_stage(ewt_tree const& t) {
  StagePlan p{0, 0, 0};
  size_t b = t.L * sizeof(ArrayMeta) + (t.L + 1) * 8;
  b = (b + 15) & ~size_t(15);
  if (b + t.sigma * 8 <= kStageLimitBytes / 2) {
    p.stage_counts = 1;
    b += t.sigma * 8;
  }
  if (b + t.nodes.size() * 8 <= kStageLimitBytes) {
    p.stage_ranks = 1;
    b += t.nodes.size() * 8;
  }
  p.bytes = b;
  return p;
}

template <class T, int K>
__global__ void __launch_bounds__(kMaxQueryThreads)
query_kernel(TreeView t, uint8_t const* __restrict__ types,
             void const* __restrict__ in, uint64_t m, void* __restrict__ out,
             uint32_t* __restrict__ err, uint32_t stage_counts,
             uint32_t stage_ranks) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint32_t const L = t.levels;
  ArrayMeta* meta = reinterpret_cast<ArrayMeta*>(smem);
  uint64_t* node_base = reinterpret_cast<uint64_t*>(meta + L);
  size_t off = L * sizeof(ArrayMeta) + (L + 1) * 8;
  off = (off + 15) & ~size_t(15);
  uint64_t const* counts = t.counts;
  uint64_t const* ranks = t.node_ranks;
  {
    uint64_t const* gm = reinterpret_cast<uint64_t const*>(t.rs.meta);
    uint64_t* sm = reinterpret_cast<uint64_t*>(meta);
    uint32_t const mw = L * (sizeof(ArrayMeta) / 8);
    for (uint32_t i = threadIdx.x; i < mw; i += blockDim.x) sm[i] = gm[i];
    for (uint32_t i = threadIdx.x; i <= L; i += blockDim.x)
      node_base[i] = t.node_base[i];
    if (stage_counts) {
      uint64_t* sc = reinterpret_cast<uint64_t*>(smem + off);
      for (uint64_t i = threadIdx.x; i < t.sigma; i += blockDim.x)
        sc[i] = t.counts[i];
      counts = sc;
      off += t.sigma * 8;
    }
    if (stage_ranks) {
      uint64_t* sr = reinterpret_cast<uint64_t*>(smem + off);
      for (uint64_t i = threadIdx.x; i < t.num_ranks; i += blockDim.x)
        sr[i] = t.node_ranks[i];
      ranks = sr;
    }
  }
  __syncthreads();
  uint32_t bad = 0;
  uint64_t const stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < m;
       i += stride) {
    int kind = K;
    if (K == kMixed) kind = types[i];
    if (kind == kAccess) {
      uint64_t idx;
      if (K == kMixed)
        idx = static_cast<QueryRec<T> const*>(in)[i].index;
      else
        idx = static_cast<uint64_t const*>(in)[i];
      T res = 0;
      if (idx < t.n)
        res = from_minimal<T>(
            t, wt_access(t, meta, counts, ranks, node_base, idx));
      if (K == kMixed)
        static_cast<uint64_t*>(out)[i] = res;
      else
        static_cast<T*>(out)[i] = res;
      continue;
    }
    QueryRec<T> const q = static_cast<QueryRec<T> const*>(in)[i];
    uint64_t const c = to_minimal<T>(t, q.symbol);
    uint64_t res;
    if (kind == kRank) {
      if (c >= t.sigma || q.index > t.n) {
        res = UINT64_MAX;
        bad = 1;
      } else {
        res = wt_rank(t, meta, counts, ranks, node_base, c, q.index);
      }
    } else if (kind == kSelect) {
      if (c >= t.sigma || q.index == 0) {
        res = UINT64_MAX;
        bad = 1;
      } else {
        res = wt_select(t, meta, counts, ranks, node_base, c, q.index);
      }
    } else {
      res = UINT64_MAX;
      bad = 1;
    }
    static_cast<uint64_t*>(out)[i] = res;
  }
  if (bad) atomicOr(err, 1u);
}

// Batched mixed form: CTAs take 2048-query chunks of the interleaved batch,
// sort each chunk's query numbers by type in shared memory (warp ballots),
// then walk the access, rank and select lists in turn, so every warp runs
// one kind of walk.  Results go straight to their original slots.
constexpr uint32_t kMixChunk = 2048;

template <class T>
__global__ void __launch_bounds__(kMaxQueryThreads)
mixed_kernel(TreeView t, uint8_t const* __restrict__ types,
             QueryRec<T> const* __restrict__ in, uint64_t m,
             uint64_t* __restrict__ out, uint32_t* __restrict__ err,
             uint32_t stage_counts, uint32_t stage_ranks, uint32_t* queue) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint16_t lists[3][kMixChunk];
  __shared__ uint32_t list_len[3];
  __shared__ uint32_t next_chunk;
  uint32_t const L = t.levels;
  ArrayMeta* meta = reinterpret_cast<ArrayMeta*>(smem);
  uint64_t* node_base = reinterpret_cast<uint64_t*>(meta + L);
  size_t off = L * sizeof(ArrayMeta) + (L + 1) * 8;
  off = (off + 15) & ~size_t(15);
  uint64_t const* counts = t.counts;
  uint64_t const* ranks = t.node_ranks;
  {
    uint64_t const* gm = reinterpret_cast<uint64_t const*>(t.rs.meta);
    uint64_t* sm = reinterpret_cast<uint64_t*>(meta);
    uint32_t const mw = L * (sizeof(ArrayMeta) / 8);
    for (uint32_t i = threadIdx.x; i < mw; i += blockDim.x) sm[i] = gm[i];
    for (uint32_t i = threadIdx.x; i <= L; i += blockDim.x)
      node_base[i] = t.node_base[i];
    if (stage_counts) {
      uint64_t* sc = reinterpret_cast<uint64_t*>(smem + off);
      for (uint64_t i = threadIdx.x; i < t.sigma; i += blockDim.x)
        sc[i] = t.counts[i];
      counts = sc;
      off += t.sigma * 8;
    }
    if (stage_ranks) {
      uint64_t* sr = reinterpret_cast<uint64_t*>(smem + off);
      for (uint64_t i = threadIdx.x; i < t.num_ranks; i += blockDim.x)
        sr[i] = t.node_ranks[i];
      ranks = sr;
    }
  }
  uint32_t const lane = threadIdx.x & 31;
  uint32_t const lt = (1u << lane) - 1u;
  uint32_t bad = 0;
  uint64_t const chunks = (m + kMixChunk - 1) / kMixChunk;
  for (uint64_t c = wq_take(queue, &next_chunk, 0, true); c < chunks;
       c = wq_take(queue, &next_chunk, c, false)) {
    uint64_t const base = c * kMixChunk;
    if (threadIdx.x < 3) list_len[threadIdx.x] = 0;
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < kMixChunk; j += blockDim.x) {
      uint64_t const q = base + j;
      uint32_t const ty = q < m ? types[q] : 3u;
#pragma unroll
      for (uint32_t k = 0; k < 3; ++k) {
        uint32_t const mask = __ballot_sync(0xffffffffu, ty == k);
        if (mask == 0) continue;
        uint32_t pos = 0;
        if (lane == __ffs(mask) - 1) pos = atomicAdd(&list_len[k], __popc(mask));
        pos = __shfl_sync(0xffffffffu, pos, __ffs(mask) - 1);
        if (ty == k) lists[k][pos + __popc(mask & lt)] = static_cast<uint16_t>(j);
      }
      if (ty > 2 && q < m) {
        out[q] = UINT64_MAX;
        bad = 1;
      }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < list_len[0]; i += blockDim.x) {
      uint64_t const q = base + lists[0][i];
      uint64_t const idx = in[q].index;
      out[q] = idx < t.n ? static_cast<uint64_t>(from_minimal<T>(
                               t, wt_access(t, meta, counts, ranks, node_base,
                                            idx)))
                         : 0;
    }
    for (uint32_t i = threadIdx.x; i < list_len[1]; i += blockDim.x) {
      uint64_t const q = base + lists[1][i];
      QueryRec<T> const r = in[q];
      uint64_t const sym = to_minimal<T>(t, r.symbol);
      if (sym >= t.sigma || r.index > t.n) {
        out[q] = UINT64_MAX;
        bad = 1;
      } else {
        out[q] = wt_rank(t, meta, counts, ranks, node_base, sym, r.index);
      }
    }
    for (uint32_t i = threadIdx.x; i < list_len[2]; i += blockDim.x) {
      uint64_t const q = base + lists[2][i];
      QueryRec<T> const r = in[q];
      uint64_t const sym = to_minimal<T>(t, r.symbol);
      if (sym >= t.sigma || r.index == 0) {
        out[q] = UINT64_MAX;
        bad = 1;
      } else {
        out[q] = wt_select(t, meta, counts, ranks, node_base, sym, r.index);
      }
    }
    __syncthreads();  // lists are reused by the next chunk
  }
  wq_finish(queue);
  if (bad) atomicOr(err, 1u);
}

template <int Value>
__global__ void __launch_bounds__(256)
rs_rank_kernel(RSView v, uint32_t array, uint64_t const* __restrict__ pos,
               uint64_t m, uint64_t* __restrict__ out, uint32_t* err) {
  ArrayMeta const meta = v.meta[array];
  uint64_t const stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < m;
       i += stride) {
    uint64_t const p = pos[i];
    if (p > meta.bits) {
      out[i] = UINT64_MAX;
      atomicOr(err, 1u);
      continue;
    }
    uint64_t const r1 = rs_rank1<false>(v, meta, p, nullptr);
    out[i] = Value ? r1 : p - r1;
  }
}

template <int Value>
__global__ void __launch_bounds__(256)
rs_select_kernel(RSView v, uint32_t array, uint64_t const* __restrict__ idx,
                 uint64_t m, uint64_t* __restrict__ out, uint32_t* err) {
  ArrayMeta const meta = v.meta[array];
  uint64_t const stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < m;
       i += stride) {
    uint64_t const k = idx[i];
    if (k == 0) {
      out[i] = UINT64_MAX;
      atomicOr(err, 1u);
      continue;
    }
    out[i] = rs_select<Value>(v, meta, k);
  }
}

namespace {

// One mixed_kernel launch with the tree's tuned shape (threads x CTAs per SM
// when the autotuner chose them), timed as a query phase; invalid queries
// set *err.
template <class T>
void launch_mixed_kernel(ewt_tree& t, uint8_t const* types, void const* in,
                         uint64_t m, uint64_t* out, uint32_t* err,
                         StagePlan const& p, cudaStream_t s,
                         uint32_t* queue) {
  RelaxedCapture relaxed;
  auto mk = mixed_kernel<T>;
  set_smem_limit(mk, static_cast<int>(kStageLimitBytes + 4096));
  uint32_t const threads =
      t.tune_threads[kMixed] ? t.tune_threads[kMixed] : kQueryThreads;
  int per_sm = 0;
  EWT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mk, threads,
                                                         p.bytes));
  per_sm = std::max(per_sm, 1);
  if (t.tune_blocks[kMixed]) per_sm = std::min<int>(per_sm, t.tune_blocks[kMixed]);
  uint64_t const chunks = ceil_div(m, kMixChunk);
  uint32_t const blocks = static_cast<uint32_t>(
      std::min<uint64_t>(chunks, uint64_t(per_sm) * sm_count()));
  PhaseTimer pt(EWT_PHASE_QUERY, s);
  mk<<<blocks, threads, p.bytes, s>>>(t.view, types,
                                      static_cast<QueryRec<T> const*>(in), m,
                                      out, err, p.stage_counts, p.stage_ranks,
                                      queue);
  EWT_LAUNCHED();
}

template <class T, int K>
void launch_typed(ewt_tree& t, uint8_t const* types, void const* in,
                  uint64_t m, void* out, cudaStream_t s) {
  if (m == 0) return;
  EWT_REQUIRE(in != nullptr && out != nullptr && (K != kMixed || types),
              EWT_ERR_INVALID_ARGUMENT, "null query, type or result buffer");
  EWT_REQUIRE(reinterpret_cast<uintptr_t>(in) % 8 == 0 &&
                  (K == kAccess ||
                   reinterpret_cast<uintptr_t>(out) % 8 == 0),
              EWT_ERR_INVALID_ARGUMENT,
              "query and result buffers must be 8-byte aligned");
  StagePlan const p = plan_stage(t);
  RelaxedCapture relaxed;  // these launches may be captured into a graph
  if (K == kMixed) {
    launch_mixed_kernel<T>(t, types, in, m, static_cast<uint64_t*>(out),
                           t.err_d.as<uint32_t>(), p, s, queue_slot(t));
    return;
  }
  auto k = query_kernel<T, K>;
  set_smem_limit(k, static_cast<int>(kStageLimitBytes + 4096));
  uint32_t const threads = t.tune_threads[K] ? t.tune_threads[K] : kQueryThreads;
  int per_sm = 0;
  EWT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k,
                                                         threads, p.bytes));
  per_sm = std::max(per_sm, 1);
  if (t.tune_blocks[K]) per_sm = std::min<int>(per_sm, t.tune_blocks[K]);
  uint64_t const need = ceil_div(m, threads);
  uint64_t const full = uint64_t(per_sm) * sm_count();
  uint32_t const blocks = static_cast<uint32_t>(std::min(need, full));
  PhaseTimer pt(EWT_PHASE_QUERY, s);
  k<<<blocks, threads, p.bytes, s>>>(t.view, types, in, m, out,
                                           t.err_d.as<uint32_t>(),
                                           p.stage_counts, p.stage_ranks);
  EWT_LAUNCHED();
}

template <int K>
void launch_any(ewt_tree& t, uint8_t const* types, void const* in, uint64_t m,
                void* out, cudaStream_t s) {
  switch (t.elem_size) {
    case 1: launch_typed<uint8_t, K>(t, types, in, m, out, s); break;
    case 2: launch_typed<uint16_t, K>(t, types, in, m, out, s); break;
    case 4: launch_typed<uint32_t, K>(t, types, in, m, out, s); break;
    default: launch_typed<uint64_t, K>(t, types, in, m, out, s); break;
  }
}

uint32_t grid_for(uint64_t m) {
  uint64_t const need = ceil_div(m, 256);
  uint64_t const full = uint64_t(sm_count()) * 8;
  return static_cast<uint32_t>(std::max<uint64_t>(1, std::min(need, full)));
}

}  // namespace

void launch_access(ewt_tree& t, uint64_t const* d_idx, uint64_t m, void* d_out,
                   cudaStream_t s) {
  launch_any<kAccess>(t, nullptr, d_idx, m, d_out, s);
}
void launch_rank(ewt_tree& t, void const* d_q, uint64_t m, uint64_t* d_out,
                 cudaStream_t s) {
  launch_any<kRank>(t, nullptr, d_q, m, d_out, s);
}
void launch_select(ewt_tree& t, void const* d_q, uint64_t m, uint64_t* d_out,
                   cudaStream_t s) {
  launch_any<kSelect>(t, nullptr, d_q, m, d_out, s);
}
void launch_mixed(ewt_tree& t, uint8_t const* d_types, void const* d_q,
                  uint64_t m, uint64_t* d_out, cudaStream_t s) {
  launch_any<kMixed>(t, d_types, d_q, m, d_out, s);
}

namespace {
template <class T>
void launch_mixed_raw_typed(ewt_tree& t, uint8_t const* d_types,
                            void const* d_q, uint64_t m, uint64_t* d_out,
                            uint32_t* d_err, cudaStream_t s) {
  launch_mixed_kernel<T>(t, d_types, d_q, m, d_out, d_err, plan_stage(t), s,
                         work_queue_enabled() ? d_err + 16 : nullptr);
}
}  // namespace

void launch_mixed_raw(ewt_tree& t, uint8_t const* d_types, void const* d_q,
                      uint64_t m, uint64_t* d_out, uint32_t* d_err,
                      cudaStream_t s) {
  if (m == 0) return;
  switch (t.elem_size) {
    case 1: launch_mixed_raw_typed<uint8_t>(t, d_types, d_q, m, d_out, d_err, s); break;
    case 2: launch_mixed_raw_typed<uint16_t>(t, d_types, d_q, m, d_out, d_err, s); break;
    case 4: launch_mixed_raw_typed<uint32_t>(t, d_types, d_q, m, d_out, d_err, s); break;
    default: launch_mixed_raw_typed<uint64_t>(t, d_types, d_q, m, d_out, d_err, s); break;
  }
}

// ---- random-access roofline probe -------------------------------------------
namespace {

__device__ __forceinline__ uint64_t probe_mix(uint64_t x) {  // splitmix64
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

// Chains of `depth` dependent random 32-byte reads (two 16-byte loads, as a
// query walk reads a block) over `units` 32-byte units; one chain per
// thread and iteration.
__global__ void __launch_bounds__(256)
random_chain_kernel(uint4 const* __restrict__ a, uint64_t units, uint32_t depth,
                    uint64_t chains, uint64_t* __restrict__ sink) {
  uint64_t acc = 0;
  uint64_t const stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t q = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; q < chains;
       q += stride) {
    uint64_t h = probe_mix(q + 0x1234567ull);
    for (uint32_t d = 0; d < depth; ++d) {
      uint4 const* u = a + (h % units) * 2;
      uint4 const x = __ldg(u), y = __ldg(u + 1);
      h = probe_mix(h ^ x.x ^ y.w);
    }
    acc += h;
  }
  if (acc == 0x5eedull) sink[0] = acc;  // keeps the loads
}

}  // namespace

int kernel_binary_version() {
  cudaFuncAttributes a{};
  EWT_CUDA(cudaFuncGetAttributes(&a, mixed_kernel<uint8_t>));
  return a.binaryVersion;
}

void probe_random_reads(uint64_t bytes, uint32_t depth, uint64_t chains,
                        double* reads_per_s) {
  EWT_REQUIRE(bytes >= (uint64_t(1) << 20) && depth >= 1 && depth <= 64 &&
                  chains >= 1024,
              EWT_ERR_INVALID_ARGUMENT, "probe: bytes >= 1 MiB, depth 1..64");
  cudaStream_t s = alloc_stream();
  DevBuf buf(bytes), sink(8);
  EWT_CUDA(cudaMemsetAsync(buf.get(), 0x5a, bytes, s));
  uint64_t const units = bytes / 32;
  uint32_t const grid = static_cast<uint32_t>(sm_count()) * 4;
  cudaEvent_t e0, e1;
  EWT_CUDA(cudaEventCreate(&e0));
  EWT_CUDA(cudaEventCreate(&e1));
  random_chain_kernel<<<grid, 256, 0, s>>>(buf.as<uint4>(), units, depth, chains,
                                           sink.as<uint64_t>());  // warm-up
  EWT_LAUNCHED();
  EWT_CUDA(cudaEventRecord(e0, s));
  random_chain_kernel<<<grid, 256, 0, s>>>(buf.as<uint4>(), units, depth, chains,
                                           sink.as<uint64_t>());
  EWT_LAUNCHED();
  EWT_CUDA(cudaEventRecord(e1, s));
  EWT_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  EWT_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *reads_per_s = double(chains) * depth / (ms * 1e-3);
}

// ---- autotuner -------------------------------------------------------------
namespace {


// Valid probe queries over tree t: access i in [0, n); rank c uniform, i in
// [0, n]; select c uniform, k in [1, count(c)] (k = 1 when c is absent);
// kind 3 mixes them 40/40/20.
template <class T>
__global__ void __launch_bounds__(256)
probe_kernel(TreeView t, int kind, uint64_t m, uint64_t seed,
             uint8_t* __restrict__ types, QueryRec<T>* __restrict__ rec,
             uint64_t* __restrict__ idx) {
  uint64_t const stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < m;
       i += stride) {
    uint64_t const h = probe_mix(seed + i);
    int ty = kind;
    if (kind == 3) {
      uint64_t const u = h % 5;
      ty = u < 2 ? 0 : (u < 4 ? 1 : 2);
    }
    uint64_t const h2 = probe_mix(h);
    uint64_t const c = h2 % t.sigma;
    uint64_t index;
    if (ty == 0) {
      index = h2 % t.n;
    } else if (ty == 1) {
      index = probe_mix(h2) % (t.n + 1);
    } else {
      uint64_t const cnt = (c + 1 < t.sigma ? t.counts[c + 1] : t.n) - t.counts[c];
      index = cnt ? 1 + probe_mix(h2) % cnt : 1;
    }
    T const sym = t.is_min ? static_cast<T>(c)
                           : static_cast<T const*>(t.alphabet)[c];
    if (kind == 0) {
      idx[i] = index;
    } else {
      rec[i].index = index;
      rec[i].symbol = sym;
      if (kind == 3) types[i] = static_cast<uint8_t>(ty);
    }
  }
}

template <class T>
void autotune_typed(ewt_tree& t, uint64_t m, ewt_tuning* out) {
  cudaStream_t const s = t.stream;
  DevBuf types(m), rec(m * 16), idx(m * 8), res(m * 8);
  uint32_t const sms = static_cast<uint32_t>(sm_count());
  cudaEvent_t e0, e1;
  EWT_CUDA(cudaEventCreate(&e0));
  EWT_CUDA(cudaEventCreate(&e1));
  uint32_t const thread_opts[2] = {128, 256};
  uint32_t const block_opts[5] = {0, 2, 4, 6, 8};  // 0: as many as fit
  for (int kind = 0; kind < 4; ++kind) {
    probe_kernel<T><<<std::min<uint64_t>(ceil_div(m, 256), uint64_t(sms) * 8), 256, 0, s>>>(
        t.view, kind, m, 0x5eed0000ull + kind, types.as<uint8_t>(),
        rec.as<QueryRec<T>>(), idx.as<uint64_t>());
    EWT_LAUNCHED();
    auto run = [&]() {
      switch (kind) {
        case 0: launch_typed<T, kAccess>(t, nullptr, idx.get(), m, res.get(), s); break;
        case 1: launch_typed<T, kRank>(t, nullptr, rec.get(), m, res.get(), s); break;
        case 2: launch_typed<T, kSelect>(t, nullptr, rec.get(), m, res.get(), s); break;
        default: launch_typed<T, kMixed>(t, types.as<uint8_t>(), rec.get(), m, res.get(), s); break;
      }
    };
    auto timed = [&]() -> float {
      run();  // warm
      EWT_CUDA(cudaEventRecord(e0, s));
      for (int r = 0; r < 3; ++r) run();
      EWT_CUDA(cudaEventRecord(e1, s));
      EWT_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      EWT_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      return ms / 3;
    };
    t.tune_threads[kind] = 0;
    t.tune_blocks[kind] = 0;
    float const base = timed();
    float sel_ms = base;
    if (kind == 2 && !t.view_shared.load() && !t.shared_store) {
      // dense select-sample rate first (select probes, default shape)
      uint32_t const start = t.rs.ds.get() ? t.rs.sel_shift : 0;
      uint32_t best_sh = start;
      float best_ms = base;
      for (uint32_t sh : {0u, 6u, 7u, 8u, 9u, 10u}) {
        if (sh == start) continue;
        set_select_rate(t, sh, s);
        float const ms = timed();
        if (ms < best_ms) {
          best_ms = ms;
          best_sh = sh;
        }
      }
      if (t.rs.sel_shift != best_sh || (best_sh && !t.rs.ds.get()))
        set_select_rate(t, best_sh, s);
      sel_ms = best_ms;
    }
    if (out) out->select_sample_rate = t.rs.ds.get() ? 1u << t.rs.sel_shift : 0u;
    float best = sel_ms;  // select: at the kept sample rate
    uint32_t bt = 0, bb = 0;
    for (uint32_t th : thread_opts)
      for (uint32_t bl : block_opts) {
        t.tune_threads[kind] = th;
        t.tune_blocks[kind] = bl;
        float const ms = timed();
        if (ms < best) {
          best = ms;
          bt = th;
          bb = bl;
        }
      }
    t.tune_threads[kind] = bt;
    t.tune_blocks[kind] = bb;
    if (out) {
      out->threads[kind] = bt ? bt : kQueryThreads;
      out->blocks_per_sm[kind] = bb;
      out->default_mq_s[kind] = m / (base * 1e3);
      out->tuned_mq_s[kind] = m / (best * 1e3);
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // the probes are valid queries; clear the invalid-query word regardless
  EWT_CUDA(cudaMemsetAsync(t.err_d.get(), 0, 4, s));
  EWT_CUDA(cudaStreamSynchronize(s));
}

}  // namespace

void autotune_queries(ewt_tree& t, uint64_t probe_queries, ewt_tuning* out) {
  switch (t.elem_size) {
    case 1: autotune_typed<uint8_t>(t, probe_queries, out); break;
    case 2: autotune_typed<uint16_t>(t, probe_queries, out); break;
    case 4: autotune_typed<uint32_t>(t, probe_queries, out); break;
    default: autotune_typed<uint64_t>(t, probe_queries, out); break;
  }
}

void launch_rs_rank(ewt_rs& r, int array, int value, uint64_t const* d_pos,
                    uint64_t m, uint64_t* d_out, cudaStream_t s) {
  if (m == 0) return;
  uint32_t* err = r.err_d.as<uint32_t>();
  RSView const v = r.rs.view();
  if (value)
    rs_rank_kernel<1><<<grid_for(m), 256, 0, s>>>(v, array, d_pos, m, d_out, err);
  else
    rs_rank_kernel<0><<<grid_for(m), 256, 0, s>>>(v, array, d_pos, m, d_out, err);
  EWT_LAUNCHED();
}

void launch_rs_select(ewt_rs& r, int array, int value, uint64_t const* d_i,
                      uint64_t m, uint64_t* d_out, cudaStream_t s) {
  if (m == 0) return;
  uint32_t* err = r.err_d.as<uint32_t>();
  RSView const v = r.rs.view();
  if (value)
    rs_select_kernel<1><<<grid_for(m), 256, 0, s>>>(v, array, d_i, m, d_out, err);
  else
    rs_select_kernel<0><<<grid_for(m), 256, 0, s>>>(v, array, d_i, m, d_out, err);
  EWT_LAUNCHED();
}

}  // namespace ewt
