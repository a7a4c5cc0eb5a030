// Many trees at once: mixed access/rank/select queries over many trees in
// one launch, and the batched construction of many texts.
//
// Queries.  A batch carries one tree id per query.  Three small kernels
// group it by tree (histogram of the ids, a plan that cuts every tree's
// queries into work items of at most kMultiChunk queries, a scatter of the
// query numbers into tree order); the multi-tree kernel then walks the work
// list: per item the CTA copies the tree's view and level metadata into
// shared memory, sorts the item's queries by type with warp ballots, and
// answers them, writing every result to its original slot.  The reference
// answers one tree per host call (wavelet_tree.cuh:956-1797); grouping by
// tree on the device replaces one call (copies, launch, synchronisation)
// per tree with one launch per batch.
//
// Construction.  ewt_build_batch builds its short texts with a given
// power-of-two minimal alphabet as segmented group builds (one per alphabet
// size, batch_build.cu) while host workers build every other text on its
// own stream; each result is a tree of its own.
#include <algorithm>
#include <atomic>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "internal.cuh"

namespace ewt {
namespace {

using namespace ecl::detail;

static_assert(sizeof(TreeView) % 8 == 0, "TreeView is copied as 8-byte words");

template <class T>
struct alignas(8) MultiRec {
  uint64_t index;
  T symbol;
};
static_assert(sizeof(MultiRec<uint8_t>) == 16, "RankSelectQuery layout");

// One work item: `count` (<= kMultiChunk) queries of tree `tree`, at
// positions [start, start + count) of the tree-ordered batch.
struct MultiItem {
  uint32_t tree, count;
  uint64_t start;
};

constexpr uint32_t kMultiChunk = 2048;
constexpr uint32_t kMultiThreads = 256;
constexpr uint32_t kPlanThreads = 1024;
constexpr uint32_t kMaxMultiTrees = 1u << 16;  // trees in one call
constexpr uint32_t kBuildWorkers = 16;          // host threads of a batch build

__global__ void __launch_bounds__(256)
tree_hist_kernel(uint32_t const* __restrict__ tree_of, uint64_t m,
                 uint32_t num_trees, uint32_t* __restrict__ cnt) {
  uint64_t const stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t q = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; q < m;
       q += stride) {
    uint32_t const t = min(tree_of[q], num_trees);  // num_trees: invalid id
    uint32_t const peers = __match_any_sync(__activemask(), t);
    if ((threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&cnt[t], __popc(peers));
  }
}

// Up to kSmemTrees trees: per-CTA shared-memory counts over a contiguous
// slice of the batch (no global atomics per query), flushed once per CTA.
constexpr uint32_t kSmemTrees = 4096;

__global__ void __launch_bounds__(256)
tree_hist_smem_kernel(uint32_t const* __restrict__ tree_of, uint64_t m,
                      uint32_t num_trees, uint32_t* __restrict__ cnt) {
  __shared__ uint32_t h[kSmemTrees + 1];
  for (uint32_t i = threadIdx.x; i <= num_trees; i += blockDim.x) h[i] = 0;
  __syncthreads();
  uint64_t const per = (m + gridDim.x - 1) / gridDim.x;
  uint64_t const s0 = min(m, blockIdx.x * per), s1 = min(m, s0 + per);
  for (uint64_t q = s0 + threadIdx.x; q < s1; q += blockDim.x)
    atomicAdd(&h[min(tree_of[q], num_trees)], 1u);  // num_trees: invalid id
  __syncthreads();
  for (uint32_t i = threadIdx.x; i <= num_trees; i += blockDim.x)
    if (h[i]) atomicAdd(&cnt[i], h[i]);
}

// Query numbers into tree order for up to kSmemTrees trees: the CTA counts
// its slice per tree, reserves one range per tree with a global atomic, and
// hands out positions inside it from shared memory.
__global__ void __launch_bounds__(256)
tree_scatter_smem_kernel(uint32_t const* __restrict__ tree_of, uint64_t m,
                         uint32_t num_trees, unsigned long long* __restrict__ cursor,
                         uint32_t* __restrict__ perm, uint64_t* __restrict__ out,
                         uint32_t* __restrict__ err) {
  __shared__ uint32_t h[kSmemTrees];
  for (uint32_t i = threadIdx.x; i < num_trees; i += blockDim.x) h[i] = 0;
  __syncthreads();
  uint64_t const per = (m + gridDim.x - 1) / gridDim.x;
  uint64_t const s0 = min(m, blockIdx.x * per), s1 = min(m, s0 + per);
  for (uint64_t q = s0 + threadIdx.x; q < s1; q += blockDim.x) {
    uint32_t const t = tree_of[q];
    if (t < num_trees) atomicAdd(&h[t], 1u);
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < num_trees; i += blockDim.x)
    if (h[i]) h[i] = static_cast<uint32_t>(atomicAdd(&cursor[i], h[i]));  // perm is < 2^32
  __syncthreads();
  for (uint64_t q = s0 + threadIdx.x; q < s1; q += blockDim.x) {
    uint32_t const t = tree_of[q];
    if (t >= num_trees) {
      out[q] = UINT64_MAX;
      atomicOr(err, 2u);
      continue;
    }
    perm[atomicAdd(&h[t], 1u)] = static_cast<uint32_t>(q);
  }
}

// One CTA: tree starts in the tree-ordered batch (cursor) and the work list.
__global__ void __launch_bounds__(kPlanThreads)
tree_plan_kernel(uint32_t const* __restrict__ cnt, uint32_t num_trees,
                 uint64_t* __restrict__ cursor, MultiItem* __restrict__ items,
                 uint32_t* __restrict__ num_items) {
  __shared__ uint64_t warp_q[32];
  __shared__ uint32_t warp_i[32];
  __shared__ uint64_t carry_q;
  __shared__ uint32_t carry_i;
  uint32_t const tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  if (tid == 0) {
    carry_q = 0;
    carry_i = 0;
  }
  __syncthreads();
  for (uint32_t base = 0; base < num_trees; base += kPlanThreads) {
    uint32_t const t = base + tid;
    uint32_t const c = t < num_trees ? cnt[t] : 0u;
    uint32_t const ni = (c + kMultiChunk - 1) / kMultiChunk;
    uint64_t iq = c;
    uint32_t ii = ni;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint64_t const yq = __shfl_up_sync(0xffffffffu, iq, o);
      uint32_t const yi = __shfl_up_sync(0xffffffffu, ii, o);
      if (lane >= static_cast<uint32_t>(o)) {
        iq += yq;
        ii += yi;
      }
    }
    if (lane == 31) {
      warp_q[wid] = iq;
      warp_i[wid] = ii;
    }
    __syncthreads();
    uint64_t bq = carry_q;
    uint32_t bi = carry_i;
    for (uint32_t w = 0; w < wid; ++w) {
      bq += warp_q[w];
      bi += warp_i[w];
    }
    uint64_t const q0 = bq + iq - c;
    uint32_t const i0 = bi + ii - ni;
    if (t < num_trees) {
      cursor[t] = q0;
      for (uint32_t j = 0; j < ni; ++j)
        items[i0 + j] = MultiItem{t, min(kMultiChunk, c - j * kMultiChunk),
                                  q0 + uint64_t(j) * kMultiChunk};
    }
    __syncthreads();
    if (tid == kPlanThreads - 1) {
      carry_q = q0 + c;
      carry_i = i0 + ni;
    }
    __syncthreads();
  }
  if (tid == 0) *num_items = carry_i;
}

// Query numbers into tree order; queries naming no tree get UINT64_MAX.
__global__ void __launch_bounds__(256)
tree_scatter_kernel(uint32_t const* __restrict__ tree_of, uint64_t m,
                    uint32_t num_trees, unsigned long long* __restrict__ cursor,
                    uint32_t* __restrict__ perm, uint64_t* __restrict__ out,
                    uint32_t* __restrict__ err) {
  uint64_t const stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t q = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; q < m;
       q += stride) {
    uint32_t const t = tree_of[q];
    if (t >= num_trees) {
      out[q] = UINT64_MAX;
      atomicOr(err, 2u);
      continue;
    }
    uint32_t const peers = __match_any_sync(__activemask(), t);
    uint32_t const leader = __ffs(peers) - 1;
    unsigned long long base = 0;
    if ((threadIdx.x & 31) == leader) base = atomicAdd(&cursor[t], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    uint32_t const rank = __popc(peers & ((1u << (threadIdx.x & 31)) - 1u));
    perm[base + rank] = static_cast<uint32_t>(q);
  }
}

template <class T>
__global__ void __launch_bounds__(kMultiThreads)
multi_kernel(TreeView const* __restrict__ views,
             MultiItem const* __restrict__ items,
             uint32_t const* __restrict__ num_items_d, uint32_t num_items_h,
             uint32_t const* __restrict__ perm,
             uint8_t const* __restrict__ types,
             MultiRec<T> const* __restrict__ in, uint64_t* __restrict__ out,
             uint32_t* __restrict__ err, uint32_t* queue) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ __align__(8) TreeView tv;
  __shared__ MultiItem it;
  __shared__ uint16_t lists[3][kMultiChunk];
  __shared__ uint32_t list_len[3];
  __shared__ uint32_t next_item;
  uint32_t const tid = threadIdx.x, lane = tid & 31;
  uint32_t const lt = (1u << lane) - 1u;
  uint32_t const n_items = num_items_d ? *num_items_d : num_items_h;
  uint32_t bad = 0;
  // work items from the device queue (or by a fixed stride without one)
  for (uint64_t w = wq_take(queue, &next_item, 0, true); w < n_items;
       w = wq_take(queue, &next_item, w, false)) {
    if (tid == 0) it = items[w];
    if (tid < 3) list_len[tid] = 0;
    __syncthreads();
    MultiItem const item = it;
    {
      uint64_t const* src = reinterpret_cast<uint64_t const*>(views + item.tree);
      uint64_t* dst = reinterpret_cast<uint64_t*>(&tv);
      for (uint32_t i = tid; i < sizeof(TreeView) / 8; i += blockDim.x)
        dst[i] = src[i];
    }
    __syncthreads();
    uint32_t const L = tv.levels;
    ArrayMeta* meta = reinterpret_cast<ArrayMeta*>(smem);
    uint64_t* node_base = reinterpret_cast<uint64_t*>(meta + L);
    {
      uint64_t const* gm = reinterpret_cast<uint64_t const*>(tv.rs.meta);
      uint64_t* sm = reinterpret_cast<uint64_t*>(meta);
      for (uint32_t i = tid; i < L * (sizeof(ArrayMeta) / 8); i += blockDim.x)
        sm[i] = gm[i];
      for (uint32_t i = tid; i <= L; i += blockDim.x) node_base[i] = tv.node_base[i];
    }
    // sort the item's query slots by type (warp ballots)
    for (uint32_t j = tid; j < kMultiChunk; j += blockDim.x) {
      uint32_t ty = 3u;
      uint64_t q = 0;
      if (j < item.count) {
        q = perm ? perm[item.start + j] : item.start + j;
        ty = types[q];
      }
#pragma unroll
      for (uint32_t k = 0; k < 3; ++k) {
        uint32_t const mask = __ballot_sync(0xffffffffu, ty == k);
        if (mask == 0) continue;
        uint32_t pos = 0;
        if (lane == __ffs(mask) - 1) pos = atomicAdd(&list_len[k], __popc(mask));
        pos = __shfl_sync(0xffffffffu, pos, __ffs(mask) - 1);
        if (ty == k) lists[k][pos + __popc(mask & lt)] = static_cast<uint16_t>(j);
      }
      if (ty > 2 && j < item.count) {
        out[q] = UINT64_MAX;
        bad = 1;
      }
    }
    __syncthreads();
    auto slot = [&](uint32_t j) -> uint64_t {
      return perm ? perm[item.start + j] : item.start + j;
    };
    for (uint32_t i = tid; i < list_len[0]; i += blockDim.x) {
      uint64_t const q = slot(lists[0][i]);
      uint64_t const idx = in[q].index;
      out[q] = idx < tv.n ? static_cast<uint64_t>(from_minimal<T>(
                                tv, wt_access(tv, meta, tv.counts, tv.node_ranks,
                                              node_base, idx)))
                          : 0;
    }
    for (uint32_t i = tid; i < list_len[1]; i += blockDim.x) {
      uint64_t const q = slot(lists[1][i]);
      MultiRec<T> const r = in[q];
      uint64_t const sym = to_minimal<T>(tv, r.symbol);
      if (sym >= tv.sigma || r.index > tv.n) {
        out[q] = UINT64_MAX;
        bad = 1;
      } else {
        out[q] = wt_rank(tv, meta, tv.counts, tv.node_ranks, node_base, sym, r.index);
      }
    }
    for (uint32_t i = tid; i < list_len[2]; i += blockDim.x) {
      uint64_t const q = slot(lists[2][i]);
      MultiRec<T> const r = in[q];
      uint64_t const sym = to_minimal<T>(tv, r.symbol);
      if (sym >= tv.sigma || r.index == 0) {
        out[q] = UINT64_MAX;
        bad = 1;
      } else {
        out[q] = wt_select(tv, meta, tv.counts, tv.node_ranks, node_base, sym, r.index);
      }
    }
    __syncthreads();  // tv, meta and lists are reused by the next item
  }
  wq_finish(queue);
  if (bad) atomicOr(err, 1u);
}

// Zero-copy form for the serving engine: work items name a request whose
// descriptor points at the caller's buffers (host memory the GPU reads and
// writes in place when it can access pageable memory); invalid queries set
// the request's error flag.
struct ServeReq {
  uint8_t const* types;
  void const* queries;
  uint64_t* results;
  uint32_t tree, pad;
};
struct ServeItemD {
  uint32_t req, count;
  uint64_t start;
};

template <class T>
__global__ void __launch_bounds__(kMultiThreads)
serve_kernel(TreeView const* __restrict__ views, ServeReq const* __restrict__ reqs,
             ServeItemD const* __restrict__ items, uint32_t n_items,
             uint32_t* __restrict__ req_err) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ __align__(8) TreeView tv;
  __shared__ ServeItemD it;
  __shared__ ServeReq rq;
  __shared__ uint16_t lists[3][kMultiChunk];
  __shared__ uint32_t list_len[3];
  uint32_t const tid = threadIdx.x, lane = tid & 31;
  uint32_t const lt = (1u << lane) - 1u;
  for (uint32_t w = blockIdx.x; w < n_items; w += gridDim.x) {
    if (tid == 0) {
      it = items[w];
      rq = reqs[it.req];
    }
    if (tid < 3) list_len[tid] = 0;
    __syncthreads();
    ServeItemD const item = it;
    uint8_t const* types = rq.types + item.start;
    MultiRec<T> const* in = static_cast<MultiRec<T> const*>(rq.queries) + item.start;
    uint64_t* out = rq.results + item.start;
    {
      uint64_t const* src = reinterpret_cast<uint64_t const*>(views + rq.tree);
      uint64_t* dst = reinterpret_cast<uint64_t*>(&tv);
      for (uint32_t i = tid; i < sizeof(TreeView) / 8; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    uint32_t const L = tv.levels;
    ArrayMeta* meta = reinterpret_cast<ArrayMeta*>(smem);
    uint64_t* node_base = reinterpret_cast<uint64_t*>(meta + L);
    {
      uint64_t const* gm = reinterpret_cast<uint64_t const*>(tv.rs.meta);
      uint64_t* sm = reinterpret_cast<uint64_t*>(meta);
      for (uint32_t i = tid; i < L * (sizeof(ArrayMeta) / 8); i += blockDim.x) sm[i] = gm[i];
      for (uint32_t i = tid; i <= L; i += blockDim.x) node_base[i] = tv.node_base[i];
    }
    uint32_t bad = 0;
    for (uint32_t j = tid; j < kMultiChunk; j += blockDim.x) {
      uint32_t const ty = j < item.count ? types[j] : 3u;
#pragma unroll
      for (uint32_t k = 0; k < 3; ++k) {
        uint32_t const mask = __ballot_sync(0xffffffffu, ty == k);
        if (mask == 0) continue;
        uint32_t pos = 0;
        if (lane == __ffs(mask) - 1) pos = atomicAdd(&list_len[k], __popc(mask));
        pos = __shfl_sync(0xffffffffu, pos, __ffs(mask) - 1);
        if (ty == k) lists[k][pos + __popc(mask & lt)] = static_cast<uint16_t>(j);
      }
      if (ty > 2 && j < item.count) {
        out[j] = UINT64_MAX;
        bad = 1;
      }
    }
    __syncthreads();
    for (uint32_t i = tid; i < list_len[0]; i += blockDim.x) {
      uint32_t const j = lists[0][i];
      uint64_t const idx = in[j].index;
      out[j] = idx < tv.n ? static_cast<uint64_t>(from_minimal<T>(
                                tv, wt_access(tv, meta, tv.counts, tv.node_ranks,
                                              node_base, idx)))
                          : 0;
    }
    for (uint32_t i = tid; i < list_len[1]; i += blockDim.x) {
      uint32_t const j = lists[1][i];
      MultiRec<T> const r = in[j];
      uint64_t const sym = to_minimal<T>(tv, r.symbol);
      if (sym >= tv.sigma || r.index > tv.n) {
        out[j] = UINT64_MAX;
        bad = 1;
      } else {
        out[j] = wt_rank(tv, meta, tv.counts, tv.node_ranks, node_base, sym, r.index);
      }
    }
    for (uint32_t i = tid; i < list_len[2]; i += blockDim.x) {
      uint32_t const j = lists[2][i];
      MultiRec<T> const r = in[j];
      uint64_t const sym = to_minimal<T>(tv, r.symbol);
      if (sym >= tv.sigma || r.index == 0) {
        out[j] = UINT64_MAX;
        bad = 1;
      } else {
        out[j] = wt_select(tv, meta, tv.counts, tv.node_ranks, node_base, sym, r.index);
      }
    }
    if (bad) req_err[item.req] = 1u;  // the same value from every writer
    __syncthreads();  // tv, rq, meta and lists are reused by the next item
  }
}

template <class T>
void launch_serve_typed(TreeView const* views, ServeReq const* reqs,
                        ServeItemD const* items, uint32_t n_items,
                        uint32_t max_levels, uint32_t* req_err, cudaStream_t s) {
  size_t const smem = max_levels * sizeof(ArrayMeta) + (max_levels + 1) * 8;
  thread_local int cached[65] = {};
  int& per_sm = cached[std::min<uint32_t>(max_levels, 64)];
  if (per_sm == 0) {
    EWT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, serve_kernel<T>, kMultiThreads, smem));
    per_sm = std::max(per_sm, 1);
  }
  uint32_t const blocks = static_cast<uint32_t>(std::max<uint64_t>(
      1, std::min<uint64_t>(n_items, uint64_t(per_sm) * sm_count())));
  serve_kernel<T><<<blocks, kMultiThreads, smem, s>>>(views, reqs, items, n_items,
                                                      req_err);
  EWT_LAUNCHED();
}

template <class T>
void launch_multi_typed(TreeView const* d_views, MultiItem const* d_items,
                        uint32_t const* d_num_items, uint32_t h_num_items,
                        uint64_t max_items, uint32_t max_levels,
                        uint32_t const* d_perm, uint8_t const* d_types,
                        void const* d_q, uint64_t* d_out, uint32_t* d_err,
                        uint32_t* d_queue, cudaStream_t s) {
  size_t const smem = max_levels * sizeof(ArrayMeta) + (max_levels + 1) * 8;
  // resident CTAs per SM, looked up once per thread and level count
  thread_local int cached[65] = {};
  int& per_sm = cached[std::min<uint32_t>(max_levels, 64)];
  if (per_sm == 0) {
    EWT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, multi_kernel<T>, kMultiThreads, smem));
    per_sm = std::max(per_sm, 1);
  }
  uint32_t const blocks = static_cast<uint32_t>(std::max<uint64_t>(
      1, std::min<uint64_t>(max_items, uint64_t(per_sm) * sm_count())));
  multi_kernel<T><<<blocks, kMultiThreads, smem, s>>>(
      d_views, d_items, d_num_items, h_num_items, d_perm, d_types,
      static_cast<MultiRec<T> const*>(d_q), d_out, d_err, d_queue);
  EWT_LAUNCHED();
}

void launch_multi(uint32_t elem_size, TreeView const* d_views,
                  MultiItem const* d_items, uint32_t const* d_num_items,
                  uint32_t h_num_items, uint64_t max_items, uint32_t max_levels,
                  uint32_t const* d_perm, uint8_t const* d_types,
                  void const* d_q, uint64_t* d_out, uint32_t* d_err,
                  uint32_t* d_queue, cudaStream_t s) {
  switch (elem_size) {
    case 1: launch_multi_typed<uint8_t>(d_views, d_items, d_num_items, h_num_items, max_items, max_levels, d_perm, d_types, d_q, d_out, d_err, d_queue, s); break;
    case 2: launch_multi_typed<uint16_t>(d_views, d_items, d_num_items, h_num_items, max_items, max_levels, d_perm, d_types, d_q, d_out, d_err, d_queue, s); break;
    case 4: launch_multi_typed<uint32_t>(d_views, d_items, d_num_items, h_num_items, max_items, max_levels, d_perm, d_types, d_q, d_out, d_err, d_queue, s); break;
    default: launch_multi_typed<uint64_t>(d_views, d_items, d_num_items, h_num_items, max_items, max_levels, d_perm, d_types, d_q, d_out, d_err, d_queue, s); break;
  }
}

// Checks the trees of one multi-tree call and uploads their views.
struct ViewSet {
  DevBuf views;
  uint32_t elem_size = 0, max_levels = 0, device = 0;
};
ViewSet upload_views(ewt_tree* const* trees, uint32_t num_trees, cudaStream_t s) {
  EWT_REQUIRE(trees != nullptr && num_trees > 0, EWT_ERR_INVALID_ARGUMENT,
              "no trees given");
  EWT_REQUIRE(num_trees <= kMaxMultiTrees, EWT_ERR_TOO_LARGE,
              "too many trees in one call");
  ViewSet vs;
  std::vector<TreeView> h(num_trees);
  for (uint32_t i = 0; i < num_trees; ++i) {
    EWT_REQUIRE(trees[i] != nullptr, EWT_ERR_INVALID_ARGUMENT, "a tree is null");
    if (i == 0) {
      vs.elem_size = trees[0]->elem_size;
      vs.device = trees[0]->device;
    }
    EWT_REQUIRE(trees[i]->elem_size == vs.elem_size, EWT_ERR_INVALID_ARGUMENT,
                "all trees of one call must have the same symbol size");
    EWT_REQUIRE(static_cast<uint32_t>(trees[i]->device) == vs.device,
                EWT_ERR_INVALID_ARGUMENT, "all trees of one call must be on one GPU");
    h[i] = trees[i]->view;
    vs.max_levels = std::max(vs.max_levels, trees[i]->L);
  }
  vs.views.alloc(num_trees * sizeof(TreeView));
  EWT_CUDA(cudaMemcpyAsync(vs.views.get(), h.data(), num_trees * sizeof(TreeView),
                           cudaMemcpyHostToDevice, s));
  return vs;
}

// The grouped multi-tree batch over device buffers; d_err receives 1 for
// invalid queries and 2 for tree ids >= num_trees.
void multi_device(ViewSet const& vs, uint32_t num_trees, uint32_t const* d_tree_of,
                  uint8_t const* d_types, void const* d_q, uint64_t m,
                  uint64_t* d_out, uint32_t* d_err, cudaStream_t s) {
  EWT_REQUIRE(m < (uint64_t(1) << 32), EWT_ERR_TOO_LARGE,
              "a multi-tree batch holds fewer than 2^32 queries");
  uint64_t const max_items = m / kMultiChunk + num_trees + 1;
  DevBuf cnt((num_trees + 1) * 4), cursor(num_trees * 8),
      items(max_items * sizeof(MultiItem)), nitems(4), perm(std::max<uint64_t>(m, 1) * 4),
      queue(8);
  EWT_CUDA(cudaMemsetAsync(cnt.get(), 0, (num_trees + 1) * 4, s));
  EWT_CUDA(cudaMemsetAsync(queue.get(), 0, 8, s));
  uint32_t const grid = static_cast<uint32_t>(
      std::max<uint64_t>(1, std::min<uint64_t>(ceil_div(m, 256), uint64_t(sm_count()) * 8)));
  PhaseTimer pt(EWT_PHASE_QUERY, s);
  bool const smem_groups = num_trees <= kSmemTrees;
  if (smem_groups)
    tree_hist_smem_kernel<<<grid, 256, 0, s>>>(d_tree_of, m, num_trees, cnt.as<uint32_t>());
  else
    tree_hist_kernel<<<grid, 256, 0, s>>>(d_tree_of, m, num_trees, cnt.as<uint32_t>());
  EWT_LAUNCHED();
  tree_plan_kernel<<<1, kPlanThreads, 0, s>>>(cnt.as<uint32_t>(), num_trees,
                                              cursor.as<uint64_t>(),
                                              items.as<MultiItem>(),
                                              nitems.as<uint32_t>());
  EWT_LAUNCHED();
  if (smem_groups)
    tree_scatter_smem_kernel<<<grid, 256, 0, s>>>(
        d_tree_of, m, num_trees, cursor.as<unsigned long long>(),
        perm.as<uint32_t>(), d_out, d_err);
  else
    tree_scatter_kernel<<<grid, 256, 0, s>>>(
        d_tree_of, m, num_trees, cursor.as<unsigned long long>(),
        perm.as<uint32_t>(), d_out, d_err);
  EWT_LAUNCHED();
  launch_multi(vs.elem_size, vs.views.as<TreeView>(), items.as<MultiItem>(),
               nitems.as<uint32_t>(), 0, max_items, vs.max_levels,
               perm.as<uint32_t>(), d_types, d_q, d_out, d_err,
               work_queue_enabled() ? queue.as<uint32_t>() : nullptr, s);
}

std::mutex g_multi_mu;            // host multi-tree calls share one stream
cudaStream_t g_multi_stream[64] = {};

cudaStream_t multi_stream(uint32_t dev) {
  EWT_REQUIRE(dev < 64, EWT_ERR_INVALID_ARGUMENT, "device index out of range");
  if (!g_multi_stream[dev])
    EWT_CUDA(cudaStreamCreateWithFlags(&g_multi_stream[dev], cudaStreamNonBlocking));
  return g_multi_stream[dev];
}

}  // namespace

// Loads the serving kernels of one symbol size (module loading is lazy,
// and the first launch would otherwise pay for it inside a request).
void prepare_serve_kernels(uint32_t elem_size) {
  cudaFuncAttributes a{};
  switch (elem_size) {
    case 1: EWT_CUDA(cudaFuncGetAttributes(&a, serve_kernel<uint8_t>)); EWT_CUDA(cudaFuncGetAttributes(&a, multi_kernel<uint8_t>)); break;
    case 2: EWT_CUDA(cudaFuncGetAttributes(&a, serve_kernel<uint16_t>)); EWT_CUDA(cudaFuncGetAttributes(&a, multi_kernel<uint16_t>)); break;
    case 4: EWT_CUDA(cudaFuncGetAttributes(&a, serve_kernel<uint32_t>)); EWT_CUDA(cudaFuncGetAttributes(&a, multi_kernel<uint32_t>)); break;
    default: EWT_CUDA(cudaFuncGetAttributes(&a, serve_kernel<uint64_t>)); EWT_CUDA(cudaFuncGetAttributes(&a, multi_kernel<uint64_t>)); break;
  }
}

// Zero-copy work-list launch of the serving engine (see ServeReq).
void launch_serve_items(uint32_t elem_size, TreeView const* d_views,
                        void const* reqs, void const* items, uint32_t num_items,
                        uint32_t max_levels, uint32_t* req_err, cudaStream_t s) {
  if (num_items == 0) return;
  auto const* r = static_cast<ServeReq const*>(reqs);
  auto const* it = static_cast<ServeItemD const*>(items);
  switch (elem_size) {
    case 1: launch_serve_typed<uint8_t>(d_views, r, it, num_items, max_levels, req_err, s); break;
    case 2: launch_serve_typed<uint16_t>(d_views, r, it, num_items, max_levels, req_err, s); break;
    case 4: launch_serve_typed<uint32_t>(d_views, r, it, num_items, max_levels, req_err, s); break;
    default: launch_serve_typed<uint64_t>(d_views, r, it, num_items, max_levels, req_err, s); break;
  }
}

// Work-list launch used by the serving engine: items are already grouped.
void launch_multi_items(uint32_t elem_size, TreeView const* d_views,
                        void const* d_items, uint32_t num_items,
                        uint32_t max_levels, uint8_t const* d_types,
                        void const* d_q, uint64_t* d_out, uint32_t* d_err,
                        cudaStream_t s) {
  if (num_items == 0) return;
  launch_multi(elem_size, d_views, static_cast<MultiItem const*>(d_items),
               nullptr, num_items, num_items, max_levels, nullptr, d_types, d_q,
               d_out, d_err, nullptr, s);
}

}  // namespace ewt

using namespace ewt;

extern "C" int ewt_mixed_multi_device(ewt_tree* const* trees, uint32_t num_trees,
                                      const uint32_t* d_tree_of,
                                      const uint8_t* d_types, const void* d_queries,
                                      uint64_t m, uint64_t* d_results,
                                      uint32_t* d_err, void* stream) {
  return run_guarded([&] {
    if (m == 0) return;
    EWT_REQUIRE(d_tree_of && d_types && d_queries && d_results && d_err,
                EWT_ERR_INVALID_ARGUMENT, "null device buffer");
    EWT_REQUIRE(trees != nullptr && trees[0] != nullptr, EWT_ERR_INVALID_ARGUMENT,
                "no trees given");
    DeviceGuard g(trees[0]->device);
    cudaStream_t const s = static_cast<cudaStream_t>(stream);
    AllocStream as(s);
    ViewSet const vs = upload_views(trees, num_trees, s);
    multi_device(vs, num_trees, d_tree_of, d_types, d_queries, m, d_results, d_err, s);
  });
}

extern "C" int ewt_mixed_multi(ewt_tree* const* trees, uint32_t num_trees,
                               const uint32_t* tree_of, const uint8_t* types,
                               const void* queries, uint64_t m, uint64_t* results) {
  return run_guarded([&] {
    if (m == 0) return;
    EWT_REQUIRE(tree_of && types && queries && results, EWT_ERR_INVALID_ARGUMENT,
                "null query, type, tree or result buffer");
    EWT_REQUIRE(trees != nullptr && trees[0] != nullptr, EWT_ERR_INVALID_ARGUMENT,
                "no trees given");
    std::lock_guard<std::mutex> lk(g_multi_mu);
    DeviceGuard g(trees[0]->device);
    cudaStream_t const s = multi_stream(static_cast<uint32_t>(trees[0]->device));
    AllocStream as(s);
    ViewSet const vs = upload_views(trees, num_trees, s);
    DevBuf d_tree(m * 4), d_types(m), d_q(m * 16), d_out(m * 8), d_err(4);
    EWT_CUDA(cudaMemsetAsync(d_err.get(), 0, 4, s));
    EWT_CUDA(cudaMemcpyAsync(d_tree.get(), tree_of, m * 4, cudaMemcpyDefault, s));
    EWT_CUDA(cudaMemcpyAsync(d_types.get(), types, m, cudaMemcpyDefault, s));
    EWT_CUDA(cudaMemcpyAsync(d_q.get(), queries, m * 16, cudaMemcpyDefault, s));
    multi_device(vs, num_trees, d_tree.as<uint32_t>(), d_types.as<uint8_t>(),
                 d_q.get(), m, d_out.as<uint64_t>(), d_err.as<uint32_t>(), s);
    EWT_CUDA(cudaMemcpyAsync(results, d_out.get(), m * 8, cudaMemcpyDefault, s));
    uint32_t bad = 0;
    EWT_CUDA(cudaMemcpyAsync(&bad, d_err.get(), 4, cudaMemcpyDeviceToHost, s));
    EWT_CUDA(cudaStreamSynchronize(s));
    EWT_REQUIRE(!(bad & 2), EWT_ERR_QUERY,
                "the batch named trees that were not given (their results are "
                "UINT64_MAX)");
    EWT_REQUIRE(!bad, EWT_ERR_QUERY,
                "the batch held invalid queries (their results are UINT64_MAX)");
  });
}

extern "C" int ewt_build_batch(const void* const* texts, const uint64_t* lengths,
                               uint32_t count, int elem_size,
                               const void* const* alphabets,
                               const uint64_t* sigmas, int gpu_index,
                               ewt_tree** out, int* statuses) {
  return run_guarded([&] {
    EWT_REQUIRE(texts && lengths && out && count > 0, EWT_ERR_INVALID_ARGUMENT,
                "texts, lengths and out must be given");
    for (uint32_t i = 0; i < count; ++i) out[i] = nullptr;
    {
      // Grow the library pool once for the whole batch (about four bytes
      // of trees and build scratch per text byte): the builds then carve
      // their buffers out of it instead of each growing the pool.
      DeviceGuard g(gpu_index);
      uint64_t need = 0;
      for (uint32_t i = 0; i < count; ++i)
        need += lengths[i] * uint64_t(elem_size > 0 ? elem_size : 1) * 4 + (uint64_t(2) << 20);
      size_t free_b = 0, total_b = 0;
      if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && need < free_b / 2) {
        void* p = nullptr;
        if (cudaMallocFromPoolAsync(&p, need, lib_pool(), nullptr) == cudaSuccess) {
          cudaFreeAsync(p, nullptr);
          cudaStreamSynchronize(nullptr);
        }
      }
      (void)cudaGetLastError();  // best effort
    }
    std::mutex mu;
    int first_status = EWT_OK;
    std::string first_msg;
    {  // device-resident texts: ordered after the caller's work once
      DeviceGuard g(gpu_index);
      EWT_CUDA(cudaDeviceSynchronize());
    }
    // Short texts with a given power-of-two minimal alphabet go to segmented
    // group builds (batch_build.cu), one per alphabet size, on this thread;
    // the others are built one per text by the workers meanwhile.
    std::vector<std::vector<uint32_t>> small(13);
    std::vector<uint32_t> rest;
    for (uint32_t i = 0; i < count; ++i) {
      void const* a = alphabets ? alphabets[i] : nullptr;
      uint64_t const sg = sigmas ? sigmas[i] : 0;
      if (texts[i] && small_batch_eligible(lengths[i], elem_size, a, sg)) {
        uint32_t L = 0;
        while ((uint64_t(1) << L) < sg) ++L;
        small[L].push_back(i);
      } else {
        rest.push_back(i);
      }
    }
    std::atomic<size_t> next{0};
    auto build_one = [&](uint32_t i) {
      int const st = ewt_build(texts[i], lengths[i], elem_size,
                               alphabets ? alphabets[i] : nullptr,
                               sigmas ? sigmas[i] : 0, gpu_index, &out[i]);
      if (statuses) statuses[i] = st;
      if (st != EWT_OK) {
        std::lock_guard<std::mutex> lk(mu);
        if (first_status == EWT_OK) {
          first_status = st;
          first_msg = "text " + std::to_string(i) + ": " + ewt_last_error();
        }
      }
    };
    auto work = [&] {
      set_texts_synchronized(true);
      set_batch_member(true);
      for (size_t j = next++; j < rest.size(); j = next++) build_one(rest[j]);
      set_texts_synchronized(false);
      set_batch_member(false);
    };
    uint32_t const hw = std::max(1u, std::thread::hardware_concurrency());
    uint32_t const workers =
        std::min<uint32_t>({static_cast<uint32_t>(rest.size()), kBuildWorkers, hw});
    std::vector<std::thread> pool;
    for (uint32_t w = 0; w < workers; ++w) pool.emplace_back(work);
    std::vector<uint32_t> retry;  // texts of groups that failed as a group
    for (uint32_t L = 0; L < small.size(); ++L) {
      if (small[L].empty()) continue;
      try {
        build_small_texts(texts, lengths, small[L], elem_size, L, gpu_index, out);
        if (statuses)
          for (uint32_t i : small[L]) statuses[i] = EWT_OK;
      } catch (...) {
        for (uint32_t i : small[L]) {
          if (out[i]) ewt_free(out[i]);
          out[i] = nullptr;
          retry.push_back(i);
        }
      }
    }
    for (auto& th : pool) th.join();
    // one by one, so that each failing text reports its own status
    set_texts_synchronized(true);
    for (uint32_t i : retry) build_one(i);
    set_texts_synchronized(false);
    if (first_status != EWT_OK) throw Error(first_status, first_msg);
  });
}
