/*
 * Drop-in ecl::WaveletTree<T> of the GB300 wavelet tree.
 *
 * Keeps the public API of include/ecl_wavelet/tree/wavelet_tree.cuh in
 * mfranzreb/ECL_wavelet:
 *   - WaveletTree(data, n, std::vector<T>&& alphabet, GPU_index) builds the
 *     tree (an empty alphabet means "detect it"); throws
 *     std::runtime_error("Not enough memory available for the wavelet
 *     tree.") when the GPU runs out of memory;
 *   - access / rank / select host batches return a std::span aliasing an
 *     internal pinned pool, valid until the next call of the same kind;
 *   - copies are shallow and non-owning, so a WaveletTree<T> can be passed
 *     by value into a kernel and queried there with deviceAccess /
 *     deviceRank / deviceSelect (symbols in the minimal alphabet 0..s-1,
 *     as in the reference's device API);
 *   - the getters and createMinimalCodes.
 * The host side runs over the C ABI of libewt.so (ewt.h); the device side
 * is inline (ecl_wavelet/detail/device_ops.cuh) and identical to the code
 * of the library's own kernels.
 *
 * Differences from the reference, all documented in ewt.h: rank/select do
 * not rewrite the caller's query symbols in place; invalid queries (select
 * with k == 0, rank with index > n) raise std::runtime_error after the
 * batch instead of tripping an assert; access at index >= n yields T(0).
 */
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <span>
#include <stdexcept>
#include <string>
#include <vector>

#include "ewt.h"
#include "ecl_wavelet/bitarray/rank_select.cuh"
#include "ecl_wavelet/utils/utils.cuh"

namespace ecl {

template <typename T>
class WaveletTree {
  static_assert(std::is_integral<T>::value && std::is_unsigned<T>::value,
                "T must be an unsigned integral type");

 public:
  struct Code {
    uint8_t len_;
    T code_;
  };

  RankSelect rank_select_;

  WaveletTree() = default;

  __host__ WaveletTree(T const* data, size_t data_size,
                       std::vector<T>&& alphabet, uint32_t GPU_index)
      : is_copy_(false) {
    int const st = ewt_build(data, data_size, sizeof(T),
                             alphabet.empty() ? nullptr : alphabet.data(),
                             alphabet.size(), static_cast<int>(GPU_index),
                             &handle_);
    if (st == EWT_ERR_OUT_OF_MEMORY)
      throw std::runtime_error(
          "Not enough memory available for the wavelet tree.");
    if (st != EWT_OK) throw std::runtime_error(ewt_last_error());
    init_from_handle();
  }

  /* Shallow, non-owning copy (what a kernel receives). */
  __host__ WaveletTree(WaveletTree const& o)
      : rank_select_(o.rank_select_),
        handle_(o.handle_),
        view_(o.view_),
        host_(o.host_),
        is_copy_(true) {}
  WaveletTree& operator=(WaveletTree const&) = delete;
  WaveletTree(WaveletTree&&) = delete;
  __host__ WaveletTree& operator=(WaveletTree&& o) {
    if (this != &o) {
      release();
      handle_ = o.handle_;
      view_ = o.view_;
      host_ = o.host_;
      is_copy_ = o.is_copy_;
      rank_select_ = RankSelect(view_.rs, host_ ? host_->level_bits.data()
                                                : nullptr);
      o.is_copy_ = true;
    }
    return *this;
  }
  __host__ ~WaveletTree() { release(); }

  /* ---- host batches --------------------------------------------------- */
  __host__ std::span<T> access(size_t* indices, size_t const num_indices) {
    T* out = pool<T>(host_->access_pool, host_->access_cap, num_indices);
    check(ewt_access(handle_, reinterpret_cast<uint64_t const*>(indices),
                     num_indices, out));
    return std::span<T>(out, num_indices);
  }
  __host__ std::span<size_t> rank(RankSelectQuery<T>* queries,
                                  size_t const num_queries) {
    size_t* out = pool<size_t>(host_->rank_pool, host_->rank_cap, num_queries);
    check(ewt_rank(handle_, queries, num_queries,
                   reinterpret_cast<uint64_t*>(out)));
    return std::span<size_t>(out, num_queries);
  }
  __host__ std::span<size_t> select(RankSelectQuery<T>* queries,
                                    size_t const num_queries) {
    size_t* out =
        pool<size_t>(host_->select_pool, host_->select_cap, num_queries);
    check(ewt_select(handle_, queries, num_queries,
                     reinterpret_cast<uint64_t*>(out)));
    return std::span<size_t>(out, num_queries);
  }

  /* ---- device queries (symbols in the minimal alphabet) ---------------
   * ThreadsPerQuery is accepted as in the reference; every lane walks the
   * tree on its own (one 32-byte block read per group level, served once for
   * lanes reading the same address), so any group size gives the same
   * answer in every lane.  RankSelect::rank / select (rank_select_) do split
   * a query over NumThreads lanes. */
  template <int ThreadsPerQuery>
  __device__ T deviceAccess(size_t index, bool /*is_pow_two*/,
                            size_t* counts = nullptr,
                            size_t* /*offsets*/ = nullptr,
                            size_t* ranks = nullptr) {
    static_assert(ThreadsPerQuery > 0 && ThreadsPerQuery <= 32 &&
                      32 % ThreadsPerQuery == 0,
                  "ThreadsPerQuery must divide 32");
    return static_cast<T>(detail::wt_access(
        view_, view_.rs.meta, counts_or(counts), ranks_or(ranks),
        view_.node_base, index));
  }
  template <int ThreadsPerQuery>
  __device__ size_t deviceRank(RankSelectQuery<T> const& q,
                               bool /*is_pow_two*/, size_t* counts = nullptr,
                               size_t* /*offsets*/ = nullptr,
                               size_t* ranks = nullptr) {
    static_assert(ThreadsPerQuery > 0 && ThreadsPerQuery <= 32 &&
                      32 % ThreadsPerQuery == 0,
                  "ThreadsPerQuery must divide 32");
    return detail::wt_rank(view_, view_.rs.meta, counts_or(counts),
                           ranks_or(ranks), view_.node_base, q.symbol_,
                           q.index_);
  }
  template <int ThreadsPerQuery>
  __device__ size_t deviceSelect(RankSelectQuery<T> const& q,
                                 bool /*is_pow_two*/,
                                 size_t* ranks = nullptr) {
    static_assert(ThreadsPerQuery > 0 && ThreadsPerQuery <= 32 &&
                      32 % ThreadsPerQuery == 0,
                  "ThreadsPerQuery must divide 32");
    return detail::wt_select(view_, view_.rs.meta, view_.counts,
                             ranks_or(ranks), view_.node_base, q.symbol_,
                             q.index_);
  }

  /* ---- getters ---------------------------------------------------------- */
  __host__ __device__ size_t getAlphabetSize() const { return view_.sigma; }
  __host__ std::vector<T> const& getAlphabet() const { return host_->alphabet; }
  __host__ __device__ uint8_t getNumLevels() const {
    return static_cast<uint8_t>(view_.levels);
  }
  __host__ __device__ size_t getCounts(size_t i) const {
#ifdef __CUDA_ARCH__
    return view_.counts[i];
#else
    return host_->counts[i];
#endif
  }
  __host__ __device__ size_t getTotalAppearances(size_t i) const {
    size_t const end = (i + 1 == view_.sigma) ? view_.n : getCounts(i + 1);
    return end - getCounts(i);
  }
  __host__ __device__ bool isMinAlphabet() const { return view_.is_min; }
  __host__ __device__ T getCodesStart() const {
    return static_cast<T>(view_.codes_start);
  }
  template <bool IsPowTwo>
  __device__ T getNodePosAtLevel(T symbol, uint8_t const level) const {
    return static_cast<T>(
        detail::node_index(view_, view_.node_base, symbol, level) -
        view_.node_base[level]);
  }
  __device__ size_t getPrecomputedRank(T const i) const {
    return view_.node_ranks[i];
  }
  /* Overwrites node rank i, the value getPrecomputedRank(i) returns and the
   * walks over binary levels read (walks over group levels use their own
   * per-node digit counts). */
  __device__ void setPrecomputedRank(T const i, size_t const rank) {
    const_cast<uint64_t*>(view_.node_ranks)[i] = rank;
  }
  __device__ T getNumNodesAtLevel(uint8_t const level) const {
    return static_cast<T>(view_.nodes_at_level[level]);
  }
  __host__ __device__ detail::TreeView const& view() const { return view_; }
  __host__ ewt_tree* handle() const { return handle_; }

  /* Shortened codes of the last symbols when the alphabet size is not a
   * power of two (createMinimalCodes): the library's own codes, the ones
   * its builds use. */
  __host__ static std::vector<Code> createMinimalCodes(
      std::vector<T> const& alphabet) {
    uint64_t const sigma = alphabet.size();
    if (sigma < 2 || utils::isPowTwo<uint64_t>(sigma)) return {};
    uint64_t count = 0;
    if (ewt_minimal_codes(sigma, nullptr, nullptr, 0, &count) != EWT_OK)
      throw std::runtime_error(ewt_last_error());
    std::vector<uint64_t> len(count), code(count);
    ewt_minimal_codes(sigma, len.data(), code.data(), count, &count);
    std::vector<Code> out(count);
    for (uint64_t i = 0; i < count; ++i)
      out[i] = Code{static_cast<uint8_t>(len[i]), static_cast<T>(code[i])};
    return out;
  }

  /* Upper bound of the device bytes a build of data_size symbols over
   * alphabet_size symbols holds at its peak (the finished tree included);
   * num_levels and num_codes follow from the alphabet size here. */
  __host__ static size_t getNeededGPUMemory(size_t const data_size,
                                            size_t const alphabet_size,
                                            uint8_t const /*num_levels*/,
                                            T const /*num_codes*/) {
    uint64_t b = 0;
    ewt_needed_memory(EWT_MEM_TREE, data_size, sizeof(T), alphabet_size, &b);
    return b;
  }

 private:
  struct HostState {
    std::vector<T> alphabet;
    std::vector<size_t> counts;
    std::vector<uint64_t> level_bits;
    T* access_pool = nullptr;
    size_t* rank_pool = nullptr;
    size_t* select_pool = nullptr;
    size_t access_cap = 0, rank_cap = 0, select_cap = 0;
  };

  template <class P>
  static P* pool(P*& p, size_t& cap, size_t need) {
    if (need > cap) {
      if (p) cudaFreeHost(p);
      p = nullptr;
      if (cudaHostAlloc(reinterpret_cast<void**>(&p), need * sizeof(P),
                        cudaHostAllocPortable) != cudaSuccess) {
        cap = 0;
        throw std::runtime_error("pinned result pool allocation failed");
      }
      cap = need;
    }
    return p;
  }

  static void check(int st) {
    if (st == EWT_ERR_OUT_OF_MEMORY)
      throw std::runtime_error(
          "Not enough GPU memory available for the queries.");
    if (st != EWT_OK) throw std::runtime_error(ewt_last_error());
  }

  __host__ void init_from_handle() {
    ewt_get_device_view(handle_, &view_, sizeof(view_));
    host_ = new HostState();
    ewt_info info;
    ewt_get_info(handle_, &info);
    std::vector<uint64_t> buf(info.sigma);
    uint64_t size = 0;
    ewt_export(handle_, EWT_EXP_ALPHABET, 0, buf.data(), buf.size() * 8, &size);
    host_->alphabet.assign(buf.begin(), buf.end());
    ewt_export(handle_, EWT_EXP_COUNTS, 0, buf.data(), buf.size() * 8, &size);
    host_->counts.assign(buf.begin(), buf.end());
    host_->level_bits.resize(info.levels);
    ewt_export(handle_, EWT_EXP_LEVEL_SIZES, 0, host_->level_bits.data(),
               info.levels * 8, &size);
    rank_select_ = RankSelect(view_.rs, host_->level_bits.data());
  }

  __device__ uint64_t const* counts_or(size_t* c) const {
    return c ? reinterpret_cast<uint64_t const*>(c) : view_.counts;
  }
  __device__ uint64_t const* ranks_or(size_t* r) const {
    return r ? reinterpret_cast<uint64_t const*>(r) : view_.node_ranks;
  }

  __host__ void release() {
    if (!is_copy_) {
      if (handle_) ewt_free(handle_);
      if (host_) {
        if (host_->access_pool) cudaFreeHost(host_->access_pool);
        if (host_->rank_pool) cudaFreeHost(host_->rank_pool);
        if (host_->select_pool) cudaFreeHost(host_->select_pool);
        delete host_;
      }
    }
    handle_ = nullptr;
    host_ = nullptr;
    is_copy_ = true;
  }

  ewt_tree* handle_ = nullptr;
  detail::TreeView view_{};
  HostState* host_ = nullptr;
  bool is_copy_ = true;
};

/* Free kernels with the reference's names: one thread per query over
 * device-resident queries (the library's own batch kernels are faster and
 * are what WaveletTree::access/rank/select use). */
template <typename T, int ThreadsPerQuery = 1>
__global__ void accessKernel(WaveletTree<T> tree, size_t* const indices,
                             size_t const num_indices, T* results) {
  size_t const stride = size_t(gridDim.x) * blockDim.x;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
       i < num_indices; i += stride) {
    if (indices[i] >= tree.view().n) continue;
    results[i] = tree.template deviceAccess<ThreadsPerQuery>(indices[i], false);
  }
}

template <typename T, int ThreadsPerQuery = 1>
__global__ void rankKernel(WaveletTree<T> tree,
                           RankSelectQuery<T>* const queries,
                           size_t const num_queries, size_t* const results) {
  size_t const stride = size_t(gridDim.x) * blockDim.x;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
       i < num_queries; i += stride)
    results[i] = tree.template deviceRank<ThreadsPerQuery>(queries[i], false);
}

template <typename T, int ThreadsPerQuery = 1>
__global__ void selectKernel(WaveletTree<T> tree,
                             RankSelectQuery<T>* const queries,
                             size_t const num_queries, size_t* const results) {
  size_t const stride = size_t(gridDim.x) * blockDim.x;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
       i < num_queries; i += stride)
    results[i] = tree.template deviceSelect<ThreadsPerQuery>(queries[i], false);
}

}  // namespace ecl
