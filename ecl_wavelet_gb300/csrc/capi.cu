// extern "C" entry points of libewt.so (declared in include/ewt.h).
//
// Every entry point converts the library's internal exceptions into an int
// status exactly once and records the message for ewt_last_error().  Host
// batch calls serialise on a per-object mutex because they share scratch
// buffers (the reference's host API is not thread-safe at all,
// wavelet_tree.cuh:80 and :1025-1027).
#include <algorithm>
#include <cstring>
#include <memory>
#include <new>
#include <string>

#ifdef __linux__
#include <sys/mman.h>
#include <unistd.h>
#endif

#include "internal.cuh"

namespace ewt {

cudaMemPool_t lib_pool() {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  int dev = 0;
  EWT_CUDA(cudaGetDevice(&dev));
  EWT_REQUIRE(dev >= 0 && dev < 64, EWT_ERR_INVALID_ARGUMENT, "device index out of range");
  std::lock_guard<std::mutex> lock(mu);
  if (!pools[dev]) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    EWT_CUDA(cudaMemPoolCreate(&pools[dev], &props));
    uint64_t keep = UINT64_MAX;
    EWT_CUDA(cudaMemPoolSetAttribute(pools[dev], cudaMemPoolAttrReleaseThreshold, &keep));
    // A block freed on one stream is handed to another stream only once the
    // free has completed, never with an inserted wait on the first stream:
    // builds and query batches on different streams (a batch build runs
    // one stream per text) must not serialise through reused blocks.
    int no = 0;
    EWT_CUDA(cudaMemPoolSetAttribute(
        pools[dev], cudaMemPoolReuseAllowInternalDependencies, &no));
  }
  return pools[dev];
}

namespace {
thread_local std::string g_last_error;
std::atomic<uint64_t> g_launches{0};

template <class F>
int guarded(F&& f) {
  try {
    f();
    g_last_error.clear();
    return EWT_OK;
  } catch (Error const& e) {
    g_last_error = e.what();
    return e.status;
  } catch (std::bad_alloc const&) {
    g_last_error = "host allocation failed";
    return EWT_ERR_OUT_OF_MEMORY;
  } catch (std::exception const& e) {
    g_last_error = e.what();
    return EWT_ERR_CUDA;
  }
}

// Whether kernels on `dev` can read and write pageable host memory
// (address translation through the host's page tables); looked up once.
bool pageable_access(int dev) {
  static std::mutex mu;
  static int cached[64];
  static bool init = false;
  std::lock_guard<std::mutex> lk(mu);
  if (!init) {
    for (int& c : cached) c = -1;
    init = true;
  }
  if (dev < 0 || dev >= 64) return false;
  if (cached[dev] < 0) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
      (void)cudaGetLastError();
      v = 0;
    }
    cached[dev] = v == 1 ? 1 : 0;
  }
  return cached[dev] == 1;
}

// Result buffers the GPU will write in place: pageable pages that were never
// touched would be populated one GPU-initiated fault at a time (tens of
// times slower than the batch itself), so a buffer whose first or last page
// is not resident is populated from the host first.  Pinned or registered
// memory, and buffers already in use, are left alone.
void populate_for_write(void* p, size_t bytes) {
#ifdef __linux__
#ifndef MADV_POPULATE_WRITE
#define MADV_POPULATE_WRITE 23
#endif
  if (!p || bytes == 0) return;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return;
  }
  if (a.type != cudaMemoryTypeUnregistered) return;
  uintptr_t const page = static_cast<uintptr_t>(sysconf(_SC_PAGESIZE));
  uintptr_t const b = reinterpret_cast<uintptr_t>(p) & ~(page - 1);
  uintptr_t const e = reinterpret_cast<uintptr_t>(p) + bytes;
  uintptr_t const last = (e - 1) & ~(page - 1);
  unsigned char r0 = 0, r1 = 0;
  if (mincore(reinterpret_cast<void*>(b), 1, &r0) == 0 &&
      mincore(reinterpret_cast<void*>(last), 1, &r1) == 0 && (r0 & 1) && (r1 & 1))
    return;
  (void)madvise(reinterpret_cast<void*>(b), e - b, MADV_POPULATE_WRITE);
#else
  (void)p;
  (void)bytes;
#endif
}

// Largest batch moved through the device scratch in one piece.
constexpr uint64_t kChunk = uint64_t(1) << 25;
// Host batches from this size on run pipelined (QueryPipe).
constexpr uint64_t kPipeMin = uint64_t(1) << 21;

void ensure(DevBuf& b, size_t& cap, size_t bytes) {
  if (bytes <= cap && b.get()) return;
  b.alloc(bytes);
  cap = bytes;
}

// Reads and clears the tree's invalid-query word.
int take_query_status(DevBuf& err, cudaStream_t s) {
  uint32_t e = 0;
  EWT_CUDA(cudaMemcpyAsync(&e, err.get(), 4, cudaMemcpyDeviceToHost, s));
  EWT_CUDA(cudaMemsetAsync(err.get(), 0, 4, s));
  EWT_CUDA(cudaStreamSynchronize(s));
  return e ? EWT_ERR_QUERY : EWT_OK;
}

__global__ void mask_tails_kernel(uint32_t* words, ArrayMeta const* meta,
                                  uint32_t count) {
  uint32_t const a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= count) return;
  ArrayMeta const m = meta[a];
  if (m.bits % 32)
    words[m.word_off + m.bits / 32] &= (1u << (m.bits % 32)) - 1u;
}

// Bits past each array's end -- in its last word and in the padding words
// up to the next 32-word boundary -- set to zero (arrays filled by callers).
__global__ void clear_tails_kernel(uint32_t* words, ArrayMeta const* meta,
                                   uint32_t count) {
  uint32_t const a = blockIdx.x;
  if (a >= count) return;
  ArrayMeta const m = meta[a];
  uint64_t const w = (m.bits + 31) / 32;
  uint64_t const padded = (w + 31) / 32 * 32;
  uint32_t const t = threadIdx.x;  // 32 threads
  if (t == 0 && m.bits % 32)
    words[m.word_off + m.bits / 32] &= (1u << (m.bits % 32)) - 1u;
  if (w + t < padded) words[m.word_off + w + t] = 0u;
}

}  // namespace

namespace {
std::atomic<bool> g_work_queue{true};
}  // namespace
bool work_queue_enabled() { return g_work_queue.load(std::memory_order_relaxed); }

namespace {
std::atomic<bool> g_timing{false};
std::mutex g_timing_mu;
ewt_phase_times g_times{};
}  // namespace

bool timing_enabled() { return g_timing.load(std::memory_order_relaxed); }
void add_phase_time(int phase, double ms) {
  if (phase < 0 || phase >= EWT_NUM_PHASES) return;
  std::lock_guard<std::mutex> lk(g_timing_mu);
  g_times.ms[phase] += ms;
  g_times.launches[phase] += 1;
}

void set_last_error(std::string const& msg) { g_last_error = msg; }
void count_launch(uint64_t k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

}  // namespace ewt

uint64_t ewt_tree::device_bytes() const {
  return (shared_store ? rs_share_bytes : rs.device_bytes()) + groups.bytes() +
         counts_d.bytes() + ranks_d.bytes() +
         node_base_d.bytes() + nodes_at_level_d.bytes() + code_len_d.bytes() +
         code_bits_d.bytes() + alphabet_d.bytes() + err_d.bytes();
}

using namespace ewt;

namespace {

// Host batch: copy queries in, launch, copy results out, chunk by chunk.
template <class Launch>
int host_batch(ewt_tree* t, void const* in, size_t in_rec, uint8_t const* types,
               uint64_t m, void* out, size_t out_rec, Launch&& launch) {
  return guarded([&] {
    EWT_REQUIRE(t != nullptr, EWT_ERR_INVALID_ARGUMENT, "tree is null");
    if (m == 0) return;
    EWT_REQUIRE(in != nullptr && out != nullptr, EWT_ERR_INVALID_ARGUMENT,
                "null query or result buffer");
    std::lock_guard<std::mutex> lk(t->query_mu);
    DeviceGuard g(t->device);
    AllocStream as(t->stream);
    cudaStream_t s = t->stream;
    if (m >= kPipeMin) {
      // large batches: copies in and out overlap the kernels chunk by chunk
      // (copy engines reach the C2C bandwidth; the kernel then works on
      // device memory only)
      populate_for_write(out, m * out_rec);
      QueryPipe& P = t->pipe;
      P.init();
      uint64_t const chunk = std::max<uint64_t>(kPipeMin / 4, ceil_div(m, 8));
      for (int x = 0; x < 2; ++x) {  // allocated on s, before the copy streams start
        ensure(P.in[x], P.cap_in[x], chunk * in_rec);
        ensure(P.out[x], P.cap_out[x], chunk * out_rec);
        if (types) ensure(P.types[x], P.cap_types[x], chunk);
      }
      EWT_CUDA(cudaEventRecord(P.start, s));
      EWT_CUDA(cudaStreamWaitEvent(P.s_in, P.start, 0));
      uint64_t i = 0;
      for (uint64_t b = 0; b < m; b += chunk, ++i) {
        int const x = static_cast<int>(i & 1);
        uint64_t const k = std::min(chunk, m - b);
        if (i >= 2) EWT_CUDA(cudaStreamWaitEvent(P.s_in, P.k_done[x], 0));
        EWT_CUDA(cudaMemcpyAsync(P.in[x].get(), static_cast<char const*>(in) + b * in_rec,
                                 k * in_rec, cudaMemcpyDefault, P.s_in));
        if (types)
          EWT_CUDA(cudaMemcpyAsync(P.types[x].get(), types + b, k, cudaMemcpyDefault,
                                   P.s_in));
        EWT_CUDA(cudaEventRecord(P.in_done[x], P.s_in));
        EWT_CUDA(cudaStreamWaitEvent(s, P.in_done[x], 0));
        if (i >= 2) EWT_CUDA(cudaStreamWaitEvent(s, P.out_done[x], 0));
        launch(P.types[x].as<uint8_t>(), P.in[x].get(), k, P.out[x].get(), s);
        EWT_CUDA(cudaEventRecord(P.k_done[x], s));
        EWT_CUDA(cudaStreamWaitEvent(P.s_out, P.k_done[x], 0));
        EWT_CUDA(cudaMemcpyAsync(static_cast<char*>(out) + b * out_rec, P.out[x].get(),
                                 k * out_rec, cudaMemcpyDefault, P.s_out));
        EWT_CUDA(cudaEventRecord(P.out_done[x], P.s_out));
      }
      EWT_CUDA(cudaStreamWaitEvent(s, P.out_done[(i - 1) & 1], 0));
      int const st = take_query_status(t->err_d, s);
      if (st != EWT_OK)
        throw Error(st, "the batch held invalid queries (their results are "
                        "UINT64_MAX)");
      return;
    }
    if (pageable_access(t->device)) {
      // the kernel reads the caller's queries and writes its results in
      // place (host page tables): no staging copies
      populate_for_write(out, m * out_rec);
      launch(types, in, m, out, s);
      int const st = take_query_status(t->err_d, s);
      if (st != EWT_OK)
        throw Error(st, "the batch held invalid queries (their results are "
                        "UINT64_MAX)");
      return;
    }
    QueryScratch& sc = t->scratch;
    uint64_t const chunk = std::min(m, kChunk);
    ensure(sc.in, sc.in_cap, chunk * in_rec);
    ensure(sc.out, sc.out_cap, chunk * out_rec);
    if (types) ensure(sc.types, sc.types_cap, chunk);
    for (uint64_t b = 0; b < m; b += chunk) {
      uint64_t const k = std::min(chunk, m - b);
      EWT_CUDA(cudaMemcpyAsync(sc.in.get(),
                               static_cast<char const*>(in) + b * in_rec,
                               k * in_rec, cudaMemcpyDefault, s));
      if (types)
        EWT_CUDA(cudaMemcpyAsync(sc.types.get(), types + b, k,
                                 cudaMemcpyDefault, s));
      launch(sc.types.as<uint8_t>(), sc.in.get(), k, sc.out.get(), s);
      EWT_CUDA(cudaMemcpyAsync(static_cast<char*>(out) + b * out_rec,
                               sc.out.get(), k * out_rec, cudaMemcpyDefault,
                               s));
    }
    int const st = take_query_status(t->err_d, s);
    if (st != EWT_OK)
      throw Error(st, "the batch held invalid queries (their results are "
                      "UINT64_MAX)");
  });
}

template <class Launch>
int rs_host_batch(ewt_rs* r, uint64_t const* in, uint64_t m, uint64_t* out,
                  Launch&& launch) {
  return guarded([&] {
    EWT_REQUIRE(r != nullptr, EWT_ERR_INVALID_ARGUMENT, "rank/select is null");
    if (m == 0) return;
    EWT_REQUIRE(in != nullptr && out != nullptr, EWT_ERR_INVALID_ARGUMENT,
                "null query or result buffer");
    std::lock_guard<std::mutex> lk(r->query_mu);
    DeviceGuard g(r->device);
    AllocStream as(r->stream);
    if (pageable_access(r->device)) {  // in place, as host_batch
      populate_for_write(out, m * 8);
      launch(in, m, out, r->stream);
      int const st = take_query_status(r->err_d, r->stream);
      if (st != EWT_OK)
        throw Error(st, "the batch held invalid queries (their results are "
                        "UINT64_MAX)");
      return;
    }
    QueryScratch& sc = r->scratch;
    uint64_t const chunk = std::min(m, kChunk);
    ensure(sc.in, sc.in_cap, chunk * 8);
    ensure(sc.out, sc.out_cap, chunk * 8);
    cudaStream_t s = r->stream;
    for (uint64_t b = 0; b < m; b += chunk) {
      uint64_t const k = std::min(chunk, m - b);
      EWT_CUDA(cudaMemcpyAsync(sc.in.get(), in + b, k * 8, cudaMemcpyDefault, s));
      launch(sc.in.as<uint64_t>(), k, sc.out.as<uint64_t>(), s);
      EWT_CUDA(cudaMemcpyAsync(out + b, sc.out.get(), k * 8, cudaMemcpyDefault,
                               s));
    }
    int const st = take_query_status(r->err_d, s);
    if (st != EWT_OK)
      throw Error(st, "the batch held invalid queries (their results are "
                      "UINT64_MAX)");
  });
}

template <class V>
int put_host(std::vector<V> const& v, void* buf, uint64_t cap, uint64_t* size) {
  uint64_t const bytes = v.size() * sizeof(V);
  if (size) *size = bytes;
  if (!buf) return EWT_OK;
  EWT_REQUIRE(cap >= bytes, EWT_ERR_INVALID_ARGUMENT, "export buffer too small");
  if (bytes) std::memcpy(buf, v.data(), bytes);
  return EWT_OK;
}

int put_device(void const* src, uint64_t bytes, void* buf, uint64_t cap,
               uint64_t* size) {
  if (size) *size = bytes;
  if (!buf) return EWT_OK;
  EWT_REQUIRE(cap >= bytes, EWT_ERR_INVALID_ARGUMENT, "export buffer too small");
  if (bytes) EWT_CUDA(cudaMemcpy(buf, src, bytes, cudaMemcpyDeviceToHost));
  return EWT_OK;
}

int export_array(RSStore const& rs, int comp, int a, void* buf, uint64_t cap,
                 uint64_t* size) {
  EWT_REQUIRE(a >= 0 && size_t(a) < rs.meta.size(), EWT_ERR_INVALID_ARGUMENT,
              "level / array index out of range");
  ArrayMeta const& m = rs.meta[a];
  switch (comp) {
    case EWT_EXP_LEVEL_WORDS:
      return put_device(rs.words.as<uint32_t>() + m.word_off,
                        ceil_div(m.bits, 32) * 4, buf, cap, size);
    case EWT_EXP_L1:
      return put_device(rs.l1.as<uint64_t>() + m.l1_off, m.num_l1 * 8, buf, cap,
                        size);
    case EWT_EXP_L2:
      return put_device(rs.l2.as<uint16_t>() + m.l2_off,
                        ((m.num_l1 - 1) * ecl::detail::kL2PerL1 + m.num_last_l2) *
                            2,
                        buf, cap, size);
    case EWT_EXP_SAMPLES0:
      return put_device(rs.s0.as<uint64_t>() + m.s0_off,
                        ((m.bits - m.ones) / ecl::detail::kSampleRate) * 8, buf,
                        cap, size);
    case EWT_EXP_SAMPLES1:
      return put_device(rs.s1.as<uint64_t>() + m.s1_off,
                        (m.ones / ecl::detail::kSampleRate) * 8, buf, cap, size);
  }
  throw Error(EWT_ERR_INVALID_ARGUMENT, "unknown export component");
}

int export_per_array(RSStore const& rs, int comp, void* buf, uint64_t cap,
                     uint64_t* size) {
  std::vector<uint64_t> v;
  for (auto const& m : rs.meta) {
    if (comp == EWT_EXP_TOTAL_ONES) v.push_back(m.ones);
    else if (comp == EWT_EXP_LEVEL_SIZES) v.push_back(m.bits);
    else v.push_back(m.num_last_l2);
  }
  return put_host(v, buf, cap, size);
}

}  // namespace

extern "C" {

int ewt_build(const void* data, uint64_t n, int elem_size,
              const void* alphabet, uint64_t sigma, int gpu_index,
              ewt_tree** out) {
  return guarded([&] {
    EWT_REQUIRE(out != nullptr, EWT_ERR_INVALID_ARGUMENT, "out is null");
    *out = nullptr;
    EWT_REQUIRE(data != nullptr && n > 0, EWT_ERR_INVALID_ARGUMENT,
                "text must be non-empty");
    EWT_REQUIRE(elem_size == 1 || elem_size == 2 || elem_size == 4 ||
                    elem_size == 8,
                EWT_ERR_INVALID_ARGUMENT, "elem_size must be 1, 2, 4 or 8");
    EWT_REQUIRE(sigma == 0 || alphabet != nullptr, EWT_ERR_INVALID_ARGUMENT,
                "alphabet is null");
    DeviceGuard g(gpu_index);
    auto t = std::make_unique<ewt_tree>();
    t->device = gpu_index;
    EWT_CUDA(cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking));
    cudaStream_t const st = t->stream;
    try {
      AllocStream as(st);
      build_tree(*t, data, n, elem_size, alphabet, sigma, st);
    } catch (...) {
      // buffers are returned to the pool in the stream's order, then the
      // stream goes
      cudaStreamSynchronize(st);
      t.reset();
      cudaStreamSynchronize(st);
      cudaStreamDestroy(st);
      throw;
    }
    *out = t.release();
  });
}

int ewt_build_u8(const uint8_t* d, uint64_t n, const uint8_t* a, uint64_t s,
                 uint32_t gpu, ewt_tree** out) {
  return ewt_build(d, n, 1, a, s, int(gpu), out);
}
int ewt_build_u16(const uint16_t* d, uint64_t n, const uint16_t* a, uint64_t s,
                  uint32_t gpu, ewt_tree** out) {
  return ewt_build(d, n, 2, a, s, int(gpu), out);
}
int ewt_build_u32(const uint32_t* d, uint64_t n, const uint32_t* a, uint64_t s,
                  uint32_t gpu, ewt_tree** out) {
  return ewt_build(d, n, 4, a, s, int(gpu), out);
}
int ewt_build_u64(const uint64_t* d, uint64_t n, const uint64_t* a, uint64_t s,
                  uint32_t gpu, ewt_tree** out) {
  return ewt_build(d, n, 8, a, s, int(gpu), out);
}

int ewt_free(ewt_tree* t) {
  return guarded([&] {
    if (!t) return;
    {
      DeviceGuard g(t->device);
      cudaStream_t const st = t->stream;
      if (st) cudaStreamSynchronize(st);
      delete t;  // device buffers are freed in the stream's order
      if (st) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
      }
    }
  });
}

int ewt_get_info(const ewt_tree* t, ewt_info* info) {
  return guarded([&] {
    EWT_REQUIRE(t && info, EWT_ERR_INVALID_ARGUMENT, "null argument");
    std::memset(info, 0, sizeof(*info));
    info->n = t->n;
    info->sigma = t->sigma;
    info->num_ranks = t->nodes.size();
    info->codes_start = t->codes_start;
    info->num_codes = t->codes.size();
    info->num_nodes_until_last_level = t->nodes_until_last;
    info->levels = t->L;
    info->elem_size = t->elem_size;
    info->is_min_alphabet = t->is_min;
    info->is_pow2 = t->pow2;
    info->device_bytes = t->device_bytes();
  });
}

int ewt_export(const ewt_tree* t, int comp, int level, void* buf, uint64_t cap,
               uint64_t* size) {
  return guarded([&] {
    EWT_REQUIRE(t != nullptr, EWT_ERR_INVALID_ARGUMENT, "tree is null");
    DeviceGuard g(t->device);
    std::vector<uint64_t> v;
    switch (comp) {
      case EWT_EXP_COUNTS: put_host(t->counts, buf, cap, size); return;
      case EWT_EXP_ALPHABET: put_host(t->alphabet, buf, cap, size); return;
      case EWT_EXP_NODE_RANKS:
        put_device(t->ranks_d.get(), t->nodes.size() * 8, buf, cap, size);
        return;
      case EWT_EXP_NODE_INFOS:
        for (auto const& nd : t->nodes) {
          v.push_back(nd.start);
          v.push_back(nd.level);
        }
        put_host(v, buf, cap, size);
        return;
      case EWT_EXP_CODES:
        for (auto const& c : t->codes) {
          v.push_back(c.len);
          v.push_back(c.code);
        }
        put_host(v, buf, cap, size);
        return;
      case EWT_EXP_NODES_AT_LEVEL:
        put_host(t->nodes_at_level, buf, cap, size);
        return;
      case EWT_EXP_TOTAL_ONES:
      case EWT_EXP_LEVEL_SIZES:
      case EWT_EXP_NUM_LAST_L2:
        export_per_array(t->rs, comp, buf, cap, size);
        return;
    }
    export_array(t->rs, comp, level, buf, cap, size);
  });
}

int ewt_access(ewt_tree* t, const uint64_t* indices, uint64_t m, void* results) {
  uint64_t const es = t ? t->elem_size : 1;
  return host_batch(t, indices, 8, nullptr, m, results, es,
                    [&](uint8_t const*, void const* in, uint64_t k, void* out,
                        cudaStream_t s) {
                      launch_access(*t, static_cast<uint64_t const*>(in), k,
                                    out, s);
                    });
}

int ewt_rank(ewt_tree* t, const void* queries, uint64_t m, uint64_t* results) {
  return host_batch(t, queries, 16, nullptr, m, results, 8,
                    [&](uint8_t const*, void const* in, uint64_t k, void* out,
                        cudaStream_t s) {
                      launch_rank(*t, in, k, static_cast<uint64_t*>(out), s);
                    });
}

int ewt_select(ewt_tree* t, const void* queries, uint64_t m,
               uint64_t* results) {
  return host_batch(t, queries, 16, nullptr, m, results, 8,
                    [&](uint8_t const*, void const* in, uint64_t k, void* out,
                        cudaStream_t s) {
                      launch_select(*t, in, k, static_cast<uint64_t*>(out), s);
                    });
}

int ewt_mixed(ewt_tree* t, const uint8_t* types, const void* queries,
              uint64_t m, uint64_t* results) {
  if (t && m > 0 && types == nullptr) {
    set_last_error("types is null");
    return EWT_ERR_INVALID_ARGUMENT;
  }
  return host_batch(t, queries, 16, types, m, results, 8,
                    [&](uint8_t const* ty, void const* in, uint64_t k,
                        void* out, cudaStream_t s) {
                      launch_mixed(*t, ty, in, k, static_cast<uint64_t*>(out),
                                   s);
                    });
}

int ewt_access_device(ewt_tree* t, const uint64_t* d_idx, uint64_t m,
                      void* d_out, void* stream) {
  return guarded([&] {
    EWT_REQUIRE(t != nullptr, EWT_ERR_INVALID_ARGUMENT, "tree is null");
    DeviceGuard g(t->device);
    launch_access(*t, d_idx, m, d_out, static_cast<cudaStream_t>(stream));
  });
}

int ewt_rank_device(ewt_tree* t, const void* d_q, uint64_t m, uint64_t* d_out,
                    void* stream) {
  return guarded([&] {
    EWT_REQUIRE(t != nullptr, EWT_ERR_INVALID_ARGUMENT, "tree is null");
    DeviceGuard g(t->device);
    launch_rank(*t, d_q, m, d_out, static_cast<cudaStream_t>(stream));
  });
}

int ewt_select_device(ewt_tree* t, const void* d_q, uint64_t m,
                      uint64_t* d_out, void* stream) {
  return guarded([&] {
    EWT_REQUIRE(t != nullptr, EWT_ERR_INVALID_ARGUMENT, "tree is null");
    DeviceGuard g(t->device);
    launch_select(*t, d_q, m, d_out, static_cast<cudaStream_t>(stream));
  });
}

int ewt_mixed_device(ewt_tree* t, const uint8_t* d_types, const void* d_q,
                     uint64_t m, uint64_t* d_out, void* stream) {
  return guarded([&] {
    EWT_REQUIRE(t != nullptr, EWT_ERR_INVALID_ARGUMENT, "tree is null");
    DeviceGuard g(t->device);
    launch_mixed(*t, d_types, d_q, m, d_out, static_cast<cudaStream_t>(stream));
  });
}

int ewt_query_status(ewt_tree* t, void* stream) {
  int st = EWT_OK;
  int const g = guarded([&] {
    EWT_REQUIRE(t != nullptr, EWT_ERR_INVALID_ARGUMENT, "tree is null");
    DeviceGuard dg(t->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    EWT_CUDA(cudaStreamSynchronize(s));
    st = take_query_status(t->err_d, t->stream);
  });
  if (g != EWT_OK) return g;
  if (st != EWT_OK) set_last_error("a batch held invalid queries");
  return st;
}

int ewt_get_device_view(const ewt_tree* t, void* view_out, uint64_t view_size) {
  return guarded([&] {
    EWT_REQUIRE(t && view_out, EWT_ERR_INVALID_ARGUMENT, "null argument");
    EWT_REQUIRE(view_size == sizeof(TreeView), EWT_ERR_INVALID_ARGUMENT,
                "view size does not match this library's TreeView");
    t->view_shared.store(true);
    std::memcpy(view_out, &t->view, sizeof(TreeView));
  });
}

int ewt_rs_build(const uint32_t* words, const uint64_t* bits,
                 uint32_t num_arrays, int gpu_index, ewt_rs** out) {
  return guarded([&] {
    EWT_REQUIRE(out != nullptr, EWT_ERR_INVALID_ARGUMENT, "out is null");
    *out = nullptr;
    EWT_REQUIRE(words && bits && num_arrays > 0, EWT_ERR_INVALID_ARGUMENT,
                "words, bits and num_arrays must be given");
    std::vector<uint64_t> b(bits, bits + num_arrays);
    for (auto x : b)
      EWT_REQUIRE(x > 0, EWT_ERR_INVALID_ARGUMENT, "empty bit array");
    DeviceGuard g(gpu_index);
    auto r = std::make_unique<ewt_rs>();
    r->device = gpu_index;
    EWT_CUDA(cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking));
    cudaStream_t const st = r->stream;
    try {
      AllocStream as(st);
      r->err_d.alloc(16);
      EWT_CUDA(cudaMemsetAsync(r->err_d.get(), 0, 16, st));
      r->rs.layout(b);
      if (is_device_pointer(words)) EWT_CUDA(cudaDeviceSynchronize());
      uint64_t off = 0;
      for (uint32_t a = 0; a < num_arrays; ++a) {
        uint64_t const w = ceil_div(b[a], 32);
        EWT_CUDA(cudaMemcpyAsync(r->rs.words.as<uint32_t>() + r->rs.meta[a].word_off,
                                 words + off, w * 4, cudaMemcpyDefault, st));
        off += w;
      }
      EWT_CUDA(cudaMemcpyAsync(r->rs.meta_d.get(), r->rs.meta.data(),
                               num_arrays * sizeof(ArrayMeta),
                               cudaMemcpyHostToDevice, st));
      mask_tails_kernel<<<ceil_div(num_arrays, 128), 128, 0, st>>>(
          r->rs.words.as<uint32_t>(), r->rs.meta_d.as<ArrayMeta>(), num_arrays);
      EWT_LAUNCHED();
      build_rs_counts(r->rs, 0, num_arrays, st);
      build_rs_samples(r->rs, st);
      build_rank_blocks(r->rs, st);
      EWT_CUDA(cudaStreamSynchronize(st));
    } catch (...) {
      cudaStreamSynchronize(st);
      r.reset();
      cudaStreamSynchronize(st);
      cudaStreamDestroy(st);
      throw;
    }
    *out = r.release();
  });
}

int ewt_bitarray_create(const uint64_t* bits, uint32_t num_arrays,
                        int init_value, int gpu_index, ewt_rs** out) {
  return guarded([&] {
    EWT_REQUIRE(out != nullptr, EWT_ERR_INVALID_ARGUMENT, "out is null");
    *out = nullptr;
    EWT_REQUIRE(bits && num_arrays > 0 && num_arrays < 256,
                EWT_ERR_INVALID_ARGUMENT,
                "bits must be given for 1 to 255 arrays");
    EWT_REQUIRE(init_value == 0 || init_value == 1, EWT_ERR_INVALID_ARGUMENT,
                "init_value must be 0 or 1");
    std::vector<uint64_t> b(bits, bits + num_arrays);
    for (auto x : b)
      EWT_REQUIRE(x > 0, EWT_ERR_INVALID_ARGUMENT, "empty bit array");
    DeviceGuard g(gpu_index);
    auto r = std::make_unique<ewt_rs>();
    r->device = gpu_index;
    r->built = false;
    EWT_CUDA(cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking));
    cudaStream_t const st = r->stream;
    try {
      AllocStream as(st);
      r->err_d.alloc(16);
      EWT_CUDA(cudaMemsetAsync(r->err_d.get(), 0, 16, st));
      r->rs.layout(b);
      EWT_CUDA(cudaMemsetAsync(r->rs.words.get(), init_value ? 0xFF : 0,
                               r->rs.words.bytes(), st));
      EWT_CUDA(cudaMemsetAsync(r->rs.l1.get(), 0, r->rs.l1.bytes(), st));
      EWT_CUDA(cudaMemsetAsync(r->rs.l2.get(), 0, r->rs.l2.bytes(), st));
      EWT_CUDA(cudaStreamSynchronize(st));
    } catch (...) {
      cudaStreamSynchronize(st);
      r.reset();
      cudaStreamDestroy(st);
      throw;
    }
    *out = r.release();
  });
}

int ewt_rs_build_in_place(ewt_rs* r) {
  return guarded([&] {
    EWT_REQUIRE(r != nullptr, EWT_ERR_INVALID_ARGUMENT, "rank/select is null");
    std::lock_guard<std::mutex> lk(r->query_mu);
    EWT_REQUIRE(!r->built, EWT_ERR_INVALID_ARGUMENT,
                "the rank/select support of these arrays is already built");
    DeviceGuard g(r->device);
    // the caller's kernels that wrote the words may run on any stream
    EWT_CUDA(cudaDeviceSynchronize());
    cudaStream_t const st = r->stream;
    AllocStream as(st);
    uint32_t const count = static_cast<uint32_t>(r->rs.meta.size());
    clear_tails_kernel<<<count, 32, 0, st>>>(r->rs.words.as<uint32_t>(),
                                             r->rs.meta_d.as<ArrayMeta>(), count);
    EWT_LAUNCHED();
    build_rs_counts(r->rs, 0, count, st);
    build_rs_samples(r->rs, st);
    build_rank_blocks(r->rs, st);
    EWT_CUDA(cudaStreamSynchronize(st));
    r->built = true;
  });
}

int ewt_needed_memory(int kind, uint64_t n, uint32_t arrays_or_elem_size,
                      uint64_t sigma, uint64_t* bytes) {
  return guarded([&] {
    EWT_REQUIRE(bytes != nullptr, EWT_ERR_INVALID_ARGUMENT, "bytes is null");
    switch (kind) {
      case EWT_MEM_BITARRAY:
        *bytes = rs_bytes_bound(n, arrays_or_elem_size, false);
        return;
      case EWT_MEM_RANKSELECT:
        *bytes = rs_bytes_bound(n, arrays_or_elem_size, true);
        return;
      case EWT_MEM_TREE:
        EWT_REQUIRE(arrays_or_elem_size == 1 || arrays_or_elem_size == 2 ||
                        arrays_or_elem_size == 4 || arrays_or_elem_size == 8,
                    EWT_ERR_INVALID_ARGUMENT, "elem_size must be 1, 2, 4 or 8");
        *bytes = build_bytes_bound(n, arrays_or_elem_size, sigma);
        return;
    }
    throw Error(EWT_ERR_INVALID_ARGUMENT, "unknown memory kind");
  });
}

int ewt_minimal_codes(uint64_t sigma, uint64_t* lens, uint64_t* codes,
                      uint64_t cap, uint64_t* count) {
  return guarded([&] {
    EWT_REQUIRE(sigma >= 2, EWT_ERR_INVALID_ARGUMENT, "sigma must be >= 2");
    std::vector<uint64_t> l, c;
    minimal_codes(sigma, l, c);
    if (count) *count = l.size();
    for (uint64_t i = 0; i < l.size() && i < cap; ++i) {
      if (lens) lens[i] = l[i];
      if (codes) codes[i] = c[i];
    }
  });
}

int ewt_rs_free(ewt_rs* r) {
  return guarded([&] {
    if (!r) return;
    DeviceGuard g(r->device);
    cudaStream_t const st = r->stream;
    if (st) cudaStreamSynchronize(st);
    delete r;  // device buffers are freed in the stream's order
    if (st) {
      cudaStreamSynchronize(st);
      cudaStreamDestroy(st);
    }
  });
}

int ewt_rs_export(const ewt_rs* r, int comp, int array, void* buf,
                  uint64_t cap, uint64_t* size) {
  return guarded([&] {
    EWT_REQUIRE(r != nullptr, EWT_ERR_INVALID_ARGUMENT, "rank/select is null");
    DeviceGuard g(r->device);
    if (comp == EWT_EXP_TOTAL_ONES || comp == EWT_EXP_LEVEL_SIZES ||
        comp == EWT_EXP_NUM_LAST_L2) {
      export_per_array(r->rs, comp, buf, cap, size);
      return;
    }
    export_array(r->rs, comp, array, buf, cap, size);
  });
}

int ewt_rs_rank(ewt_rs* r, int array, int value, const uint64_t* pos,
                uint64_t m, uint64_t* results) {
  if (r && !r->built) {
    set_last_error("rank/select support not built (ewt_rs_build_in_place)");
    return EWT_ERR_INVALID_ARGUMENT;
  }
  if (r && (array < 0 || size_t(array) >= r->rs.meta.size())) {
    set_last_error("array index out of range");
    return EWT_ERR_INVALID_ARGUMENT;
  }
  return rs_host_batch(r, pos, m, results,
                       [&](uint64_t const* in, uint64_t k, uint64_t* out,
                           cudaStream_t s) {
                         launch_rs_rank(*r, array, value, in, k, out, s);
                       });
}

int ewt_rs_select(ewt_rs* r, int array, int value, const uint64_t* idx,
                  uint64_t m, uint64_t* results) {
  if (r && !r->built) {
    set_last_error("rank/select support not built (ewt_rs_build_in_place)");
    return EWT_ERR_INVALID_ARGUMENT;
  }
  if (r && (array < 0 || size_t(array) >= r->rs.meta.size())) {
    set_last_error("array index out of range");
    return EWT_ERR_INVALID_ARGUMENT;
  }
  return rs_host_batch(r, idx, m, results,
                       [&](uint64_t const* in, uint64_t k, uint64_t* out,
                           cudaStream_t s) {
                         launch_rs_select(*r, array, value, in, k, out, s);
                       });
}

int ewt_rs_get_device_view(const ewt_rs* r, void* view_out, uint64_t view_size) {
  return guarded([&] {
    EWT_REQUIRE(r && view_out, EWT_ERR_INVALID_ARGUMENT, "null argument");
    EWT_REQUIRE(view_size == sizeof(RSView), EWT_ERR_INVALID_ARGUMENT,
                "view size does not match this library's RSView");
    r->view_shared.store(true);
    RSView const v = r->rs.view();
    std::memcpy(view_out, &v, sizeof(RSView));
  });
}

namespace {
uint32_t sample_shift(uint32_t rate) {
  EWT_REQUIRE(rate == 0 || (rate >= 32 && rate <= 65536 && (rate & (rate - 1)) == 0),
              EWT_ERR_INVALID_ARGUMENT,
              "select sample rate must be 0 or a power of two in [32, 65536]");
  uint32_t sh = 0;
  while (rate > 1) {
    rate >>= 1;
    ++sh;
  }
  return sh;
}
}  // namespace

int ewt_set_select_samples(ewt_tree* t, uint32_t rate) {
  return guarded([&] {
    EWT_REQUIRE(t != nullptr, EWT_ERR_INVALID_ARGUMENT, "tree is null");
    uint32_t const sh = sample_shift(rate);
    std::lock_guard<std::mutex> lk(t->query_mu);
    EWT_REQUIRE(!t->view_shared.load(), EWT_ERR_INVALID_ARGUMENT,
                "the tree's device view was copied out; its samples stay");
    EWT_REQUIRE(!t->shared_store, EWT_ERR_UNSUPPORTED,
                "a short text of a batch build shares its rank/select store "
                "with the other texts of its group; its samples stay");
    DeviceGuard g(t->device);
    AllocStream as(t->stream);
    set_select_rate(*t, sh, t->stream);
  });
}

int ewt_rs_set_select_samples(ewt_rs* r, uint32_t rate) {
  return guarded([&] {
    EWT_REQUIRE(r != nullptr, EWT_ERR_INVALID_ARGUMENT, "rank/select is null");
    uint32_t const sh = sample_shift(rate);
    std::lock_guard<std::mutex> lk(r->query_mu);
    EWT_REQUIRE(!r->view_shared.load(), EWT_ERR_INVALID_ARGUMENT,
                "the device view was copied out; its samples stay");
    DeviceGuard g(r->device);
    AllocStream as(r->stream);
    build_dense_samples(r->rs, sh, r->stream);
  });
}

void ewt_set_timing(int enable) { ewt::g_timing.store(enable != 0); }

void ewt_get_timing(ewt_phase_times* out, int reset) {
  std::lock_guard<std::mutex> lk(ewt::g_timing_mu);
  if (out) *out = ewt::g_times;
  if (reset) std::memset(&ewt::g_times, 0, sizeof(ewt::g_times));
}

const char* ewt_last_error(void) { return g_last_error.c_str(); }
int ewt_abi_version(void) { return EWT_ABI_VERSION; }

int ewt_probe_random_reads(int gpu_index, uint64_t bytes, uint32_t depth,
                           uint64_t chains, double* reads_per_s) {
  return guarded([&] {
    EWT_REQUIRE(reads_per_s != nullptr, EWT_ERR_INVALID_ARGUMENT, "null argument");
    DeviceGuard g(gpu_index);
    cudaStream_t st = nullptr;
    EWT_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    try {
      AllocStream as(st);
      probe_random_reads(bytes, depth, chains, reads_per_s);
    } catch (...) {
      cudaStreamSynchronize(st);
      cudaStreamDestroy(st);
      throw;
    }
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
  });
}

int ewt_autotune(ewt_tree* t, uint64_t probe_queries, ewt_tuning* out) {
  return guarded([&] {
    EWT_REQUIRE(t != nullptr, EWT_ERR_INVALID_ARGUMENT, "tree is null");
    EWT_REQUIRE(probe_queries >= 1024 && probe_queries <= (uint64_t(1) << 28),
                EWT_ERR_INVALID_ARGUMENT, "probe_queries must be in [2^10, 2^28]");
    std::lock_guard<std::mutex> lk(t->query_mu);
    DeviceGuard g(t->device);
    AllocStream as(t->stream);
    if (out) std::memset(out, 0, sizeof(*out));
    autotune_queries(*t, probe_queries, out);
  });
}

int ewt_release_cached_memory(int gpu_index) {
  return guarded([&] {
    DeviceGuard g(gpu_index);
    EWT_CUDA(cudaDeviceSynchronize());
    EWT_CUDA(cudaMemPoolTrimTo(lib_pool(), 0));
  });
}
uint64_t ewt_launch_count(void) { return g_launches.load(); }

void ewt_set_work_queue(int enable) { g_work_queue.store(enable != 0); }

int ewt_binary_version(int gpu_index, int* version) {
  return guarded([&] {
    EWT_REQUIRE(version != nullptr, EWT_ERR_INVALID_ARGUMENT, "null argument");
    DeviceGuard g(gpu_index);
    *version = kernel_binary_version();
  });
}

}  // extern "C"
