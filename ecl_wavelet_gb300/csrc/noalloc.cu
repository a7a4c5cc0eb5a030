// ewt_mixed_noalloc: the mixed access/rank/select host batch without any
// device allocation.
//
// Who needs it: callers that are not allowed to allocate device memory once
// they are running — serving loops that hand all free HBM to their own arena
// or caching allocator at start-up (a cudaMalloc from the library would fail
// or steal the arena's headroom), hosts that fix every component's device
// budget in advance, and latency-critical paths where an allocation that
// misses the pool, or cudaFree's implicit device-wide synchronisation, would
// stall every other stream.  ewt_mixed grows per-tree device scratch on
// demand; this entry point stages the batch in a fixed array compiled into
// the library instead.
//
// The scratch is one file-scope __device__ array of kScratchBytes per GPU
// (about 6.3 MB), present on every GPU that loads libewt.so until the
// process exits.  Its device address is fetched once per GPU with
// cudaGetSymbolAddress, on the first call made on that GPU, with that GPU
// current; that first call should come before any stream capture.  The
// address is kept for the life of the process, so resetting a device
// (cudaDeviceReset) after that first call is not supported.
// All calls share the array and it keeps the last call's contents: the
// invalid-query word and the work-queue counters are cleared on every call.  Calls are serialised by a
// process-wide lock (taken before the tree's own query lock, so calls that
// change the tree — autotuning, select-sample rates — cannot interleave) and
// each returns only after its GPU work has finished, so two calls never use
// the array at the same time; GPU work of one call that overlapped another
// call would race on it.  The launch uses the tree's tuned shape and is
// timed as a query phase, exactly as ewt_mixed's kernel.
#include <array>
#include <mutex>
#include <string>

#include "internal.cuh"

namespace {

// Largest batch one call accepts.
constexpr uint64_t kNoAllocMaxQueries = uint64_t(1) << 18;  // 262,144
constexpr size_t kErrBytes = 256;  // invalid-query word + queue counters
constexpr size_t kQueryBytes = kNoAllocMaxQueries * 16;  // RankSelectQuery
constexpr size_t kResultBytes = kNoAllocMaxQueries * 8;
constexpr size_t kTypeBytes = kNoAllocMaxQueries;
constexpr size_t kScratchBytes =
    kErrBytes + kQueryBytes + kResultBytes + kTypeBytes;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;  // guards the array and the address table
std::array<void*, kMaxDevices> g_scratch_addr{};

// Device address of the scratch on `dev` (which must be current); looked up
// once per device.
unsigned char* scratch_on(int dev) {
  EWT_REQUIRE(dev >= 0 && dev < kMaxDevices, EWT_ERR_INVALID_ARGUMENT,
              "device index out of range for the no-allocation scratch");
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    cudaError_t const e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      throw ewt::Error(EWT_ERR_CUDA,
                       std::string("cudaGetSymbolAddress of the "
                                   "no-allocation scratch: ") +
                           cudaGetErrorString(e));
    }
    g_scratch_addr[dev] = p;
  }
  return static_cast<unsigned char*>(g_scratch_addr[dev]);
}

}  // namespace

extern "C" int ewt_mixed_noalloc(ewt_tree* t, const uint8_t* types,
                                 const void* queries, uint64_t m,
                                 uint64_t* results) {
  try {
    EWT_REQUIRE(t != nullptr, EWT_ERR_INVALID_ARGUMENT, "tree is null");
    if (m == 0) return EWT_OK;
    EWT_REQUIRE(m <= kNoAllocMaxQueries, EWT_ERR_TOO_LARGE,
                "ewt_mixed_noalloc takes at most 262144 queries per call; "
                "split the batch");
    EWT_REQUIRE(types && queries && results, EWT_ERR_INVALID_ARGUMENT,
                "null type, query or result buffer");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    std::lock_guard<std::mutex> tree_lk(t->query_mu);
    ewt::DeviceGuard g(t->device);
    unsigned char* base = scratch_on(t->device);
    uint32_t* d_err = reinterpret_cast<uint32_t*>(base);
    unsigned char* d_q = base + kErrBytes;
    uint64_t* d_out = reinterpret_cast<uint64_t*>(d_q + kQueryBytes);
    uint8_t* d_types = reinterpret_cast<uint8_t*>(d_q + kQueryBytes +
                                                  kResultBytes);
    cudaStream_t const s = t->stream;
    // the invalid-query word and the launch's work-queue counters (bytes
    // 64..71 of the same 256-byte region) start at zero
    EWT_CUDA(cudaMemsetAsync(d_err, 0, kErrBytes, s));
    EWT_CUDA(cudaMemcpyAsync(d_q, queries, m * 16, cudaMemcpyDefault, s));
    EWT_CUDA(cudaMemcpyAsync(d_types, types, m, cudaMemcpyDefault, s));
    ewt::launch_mixed_raw(*t, d_types, d_q, m, d_out, d_err, s);
    EWT_CUDA(cudaMemcpyAsync(results, d_out, m * 8, cudaMemcpyDefault, s));
    uint32_t bad = 0;
    EWT_CUDA(cudaMemcpyAsync(&bad, d_err, sizeof(bad), cudaMemcpyDeviceToHost,
                             s));
    EWT_CUDA(cudaStreamSynchronize(s));
    if (bad) {
      ewt::set_last_error(
          "the batch held invalid queries (their results are UINT64_MAX)");
      return EWT_ERR_QUERY;
    }
    ewt::set_last_error("");
    return EWT_OK;
  } catch (ewt::Error const& e) {
    ewt::set_last_error(e.what());
    return e.status;
  } catch (std::exception const& e) {
    ewt::set_last_error(e.what());
    return EWT_ERR_CUDA;
  }
}
