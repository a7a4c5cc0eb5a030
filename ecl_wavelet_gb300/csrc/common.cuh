// Host-side plumbing shared by the libewt.so translation units: status
// codes from CUDA errors, the per-thread error message behind
// ewt_last_error(), a launch counter, and small RAII device buffers.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <mutex>
#include <set>
#include <utility>
#include <cstdio>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "ewt.h"

namespace ewt {

// Status carried through the host code as an exception so that every C-ABI
// entry point can convert it into an int exactly once.
struct Error : std::runtime_error {
  int status;
  Error(int st, std::string const& msg) : std::runtime_error(msg), status(st) {}
};

void set_last_error(std::string const& msg);
void count_launch(uint64_t k = 1);

inline int status_of(cudaError_t e) {
  return e == cudaErrorMemoryAllocation ? EWT_ERR_OUT_OF_MEMORY : EWT_ERR_CUDA;
}

#define EWT_CUDA(expr)                                                      \
  do {                                                                      \
    cudaError_t _e = (expr);                                                \
    if (_e != cudaSuccess) {                                                \
      (void)cudaGetLastError();                                             \
      throw ::ewt::Error(::ewt::status_of(_e),                              \
                         std::string(#expr) + ": " + cudaGetErrorString(_e)); \
    }                                                                       \
  } while (0)

// Check a kernel launch and count it.
#define EWT_LAUNCHED()                                                      \
  do {                                                                      \
    ::ewt::count_launch();                                                  \
    cudaError_t _e = cudaGetLastError();                                    \
    if (_e != cudaSuccess)                                                  \
      throw ::ewt::Error(::ewt::status_of(_e),                              \
                         std::string("kernel launch: ") +                  \
                             cudaGetErrorString(_e));                       \
  } while (0)

#define EWT_REQUIRE(cond, st, msg)                                          \
  do {                                                                      \
    if (!(cond)) throw ::ewt::Error((st), (msg));                           \
  } while (0)

// The stream that device allocations and frees of the running library
// call are ordered on (set for the call's duration by AllocStream).
inline cudaStream_t& alloc_stream() {
  thread_local cudaStream_t s = nullptr;
  return s;
}
class AllocStream {
 public:
  explicit AllocStream(cudaStream_t s) : prev_(alloc_stream()) { alloc_stream() = s; }
  ~AllocStream() { alloc_stream() = prev_; }
  AllocStream(AllocStream const&) = delete;
  AllocStream& operator=(AllocStream const&) = delete;

 private:
  cudaStream_t prev_;
};

// Library memory pool of the current device: stream-ordered allocations
// that keep freed blocks for reuse (release threshold: never), so repeated
// builds do not pay cudaMalloc / cudaFree (whose frees synchronise the
// device).  ewt_release_cached_memory() returns the cached blocks.
cudaMemPool_t lib_pool();

// Owning device allocation.  With an allocation stream set: from the
// library pool, allocated and freed in that stream's order; otherwise
// cudaMalloc / cudaFree.  A view (view()) names memory another owner keeps
// and frees nothing.
class DevBuf {
 public:
  DevBuf() = default;
  explicit DevBuf(size_t bytes) { alloc(bytes); }
  DevBuf(DevBuf const&) = delete;
  DevBuf& operator=(DevBuf const&) = delete;
  DevBuf(DevBuf&& o) noexcept
      : p_(o.p_), n_(o.n_), s_(o.s_), pooled_(o.pooled_), view_(o.view_) {
    o.p_ = nullptr;
    o.n_ = 0;
  }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      reset();
      p_ = o.p_; n_ = o.n_; s_ = o.s_; pooled_ = o.pooled_; view_ = o.view_;
      o.p_ = nullptr; o.n_ = 0;
    }
    return *this;
  }
  ~DevBuf() { reset(); }
  void alloc(size_t bytes) {
    reset();
    if (bytes == 0) bytes = 16;
    s_ = alloc_stream();
    pooled_ = s_ != nullptr;
    if (pooled_)
      EWT_CUDA(cudaMallocFromPoolAsync(&p_, bytes, lib_pool(), s_));
    else
      EWT_CUDA(cudaMalloc(&p_, bytes));
    n_ = bytes;
  }
  void view(void* p, size_t bytes) {
    reset();
    p_ = p;
    n_ = bytes;
    view_ = true;
  }
  bool is_view() const { return view_; }
  void reset() {
    if (p_ && !view_) {
      if (pooled_) cudaFreeAsync(p_, s_);
      else cudaFree(p_);
    }
    p_ = nullptr;
    n_ = 0;
    view_ = false;
  }
  template <class T> T* as() const { return static_cast<T*>(p_); }
  void* get() const { return p_; }
  size_t bytes() const { return n_; }

 private:
  void* p_ = nullptr;
  size_t n_ = 0;
  cudaStream_t s_ = nullptr;
  bool pooled_ = false;
  bool view_ = false;
};

// Runs an entry point's body: library exceptions become an int status and
// the calling thread's last-error message.
template <class F>
int run_guarded(F&& f) {
  try {
    f();
    set_last_error("");
    return EWT_OK;
  } catch (Error const& e) {
    set_last_error(e.what());
    return e.status;
  } catch (std::bad_alloc const&) {
    set_last_error("host allocation failed");
    return EWT_ERR_OUT_OF_MEMORY;
  } catch (std::exception const& e) {
    set_last_error(e.what());
    return EWT_ERR_CUDA;
  }
}

// Owning pinned host allocation.
class PinnedBuf {
 public:
  PinnedBuf() = default;
  PinnedBuf(PinnedBuf const&) = delete;
  PinnedBuf& operator=(PinnedBuf const&) = delete;
  ~PinnedBuf() { reset(); }
  void ensure(size_t bytes) {
    if (bytes <= n_) return;
    reset();
    EWT_CUDA(cudaHostAlloc(&p_, bytes, cudaHostAllocPortable));
    n_ = bytes;
  }
  void reset() {
    if (p_) cudaFreeHost(p_);
    p_ = nullptr;
    n_ = 0;
  }
  template <class T> T* as() const { return static_cast<T*>(p_); }
  void* get() const { return p_; }
  size_t bytes() const { return n_; }

 private:
  void* p_ = nullptr;
  size_t n_ = 0;
};

// Device the calling thread should use; restores the previous one on exit.
class DeviceGuard {
 public:
  explicit DeviceGuard(int dev) {
    EWT_CUDA(cudaGetDevice(&prev_));
    if (prev_ != dev) EWT_CUDA(cudaSetDevice(dev));
  }
  ~DeviceGuard() { cudaSetDevice(prev_); }

 private:
  int prev_ = 0;
};

inline bool is_device_pointer(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

inline int sm_count() {
  static int cached = -1;
  if (cached < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    cached = v > 0 ? v : 1;
  }
  return cached;
}

inline uint64_t ceil_div(uint64_t a, uint64_t b) { return (a + b - 1) / b; }

// Raises kernel `f`'s dynamic shared-memory limit to `bytes` on the current
// device, once per (kernel, device): the attribute belongs to the kernel's
// instance in that device's context.
template <class Kernel>
void set_smem_limit(Kernel f, int bytes) {
  static std::mutex mu;
  static std::set<std::pair<void const*, int>> done;
  int dev = 0;
  EWT_CUDA(cudaGetDevice(&dev));
  auto const key = std::make_pair(reinterpret_cast<void const*>(f), dev);
  std::lock_guard<std::mutex> lk(mu);
  if (done.count(key)) return;
  EWT_CUDA(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  done.insert(key);
}

// Puts this thread's stream-capture mode to relaxed for its scope, so that
// the host-side launch preparation (kernel attributes, occupancy queries) of
// a launch made while the caller captures a CUDA graph is permitted in every
// capture mode; restores the caller's mode on exit.
// Device work queue of one launch.  CTAs take their next chunk from a
// counter in device memory (q[0]) instead of a fixed stride, so a CTA that
// drew cheap chunks (mostly access and rank walks) takes more of them than
// one that drew select-heavy chunks; the CTA that finishes last resets the
// counter (q[1] counts finished CTAs), so the next launch that uses the same
// pair finds it at zero.  With q == nullptr CTA b takes chunks b, b + G, ...
// Every thread of the CTA calls both functions (they hold a barrier).
__device__ __forceinline__ uint64_t wq_take(uint32_t* q, uint32_t* s_next,
                                            uint64_t prev, bool first) {
  if (q == nullptr) return first ? blockIdx.x : prev + gridDim.x;
  if (threadIdx.x == 0) *s_next = atomicAdd(q, 1u);
  __syncthreads();
  return *s_next;
}
__device__ __forceinline__ void wq_finish(uint32_t* q) {
  if (q == nullptr || threadIdx.x != 0) return;
  __threadfence();
  if (atomicAdd(q + 1, 1u) == gridDim.x - 1) {
    q[0] = 0u;  // every CTA has made its last take
    q[1] = 0u;
  }
}

class RelaxedCapture {
 public:
  RelaxedCapture() { cudaThreadExchangeStreamCaptureMode(&mode_); }
  ~RelaxedCapture() { cudaThreadExchangeStreamCaptureMode(&mode_); }
  RelaxedCapture(RelaxedCapture const&) = delete;
  RelaxedCapture& operator=(RelaxedCapture const&) = delete;

 private:
  cudaStreamCaptureMode mode_ = cudaStreamCaptureModeRelaxed;
};

// Event-timed phase on one stream (ewt_set_timing / ewt_get_timing).  When
// timing is off the guard does nothing.
bool timing_enabled();
void add_phase_time(int phase, double ms);

class PhaseTimer {
 public:
  PhaseTimer(int phase, cudaStream_t s) : phase_(phase), s_(s) {
    if (!timing_enabled()) return;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s_, &cs) != cudaSuccess ||
        cs != cudaStreamCaptureStatusNone) {  // a graph is being captured
      (void)cudaGetLastError();
      return;
    }
    if (cudaEventCreate(&a_) != cudaSuccess || cudaEventCreate(&b_) != cudaSuccess) {
      (void)cudaGetLastError();
      return;
    }
    cudaEventRecord(a_, s_);
    on_ = true;
  }
  PhaseTimer(PhaseTimer const&) = delete;
  PhaseTimer& operator=(PhaseTimer const&) = delete;
  ~PhaseTimer() {
    if (!on_) return;
    float ms = 0.f;
    if (cudaEventRecord(b_, s_) == cudaSuccess &&
        cudaEventSynchronize(b_) == cudaSuccess &&
        cudaEventElapsedTime(&ms, a_, b_) == cudaSuccess)
      add_phase_time(phase_, ms);
    (void)cudaGetLastError();
    cudaEventDestroy(a_);
    cudaEventDestroy(b_);
  }

 private:
  int phase_;
  cudaStream_t s_;
  cudaEvent_t a_ = nullptr, b_ = nullptr;
  bool on_ = false;
};

}  // namespace ewt
