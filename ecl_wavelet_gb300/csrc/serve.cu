// Serving engine: resident trees, continuous batching of query requests,
// builds admitted by device-memory footprint, p50/p99 latency.
//
// Threads: callers submit requests (any thread); the dispatcher takes the
// next batch from the scheduler (serve_sched.h) whenever one of the `inflight`
// batch slots is free, packs the requests' queries into the slot's pinned
// buffers, and launches copy-in, the multi-tree kernel (multi.cu) and
// copy-out on the slot's stream; the completer waits for the slots in
// launch order, copies every request's results to its buffer and completes
// it; the builder runs admitted builds on their own streams.  So requests
// that arrive while batches are on the GPU are admitted into the next slot
// as soon as one frees up, and copies, kernels and builds of different
// slots overlap on the device.
//
// The reference answers one synchronous host call at a time
// (wavelet_tree.cuh:956-1797); it has no serving layer.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <random>
#include <thread>
#include <unordered_map>
#include <vector>

#include "internal.cuh"
#include "serve_sched.h"

namespace ewt {
namespace {

constexpr uint32_t kMaxServerTrees = 4096;
constexpr uint32_t kServeChunk = 2048;  // queries per work item (multi.cu)

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct ServeItem {  // multi.cu's work item layout
  uint32_t tree, count;
  uint64_t start;
};
static_assert(sizeof(ServeItem) == 16, "work item layout");

struct ServeReqH {  // multi.cu's request descriptor layout
  uint8_t const* types;
  void const* queries;
  uint64_t* results;
  uint32_t tree, pad;
};
static_assert(sizeof(ServeReqH) == 32, "request descriptor layout");

struct Slot {
  cudaStream_t st = nullptr;
  cudaEvent_t done = nullptr;
  PinnedBuf h_q, h_types, h_items, h_out, h_err, h_reqs, h_reqerr;
  DevBuf d_q, d_types, d_items, d_out, d_err;
  std::vector<sched::Request*> reqs;
  std::vector<uint64_t> offs;
  bool busy = false;
};

struct BuildJob {
  const void* text = nullptr;
  uint64_t n = 0;
  const void* alphabet = nullptr;
  uint64_t sigma = 0;
};

}  // namespace
}  // namespace ewt

struct ewt_server {
  int device = 0;
  ewt_server_config cfg{};
  std::mutex mu;
  std::condition_variable cv_work, cv_launched, cv_done, cv_build;
  ewt::sched::Scheduler sched;
  std::vector<ewt_tree*> trees;
  std::vector<bool> owned;
  std::vector<uint64_t> tree_bytes;
  ewt::TreeView* views_d = nullptr;  // kMaxServerTrees views
  uint32_t max_levels = 1;
  std::deque<ewt::Slot> slots;  // deque: slots are not movable
  std::deque<int> launched;
  std::unordered_map<uint64_t, ewt::BuildJob> build_jobs;
  std::thread dispatcher, completer, builder;
  bool stop = false;
  bool zero_copy = false;  // kernels read requests and write results in place
  std::string fatal;  // set when a worker thread failed

  ewt_server(ewt_server_config const& c)
      : cfg(c), sched(c.batch_queries, c.batch_requests, c.memory_budget) {}
};

namespace ewt {
namespace {

uint64_t build_footprint(uint64_t n, uint32_t elem_size) {
  // text copy + two level orders + bits and rank blocks of up to 8 * size
  // levels + counts and samples (conservative)
  uint64_t const levels = 8ull * elem_size;
  return n * elem_size * 3 + (n * levels / 8) * 23 / 10 + (64ull << 20);
}

void dispatcher_loop(ewt_server* S) {
  DeviceGuard g(S->device);
  for (;;) {
    int si = -1;
    std::vector<sched::Request*> batch;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_work.wait(lk, [&] {
        if (S->stop && !S->sched.has_queries()) return true;
        if (!S->sched.has_queries()) return false;
        for (auto const& sl : S->slots)
          if (!sl.busy) return true;
        return false;
      });
      if (S->stop && !S->sched.has_queries()) return;
      for (size_t i = 0; i < S->slots.size(); ++i)
        if (!S->slots[i].busy) {
          si = static_cast<int>(i);
          break;
        }
      batch = S->sched.take_batch(now_s());
      S->slots[si].busy = true;
    }
    Slot& sl = S->slots[si];
    sl.reqs = batch;
    sl.offs.clear();
    if (S->zero_copy) {
      // descriptors of the callers' buffers; the kernel reads the queries
      // and writes the results in place
      auto* reqs = sl.h_reqs.as<ServeReqH>();
      auto* items = sl.h_items.as<ServeItem>();
      auto* rerr = sl.h_reqerr.as<uint32_t>();
      uint32_t nitems = 0;
      for (size_t i = 0; i < batch.size(); ++i) {
        sched::Request* r = batch[i];
        reqs[i] = ServeReqH{r->types, r->queries, r->results, r->tree, 0};
        rerr[i] = 0;
        for (uint64_t j = 0; j < r->m; j += kServeChunk)
          items[nitems++] = ServeItem{static_cast<uint32_t>(i),
                                      static_cast<uint32_t>(std::min<uint64_t>(kServeChunk, r->m - j)),
                                      j};
      }
      try {
        launch_serve_items(S->cfg.elem_size, S->views_d, reqs, items, nitems,
                           S->max_levels, rerr, sl.st);
        EWT_CUDA(cudaEventRecord(sl.done, sl.st));
      } catch (std::exception const& e) {
        std::lock_guard<std::mutex> lk(S->mu);
        S->fatal = e.what();
        for (auto* r : batch) S->sched.complete(r->id, EWT_ERR_CUDA, now_s());
        sl.busy = false;
        S->cv_done.notify_all();
        S->cv_work.notify_all();
        continue;
      }
      {
        std::lock_guard<std::mutex> lk(S->mu);
        S->launched.push_back(si);
      }
      S->cv_launched.notify_one();
      continue;
    }
    uint64_t off = 0;
    uint32_t nitems = 0;
    auto* items = sl.h_items.as<ServeItem>();
    for (auto* r : batch) {
      sl.offs.push_back(off);
      std::memcpy(sl.h_types.as<uint8_t>() + off, r->types, r->m);
      std::memcpy(sl.h_q.as<unsigned char>() + off * 16, r->queries, r->m * 16);
      for (uint64_t j = 0; j < r->m; j += kServeChunk)
        items[nitems++] = ServeItem{r->tree,
                                    static_cast<uint32_t>(std::min<uint64_t>(kServeChunk, r->m - j)),
                                    off + j};
      off += r->m;
    }
    try {
      *sl.h_err.as<uint32_t>() = 0;
      EWT_CUDA(cudaMemcpyAsync(sl.d_err.get(), sl.h_err.get(), 4, cudaMemcpyHostToDevice, sl.st));
      EWT_CUDA(cudaMemcpyAsync(sl.d_q.get(), sl.h_q.get(), off * 16, cudaMemcpyHostToDevice, sl.st));
      EWT_CUDA(cudaMemcpyAsync(sl.d_types.get(), sl.h_types.get(), off, cudaMemcpyHostToDevice, sl.st));
      EWT_CUDA(cudaMemcpyAsync(sl.d_items.get(), sl.h_items.get(), nitems * sizeof(ServeItem),
                               cudaMemcpyHostToDevice, sl.st));
      launch_multi_items(S->cfg.elem_size, S->views_d, sl.d_items.get(), nitems,
                         S->max_levels, sl.d_types.as<uint8_t>(), sl.d_q.get(),
                         sl.d_out.as<uint64_t>(), sl.d_err.as<uint32_t>(), sl.st);
      EWT_CUDA(cudaMemcpyAsync(sl.h_out.get(), sl.d_out.get(), off * 8, cudaMemcpyDeviceToHost, sl.st));
      EWT_CUDA(cudaMemcpyAsync(sl.h_err.get(), sl.d_err.get(), 4, cudaMemcpyDeviceToHost, sl.st));
      EWT_CUDA(cudaEventRecord(sl.done, sl.st));
    } catch (std::exception const& e) {
      std::lock_guard<std::mutex> lk(S->mu);
      S->fatal = e.what();
      for (auto* r : batch) S->sched.complete(r->id, EWT_ERR_CUDA, now_s());
      sl.busy = false;
      S->cv_done.notify_all();
      S->cv_work.notify_all();
      continue;
    }
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->launched.push_back(si);
    }
    S->cv_launched.notify_one();
  }
}

void completer_loop(ewt_server* S) {
  DeviceGuard g(S->device);
  for (;;) {
    int si;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_launched.wait(lk, [&] {
        if (!S->launched.empty()) return true;
        // stop once nothing is queued, launched or being packed
        if (!S->stop || S->sched.has_queries()) return false;
        for (auto const& sl : S->slots)
          if (sl.busy) return false;
        return true;
      });
      if (S->launched.empty()) return;
      si = S->launched.front();
      S->launched.pop_front();
    }
    Slot& sl = S->slots[si];
    cudaError_t const e = cudaEventSynchronize(sl.done);
    double const t = now_s();
    std::vector<int> status(sl.reqs.size(), EWT_OK);
    if (e == cudaSuccess && S->zero_copy) {
      uint32_t const* rerr = sl.h_reqerr.as<uint32_t>();
      for (size_t i = 0; i < sl.reqs.size(); ++i)
        if (rerr[i]) status[i] = EWT_ERR_QUERY;
    } else if (e == cudaSuccess) {
      uint64_t const* out = sl.h_out.as<uint64_t>();
      // the batch's invalid-query word says whether any request must be
      // scanned for the UINT64_MAX results of invalid queries
      bool const any_bad = *sl.h_err.as<uint32_t>() != 0;
      for (size_t i = 0; i < sl.reqs.size(); ++i) {
        sched::Request* r = sl.reqs[i];
        uint64_t const o = sl.offs[i];
        std::memcpy(r->results, out + o, r->m * 8);
        if (any_bad)
          for (uint64_t j = 0; j < r->m; ++j)
            if (r->types[j] != 0 && out[o + j] == UINT64_MAX) {
              status[i] = EWT_ERR_QUERY;
              break;
            }
      }
    } else {
      (void)cudaGetLastError();
      for (auto& s : status) s = EWT_ERR_CUDA;
    }
    {
      std::lock_guard<std::mutex> lk(S->mu);
      for (size_t i = 0; i < sl.reqs.size(); ++i)
        S->sched.complete(sl.reqs[i]->id, status[i], t);
      sl.reqs.clear();
      sl.busy = false;
    }
    S->cv_done.notify_all();
    S->cv_work.notify_all();
    S->cv_launched.notify_all();
  }
}

uint32_t register_tree(ewt_server* S, ewt_tree* t, bool owned) {
  // caller holds S->mu
  EWT_REQUIRE(S->trees.size() < kMaxServerTrees, EWT_ERR_TOO_LARGE,
              "the server holds at most 4096 trees");
  EWT_REQUIRE(t->elem_size == S->cfg.elem_size, EWT_ERR_INVALID_ARGUMENT,
              "the tree's symbol size differs from the server's");
  EWT_REQUIRE(t->device == S->device, EWT_ERR_INVALID_ARGUMENT,
              "the tree lives on another GPU");
  uint32_t const id = static_cast<uint32_t>(S->trees.size());
  t->view_shared.store(true);
  EWT_CUDA(cudaMemcpy(S->views_d + id, &t->view, sizeof(TreeView), cudaMemcpyHostToDevice));
  S->trees.push_back(t);
  S->owned.push_back(owned);
  S->tree_bytes.push_back(t->device_bytes());
  S->max_levels = std::max(S->max_levels, t->L);
  return id;
}

void builder_loop(ewt_server* S) {
  DeviceGuard g(S->device);
  for (;;) {
    sched::Request* r = nullptr;
    BuildJob job;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_build.wait(lk, [&] {
        if (S->stop) return true;
        r = S->sched.take_build(now_s());
        return r != nullptr;
      });
      if (!r) return;  // stopping; pending builds stay pending
      job = S->build_jobs[r->id];
      S->build_jobs.erase(r->id);
    }
    ewt_tree* t = nullptr;
    int const st = ewt_build(job.text, job.n, static_cast<int>(S->cfg.elem_size),
                             job.alphabet, job.sigma, S->device, &t);
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->sched.release(r->footprint);
      int status = st;
      if (st == EWT_OK) {
        try {
          r->built_tree = register_tree(S, t, true);
          S->sched.reserve(S->tree_bytes.back());
        } catch (Error const& e) {
          status = e.status;
          ewt_free(t);
        }
      }
      S->sched.complete(r->id, status, now_s());
    }
    S->cv_done.notify_all();
    S->cv_build.notify_all();
  }
}

}  // namespace
}  // namespace ewt

using namespace ewt;

extern "C" int ewt_server_create(int gpu_index, const ewt_server_config* cfg,
                                 ewt_server** out) {
  return run_guarded([&] {
    EWT_REQUIRE(cfg && out, EWT_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    EWT_REQUIRE(cfg->batch_queries >= 1 && cfg->batch_requests >= 1 &&
                    cfg->inflight >= 1 && cfg->inflight <= 8,
                EWT_ERR_INVALID_ARGUMENT, "invalid batch capacities");
    EWT_REQUIRE(cfg->elem_size == 1 || cfg->elem_size == 2 || cfg->elem_size == 4 ||
                    cfg->elem_size == 8,
                EWT_ERR_INVALID_ARGUMENT, "elem_size must be 1, 2, 4 or 8");
    DeviceGuard g(gpu_index);
    auto S = std::make_unique<ewt_server>(*cfg);
    S->device = gpu_index;
    EWT_CUDA(cudaMalloc(&S->views_d, kMaxServerTrees * sizeof(TreeView)));
    uint64_t const q = cfg->batch_queries;
    uint64_t const items = q / kServeChunk + cfg->batch_requests + 1;
    // With pageable-memory access (address translation through the host's
    // page tables, as on Grace-hosted GPUs) kernels read the callers' query
    // buffers and write their result buffers in place: no staging copies.
    int pageable = 0;
    EWT_CUDA(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, gpu_index));
    S->zero_copy = pageable == 1 && !cfg->force_staging;
    prepare_serve_kernels(cfg->elem_size);
    for (uint32_t i = 0; i < cfg->inflight; ++i) S->slots.emplace_back();
    for (auto& sl : S->slots) {
      EWT_CUDA(cudaStreamCreateWithFlags(&sl.st, cudaStreamNonBlocking));
      EWT_CUDA(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming));
      sl.h_items.ensure(items * sizeof(ServeItem));
      sl.h_err.ensure(16);
      if (S->zero_copy) {
        sl.h_reqs.ensure(cfg->batch_requests * sizeof(ServeReqH));
        sl.h_reqerr.ensure(cfg->batch_requests * 4);
        continue;
      }
      sl.h_q.ensure(q * 16);
      sl.h_types.ensure(q);
      sl.h_out.ensure(q * 8);
      sl.d_q.alloc(q * 16);
      sl.d_types.alloc(q);
      sl.d_items.alloc(items * sizeof(ServeItem));
      sl.d_out.alloc(q * 8);
      sl.d_err.alloc(16);
    }
    ewt_server* raw = S.get();
    S->dispatcher = std::thread(dispatcher_loop, raw);
    S->completer = std::thread(completer_loop, raw);
    S->builder = std::thread(builder_loop, raw);
    *out = S.release();
  });
}

extern "C" int ewt_server_destroy(ewt_server* S) {
  return run_guarded([&] {
    if (!S) return;
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->stop = true;
    }
    S->cv_work.notify_all();
    S->cv_launched.notify_all();
    S->cv_build.notify_all();
    S->dispatcher.join();
    S->completer.join();
    S->builder.join();
    DeviceGuard g(S->device);
    for (auto& sl : S->slots) {
      cudaStreamSynchronize(sl.st);
      cudaEventDestroy(sl.done);
      cudaStreamDestroy(sl.st);
    }
    for (size_t i = 0; i < S->trees.size(); ++i)
      if (S->owned[i] && S->trees[i]) ewt_free(S->trees[i]);
    cudaFree(S->views_d);
    delete S;
  });
}

extern "C" int ewt_server_add_tree(ewt_server* S, ewt_tree* tree, uint32_t* tree_id) {
  return run_guarded([&] {
    EWT_REQUIRE(S && tree && tree_id, EWT_ERR_INVALID_ARGUMENT, "null argument");
    DeviceGuard g(S->device);
    std::lock_guard<std::mutex> lk(S->mu);
    *tree_id = register_tree(S, tree, false);
    S->sched.reserve(S->tree_bytes.back());
  });
}

extern "C" int ewt_server_submit(ewt_server* S, uint32_t tree_id,
                                 const uint8_t* types, const void* queries,
                                 uint64_t m, uint64_t* results,
                                 uint64_t* request_id) {
  return run_guarded([&] {
    EWT_REQUIRE(S && types && queries && results && request_id,
                EWT_ERR_INVALID_ARGUMENT, "null argument");
    {
      std::lock_guard<std::mutex> lk(S->mu);
      EWT_REQUIRE(tree_id < S->trees.size() && S->trees[tree_id],
                  EWT_ERR_INVALID_ARGUMENT, "unknown tree id");
      EWT_REQUIRE(!S->stop, EWT_ERR_INVALID_ARGUMENT, "the server is stopping");
      try {
        *request_id = S->sched.submit_query(tree_id, m, types, queries, results, now_s());
      } catch (std::length_error const&) {
        throw Error(EWT_ERR_TOO_LARGE,
                    "a request holds 1 .. batch_queries queries");
      }
    }
    S->cv_work.notify_one();
  });
}

extern "C" int ewt_server_submit_build(ewt_server* S, const void* text, uint64_t n,
                                       const void* alphabet, uint64_t sigma,
                                       uint64_t* request_id) {
  return run_guarded([&] {
    EWT_REQUIRE(S && text && n && request_id, EWT_ERR_INVALID_ARGUMENT, "null argument");
    {
      std::lock_guard<std::mutex> lk(S->mu);
      EWT_REQUIRE(!S->stop, EWT_ERR_INVALID_ARGUMENT, "the server is stopping");
      uint64_t id = 0;
      try {
        id = S->sched.submit_build(build_footprint(n, S->cfg.elem_size), now_s());
      } catch (std::length_error const&) {
        throw Error(EWT_ERR_OUT_OF_MEMORY,
                    "the build does not fit the server's memory budget");
      }
      S->build_jobs[id] = BuildJob{text, n, alphabet, sigma};
      *request_id = id;
    }
    S->cv_build.notify_one();
  });
}

extern "C" int ewt_server_wait(ewt_server* S, uint64_t request_id, int* status,
                               double* latency_ms, uint32_t* tree_id) {
  return run_guarded([&] {
    EWT_REQUIRE(S, EWT_ERR_INVALID_ARGUMENT, "server is null");
    std::unique_lock<std::mutex> lk(S->mu);
    EWT_REQUIRE(S->sched.find(request_id), EWT_ERR_INVALID_ARGUMENT,
                "unknown request id (or already waited for)");
    S->cv_done.wait(lk, [&] {
      auto const* r = S->sched.find(request_id);
      return r->state == sched::kDone || r->state == sched::kCancelled;
    });
    auto const* r = S->sched.find(request_id);
    if (status) *status = r->state == sched::kCancelled ? EWT_ERR_CANCELLED : r->status;
    if (latency_ms) *latency_ms = (r->t_done - r->t_submit) * 1e3;
    if (tree_id) *tree_id = r->built_tree;
    S->sched.forget(request_id);
  });
}

extern "C" int ewt_server_cancel(ewt_server* S, uint64_t request_id) {
  return run_guarded([&] {
    EWT_REQUIRE(S, EWT_ERR_INVALID_ARGUMENT, "server is null");
    bool ok;
    {
      std::lock_guard<std::mutex> lk(S->mu);
      ok = S->sched.cancel(request_id, now_s());
      if (ok) S->build_jobs.erase(request_id);
    }
    S->cv_done.notify_all();
    EWT_REQUIRE(ok, EWT_ERR_INVALID_ARGUMENT,
                "the request is unknown or already running");
  });
}

extern "C" int ewt_server_remove_tree(ewt_server* S, uint32_t tree_id) {
  return run_guarded([&] {
    EWT_REQUIRE(S, EWT_ERR_INVALID_ARGUMENT, "server is null");
    ewt_tree* t = nullptr;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      EWT_REQUIRE(tree_id < S->trees.size() && S->trees[tree_id],
                  EWT_ERR_INVALID_ARGUMENT, "unknown tree id");
      // no batch may still reference it: wait for all queued and running
      S->cv_done.wait(lk, [&] {
        if (S->sched.has_queries()) return false;
        for (auto const& sl : S->slots)
          if (sl.busy) return false;
        return true;
      });
      if (S->owned[tree_id]) t = S->trees[tree_id];
      S->trees[tree_id] = nullptr;
      S->sched.release(S->tree_bytes[tree_id]);
    }
    if (t) ewt_free(t);
    S->cv_build.notify_all();
  });
}

extern "C" int ewt_server_stats(ewt_server* S, ewt_sched_stats* out, int reset) {
  return run_guarded([&] {
    EWT_REQUIRE(S && out, EWT_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    auto const st = S->sched.stats();
    out->submitted = st.submitted;
    out->completed = st.completed;
    out->cancelled = st.cancelled;
    out->failed = st.failed;
    out->batches = st.batches;
    out->batched_requests = st.batched_requests;
    out->queries = st.queries;
    out->p50_ms = st.p50_ms;
    out->p99_ms = st.p99_ms;
    out->max_ms = st.max_ms;
    out->mean_ms = st.mean_ms;
    if (reset) S->sched.reset_latencies();
  });
}

// ---- native load generator ------------------------------------------------
namespace ewt {
namespace {

// A pool of valid mixed queries for one tree (ranges of the reference's
// generators: access i in [0, n), rank c uniform, i in [0, n], select c
// uniform over present symbols, k in [1, count(c)]).
struct QueryPool {
  std::vector<uint8_t> types;
  std::vector<unsigned char> recs;  // 16-byte RankSelectQuery records
};

QueryPool make_pool(ewt_tree const& t, uint64_t size, double fa, double fr,
                    std::mt19937_64& rng) {
  QueryPool p;
  p.types.resize(size);
  p.recs.assign(size * 16, 0);
  std::uniform_real_distribution<double> u01(0.0, 1.0);
  std::vector<uint64_t> present;
  for (uint64_t c = 0; c < t.sigma; ++c)
    if (t.occ[c]) present.push_back(c);
  for (uint64_t i = 0; i < size; ++i) {
    double const x = u01(rng);
    uint8_t ty = x < fa ? 0 : (x < fa + fr ? 1 : 2);
    uint64_t index = 0, sym = 0;
    if (ty == 0) {
      index = rng() % t.n;
    } else if (ty == 1) {
      sym = rng() % t.sigma;
      index = rng() % (t.n + 1);
    } else {
      uint64_t const c = present[rng() % present.size()];
      sym = c;
      index = 1 + rng() % t.occ[c];
    }
    uint64_t const orig = t.is_min ? sym : t.alphabet[sym];
    p.types[i] = ty;
    std::memcpy(&p.recs[i * 16], &index, 8);
    std::memcpy(&p.recs[i * 16 + 8], &orig, t.elem_size);
  }
  return p;
}

double pct(std::vector<double>& v, double p) {
  if (v.empty()) return 0;
  std::sort(v.begin(), v.end());
  size_t const k = static_cast<size_t>(p * (v.size() - 1) + 0.5);
  return v[std::min(k, v.size() - 1)];
}

}  // namespace
}  // namespace ewt

extern "C" int ewt_server_run_load(ewt_server* S, const ewt_load_config* cfg,
                                   ewt_load_result* res) {
  return run_guarded([&] {
    EWT_REQUIRE(S && cfg && res, EWT_ERR_INVALID_ARGUMENT, "null argument");
    EWT_REQUIRE(cfg->rate > 0 && cfg->duration_s > 0 && cfg->max_request >= 1 &&
                    cfg->num_trees >= 1,
                EWT_ERR_INVALID_ARGUMENT, "invalid load parameters");
    std::memset(res, 0, sizeof(*res));
    std::vector<ewt_tree*> targets;
    {
      std::lock_guard<std::mutex> lk(S->mu);
      for (uint32_t i = 0; i < cfg->num_trees; ++i) {
        uint32_t const id = cfg->first_tree + i;
        EWT_REQUIRE(id < S->trees.size() && S->trees[id], EWT_ERR_INVALID_ARGUMENT,
                    "unknown target tree");
        targets.push_back(S->trees[id]);
      }
      EWT_REQUIRE(cfg->max_request <= S->cfg.batch_queries, EWT_ERR_TOO_LARGE,
                  "max_request exceeds the server's batch size");
      S->sched.reset_latencies();
    }
    std::mt19937_64 rng(cfg->seed);
    uint64_t const pool_size = std::max<uint64_t>(uint64_t(1) << 17, 2ull * cfg->max_request);
    std::vector<QueryPool> pools;
    for (auto* t : targets)
      pools.push_back(make_pool(*t, pool_size, cfg->frac_access, cfg->frac_rank, rng));
    // results land in a ring; requests in flight at once stay far below it
    uint64_t const ring = uint64_t(1) << 24;
    std::vector<uint64_t> results(ring + cfg->max_request);
    uint64_t cursor = 0;
    std::exponential_distribution<double> gap(cfg->rate);
    std::uniform_real_distribution<double> u01(0.0, 1.0);
    double const lmax = std::log(double(cfg->max_request));
    struct Arrival {
      uint32_t tree;
      uint64_t off, m, res;
      double t;
    };
    std::vector<Arrival> arrivals;
    for (double t = 0; t < cfg->duration_s; t += gap(rng)) {
      Arrival a;
      a.tree = static_cast<uint32_t>(rng() % targets.size());
      a.m = std::min<uint64_t>(cfg->max_request,
                               static_cast<uint64_t>(std::exp(u01(rng) * lmax)));
      a.m = std::max<uint64_t>(a.m, 1);
      a.off = rng() % (pool_size - a.m + 1);
      if (cursor + a.m > ring) cursor = 0;
      a.res = cursor;
      cursor += a.m;
      a.t = t;
      arrivals.push_back(a);
    }
    // build requests of sigma-4 uint8 texts, if asked
    std::vector<uint8_t> build_text;
    if (cfg->build_n && S->cfg.elem_size == 1) {
      build_text.resize(cfg->build_n);
      for (auto& c : build_text) c = static_cast<uint8_t>(rng() & 3);
    }
    uint8_t const alpha4[4] = {0, 1, 2, 3};
    std::vector<double> lat;
    lat.reserve(arrivals.size());
    uint64_t queries = 0;
    double const t0 = now_s();
    if (!cfg->plain) {
      std::vector<uint64_t> ids, build_ids;
      ids.reserve(arrivals.size());
      double next_build = cfg->build_interval_s > 0 ? cfg->build_interval_s : 1e300;
      for (auto const& a : arrivals) {
        while (now_s() - t0 < a.t) {
        }
        if (!build_text.empty() && a.t >= next_build) {
          uint64_t bid = 0;
          if (ewt_server_submit_build(S, build_text.data(), build_text.size(), alpha4,
                                      4, &bid) == EWT_OK)
            build_ids.push_back(bid);
          next_build += cfg->build_interval_s;
        }
        QueryPool const& p = pools[a.tree];
        uint64_t id = 0;
        int const st = ewt_server_submit(S, cfg->first_tree + a.tree, p.types.data() + a.off,
                                         p.recs.data() + a.off * 16, a.m,
                                         results.data() + a.res, &id);
        if (st != EWT_OK) throw Error(st, ewt_last_error());
        ids.push_back(id);
        queries += a.m;
      }
      for (uint64_t id : ids) {
        int st = 0;
        double ms = 0;
        int const w = ewt_server_wait(S, id, &st, &ms, nullptr);
        if (w != EWT_OK) throw Error(w, ewt_last_error());
        lat.push_back(ms);
      }
      std::vector<double> blat;
      for (uint64_t id : build_ids) {
        int st = 0;
        double ms = 0;
        if (ewt_server_wait(S, id, &st, &ms, nullptr) == EWT_OK && st == EWT_OK)
          blat.push_back(ms);
      }
      res->builds = blat.size();
      res->build_p50_ms = pct(blat, 0.5);
      ewt_sched_stats ss{};
      ewt_server_stats(S, &ss, 0);
      res->batches = ss.batches;
    } else {
      // plain per-request path: one synchronous host call per request, in
      // arrival order, from one worker
      std::mutex qm;
      std::condition_variable qcv;
      std::deque<std::pair<size_t, double>> queue;  // arrival index, submit time
      bool done = false;
      std::thread worker([&] {
        for (;;) {
          std::pair<size_t, double> job;
          {
            std::unique_lock<std::mutex> lk(qm);
            qcv.wait(lk, [&] { return done || !queue.empty(); });
            if (queue.empty()) return;
            job = queue.front();
            queue.pop_front();
          }
          Arrival const& a = arrivals[job.first];
          QueryPool const& p = pools[a.tree];
          (void)ewt_mixed(targets[a.tree], p.types.data() + a.off,
                          p.recs.data() + a.off * 16, a.m, results.data() + a.res);
          lat.push_back((now_s() - job.second) * 1e3);
        }
      });
      for (size_t i = 0; i < arrivals.size(); ++i) {
        while (now_s() - t0 < arrivals[i].t) {
        }
        {
          std::lock_guard<std::mutex> lk(qm);
          queue.emplace_back(i, now_s());
        }
        qcv.notify_one();
        queries += arrivals[i].m;
      }
      {
        std::lock_guard<std::mutex> lk(qm);
        done = true;
      }
      qcv.notify_one();
      worker.join();
    }
    double const wall = now_s() - t0;
    res->requests = arrivals.size();
    res->queries = queries;
    res->wall_s = wall;
    res->qps = queries / wall;
    double sum = 0;
    for (double x : lat) sum += x;
    res->mean_ms = lat.empty() ? 0 : sum / lat.size();
    res->p50_ms = pct(lat, 0.50);
    res->p99_ms = pct(lat, 0.99);
    res->max_ms = lat.empty() ? 0 : lat.back();
  });
}
