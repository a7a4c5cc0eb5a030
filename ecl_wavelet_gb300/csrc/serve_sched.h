// Scheduling core of the serving engine: no CUDA, so that it can be
// compiled and tested on a host without a GPU.
//
// Requests are queries against one resident tree, or builds of a new text.
// Query requests wait in FIFO order and are admitted into a batch while it
// has room (at most batch_queries queries and batch_requests requests); a
// batch is taken whenever the GPU has a free batch slot, so requests that
// arrive while earlier batches run join the next one (continuous batching).
// Build requests are admitted by device-memory footprint: the first pending
// build whose estimate fits into budget - used starts; memory is returned
// with release().  A request can be cancelled until it is taken.
#pragma once
#include <algorithm>
#include <cstdint>
#include <deque>
#include <stdexcept>
#include <unordered_map>
#include <vector>

namespace ewt {
namespace sched {

enum Kind { kQuery = 0, kBuild = 1 };
enum State { kPending = 0, kRunning = 1, kDone = 2, kCancelled = 3 };

struct Request {
  uint64_t id = 0;
  int kind = kQuery;
  int state = kPending;
  int status = 0;
  // query requests
  uint32_t tree = 0;
  uint64_t m = 0;
  const uint8_t* types = nullptr;
  const void* queries = nullptr;
  uint64_t* results = nullptr;
  // build requests
  uint64_t footprint = 0;
  uint32_t built_tree = 0;
  // host clock, seconds
  double t_submit = 0, t_start = 0, t_done = 0;
};

struct Stats {
  uint64_t submitted = 0, completed = 0, cancelled = 0, failed = 0;
  uint64_t batches = 0, batched_requests = 0, queries = 0;
  double p50_ms = 0, p99_ms = 0, max_ms = 0, mean_ms = 0;
};

class Scheduler {
 public:
  Scheduler(uint64_t batch_queries, uint32_t batch_requests, uint64_t budget)
      : batch_queries_(batch_queries), batch_requests_(batch_requests),
        budget_(budget) {
    if (batch_queries == 0 || batch_requests == 0)
      throw std::invalid_argument("batch capacity must be positive");
  }

  uint64_t submit_query(uint32_t tree, uint64_t m, const uint8_t* types,
                        const void* queries, uint64_t* results, double now) {
    if (m == 0 || m > batch_queries_)
      throw std::length_error("a request holds 1 .. batch_queries queries");
    Request r;
    r.id = next_id_++;
    r.kind = kQuery;
    r.tree = tree;
    r.m = m;
    r.types = types;
    r.queries = queries;
    r.results = results;
    r.t_submit = now;
    reqs_[r.id] = r;
    queue_.push_back(r.id);
    ++stats_.submitted;
    return r.id;
  }

  uint64_t submit_build(uint64_t footprint, double now) {
    if (footprint > budget_)
      throw std::length_error("the build's footprint exceeds the memory budget");
    Request r;
    r.id = next_id_++;
    r.kind = kBuild;
    r.footprint = footprint;
    r.t_submit = now;
    reqs_[r.id] = r;
    builds_.push_back(r.id);
    ++stats_.submitted;
    return r.id;
  }

  // Cancels a request that has not been taken yet.
  bool cancel(uint64_t id, double now) {
    auto it = reqs_.find(id);
    if (it == reqs_.end() || it->second.state != kPending) return false;
    auto& q = it->second.kind == kQuery ? queue_ : builds_;
    q.erase(std::remove(q.begin(), q.end(), id), q.end());
    it->second.state = kCancelled;
    it->second.t_done = now;
    ++stats_.cancelled;
    return true;
  }

  bool has_queries() const { return !queue_.empty(); }
  bool has_builds() const { return !builds_.empty(); }

  // The FIFO prefix of pending query requests that fits one batch.
  std::vector<Request*> take_batch(double now) {
    std::vector<Request*> out;
    uint64_t q = 0;
    while (!queue_.empty() && out.size() < batch_requests_) {
      Request& r = reqs_.at(queue_.front());
      if (q + r.m > batch_queries_) break;
      q += r.m;
      r.state = kRunning;
      r.t_start = now;
      out.push_back(&r);
      queue_.pop_front();
    }
    if (!out.empty()) {
      ++stats_.batches;
      stats_.batched_requests += out.size();
      stats_.queries += q;
    }
    return out;
  }

  // The first pending build whose footprint fits; its memory is reserved.
  Request* take_build(double now) {
    for (auto it = builds_.begin(); it != builds_.end(); ++it) {
      Request& r = reqs_.at(*it);
      if (used_ + r.footprint <= budget_) {
        used_ += r.footprint;
        r.state = kRunning;
        r.t_start = now;
        builds_.erase(it);
        return &r;
      }
    }
    return nullptr;
  }

  // Device memory accounting (resident trees, running builds).
  void reserve(uint64_t bytes) { used_ += bytes; }
  void release(uint64_t bytes) { used_ -= std::min(used_, bytes); }
  uint64_t used() const { return used_; }
  uint64_t budget() const { return budget_; }

  void complete(uint64_t id, int status, double now) {
    Request& r = reqs_.at(id);
    r.state = kDone;
    r.status = status;
    r.t_done = now;
    ++stats_.completed;
    if (status != 0) ++stats_.failed;
    lat_ms_.push_back((r.t_done - r.t_submit) * 1e3);
  }

  Request const* find(uint64_t id) const {
    auto it = reqs_.find(id);
    return it == reqs_.end() ? nullptr : &it->second;
  }
  Request* find(uint64_t id) {
    auto it = reqs_.find(id);
    return it == reqs_.end() ? nullptr : &it->second;
  }
  void forget(uint64_t id) { reqs_.erase(id); }

  // Latency percentiles over the completed requests (nearest rank).
  Stats stats() const {
    Stats s = stats_;
    if (!lat_ms_.empty()) {
      std::vector<double> v(lat_ms_);
      std::sort(v.begin(), v.end());
      auto pct = [&](double p) {
        size_t const k = static_cast<size_t>(p * (v.size() - 1) + 0.5);
        return v[std::min(k, v.size() - 1)];
      };
      s.p50_ms = pct(0.50);
      s.p99_ms = pct(0.99);
      s.max_ms = v.back();
      double sum = 0;
      for (double x : v) sum += x;
      s.mean_ms = sum / v.size();
    }
    return s;
  }
  void reset_latencies() { lat_ms_.clear(); }

 private:
  uint64_t batch_queries_;
  uint32_t batch_requests_;
  uint64_t budget_, used_ = 0;
  uint64_t next_id_ = 1;
  std::unordered_map<uint64_t, Request> reqs_;
  std::deque<uint64_t> queue_, builds_;
  std::vector<double> lat_ms_;
  Stats stats_;
};

}  // namespace sched
}  // namespace ewt
