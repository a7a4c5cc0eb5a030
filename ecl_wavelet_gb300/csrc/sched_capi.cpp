// C ABI of the serving engine's scheduling core (include/ewt_sched.h).
// Plain C++: built into libewt.so and, without CUDA, into libewt_sched.so.
#include "ewt_sched.h"

#include <new>

#include "serve_sched.h"

using ewt::sched::Scheduler;

struct ewt_sched {
  Scheduler core;
  ewt_sched(uint64_t q, uint32_t r, uint64_t b) : core(q, r, b) {}
};

extern "C" {

ewt_sched* ewt_sched_create(uint64_t batch_queries, uint32_t batch_requests,
                            uint64_t budget_bytes) {
  try {
    return new ewt_sched(batch_queries, batch_requests, budget_bytes);
  } catch (...) {
    return nullptr;
  }
}

void ewt_sched_destroy(ewt_sched* s) { delete s; }

uint64_t ewt_sched_submit_query(ewt_sched* s, uint32_t tree, uint64_t m,
                                double now) {
  try {
    return s->core.submit_query(tree, m, nullptr, nullptr, nullptr, now);
  } catch (...) {
    return 0;
  }
}

uint64_t ewt_sched_submit_build(ewt_sched* s, uint64_t footprint, double now) {
  try {
    return s->core.submit_build(footprint, now);
  } catch (...) {
    return 0;
  }
}

int ewt_sched_cancel(ewt_sched* s, uint64_t id, double now) {
  return s->core.cancel(id, now) ? 1 : 0;
}

uint32_t ewt_sched_take_batch(ewt_sched* s, double now, uint64_t* ids,
                              uint32_t cap) {
  auto batch = s->core.take_batch(now);
  uint32_t n = 0;
  for (auto* r : batch) {
    if (n < cap) ids[n] = r->id;
    ++n;
  }
  return n;
}

uint64_t ewt_sched_take_build(ewt_sched* s, double now) {
  auto* r = s->core.take_build(now);
  return r ? r->id : 0;
}

void ewt_sched_reserve(ewt_sched* s, uint64_t bytes) { s->core.reserve(bytes); }
void ewt_sched_release(ewt_sched* s, uint64_t bytes) { s->core.release(bytes); }
uint64_t ewt_sched_used(const ewt_sched* s) { return s->core.used(); }

void ewt_sched_complete(ewt_sched* s, uint64_t id, int status, double now) {
  if (s->core.find(id)) s->core.complete(id, status, now);
}

int ewt_sched_state(const ewt_sched* s, uint64_t id) {
  auto const* r = s->core.find(id);
  return r ? r->state : -1;
}

void ewt_sched_get_stats(const ewt_sched* s, ewt_sched_stats* out) {
  auto const st = s->core.stats();
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
}

}  // extern "C"
