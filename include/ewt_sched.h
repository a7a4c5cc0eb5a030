/* Scheduling core of the serving engine (ewt_server_* in ewt.h), exposed
 * on its own so that admission, batching, cancellation and latency
 * accounting can be exercised without a GPU.  Exported by libewt.so and by
 * the CUDA-free libewt_sched.so.  No reference counterpart: the reference
 * has no serving layer (its host API answers one synchronous call at a
 * time, wavelet_tree.cuh:956-1797).  Times are host seconds. */
#ifndef EWT_SCHED_H
#define EWT_SCHED_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct ewt_sched ewt_sched;

/* A batch holds at most batch_queries queries and batch_requests
 * requests; builds are admitted while their footprints fit into
 * budget_bytes.  NULL on invalid capacities. */
ewt_sched* ewt_sched_create(uint64_t batch_queries, uint32_t batch_requests,
                            uint64_t budget_bytes);
void ewt_sched_destroy(ewt_sched* s);
/* Request ids (> 0), or 0 when the request is refused (m == 0, m above
 * batch_queries, footprint above the budget). */
uint64_t ewt_sched_submit_query(ewt_sched* s, uint32_t tree, uint64_t m,
                                double now);
uint64_t ewt_sched_submit_build(ewt_sched* s, uint64_t footprint, double now);
/* 1 when the request was still pending and is now cancelled, else 0. */
int ewt_sched_cancel(ewt_sched* s, uint64_t id, double now);
/* Takes the next batch (FIFO prefix that fits); writes up to cap ids and
 * returns how many were taken. */
uint32_t ewt_sched_take_batch(ewt_sched* s, double now, uint64_t* ids,
                              uint32_t cap);
/* Takes the first pending build that fits the free budget (its footprint is
 * reserved); 0 when none fits. */
uint64_t ewt_sched_take_build(ewt_sched* s, double now);
void ewt_sched_reserve(ewt_sched* s, uint64_t bytes);
void ewt_sched_release(ewt_sched* s, uint64_t bytes);
uint64_t ewt_sched_used(const ewt_sched* s);
void ewt_sched_complete(ewt_sched* s, uint64_t id, int status, double now);
/* State of a request: 0 pending, 1 running, 2 done, 3 cancelled, -1
 * unknown. */
int ewt_sched_state(const ewt_sched* s, uint64_t id);

typedef struct ewt_sched_stats {
  uint64_t submitted, completed, cancelled, failed;
  uint64_t batches, batched_requests, queries;
  double p50_ms, p99_ms, max_ms, mean_ms;
} ewt_sched_stats;
void ewt_sched_get_stats(const ewt_sched* s, ewt_sched_stats* out);

#ifdef __cplusplus
}
#endif
#endif /* EWT_SCHED_H */
