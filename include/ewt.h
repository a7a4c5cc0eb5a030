/*
 * ewt.h — C ABI of the GB300 wavelet-tree library (libewt.so).
 *
 * This is the drop-in boundary for the hot path of mfranzreb/ECL_wavelet:
 * wavelet-tree construction, RankSelect support over packed bit arrays, and
 * batched access / rank / select queries.  Every entry point takes plain
 * pointers and sizes, returns an int status (EWT_OK or a negative EWT_ERR_*),
 * and never throws.  The C++ header <ecl_wavelet/tree/wavelet_tree.cuh>
 * wraps it into the reference's ecl::WaveletTree<T> class and rethrows
 * std::runtime_error with the reference's messages.
 *
 * Reference interfaces replaced (paths inside the ECL_wavelet project):
 *   ewt_build*         WaveletTree<T>::WaveletTree(data, n, alphabet, gpu)
 *                        include/ecl_wavelet/tree/wavelet_tree.cuh:576-867
 *   ewt_free           WaveletTree<T>::~WaveletTree   wavelet_tree.cuh:931-943
 *   ewt_access         WaveletTree<T>::access         wavelet_tree.cuh:956-1231
 *   ewt_rank           WaveletTree<T>::rank           wavelet_tree.cuh:1247-1551
 *   ewt_select         WaveletTree<T>::select         wavelet_tree.cuh:1567-1797
 *   ewt_*_device       accessKernel / rankKernel / selectKernel launched on
 *                        device-resident queries      wavelet_tree.cuh:373-544
 *   ewt_mixed*         no counterpart: one launch answers interleaved access,
 *                        rank and select queries (batched form)
 *   ewt_get_info       getAlphabetSize / getNumLevels / isMinAlphabet /
 *                        getCodesStart               wavelet_tree.cuh:2165-2228
 *   ewt_export         the device arrays the reference keeps private
 *                        (BitArray words, RankSelect L1/L2/samples, counts,
 *                        precomputed node ranks), copied to the host
 *   ewt_get_device_view  the by-value WaveletTree<T> copy a user kernel
 *                        receives (copy ctor wavelet_tree.cuh:870-887)
 *   ewt_rs_*           RankSelect(BitArray&&, gpu)   src/bitarray/rank_select.cu:50-304
 *                        and BitArray(sizes, init)   src/bitarray/bit_array.cu:40-100
 */
#ifndef EWT_H
#define EWT_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EWT_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
#define EWT_OK 0
#define EWT_ERR_INVALID_ARGUMENT (-1) /* null pointer, n == 0, bad elem size */
#define EWT_ERR_OUT_OF_MEMORY (-2)    /* device or pinned allocation failed  */
#define EWT_ERR_CUDA (-3)             /* any other CUDA runtime error        */
#define EWT_ERR_ALPHABET (-4) /* alphabet unsorted, < 2 symbols, or the text
                                 holds a symbol above the last one          */
#define EWT_ERR_QUERY (-5)    /* a batch held an invalid query: select with
                                 k == 0, rank with index > n, or a symbol
                                 above the alphabet's last symbol; the other
                                 answers of the batch are still written     */
#define EWT_ERR_UNSUPPORTED (-6)
#define EWT_ERR_TIMEOUT (-7) /* a bounded device-side wait gave up        */
#define EWT_ERR_TOO_LARGE (-8) /* size beyond a stated fixed maximum      */
#define EWT_ERR_CANCELLED (-9) /* the request was cancelled before it ran */

/* ---- query types of the mixed batch ----------------------------------- */
#define EWT_Q_ACCESS 0
#define EWT_Q_RANK 1
#define EWT_Q_SELECT 2

/* ---- components returned by ewt_export / ewt_rs_export ----------------- */
#define EWT_EXP_COUNTS 1         /* u64 x sigma: exclusive prefix C[c]       */
#define EWT_EXP_LEVEL_WORDS 2    /* u32 x ceil(bits/32) of one level/array   */
#define EWT_EXP_L1 3             /* u64 x num_l1 of one level/array          */
#define EWT_EXP_L2 4             /* u16 x num_l2 of one level/array          */
#define EWT_EXP_SAMPLES0 5       /* u64 select samples of zeros              */
#define EWT_EXP_SAMPLES1 6       /* u64 select samples of ones               */
#define EWT_EXP_TOTAL_ONES 7     /* u64 x levels (or arrays)                 */
#define EWT_EXP_LEVEL_SIZES 8    /* u64 x levels (or arrays): bits per array */
#define EWT_EXP_NODE_RANKS 9     /* u64 x num_ranks: rank0 at node starts    */
#define EWT_EXP_NODE_INFOS 10    /* (u64 start, u64 level) x num_ranks       */
#define EWT_EXP_CODES 11         /* (u64 len, u64 code) x num_codes          */
#define EWT_EXP_NODES_AT_LEVEL 12 /* u64 x levels                            */
#define EWT_EXP_ALPHABET 13      /* u64 x sigma, sorted                      */
#define EWT_EXP_NUM_LAST_L2 14   /* u64 x levels (or arrays)                 */

typedef struct ewt_info {
  uint64_t n;                          /* text length                      */
  uint64_t sigma;                      /* alphabet size                    */
  uint64_t num_ranks;                  /* node starts with a stored rank0  */
  uint64_t codes_start;                /* first symbol with a short code   */
  uint64_t num_codes;                  /* sigma - codes_start              */
  uint64_t num_nodes_until_last_level; /* node starts above the last level */
  uint32_t levels;                     /* ceil(log2(sigma))                */
  uint32_t elem_size;                  /* bytes per text symbol            */
  uint32_t is_min_alphabet;            /* alphabet == 0..sigma-1           */
  uint32_t is_pow2;                    /* sigma is a power of two          */
  uint64_t device_bytes;               /* device memory held by the index  */
} ewt_info;

typedef struct ewt_tree ewt_tree; /* opaque built index          */
typedef struct ewt_rs ewt_rs;     /* opaque standalone RankSelect */

/* ---- construction ------------------------------------------------------
 * data: n symbols of elem_size bytes (1, 2, 4 or 8), host OR device memory.
 * A device-resident text is read after a device-wide synchronisation, so
 * work still writing it on any stream completes first.  The call returns
 * once the tree is built.
 * alphabet: sorted distinct symbols in host memory (elem_size bytes each), or
 * NULL with sigma == 0 to detect the alphabet from the text.               */
int ewt_build(const void* data, uint64_t n, int elem_size,
              const void* alphabet, uint64_t sigma, int gpu_index,
              ewt_tree** out);
int ewt_build_u8(const uint8_t* data, uint64_t n, const uint8_t* alphabet,
                 uint64_t sigma, uint32_t gpu_index, ewt_tree** out);
int ewt_build_u16(const uint16_t* data, uint64_t n, const uint16_t* alphabet,
                  uint64_t sigma, uint32_t gpu_index, ewt_tree** out);
int ewt_build_u32(const uint32_t* data, uint64_t n, const uint32_t* alphabet,
                  uint64_t sigma, uint32_t gpu_index, ewt_tree** out);
int ewt_build_u64(const uint64_t* data, uint64_t n, const uint64_t* alphabet,
                  uint64_t sigma, uint32_t gpu_index, ewt_tree** out);
int ewt_free(ewt_tree* tree);
int ewt_get_info(const ewt_tree* tree, ewt_info* info);
int ewt_export(const ewt_tree* tree, int component, int level, void* host_buf,
               uint64_t cap_bytes, uint64_t* size_bytes);

/* ---- host batch queries (synchronous, host buffers) --------------------
 * queries: m records laid out as ecl::RankSelectQuery<T> — a uint64 index
 * (rank: position i; select: k >= 1) at byte 0 and the symbol (elem_size
 * bytes) at byte 8, 16 bytes per record.  Symbols are in the original
 * alphabet.  access results are elem_size-byte symbols; an index >= n yields
 * 0.  select with k > count(symbol) yields n.                             */
int ewt_access(ewt_tree* tree, const uint64_t* indices, uint64_t m,
               void* results);
int ewt_rank(ewt_tree* tree, const void* queries, uint64_t m,
             uint64_t* results);
int ewt_select(ewt_tree* tree, const void* queries, uint64_t m,
               uint64_t* results);
/* types[i] in {EWT_Q_ACCESS, EWT_Q_RANK, EWT_Q_SELECT}; every result is a
 * uint64 (access results are the symbol widened to 64 bits).              */
int ewt_mixed(ewt_tree* tree, const uint8_t* types, const void* queries,
              uint64_t m, uint64_t* results);

/* ---- device-resident batch queries (asynchronous on `stream`) ----------
 * Same layouts as above with device pointers.  Invalid-query reports are
 * collected on the device; ewt_query_status synchronises `stream` and
 * returns EWT_ERR_QUERY if any batch since the last call held one.        */
int ewt_access_device(ewt_tree* tree, const uint64_t* d_indices, uint64_t m,
                      void* d_results, void* stream);
int ewt_rank_device(ewt_tree* tree, const void* d_queries, uint64_t m,
                    uint64_t* d_results, void* stream);
int ewt_select_device(ewt_tree* tree, const void* d_queries, uint64_t m,
                      uint64_t* d_results, void* stream);
int ewt_mixed_device(ewt_tree* tree, const uint8_t* d_types,
                     const void* d_queries, uint64_t m, uint64_t* d_results,
                     void* stream);
int ewt_query_status(ewt_tree* tree, void* stream);

/* ---- allocation-free mixed batch (no counterpart in the reference) ------
 * Same inputs, results and statuses as ewt_mixed, for callers that must not
 * allocate device memory while querying: serving loops whose arena or
 * caching allocator owns all free HBM, hosts that fix each component's
 * device budget up front, and latency-critical paths where an allocation or
 * cudaFree's device-wide synchronisation would stall other streams.  The
 * batch is staged in a fixed array compiled into libewt.so (about 6.3 MB on
 * every GPU that loads it, held until exit); at most 262144 queries per
 * call, larger batches return EWT_ERR_TOO_LARGE without touching the GPU.
 * The first call on a GPU looks up that array's device address (kept for
 * the process; a later cudaDeviceReset is not supported); make it before
 * any stream capture.  Calls share the array and are serialised; each
 * returns after its GPU work is done.                                      */
int ewt_mixed_noalloc(ewt_tree* tree, const uint8_t* types,
                      const void* queries, uint64_t m, uint64_t* results);

/* Copies the by-value device view (ecl::detail::TreeView) that the C++
 * header's WaveletTree<T> embeds; view_size must equal sizeof(TreeView).   */
int ewt_get_device_view(const ewt_tree* tree, void* view_out,
                        uint64_t view_size);

/* ---- standalone RankSelect over caller bit arrays ----------------------
 * words: for each array in turn, ceil(bits[a]/32) packed words, bit i of an
 * array in bit i%32 of word i/32; host or device memory.                   */
int ewt_rs_build(const uint32_t* words, const uint64_t* bits,
                 uint32_t num_arrays, int gpu_index, ewt_rs** out);
int ewt_rs_free(ewt_rs* rs);
int ewt_rs_export(const ewt_rs* rs, int component, int array, void* host_buf,
                  uint64_t cap_bytes, uint64_t* size_bytes);
/* Batched binary queries on one array: value 0 or 1; rank counts `value`
 * bits in [0, pos) with pos <= bits; select returns the position of the
 * i-th `value` bit (i >= 1) or `bits` if there are fewer.  Host buffers.  */
int ewt_rs_rank(ewt_rs* rs, int array, int value, const uint64_t* pos,
                uint64_t m, uint64_t* results);
int ewt_rs_select(ewt_rs* rs, int array, int value, const uint64_t* i,
                  uint64_t m, uint64_t* results);
int ewt_rs_get_device_view(const ewt_rs* rs, void* view_out,
                           uint64_t view_size);

/* Bit arrays that the caller fills on the device, then gives rank/select
 * support.  ewt_bitarray_create lays out num_arrays arrays of bits[a] bits
 * (1 to 255 arrays, the ewt_rs_build layout: each array padded to 32
 * words) with every bit set to init_value (0 or 1); the caller's kernels
 * write them through the device view (ewt_rs_get_device_view: RSView::words
 * at ArrayMeta::word_off); rank and select are refused until
 * ewt_rs_build_in_place.  Replaces BitArray(sizes) and BitArray(sizes,
 * init_value) (bit_array.cuh:61,70; bit_array.cu:40-100; the reference leaves
 * the words of the first form uninitialised, here they are zero). */
int ewt_bitarray_create(const uint64_t* bits, uint32_t num_arrays,
                        int init_value, int gpu_index, ewt_rs** out);
/* Builds the L1/L2 counts, select samples and query-side blocks over the
 * words the caller wrote, in place (bits past an array's end are cleared);
 * first waits for all work on the device, since the kernels that wrote the
 * words may run on any stream.  Replaces RankSelect(BitArray&&, GPU_index)
 * (rank_select.cuh:94; rank_select.cu:50-304). */
int ewt_rs_build_in_place(ewt_rs* rs);

/* Upper bound of the device bytes of: EWT_MEM_BITARRAY, num_arrays bit
 * arrays of n bits each (ewt_bitarray_create); EWT_MEM_RANKSELECT, the same
 * with their rank/select support (ewt_rs_build, ewt_rs_build_in_place);
 * EWT_MEM_TREE, a build of n elem_size-byte symbols over sigma symbols at its
 * peak (the finished tree, a device copy of a host text and the build's
 * transient level orders).  Replaces BitArray::getNeededGPUMemory
 * (bit_array.cuh:332), RankSelect::getNeededGPUMemory (rank_select.cuh:818)
 * and WaveletTree::getNeededGPUMemory (wavelet_tree.cuh:2544), whose figures
 * describe the reference's own allocations. */
#define EWT_MEM_BITARRAY 0
#define EWT_MEM_RANKSELECT 1
#define EWT_MEM_TREE 2
int ewt_needed_memory(int kind, uint64_t n, uint32_t num_arrays_or_elem_size,
                      uint64_t sigma, uint64_t* bytes);

/* The shortened codes (length, code; code aligned to the top of
 * ceil(log2 sigma) bits) of the last *count symbols of 0..sigma-1 when
 * sigma is not a power of two, none otherwise; at most cap are written.
 * The codes the builds use.  Replaces WaveletTree::createMinimalCodes
 * (wavelet_tree.cuh:2100-2159). */
int ewt_minimal_codes(uint64_t sigma, uint64_t* lens, uint64_t* codes,
                      uint64_t cap, uint64_t* count);

/* ---- diagnostics ------------------------------------------------------- */
/* Per-phase device time, measured with CUDA events recorded on the stream
 * each kernel is launched on.  Off by default; enabling adds a stream
 * synchronisation after every timed phase. */
#define EWT_PHASE_HIST 0       /* histogram + remap                       */
#define EWT_PHASE_FILL 1       /* level bit packing                        */
#define EWT_PHASE_RS_COUNTS 2  /* L2/L1 counts + L1 scan                   */
#define EWT_PHASE_SPLIT 3      /* per-level stable partition               */
#define EWT_PHASE_NODE_RANKS 4 /* rank0 at node starts                     */
#define EWT_PHASE_SAMPLES 5    /* select samples                           */
#define EWT_PHASE_QUERY 6      /* query kernels                            */
#define EWT_PHASE_H2D 7        /* host-to-device text copy                 */
#define EWT_PHASE_QUAD 8       /* group (octal / quad) query levels        */
#define EWT_NUM_PHASES 9
typedef struct ewt_phase_times {
  double ms[EWT_NUM_PHASES];        /* accumulated device milliseconds    */
  uint64_t launches[EWT_NUM_PHASES]; /* timed launches per phase          */
} ewt_phase_times;
void ewt_set_timing(int enable);
/* Copies the accumulated times; resets them when reset != 0. */
void ewt_get_timing(ewt_phase_times* out, int reset);

const char* ewt_last_error(void); /* message of the calling thread's last
                                     failed call, "" if none              */
int ewt_abi_version(void);
/* Number of kernel launches this library issued since load (all threads). */
uint64_t ewt_launch_count(void);
/* Batched query launches (ewt_mixed*, ewt_mixed_multi*) hand their chunks
 * to CTAs from a device work queue, an atomic chunk counter, by default;
 * enable = 0 switches to a fixed stride (CTA b takes chunks b, b + G, ...)
 * for comparisons.  Results never depend on it.  Launches already captured
 * in a graph keep the form they were captured with.  No reference
 * counterpart (the reference strides by the grid size, wavelet_tree.cuh:
 * 373-544). */
void ewt_set_work_queue(int enable);
/* SM version (major * 10 + minor, e.g. 103) of the library code that runs
 * on GPU gpu_index, as the CUDA runtime reports it for the query kernel.
 * No reference counterpart (diagnostic). */
int ewt_binary_version(int gpu_index, int* version);

/* ---- autotuning -----------------------------------------------------------
 * Times the query kernels on probe_queries device-generated valid queries
 * over this tree and keeps the fastest configuration for every later query
 * on it: first the dense select-sample rate (every R-th zero / one, R in
 * {64, 128, 256, 512, 1024}, or none: the reference-format samples alone), timed
 * on select probes, then per kind (access, rank, select, mixed) the launch
 * shape (threads per CTA x resident CTAs per SM).  *out (may be NULL)
 * reports the choices and the default and tuned rates.  Results never
 * depend on either choice.  Once the tree's device view was copied out
 * (ewt_get_device_view, ewt_server_add_tree) the sample rate stays as it is,
 * so that view stays valid.  No reference counterpart (the reference fixes
 * its launch configuration per call site, utils.cu:42-94, and its sample
 * rate at compile time, rank_select.cuh:44-64). */
typedef struct ewt_tuning {
  uint32_t threads[4];       /* threads per CTA: access, rank, select, mixed */
  uint32_t blocks_per_sm[4]; /* resident CTAs per SM; 0 = as many as fit    */
  uint32_t select_sample_rate; /* R of the dense select samples; 0 = none  */
  uint32_t reserved;
  double default_mq_s[4], tuned_mq_s[4];
} ewt_tuning;
int ewt_autotune(ewt_tree* tree, uint64_t probe_queries, ewt_tuning* out);

/* Random-access roofline of this GPU: dependent random 32-byte reads per
 * second, `chains` chains of `depth` reads over a device buffer of `bytes`
 * (larger than L2), read the way a query walk reads its blocks.  A query
 * walk reading r blocks is bounded by reads_per_s / r queries per second.
 * No reference counterpart (measurement utility). */
int ewt_probe_random_reads(int gpu_index, uint64_t bytes, uint32_t depth,
                           uint64_t chains, double* reads_per_s);

/* Rebuilds the dense select samples (query side, beside the reference-format
 * samples, which exports keep) at one entry per `rate` zeros / ones: 0 drops
 * them (select then runs the reference's sample -> L1 -> L2 search, or on
 * group levels a search of the superblock table), else a
 * power of two in [32, 65536]; each entry costs 4 bytes.  Built at 256 by
 * default.  Octal group levels (3-bit digits) of power-of-two trees sample
 * eight times as densely (rate / 8, at least 16).  Refused (EWT_ERR_INVALID_ARGUMENT) once the device view was
 * copied out.  No reference counterpart (rank_select.cuh:44-64 fixes one
 * sample per 4096 at compile time). */
int ewt_set_select_samples(ewt_tree* tree, uint32_t rate);
int ewt_rs_set_select_samples(ewt_rs* rs, uint32_t rate);

/* ---- index files --------------------------------------------------------
 * Writes a built tree (shape, level bits, RankSelect counts and samples,
 * rank blocks, count table, node ranks) to `path`; ewt_load reads it back
 * onto a GPU without rebuilding.  Files are native-endian and versioned by
 * their magic.  No reference counterpart (the reference rebuilds). */
int ewt_save(const ewt_tree* tree, const char* path);
int ewt_load(const char* path, int gpu_index, ewt_tree** out);

/* ---- many trees at once ------------------------------------------------
 * Builds `count` texts (elem_size bytes per symbol) concurrently, each on its
 * own stream: out[i] receives tree i (NULL when its build failed, with
 * statuses[i], if given, holding its status).  alphabets / sigmas may be
 * NULL (every alphabet detected).  Returns the first failing status.
 * Texts shorter than 2^24 symbols (1 or 2 bytes each) with a given alphabet
 * 0 .. sigma-1, sigma a power of two in [4, 4096], are built together: one
 * segmented build per alphabet size runs the concatenated texts through the
 * level pipeline once (the text number above the symbol), then single
 * launches cut the levels into per-text arrays of a store the group's trees
 * share and build all their rank/select support, counts and node ranks.
 * Exports and answers are those of single builds; those trees carry rank
 * blocks on every level instead of group query levels, and their dense
 * select-sample rate is fixed (ewt_set_select_samples returns
 * EWT_ERR_UNSUPPORTED).  A group that fails is rebuilt text by text, so
 * every failing text reports its own status.  The reference builds one tree
 * per constructor call (wavelet_tree.cuh:576-867); no reference counterpart
 * for the batch. */
int ewt_build_batch(const void* const* texts, const uint64_t* lengths,
                    uint32_t count, int elem_size,
                    const void* const* alphabets, const uint64_t* sigmas,
                    int gpu_index, ewt_tree** out, int* statuses);
/* Mixed access/rank/select over several trees in one launch: query i is
 * answered on trees[tree_of[i]] (types and records as ewt_mixed; results as
 * ewt_mixed).  All trees share one symbol size and one GPU; fewer than 2^32
 * queries, at most 65536 trees.  A tree id >= num_trees yields UINT64_MAX and
 * EWT_ERR_QUERY.  Replaces one host call per tree (access/rank/select,
 * wavelet_tree.cuh:956-1797); no single reference counterpart. */
int ewt_mixed_multi(ewt_tree* const* trees, uint32_t num_trees,
                    const uint32_t* tree_of, const uint8_t* types,
                    const void* queries, uint64_t m, uint64_t* results);
/* Same over device buffers on `stream` (a cudaStream_t); asynchronous.
 * *d_err (device) is OR-ed with 1 for invalid queries and 2 for unknown
 * tree ids; the caller clears and reads it. */
int ewt_mixed_multi_device(ewt_tree* const* trees, uint32_t num_trees,
                           const uint32_t* d_tree_of, const uint8_t* d_types,
                           const void* d_queries, uint64_t m,
                           uint64_t* d_results, uint32_t* d_err, void* stream);

/* ---- serving engine ---------------------------------------------------
 * Resident trees, query requests served by continuous batching, builds
 * admitted by device-memory footprint, p50/p99 latency.  A dispatcher thread
 * packs every pending request that fits into the next free batch slot
 * (`inflight` slots, each its own stream and pinned buffers) and launches
 * one multi-tree kernel per batch; a completer thread hands results back;
 * a builder thread runs admitted builds.  Requests arriving while batches
 * run join the next batch.  No reference counterpart (the reference serves
 * one synchronous host call at a time, wavelet_tree.cuh:956-1797). */
#include "ewt_sched.h"
typedef struct ewt_server ewt_server;
typedef struct ewt_server_config {
  uint64_t batch_queries;  /* queries per batch; also the largest request */
  uint32_t batch_requests; /* requests per batch                         */
  uint32_t inflight;       /* batches on the GPU at once, 1 .. 8           */
  uint64_t memory_budget;  /* device bytes for resident trees and builds   */
  uint32_t elem_size;      /* symbol size of every tree served             */
  uint32_t force_staging;  /* 1: stage queries and results through pinned
                              buffers even when the GPU can read and write
                              the callers' pageable host buffers in place
                              (the default there)                         */
} ewt_server_config;
int ewt_server_create(int gpu_index, const ewt_server_config* cfg,
                      ewt_server** out);
/* Serves what was submitted, stops the threads, frees the trees the server
 * built (trees added by the caller stay the caller's). */
int ewt_server_destroy(ewt_server* s);
/* Registers a built tree (the caller keeps ownership and must keep it alive
 * until it is removed or the server destroyed); its device bytes count
 * against the budget. */
int ewt_server_add_tree(ewt_server* s, ewt_tree* tree, uint32_t* tree_id);
/* Waits until no queued or running batch can reference the tree, then
 * unregisters it (and frees it when the server built it). */
int ewt_server_remove_tree(ewt_server* s, uint32_t tree_id);
/* Queues m (1 .. batch_queries) mixed queries (types and records as
 * ewt_mixed) against a registered tree.  Host buffers; they must stay valid,
 * and results untouched, until the request completes. */
int ewt_server_submit(ewt_server* s, uint32_t tree_id, const uint8_t* types,
                      const void* queries, uint64_t m, uint64_t* results,
                      uint64_t* request_id);
/* Queues the build of a text (host or device pointer; alphabet as
 * ewt_build); it starts when its estimated footprint fits the budget. */
int ewt_server_submit_build(ewt_server* s, const void* text, uint64_t n,
                            const void* alphabet, uint64_t sigma,
                            uint64_t* request_id);
/* Blocks until the request completed or was cancelled; *status receives its
 * status (EWT_ERR_QUERY when it held invalid queries, EWT_ERR_CANCELLED),
 * *latency_ms submit-to-completion time, *tree_id the id of a built tree.
 * Any out pointer may be NULL.  A request can be waited for once. */
int ewt_server_wait(ewt_server* s, uint64_t request_id, int* status,
                    double* latency_ms, uint32_t* tree_id);
/* Cancels a request that has not started (EWT_ERR_INVALID_ARGUMENT if it
 * already runs or is unknown). */
int ewt_server_cancel(ewt_server* s, uint64_t request_id);
/* Counters and latency percentiles of the completed requests; reset != 0
 * clears the latency record afterwards. */
int ewt_server_stats(ewt_server* s, ewt_sched_stats* out, int reset);

/* Native load generator: Poisson arrivals of requests of log-uniform size,
 * each against a uniformly chosen tree of [first_tree, first_tree +
 * num_trees), queries drawn from valid ranges with the given access / rank
 * fractions (the rest select).  plain != 0 serves the same arrivals through
 * the plain per-request path instead: one synchronous ewt_mixed call per
 * request, in arrival order.  build_n > 0 adds the build of a sigma-4 uint8
 * text of build_n symbols every build_interval_s. */
typedef struct ewt_load_config {
  double rate, duration_s;
  uint32_t max_request, first_tree, num_trees;
  double frac_access, frac_rank;
  uint64_t seed;
  int plain;
  uint64_t build_n;
  double build_interval_s;
} ewt_load_config;
typedef struct ewt_load_result {
  uint64_t requests, queries;
  double wall_s, qps, p50_ms, p99_ms, mean_ms, max_ms;
  uint64_t batches, builds;
  double build_p50_ms;
} ewt_load_result;
int ewt_server_run_load(ewt_server* s, const ewt_load_config* cfg,
                        ewt_load_result* res);

/* Device memory of trees, rank/select structures, build scratch and query
 * scratch comes from a library-owned, stream-ordered memory pool per GPU
 * that keeps freed blocks for the next build instead of returning them to
 * the driver (so repeated builds pay no cudaMalloc / cudaFree).  This call
 * waits for the GPU and returns every unused cached block to the driver.
 * No reference counterpart (the reference calls cudaMalloc / cudaFree
 * directly, wavelet_tree.cuh:620-860). */
int ewt_release_cached_memory(int gpu_index);

#ifdef __cplusplus
}
#endif
#endif /* EWT_H */
