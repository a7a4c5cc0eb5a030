// Host-side objects behind the opaque ewt_tree / ewt_rs handles, and the
// functions the translation units share.
#pragma once
#include <atomic>
#include <memory>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "ecl_wavelet/detail/device_ops.cuh"

namespace ewt {

using ecl::detail::ArrayMeta;
using ecl::detail::RSView;
using ecl::detail::TreeView;

// Device storage of a group of bit arrays with rank/select support, laid out
// as src/bitarray/bit_array.cu:40-100 and src/bitarray/rank_select.cu:50-304
// do: arrays padded to 32-word multiples, total word count even.
struct RSStore {
  std::vector<ArrayMeta> meta;  // host copy
  DevBuf words, l1, l2, s0, s1, meta_d, jobs_d, rb, ds;
  uint64_t total_words = 0, total_l1 = 0, total_l2 = 0;
  uint64_t total_s0 = 0, total_s1 = 0;
  uint32_t sel_shift = ecl::detail::kDefaultSelShift;  // dense sample rate
  std::vector<uint8_t> skip_blocks;  // arrays built without rank blocks

  // Lays out arrays of the given bit lengths and allocates words (zeroed),
  // L1, L2 and the device meta table.  Samples are allocated by build_rs.
  void layout(std::vector<uint64_t> const& bits);
  RSView view() const;
  uint64_t device_bytes() const {
    return words.bytes() + l1.bytes() + l2.bytes() + s0.bytes() + s1.bytes() + rb.bytes() +
           ds.bytes() + meta_d.bytes();
  }
};

// Builds L2/L1/total counts for arrays [first, last) of `rs` on `stream`
// (the words must be final); totals land in the device meta table only.
// Asynchronous: no host synchronisation.
void build_rs_counts(RSStore& rs, uint32_t first, uint32_t last,
                     cudaStream_t stream);
// Allocates and fills the select samples of every array (needs counts of
// all arrays) and uploads the final meta table.
void build_rs_samples(RSStore& rs, cudaStream_t stream);
// Builds the query-side rank blocks of every array (needs the counts) and,
// when rs.sel_shift > 0, the dense select samples in the same pass; uploads
// the meta table with their offsets.
void build_rank_blocks(RSStore& rs, cudaStream_t stream);
// Rank-block start of every array (running totals; arrays without blocks
// add none) and the total block count.
uint64_t rank_block_starts(std::vector<ArrayMeta> const& meta,
                           std::vector<uint64_t>& start);
// Rebuilds the dense select samples at rate 2^shift from the rank blocks
// (shift 0 drops them: select then uses the reference-format samples).
void build_dense_samples(RSStore& rs, uint32_t shift, cudaStream_t stream);

// Group (octal / quad) query levels of a power-of-two tree (groups.cu).
struct GroupStore {
  std::vector<ecl::detail::GroupLevel> levels;  // host copy
  DevBuf blocks, sb, ds, node_ranks, levels_d;
  // transient, during a build: the symbols in level-`order_level` order as
  // the first pass wrote them, for the octal group level starting there
  DevBuf order;
  uint32_t order_level = 0;
  uint32_t sel_shift = ecl::detail::kDefaultSelShift;
  bool level0_built = false;  // octal level 0 written with the binary level 0
  ecl::detail::GroupView view() const;
  uint64_t bytes() const {
    return blocks.bytes() + sb.bytes() + ds.bytes() + node_ranks.bytes() +
           levels_d.bytes();
  }
};

struct QueryScratch {
  DevBuf in, out, types;
  PinnedBuf h_in, h_out, h_types;
  size_t in_cap = 0, out_cap = 0, types_cap = 0;
};

// Streams, events and double buffers of pipelined host batches: queries of
// chunk i+1 copied in and results of chunk i-1 copied out while chunk i is
// answered (capi.cu).  Created on first use.
struct QueryPipe {
  cudaStream_t s_in = nullptr, s_out = nullptr;
  cudaEvent_t start = nullptr, in_done[2] = {}, k_done[2] = {}, out_done[2] = {};
  DevBuf in[2], out[2], types[2];
  size_t cap_in[2] = {0, 0}, cap_out[2] = {0, 0}, cap_types[2] = {0, 0};
  void init() {
    if (s_in) return;
    EWT_CUDA(cudaStreamCreateWithFlags(&s_in, cudaStreamNonBlocking));
    EWT_CUDA(cudaStreamCreateWithFlags(&s_out, cudaStreamNonBlocking));
    EWT_CUDA(cudaEventCreateWithFlags(&start, cudaEventDisableTiming));
    for (int i = 0; i < 2; ++i) {
      EWT_CUDA(cudaEventCreateWithFlags(&in_done[i], cudaEventDisableTiming));
      EWT_CUDA(cudaEventCreateWithFlags(&k_done[i], cudaEventDisableTiming));
      EWT_CUDA(cudaEventCreateWithFlags(&out_done[i], cudaEventDisableTiming));
    }
  }
  ~QueryPipe() {
    if (!s_in) return;
    cudaStreamSynchronize(s_in);
    cudaStreamSynchronize(s_out);
    for (cudaEvent_t e : {start, in_done[0], in_done[1], k_done[0], k_done[1],
                          out_done[0], out_done[1]})
      if (e) cudaEventDestroy(e);
    cudaStreamDestroy(s_in);
    cudaStreamDestroy(s_out);
  }
};

struct CodeH {
  uint64_t len, code;
};
struct NodeInfoH {
  uint64_t start, level;
};

}  // namespace ewt

// Per-tree device words next to the query error word: kQueueSlots work-queue
// counter pairs (mixed launches take the next pair in turn, so launches that
// overlap on different streams use different pairs).
constexpr uint32_t kQueueSlots = 256;
constexpr size_t kTreeErrBytes = 16 + size_t(kQueueSlots) * 8;

struct ewt_tree {
  int device = 0;
  std::atomic<uint32_t> queue_next{0};  // next work-queue counter pair
  uint32_t elem_size = 1;
  // query launch shape per kind (access, rank, select, mixed) chosen by
  // ewt_autotune: threads per CTA and resident CTAs per SM (0 = default)
  uint32_t tune_threads[4] = {0, 0, 0, 0};
  uint32_t tune_blocks[4] = {0, 0, 0, 0};
  // set once the device view was copied out (ewt_get_device_view, a
  // server): its pointers must stay valid, so the dense select samples are
  // no longer rebuilt at another rate
  mutable std::atomic<bool> view_shared{false};
  uint64_t n = 0, sigma = 0;
  uint32_t L = 0;
  bool is_min = false, pow2 = false;
  uint64_t codes_start = 0;
  uint64_t nodes_until_last = 0;
  std::vector<uint64_t> alphabet;  // original symbols, widened
  std::vector<uint64_t> occ, counts;
  std::vector<ewt::CodeH> codes;
  std::vector<ewt::NodeInfoH> nodes;
  std::vector<uint64_t> nodes_at_level, node_base, level_bits;
  ewt::RSStore rs;
  ewt::GroupStore groups;  // octal / quad query levels (power-of-two trees)
  ewt::DevBuf counts_d, ranks_d, node_base_d, nodes_at_level_d, code_len_d,
      code_bits_d, alphabet_d, err_d;
  ecl::detail::TreeView view{};
  std::mutex query_mu;  // host batch calls share scratch buffers
  ewt::QueryScratch scratch;
  ewt::QueryPipe pipe;
  cudaStream_t stream = nullptr;  // library-owned stream for host calls
  // Trees of a batch build's short texts: their rank/select arrays and small
  // tables are views into a store shared by the batch's group, kept alive by
  // every tree of the group; rs_share_bytes is this tree's part of it.
  std::shared_ptr<void> shared_store;
  uint64_t rs_share_bytes = 0;
  uint64_t device_bytes() const;
};

struct ewt_rs {
  int device = 0;
  // false while the arrays are being filled by the caller (ewt_bitarray_create)
  // and the counts and samples do not exist yet
  bool built = true;
  mutable std::atomic<bool> view_shared{false};  // as ewt_tree::view_shared
  ewt::RSStore rs;
  ewt::DevBuf err_d;
  std::mutex query_mu;
  ewt::QueryScratch scratch;
  cudaStream_t stream = nullptr;
};

namespace ewt {
// Batched query launches distribute their chunks through a device work
// queue unless ewt_set_work_queue(0) switched it off (capi.cu).
bool work_queue_enabled();
// The next work-queue counter pair of a tree (nullptr when launches use
// static striding).
inline uint32_t* queue_slot(ewt_tree& t) {
  if (!work_queue_enabled()) return nullptr;
  uint32_t const i = t.queue_next.fetch_add(1) % kQueueSlots;
  return t.err_d.as<uint32_t>() + 4 + 2 * i;
}
// Host orchestration of one tree build (wt_build.cu).
void build_tree(ewt_tree& t, const void* data, uint64_t n, int elem_size,
                const void* alphabet, uint64_t sigma, cudaStream_t stream);
// Builds on this thread skip the device-wide synchronisation that orders a
// device-resident text after the caller's work while set (a batch of builds
// synchronises once before it starts; wt_build.cu).
void set_texts_synchronized(bool v);
bool texts_synchronized();
// Builds on this thread belong to a batch (ewt_build_batch): texts shorter
// than kBatchGroupMinSymbols get rank blocks instead of group query levels
// (those eligible for the segmented group build get them there).  At 2^24
// the 256-text C4-style batch builds in 38 ms instead of 47 ms at 2^22,
// for 3 % fewer multi-tree queries per second.
constexpr uint64_t kBatchGroupMinSymbols = uint64_t(1) << 24;
void set_batch_member(bool v);
// Whether a text goes to the segmented build of short texts: below
// kBatchGroupMinSymbols symbols of 1 or 2 bytes with the given alphabet
// 0 .. sigma-1, sigma a power of two in [4, 4096] (batch_build.cu).
bool small_batch_eligible(uint64_t n, int elem_size, void const* alphabet,
                          uint64_t sigma);
// Builds the texts `ids` (all eligible, alphabets of 2^L symbols) as
// segmented group builds; out[id] receives each tree.  Throws on failure
// (out untouched for the failing group).
void build_small_texts(void const* const* texts, uint64_t const* lengths,
                       std::vector<uint32_t> const& ids, int elem_size,
                       uint32_t L, int gpu, ewt_tree** out);
// Sets t.view from the tree's device buffers and shape (wt_build.cu).
void fill_tree_view(ewt_tree& t);
// Codes, node starts and node counts per level of a tree whose sigma, L and
// pow2 are set (wavelet_tree.cuh:618-724; wt_build.cu).
void set_tree_shape(ewt_tree& t);
// Shortened codes (length, code) of the last symbols of a non-power-of-two
// alphabet of sigma symbols; none for powers of two (wt_build.cu).
void minimal_codes(uint64_t sigma, std::vector<uint64_t>& lens,
                   std::vector<uint64_t>& codes);
// Upper bound of the device bytes a build of n elem_size-byte symbols over
// sigma symbols holds at its peak, the finished tree included (wt_build.cu).
uint64_t build_bytes_bound(uint64_t n, uint32_t elem_size, uint64_t sigma);
// Device bytes of RankSelect-supported bit arrays (words, counts, samples,
// query-side blocks) of `arrays` arrays of `bits` bits each (rs_build.cu).
uint64_t rs_bytes_bound(uint64_t bits, uint32_t arrays, bool with_support);

// Query launches on device buffers (queries.cu).
void launch_access(ewt_tree& t, const uint64_t* d_idx, uint64_t m,
                   void* d_out, cudaStream_t s);
void launch_rank(ewt_tree& t, const void* d_q, uint64_t m, uint64_t* d_out,
                 cudaStream_t s);
void launch_select(ewt_tree& t, const void* d_q, uint64_t m, uint64_t* d_out,
                   cudaStream_t s);
void launch_mixed(ewt_tree& t, const uint8_t* d_types, const void* d_q,
                  uint64_t m, uint64_t* d_out, cudaStream_t s);
// The mixed kernel over caller-provided device buffers with an explicit
// invalid-query word (its work-queue counter pair at d_err + 16, i.e. 64
// bytes in, zeroed by the caller); allocates nothing.
void launch_mixed_raw(ewt_tree& t, const uint8_t* d_types, const void* d_q,
                      uint64_t m, uint64_t* d_out, uint32_t* d_err,
                      cudaStream_t s);
// Multi-tree mixed batch over an already grouped work list (multi.cu):
// d_items holds num_items 16-byte items {uint32 tree, uint32 count, uint64
// start} (count <= 2048) naming positions of d_q / d_types / d_out.
void launch_multi_items(uint32_t elem_size, TreeView const* d_views,
                        void const* d_items, uint32_t num_items,
                        uint32_t max_levels, uint8_t const* d_types,
                        void const* d_q, uint64_t* d_out, uint32_t* d_err,
                        cudaStream_t s);
// Zero-copy serving launch (multi.cu): `reqs` holds 32-byte descriptors
// {const uint8_t* types; const void* queries; uint64_t* results; uint32
// tree; uint32 pad} of buffers the GPU reads and writes in place, `items`
// 16-byte {uint32 req, uint32 count (<= 2048), uint64 start}; req_err[r] is
// set to 1 when request r held an invalid query.
void launch_serve_items(uint32_t elem_size, TreeView const* d_views,
                        void const* reqs, void const* items, uint32_t num_items,
                        uint32_t max_levels, uint32_t* req_err, cudaStream_t s);
void prepare_serve_kernels(uint32_t elem_size);
// Group query levels (groups.cu): whether a tree gets them (power-of-two
// alphabet, two or more levels), their build from the finished binary levels
// and count table C (sigma + 1 entries), and a rebuild of their dense select
// samples at rate 2^shift (0: none).
bool groups_eligible(ewt_tree const& t);
// Digit widths of the group levels of an L-level tree, top down: octal (3)
// groups, then one or two quad (2) groups; they cover all L levels.
std::vector<uint32_t> group_widths(uint32_t L);
// sym: the tree's minimal symbols on the device (elem_size bytes each), or
// null; level 0 is then built from them directly.
void build_groups(ewt_tree& t, std::vector<uint64_t> const& C, void const* sym,
                uint32_t elem_size, cudaStream_t st);
// Octal level 0 from the minimal symbols (1- or 2-byte) before the other
// levels exist: lays out the group levels, writes the octal level-0 blocks
// and the binary level 0 (`level0`, its words) in one read of the symbols,
// and reports symbols >= 2^L in err bit 0 when `check`; build_groups finishes
// the level.
bool octal_text_eligible(ewt_tree const& t, uint32_t elem_size);
void build_octal_level0(ewt_tree& t, void const* sym, uint32_t elem_size,
                        uint32_t* level0, bool check, uint32_t* err, cudaStream_t st);
void build_group_samples(ewt_tree& t, uint32_t shift, cudaStream_t st);
// Dense select samples of the binary and group levels at rate 2^shift (0:
// none), and the tree's view updated.
void set_select_rate(ewt_tree& t, uint32_t shift, cudaStream_t st);
// Random-access roofline: dependent random 32-byte reads per second over a
// buffer of `bytes` (queries.cu).
// binaryVersion of the mixed query kernel on the current device.
int kernel_binary_version();
void probe_random_reads(uint64_t bytes, uint32_t depth, uint64_t chains,
                        double* reads_per_s);
// Times candidate launch shapes of every query kind on probe queries and
// keeps the fastest in the tree (queries.cu).
void autotune_queries(ewt_tree& t, uint64_t probe_queries, ewt_tuning* out);
void launch_rs_rank(ewt_rs& r, int array, int value, const uint64_t* d_pos,
                    uint64_t m, uint64_t* d_out, cudaStream_t s);
void launch_rs_select(ewt_rs& r, int array, int value, const uint64_t* d_i,
                      uint64_t m, uint64_t* d_out, cudaStream_t s);
}  // namespace ewt
