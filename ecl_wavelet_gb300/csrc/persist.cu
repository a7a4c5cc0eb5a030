// Index files: a built tree written to disk and read back onto a GPU without
// rebuilding (ewt_save / ewt_load).  The reference has no serialisation; a
// serving process uses this to admit prebuilt indexes.
//
// Layout (little-endian): the magic "EWTIDX03", a header of 64-bit fields,
// the host-side shape (alphabet, count table, codes, node starts, nodes per
// level, node bases, level sizes, per-array metadata), then the device arrays
// in a fixed order (level words, L1, L2, samples of zeros and ones, rank
// blocks, node-start ranks).  Big arrays move through a pinned staging
// buffer in 64 MiB pieces on the tree's stream.
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "internal.cuh"

namespace ewt {
namespace {

constexpr char kMagic[8] = {'E', 'W', 'T', 'I', 'D', 'X', '0', '3'};
constexpr size_t kPiece = size_t(64) << 20;

struct File {
  FILE* f = nullptr;
  File(std::string const& path, char const* mode) : f(std::fopen(path.c_str(), mode)) {
    EWT_REQUIRE(f != nullptr, EWT_ERR_INVALID_ARGUMENT, "cannot open " + path);
  }
  ~File() {
    if (f) std::fclose(f);
  }
  void write(void const* p, size_t n) {
    EWT_REQUIRE(std::fwrite(p, 1, n, f) == n, EWT_ERR_CUDA, "index file write failed");
  }
  void read(void* p, size_t n) {
    EWT_REQUIRE(std::fread(p, 1, n, f) == n, EWT_ERR_INVALID_ARGUMENT,
                "index file is truncated");
  }
  void put(uint64_t v) { write(&v, 8); }
  uint64_t get() {
    uint64_t v;
    read(&v, 8);
    return v;
  }
  template <class V>
  void put_vec(std::vector<V> const& v) {
    put(v.size());
    if (!v.empty()) write(v.data(), v.size() * sizeof(V));
  }
  template <class V>
  std::vector<V> get_vec(uint64_t limit) {
    uint64_t const n = get();
    EWT_REQUIRE(n <= limit, EWT_ERR_INVALID_ARGUMENT, "index file is corrupt");
    std::vector<V> v(n);
    if (n) read(v.data(), n * sizeof(V));
    return v;
  }
};

void dev_to_file(File& f, void const* d, uint64_t bytes, PinnedBuf& stage,
                 cudaStream_t s) {
  f.put(bytes);
  for (uint64_t o = 0; o < bytes; o += kPiece) {
    size_t const k = static_cast<size_t>(std::min<uint64_t>(kPiece, bytes - o));
    EWT_CUDA(cudaMemcpyAsync(stage.get(), static_cast<char const*>(d) + o, k,
                             cudaMemcpyDeviceToHost, s));
    EWT_CUDA(cudaStreamSynchronize(s));
    f.write(stage.get(), k);
  }
}

void file_to_dev(File& f, DevBuf& d, PinnedBuf& stage, cudaStream_t s,
                 uint64_t limit) {
  uint64_t const bytes = f.get();
  EWT_REQUIRE(bytes <= limit, EWT_ERR_INVALID_ARGUMENT, "index file is corrupt");
  d.alloc(bytes);
  for (uint64_t o = 0; o < bytes; o += kPiece) {
    size_t const k = static_cast<size_t>(std::min<uint64_t>(kPiece, bytes - o));
    EWT_CUDA(cudaStreamSynchronize(s));  // the staging buffer is free again
    f.read(stage.get(), k);
    EWT_CUDA(cudaMemcpyAsync(static_cast<char*>(d.get()) + o, stage.get(), k,
                             cudaMemcpyHostToDevice, s));
  }
}

template <class V>
void upload(DevBuf& d, std::vector<V> const& v, cudaStream_t s) {
  d.alloc(std::max<size_t>(v.size(), 1) * sizeof(V));
  if (!v.empty())
    EWT_CUDA(cudaMemcpyAsync(d.get(), v.data(), v.size() * sizeof(V),
                             cudaMemcpyHostToDevice, s));
}

}  // namespace
}  // namespace ewt

using namespace ewt;

extern "C" int ewt_save(const ewt_tree* t, const char* path) {
  return run_guarded([&] {
    EWT_REQUIRE(t && path, EWT_ERR_INVALID_ARGUMENT, "null argument");
    DeviceGuard g(t->device);
    cudaStream_t const s = t->stream;
    File f(path, "wb");
    f.write(kMagic, 8);
    for (uint64_t v : {uint64_t(t->elem_size), t->n, t->sigma, uint64_t(t->L),
                       uint64_t(t->is_min), uint64_t(t->pow2), t->codes_start,
                       t->nodes_until_last})
      f.put(v);
    f.put_vec(t->alphabet);
    f.put_vec(t->occ);
    f.put_vec(t->counts);
    f.put_vec(t->codes);
    f.put_vec(t->nodes);
    f.put_vec(t->nodes_at_level);
    f.put_vec(t->node_base);
    f.put_vec(t->level_bits);
    f.put_vec(t->rs.meta);
    for (uint64_t v : {t->rs.total_words, t->rs.total_l1, t->rs.total_l2,
                       t->rs.total_s0, t->rs.total_s1,
                       uint64_t(t->rs.ds.get() ? t->rs.sel_shift : 0)})
      f.put(v);
    PinnedBuf stage;
    stage.ensure(kPiece);
    dev_to_file(f, t->rs.words.get(), t->rs.words.bytes(), stage, s);
    dev_to_file(f, t->rs.l1.get(), t->rs.l1.bytes(), stage, s);
    dev_to_file(f, t->rs.l2.get(), t->rs.l2.bytes(), stage, s);
    dev_to_file(f, t->rs.s0.get(), t->rs.s0.bytes(), stage, s);
    dev_to_file(f, t->rs.s1.get(), t->rs.s1.bytes(), stage, s);
    dev_to_file(f, t->rs.rb.get(), t->rs.rb.bytes(), stage, s);
    dev_to_file(f, t->rs.ds.get(), t->rs.ds.bytes(), stage, s);
    dev_to_file(f, t->counts_d.get(), t->counts_d.bytes(), stage, s);
    dev_to_file(f, t->ranks_d.get(), t->ranks_d.bytes(), stage, s);
    // group query levels (none for other alphabets)
    f.put_vec(t->groups.levels);
    f.put(t->groups.ds.get() ? t->groups.sel_shift : 0);
    if (!t->groups.levels.empty()) {
      dev_to_file(f, t->groups.blocks.get(), t->groups.blocks.bytes(), stage, s);
      dev_to_file(f, t->groups.sb.get(), t->groups.sb.bytes(), stage, s);
      dev_to_file(f, t->groups.ds.get(), t->groups.ds.bytes(), stage, s);
      dev_to_file(f, t->groups.node_ranks.get(), t->groups.node_ranks.bytes(), stage, s);
    }
  });
}

extern "C" int ewt_load(const char* path, int gpu_index, ewt_tree** out) {
  return run_guarded([&] {
    EWT_REQUIRE(path && out, EWT_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    File f(path, "rb");
    char magic[8];
    f.read(magic, 8);
    EWT_REQUIRE(std::memcmp(magic, kMagic, 8) == 0, EWT_ERR_INVALID_ARGUMENT,
                "not an index file (bad magic)");
    DeviceGuard g(gpu_index);
    auto t = std::make_unique<ewt_tree>();
    t->device = gpu_index;
    EWT_CUDA(cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking));
    cudaStream_t const s = t->stream;
    try {
      AllocStream as(s);
      t->elem_size = static_cast<uint32_t>(f.get());
      t->n = f.get();
      t->sigma = f.get();
      t->L = static_cast<uint32_t>(f.get());
      t->is_min = f.get() != 0;
      t->pow2 = f.get() != 0;
      t->codes_start = f.get();
      t->nodes_until_last = f.get();
      EWT_REQUIRE((t->elem_size == 1 || t->elem_size == 2 || t->elem_size == 4 ||
                   t->elem_size == 8) &&
                      t->L >= 1 && t->L <= 64 && t->sigma >= 2 && t->n >= 1,
                  EWT_ERR_INVALID_ARGUMENT, "index file is corrupt");
      uint64_t const sig = t->sigma, lim_l = t->L + 1;
      t->alphabet = f.get_vec<uint64_t>(sig);
      t->occ = f.get_vec<uint64_t>(sig);
      t->counts = f.get_vec<uint64_t>(sig);
      t->codes = f.get_vec<CodeH>(sig);
      t->nodes = f.get_vec<NodeInfoH>(sig * 64);
      t->nodes_at_level = f.get_vec<uint64_t>(lim_l);
      t->node_base = f.get_vec<uint64_t>(lim_l);
      t->level_bits = f.get_vec<uint64_t>(lim_l);
      t->rs.meta = f.get_vec<ArrayMeta>(lim_l);
      EWT_REQUIRE(t->alphabet.size() == sig && t->rs.meta.size() == t->L &&
                      t->node_base.size() == t->L + 1,
                  EWT_ERR_INVALID_ARGUMENT, "index file is corrupt");
      t->rs.total_words = f.get();
      t->rs.total_l1 = f.get();
      t->rs.total_l2 = f.get();
      t->rs.total_s0 = f.get();
      t->rs.total_s1 = f.get();
      t->rs.sel_shift = static_cast<uint32_t>(f.get());
      EWT_REQUIRE(t->rs.sel_shift == 0 || (t->rs.sel_shift >= 5 && t->rs.sel_shift <= 16),
                  EWT_ERR_INVALID_ARGUMENT, "index file is corrupt");
      PinnedBuf stage;
      stage.ensure(kPiece);
      uint64_t const big = t->n * 64 + (uint64_t(1) << 30);  // sanity bound
      file_to_dev(f, t->rs.words, stage, s, big);
      file_to_dev(f, t->rs.l1, stage, s, big);
      file_to_dev(f, t->rs.l2, stage, s, big);
      file_to_dev(f, t->rs.s0, stage, s, big);
      file_to_dev(f, t->rs.s1, stage, s, big);
      file_to_dev(f, t->rs.rb, stage, s, big);
      file_to_dev(f, t->rs.ds, stage, s, big);
      EWT_REQUIRE(t->rs.sel_shift == 0 || t->rs.ds.get() != nullptr,
                  EWT_ERR_INVALID_ARGUMENT, "index file is corrupt");
      file_to_dev(f, t->counts_d, stage, s, (sig + 1) * 8);
      file_to_dev(f, t->ranks_d, stage, s, big);
      t->groups.levels = f.get_vec<ecl::detail::GroupLevel>(t->L / 2 + 1);
      t->groups.sel_shift = static_cast<uint32_t>(f.get());
      bool plan_ok = t->groups.levels.empty() ||
                     (groups_eligible(*t) && (t->groups.sel_shift == 0 ||
                                            (t->groups.sel_shift >= 5 && t->groups.sel_shift <= 16)));
      if (!t->groups.levels.empty()) {
        std::vector<uint32_t> const widths = group_widths(t->L);
        plan_ok = plan_ok && widths.size() == t->groups.levels.size();
        uint32_t l = 0;
        for (size_t j = 0; plan_ok && j < widths.size(); ++j) {
          auto const& ql = t->groups.levels[j];
          plan_ok = ql.width == widths[j] && ql.start == l && ql.sel_shift <= 16;
          l += widths[j];
        }
      }
      EWT_REQUIRE(plan_ok, EWT_ERR_INVALID_ARGUMENT, "index file is corrupt");
      if (!t->groups.levels.empty()) {
        file_to_dev(f, t->groups.blocks, stage, s, big);
        file_to_dev(f, t->groups.sb, stage, s, big);
        file_to_dev(f, t->groups.ds, stage, s, big);
        file_to_dev(f, t->groups.node_ranks, stage, s, big);
        upload(t->groups.levels_d, t->groups.levels, s);
        if (t->groups.sel_shift == 0) t->groups.ds.reset();
      }
      upload(t->rs.meta_d, t->rs.meta, s);
      upload(t->node_base_d, t->node_base, s);
      upload(t->nodes_at_level_d, t->nodes_at_level, s);
      std::vector<uint64_t> cl(std::max<size_t>(t->codes.size(), 1), 0), cb(cl.size(), 0);
      for (size_t i = 0; i < t->codes.size(); ++i) {
        cl[i] = t->codes[i].len;
        cb[i] = t->codes[i].code;
      }
      upload(t->code_len_d, cl, s);
      upload(t->code_bits_d, cb, s);
      if (!t->is_min) {
        // the alphabet in the tree's own symbol width
        std::vector<unsigned char> a(sig * t->elem_size);
        for (uint64_t i = 0; i < sig; ++i)
          std::memcpy(&a[i * t->elem_size], &t->alphabet[i], t->elem_size);
        upload(t->alphabet_d, a, s);
      }
      t->err_d.alloc(kTreeErrBytes);
      EWT_CUDA(cudaMemsetAsync(t->err_d.get(), 0, kTreeErrBytes, s));
      EWT_CUDA(cudaStreamSynchronize(s));  // host vectors above leave scope
      fill_tree_view(*t);
    } catch (...) {
      cudaStreamSynchronize(s);
      t.reset();
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
      throw;
    }
    *out = t.release();
  });
}
