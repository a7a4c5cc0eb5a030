// Driver for the reference's own GPU build (mfranzreb/ECL_wavelet), compiled
// against its unmodified headers and sources: it is how this repository
// compares its answers and speed with the reference on the same GPU.
// Everything here goes through the reference's public API: the
// WaveletTree<T>(data, n, alphabet, gpu) constructor, the host access / rank
// / select batch calls, and the public device accessors of RankSelect and
// BitArray (rank_select.cuh:530-695, bit_array.cuh:173-330), read by value
// in a kernel as the reference's own query kernels do.
//
//   ref_driver dump  TEXT ES SIGMA NUM_RANKS OUT_PREFIX
//       build from the raw text file TEXT (ES-byte symbols, alphabet
//       0..SIGMA-1); write every level's words, L1, L2, select samples and
//       the tree's counts, node ranks, total ones, last-L1 L2 counts, level
//       sizes as OUT_PREFIX.<name>[.<level>].bin
//   ref_driver query TEXT ES SIGMA QUERIES M OUT
//       answer M mixed queries (QUERIES: M type bytes, M uint64 indices, M
//       uint64 symbols) with one host call per type; write M uint64 answers
//   ref_driver bench N ES SIGMA M REPS
//       time the build of an N-symbol iid uniform text from pinned host
//       memory and M host queries of each type; print one JSON line
#include <ecl_wavelet/tree/wavelet_tree.cuh>

#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

#define CK(x)                                                              \
  do {                                                                     \
    cudaError_t e_ = (x);                                                  \
    if (e_ != cudaSuccess) {                                               \
      std::fprintf(stderr, "CUDA error %s at %s:%d\n",                      \
                   cudaGetErrorString(e_), __FILE__, __LINE__);             \
      std::exit(2);                                                        \
    }                                                                      \
  } while (0)

constexpr uint64_t kSampleRate = 4096;  // RSConfig::SELECT_SAMPLE_RATE

std::vector<char> read_file(std::string const& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) {
    std::fprintf(stderr, "cannot open %s\n", path.c_str());
    std::exit(2);
  }
  std::fseek(f, 0, SEEK_END);
  long const size = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  std::vector<char> buf(size);
  if (size && std::fread(buf.data(), 1, size, f) != size_t(size)) std::exit(2);
  std::fclose(f);
  return buf;
}

void write_file(std::string const& path, void const* p, size_t bytes) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f || (bytes && std::fwrite(p, 1, bytes, f) != bytes)) {
    std::fprintf(stderr, "cannot write %s\n", path.c_str());
    std::exit(2);
  }
  std::fclose(f);
}

// ---- reads through the public device accessors ---------------------------
enum Part { kWords, kL1, kL2, kS0, kS1, kRanks, kPerLevel };

template <class T>
__global__ void gather_kernel(ecl::WaveletTree<T> wt, int part, uint32_t level,
                              uint64_t count, uint64_t* out) {
  auto const& rs = wt.rank_select_;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < count;
       i += uint64_t(gridDim.x) * blockDim.x) {
    uint64_t v = 0;
    switch (part) {
      case kWords: v = rs.bit_array_.word(level, i); break;
      case kL1: v = rs.getL1Entry(level, i); break;
      case kL2: v = rs.getL2Entry(level, i); break;
      case kS0: v = rs.template getSelectSample<0>(level, i); break;
      case kS1: v = rs.template getSelectSample<1>(level, i); break;
      case kRanks: v = wt.getPrecomputedRank(static_cast<T>(i)); break;
      case kPerLevel: {  // 4 per level: ones, last-L1 L2, L1 and L2 blocks
        uint32_t const l = static_cast<uint32_t>(i / 4);
        switch (i % 4) {
          case 0: v = rs.template getTotalNumVals<1>(l); break;
          case 1: v = rs.getNumLastL2Blocks(l); break;
          case 2: v = rs.getNumL1Blocks(l); break;
          default: v = rs.getNumL2Blocks(l); break;
        }
        break;
      }
    }
    out[i] = v;
  }
}

template <class T>
std::vector<uint64_t> gather(ecl::WaveletTree<T>& wt, int part, uint32_t level,
                             uint64_t count) {
  std::vector<uint64_t> h(count);
  if (count == 0) return h;
  uint64_t* d = nullptr;
  CK(cudaMalloc(&d, count * 8));
  gather_kernel<T><<<1024, 256>>>(wt, part, level, count, d);
  CK(cudaGetLastError());
  CK(cudaMemcpy(h.data(), d, count * 8, cudaMemcpyDeviceToHost));
  CK(cudaFree(d));
  return h;
}

template <class V>
void write_as(std::string const& path, std::vector<uint64_t> const& v) {
  std::vector<V> out(v.begin(), v.end());
  write_file(path, out.data(), out.size() * sizeof(V));
}

template <class T>
std::vector<T> make_alphabet(uint64_t sigma) {
  std::vector<T> a(sigma);
  for (uint64_t i = 0; i < sigma; ++i) a[i] = static_cast<T>(i);
  return a;
}

// Number of precomputed node ranks, counted by the reference's own
// (protected) node-start helper, reached the way its tests reach it: through
// a subclass (tests/test_wavelet_tree.cu:17-24).
template <class T>
struct NodeCount : ecl::WaveletTree<T> {
  static uint64_t of(std::vector<T> const& alphabet) {
    auto const codes = ecl::WaveletTree<T>::createMinimalCodes(alphabet);
    return ecl::WaveletTree<T>::getNodeInfos(alphabet, codes).size();
  }
};

template <class T>
int dump(std::string const& text_path, uint64_t sigma, uint64_t num_ranks,
         std::string const& prefix) {
  if (num_ranks != NodeCount<T>::of(make_alphabet<T>(sigma))) {
    std::fprintf(stderr, "node-rank count %llu differs from the reference's %llu\n",
                 (unsigned long long)num_ranks,
                 (unsigned long long)NodeCount<T>::of(make_alphabet<T>(sigma)));
    return 4;
  }
  auto const buf = read_file(text_path);
  uint64_t const n = buf.size() / sizeof(T);
  auto const* text = reinterpret_cast<T const*>(buf.data());
  ecl::WaveletTree<T> wt(text, n, make_alphabet<T>(sigma), 0);
  CK(cudaDeviceSynchronize());
  uint32_t const L = wt.rank_select_.bit_array_.numArrays();
  std::vector<uint64_t> sizes(L);
  for (uint32_t l = 0; l < L; ++l) sizes[l] = wt.rank_select_.bit_array_.size(l);
  auto const per = gather(wt, kPerLevel, 0, 4 * uint64_t(L));
  std::vector<uint64_t> ones(L), last_l2(L), num_l1(L), num_l2(L);
  for (uint32_t l = 0; l < L; ++l) {
    ones[l] = per[4 * l];
    last_l2[l] = per[4 * l + 1];
    num_l1[l] = per[4 * l + 2];
    num_l2[l] = per[4 * l + 3];
  }
  write_as<uint64_t>(prefix + ".LEVEL_SIZES.bin", sizes);
  write_as<uint64_t>(prefix + ".TOTAL_ONES.bin", ones);
  write_as<uint64_t>(prefix + ".NUM_LAST_L2.bin", last_l2);
  std::vector<uint64_t> counts(sigma);
  for (uint64_t c = 0; c < sigma; ++c) counts[c] = wt.getCounts(c);
  write_as<uint64_t>(prefix + ".COUNTS.bin", counts);
  write_as<uint64_t>(prefix + ".NODE_RANKS.bin",
                     gather(wt, kRanks, 0, num_ranks));
  for (uint32_t l = 0; l < L; ++l) {
    uint64_t const bits = sizes[l];
    std::string const sfx = "." + std::to_string(l) + ".bin";
    write_as<uint32_t>(prefix + ".LEVEL_WORDS" + sfx,
                       gather(wt, kWords, l, (bits + 31) / 32));
    write_as<uint64_t>(prefix + ".L1" + sfx, gather(wt, kL1, l, num_l1[l]));
    write_as<uint16_t>(prefix + ".L2" + sfx, gather(wt, kL2, l, num_l2[l]));
    write_as<uint64_t>(prefix + ".SAMPLES0" + sfx,
                       gather(wt, kS0, l, (bits - ones[l]) / kSampleRate));
    write_as<uint64_t>(prefix + ".SAMPLES1" + sfx,
                       gather(wt, kS1, l, ones[l] / kSampleRate));
  }
  return 0;
}

template <class T>
int query(std::string const& text_path, uint64_t sigma,
          std::string const& q_path, uint64_t m, std::string const& out_path) {
  auto const buf = read_file(text_path);
  uint64_t const n = buf.size() / sizeof(T);
  ecl::WaveletTree<T> wt(reinterpret_cast<T const*>(buf.data()), n,
                         make_alphabet<T>(sigma), 0);
  auto const qb = read_file(q_path);
  auto const* types = reinterpret_cast<uint8_t const*>(qb.data());
  auto const* idx = reinterpret_cast<uint64_t const*>(qb.data() + m);
  auto const* sym = idx + m;
  std::vector<size_t> acc;
  std::vector<ecl::RankSelectQuery<T>> rq, sq;
  std::vector<uint64_t> where_a, where_r, where_s;
  for (uint64_t i = 0; i < m; ++i) {
    if (types[i] == 0) {
      acc.push_back(idx[i]);
      where_a.push_back(i);
    } else if (types[i] == 1) {
      rq.push_back({idx[i], static_cast<T>(sym[i])});
      where_r.push_back(i);
    } else {
      sq.push_back({idx[i], static_cast<T>(sym[i])});
      where_s.push_back(i);
    }
  }
  std::vector<uint64_t> out(m, 0);
  if (!acc.empty()) {
    auto r = wt.access(acc.data(), acc.size());
    for (size_t j = 0; j < acc.size(); ++j) out[where_a[j]] = r[j];
  }
  if (!rq.empty()) {
    auto r = wt.rank(rq.data(), rq.size());
    for (size_t j = 0; j < rq.size(); ++j) out[where_r[j]] = r[j];
  }
  if (!sq.empty()) {
    auto r = wt.select(sq.data(), sq.size());
    for (size_t j = 0; j < sq.size(); ++j) out[where_s[j]] = r[j];
  }
  write_file(out_path, out.data(), m * 8);
  return 0;
}

inline uint64_t mix64(uint64_t x) {  // splitmix64
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0)
      .count();
}

template <class T>
int bench(uint64_t n, uint64_t sigma, uint64_t m, int reps) {
  T* text = nullptr;
  CK(cudaHostAlloc(&text, n * sizeof(T), cudaHostAllocPortable));
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < int64_t(n); ++i)
    text[i] = static_cast<T>(mix64(uint64_t(i) ^ 0x5eed) % sigma);
  std::vector<double> build_s;
  ecl::WaveletTree<T> wt;
  for (int r = 0; r <= reps; ++r) {
    CK(cudaDeviceSynchronize());
    auto const t0 = std::chrono::steady_clock::now();
    wt = ecl::WaveletTree<T>(text, n, make_alphabet<T>(sigma), 0);
    CK(cudaDeviceSynchronize());
    if (r > 0) build_s.push_back(seconds_since(t0));  // first: warm-up
  }
  std::vector<uint64_t> occ(sigma);
  for (uint64_t c = 0; c < sigma; ++c) occ[c] = wt.getTotalAppearances(c);
  size_t* acc = nullptr;
  ecl::RankSelectQuery<T>*rq = nullptr, *sq = nullptr;
  CK(cudaHostAlloc(&acc, m * sizeof(size_t), cudaHostAllocPortable));
  CK(cudaHostAlloc(&rq, m * sizeof(*rq), cudaHostAllocPortable));
  CK(cudaHostAlloc(&sq, m * sizeof(*sq), cudaHostAllocPortable));
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < int64_t(m); ++i) {
    uint64_t const h = mix64(uint64_t(i) + 77);
    acc[i] = h % n;
    rq[i] = {mix64(h) % n, static_cast<T>(mix64(h + 1) % sigma)};
    T c = static_cast<T>(mix64(h + 2) % sigma);
    while (occ[c] == 0) c = static_cast<T>((c + 1) % sigma);
    sq[i] = {1 + mix64(h + 3) % occ[c], c};
  }
  auto time_call = [&](auto&& fn) {
    fn();  // warm-up
    double best = 1e30;
    for (int r = 0; r < reps; ++r) {
      auto const t0 = std::chrono::steady_clock::now();
      fn();
      best = std::min(best, seconds_since(t0));
    }
    return best;
  };
  double const ta = time_call([&] { (void)wt.access(acc, m); });
  double const tr = time_call([&] { (void)wt.rank(rq, m); });
  double const ts = time_call([&] { (void)wt.select(sq, m); });
  double mean_build = 0;
  for (double s : build_s) mean_build += s / build_s.size();
  double const best_build = *std::min_element(build_s.begin(), build_s.end());
  std::printf(
      "{\"n\": %llu, \"elem_size\": %d, \"sigma\": %llu, \"queries_per_type\": "
      "%llu, \"build_ms_mean\": %.3f, \"build_ms_best\": %.3f, "
      "\"build_GB_s\": %.4f, \"access_Mq_s\": %.2f, \"rank_Mq_s\": %.2f, "
      "\"select_Mq_s\": %.2f, \"reps\": %d}\n",
      (unsigned long long)n, int(sizeof(T)), (unsigned long long)sigma,
      (unsigned long long)m, mean_build * 1e3, best_build * 1e3,
      n * sizeof(T) / mean_build / 1e9, m / ta / 1e6, m / tr / 1e6,
      m / ts / 1e6, reps);
  CK(cudaFreeHost(acc));
  CK(cudaFreeHost(rq));
  CK(cudaFreeHost(sq));
  CK(cudaFreeHost(text));
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: ref_driver dump|query|bench ...\n");
    return 2;
  }
  std::string const mode = argv[1];
  auto u = [&](int i) { return std::strtoull(argv[i], nullptr, 10); };
  if (mode == "dump" && argc == 7) {
    int const es = int(u(3));
    if (es == 1) return dump<uint8_t>(argv[2], u(4), u(5), argv[6]);
    if (es == 2) return dump<uint16_t>(argv[2], u(4), u(5), argv[6]);
  } else if (mode == "query" && argc == 8) {
    int const es = int(u(3));
    if (es == 1) return query<uint8_t>(argv[2], u(4), argv[5], u(6), argv[7]);
    if (es == 2) return query<uint16_t>(argv[2], u(4), argv[5], u(6), argv[7]);
  } else if (mode == "bench" && argc == 7) {
    int const es = int(u(3));
    if (es == 1) return bench<uint8_t>(u(2), u(4), u(5), int(u(6)));
    if (es == 2) return bench<uint16_t>(u(2), u(4), u(5), int(u(6)));
  }
  std::fprintf(stderr, "bad arguments\n");
  return 2;
}
