// Drop-in check of the C++ API: the same calls the reference's
// example/example.cu and test suites make, against libewt.so.
//
//   dropin_example <n> <sigma> <seed> <out.bin>
//
// Builds a WaveletTree<uint8_t> over an LCG text, runs host access / rank /
// select batches and a user kernel that receives the tree by value and
// queries it with deviceAccess / deviceRank / deviceSelect and the
// RankSelect device calls.  Writes the text and every answer to out.bin for
// the Python test to check against the oracle.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "ecl_wavelet/tree/wavelet_tree.cuh"

using T = uint8_t;

__global__ void user_kernel(ecl::WaveletTree<T> tree, size_t const* idx,
                            ecl::RankSelectQuery<T> const* rq,
                            ecl::RankSelectQuery<T> const* sq, size_t m,
                            size_t* out) {
  size_t const i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i >= m) return;
  out[4 * i + 0] = tree.deviceAccess<1>(idx[i], true);
  out[4 * i + 1] = tree.deviceRank<1>(rq[i], true);
  out[4 * i + 2] = tree.deviceSelect<1>(sq[i], true);
  // binary rank of ones on level 0 before idx[i]
  out[4 * i + 3] = tree.rank_select_.rank<1, false, 1>(
      0, idx[i], tree.rank_select_.bit_array_.getOffset(0));
}

#define CK(x)                                                  \
  do {                                                         \
    cudaError_t e = (x);                                       \
    if (e != cudaSuccess) {                                    \
      std::fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e)); \
      return 2;                                                \
    }                                                          \
  } while (0)

int main(int argc, char** argv) {
  if (argc != 5) return 1;
  size_t const n = std::strtoull(argv[1], nullptr, 10);
  size_t const sigma = std::strtoull(argv[2], nullptr, 10);
  uint64_t x = std::strtoull(argv[3], nullptr, 10);
  auto next = [&]() {
    x = x * 6364136223846793005ull + 1442695040888963407ull;
    return x >> 33;
  };
  std::vector<T> text(n);
  for (auto& c : text) c = static_cast<T>(next() % sigma);
  ecl::WaveletTree<T> wt;
  try {
    wt = ecl::WaveletTree<T>(text.data(), n, std::vector<T>(), 0);
  } catch (std::runtime_error const& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 3;
  }
  size_t const m = 4096;
  std::vector<size_t> idx(m);
  std::vector<ecl::RankSelectQuery<T>> rq(m), sq(m);
  for (size_t i = 0; i < m; ++i) {
    idx[i] = next() % n;
    rq[i] = {next() % (n + 1), static_cast<T>(next() % sigma)};
    sq[i] = {1 + next() % (n / sigma + 2), static_cast<T>(next() % sigma)};
  }
  std::span<T> a = wt.access(idx.data(), m);
  std::vector<size_t> host_out(3 * m);
  for (size_t i = 0; i < m; ++i) host_out[i] = a[i];
  auto r = wt.rank(rq.data(), m);
  for (size_t i = 0; i < m; ++i) host_out[m + i] = r[i];
  auto s = wt.select(sq.data(), m);
  for (size_t i = 0; i < m; ++i) host_out[2 * m + i] = s[i];

  size_t* d_idx;
  ecl::RankSelectQuery<T>*d_rq, *d_sq;
  size_t* d_out;
  CK(cudaMalloc(&d_idx, m * sizeof(size_t)));
  CK(cudaMalloc(&d_rq, m * sizeof(rq[0])));
  CK(cudaMalloc(&d_sq, m * sizeof(sq[0])));
  CK(cudaMalloc(&d_out, 4 * m * sizeof(size_t)));
  CK(cudaMemcpy(d_idx, idx.data(), m * sizeof(size_t), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_rq, rq.data(), m * sizeof(rq[0]), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_sq, sq.data(), m * sizeof(sq[0]), cudaMemcpyHostToDevice));
  user_kernel<<<(m + 127) / 128, 128>>>(wt, d_idx, d_rq, d_sq, m, d_out);
  CK(cudaGetLastError());
  std::vector<size_t> dev_out(4 * m);
  CK(cudaMemcpy(dev_out.data(), d_out, 4 * m * sizeof(size_t),
                cudaMemcpyDeviceToHost));
  cudaFree(d_idx);
  cudaFree(d_rq);
  cudaFree(d_sq);
  cudaFree(d_out);

  std::FILE* f = std::fopen(argv[4], "wb");
  if (!f) return 4;
  uint64_t hdr[3] = {n, sigma, m};
  std::fwrite(hdr, 8, 3, f);
  std::fwrite(text.data(), 1, n, f);
  std::fwrite(idx.data(), 8, m, f);
  std::fwrite(rq.data(), sizeof(rq[0]), m, f);
  std::fwrite(sq.data(), sizeof(sq[0]), m, f);
  std::fwrite(host_out.data(), 8, 3 * m, f);
  std::fwrite(dev_out.data(), 8, 4 * m, f);
  std::fclose(f);
  std::printf("alphabet size %zu, levels %u, access[0]=%u\n",
              wt.getAlphabetSize(), unsigned(wt.getNumLevels()),
              unsigned(a[0]));
  return 0;
}
