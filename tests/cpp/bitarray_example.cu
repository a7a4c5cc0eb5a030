// Drop-in check of the standalone BitArray / RankSelect API, the way the
// reference's own tests use it (tests/test_rank_select.cu:405-555 of
// mfranzreb/ECL_wavelet): bit arrays created with BitArray(sizes[,
// init_value]), filled by a user kernel through writeWord / writeWordAtBit,
// moved into RankSelect(BitArray&&, GPU_index), then queried by a user kernel
// that receives the RankSelect by value.
//
//   bitarray_example <init_value> <seed> <out.bin>
//
// Arrays: a % 4 == 0 hashed words, 1 the 0xFFFF0000 pattern, 2 sparse hashed
// words (written with writeWordAtBit), 3 left as created.  Writes the sizes,
// every array's words as the kernel wrote them (recomputed here on the
// host), the memory bounds and every answer to out.bin for the Python test
// to check against the oracle.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "ecl_wavelet/tree/wavelet_tree.cuh"

__host__ __device__ inline uint64_t mix(uint64_t x) {  // splitmix64
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

__host__ __device__ inline uint32_t word_of(uint32_t a, uint64_t w,
                                            uint64_t seed) {
  uint64_t const h = mix(seed ^ (uint64_t(a) << 40) ^ w);
  switch (a % 4) {
    case 0: return static_cast<uint32_t>(h);
    case 1: return 0xFFFF0000u;
    default: return static_cast<uint32_t>(h & (h >> 32) & mix(h));
  }
}

__global__ void fill_kernel(ecl::BitArray ba, uint32_t a, uint64_t nwords,
                            uint64_t seed) {
  uint64_t const stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t w = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
       w < nwords; w += stride) {
    if (a % 4 == 2)
      ba.writeWordAtBit(a, w * 32 + (w % 32), word_of(a, w, seed));
    else
      ba.writeWord(a, w, word_of(a, w, seed));
  }
}

__global__ void query_kernel(ecl::RankSelect rs, uint32_t a,
                             uint64_t const* pos, uint64_t const* k1,
                             uint64_t const* k0, uint64_t m, uint64_t* out) {
  uint64_t const i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= m) return;
  size_t const off = rs.bit_array_.getOffset(a);
  out[6 * i + 0] = rs.rank<1, false, 1>(static_cast<uint8_t>(a), pos[i], off);
  auto const r0 = rs.rank<1, true, 0>(static_cast<uint8_t>(a), pos[i], off);
  out[6 * i + 1] = r0.rank;
  out[6 * i + 2] = r0.bit;
  out[6 * i + 3] = rs.select<1, 1>(a, k1[i], off);
  out[6 * i + 4] = rs.select<0, 1>(a, k0[i], off);
  out[6 * i + 5] = rs.getTotalNumVals<1>(a);
}

#define CK(x)                                                      \
  do {                                                             \
    cudaError_t e = (x);                                           \
    if (e != cudaSuccess) {                                        \
      std::fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e)); \
      return 2;                                                    \
    }                                                              \
  } while (0)

int main(int argc, char** argv) {
  if (argc != 4) return 1;
  bool const init = std::atoi(argv[1]) != 0;
  uint64_t const seed = std::strtoull(argv[2], nullptr, 10);
  std::vector<size_t> const sizes = {33,        4097,    65536,     65537,
                                     300001,    1048576, 5000003,   17,
                                     3 * 65536 + 777, 1u << 22};
  uint32_t const A = static_cast<uint32_t>(sizes.size());
  uint64_t const total = 5000003 + (1u << 22);
  size_t const need_ba = ecl::BitArray::getNeededGPUMemory(total, A);
  size_t const need_rs = ecl::RankSelect::getNeededGPUMemory(total, A);
  ecl::RankSelect rs;
  try {
    ecl::BitArray ba(sizes, init);
    for (uint32_t a = 0; a < A; ++a) {
      if (a % 4 == 3) continue;  // left as created
      uint64_t const nw = (sizes[a] + 31) / 32;
      fill_kernel<<<256, 256>>>(ba, a, nw, seed);
      CK(cudaGetLastError());
    }
    rs = ecl::RankSelect(std::move(ba), 0);
  } catch (std::runtime_error const& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 3;
  }
  uint64_t const m = 4096;
  std::FILE* f = std::fopen(argv[3], "wb");
  if (!f) return 4;
  uint64_t hdr[5] = {A, m, init ? 1u : 0u, need_ba, need_rs};
  std::fwrite(hdr, 8, 5, f);
  for (size_t s : sizes) {
    uint64_t v = s;
    std::fwrite(&v, 8, 1, f);
  }
  uint64_t *d_pos, *d_k1, *d_k0, *d_out;
  CK(cudaMalloc(&d_pos, m * 8));
  CK(cudaMalloc(&d_k1, m * 8));
  CK(cudaMalloc(&d_k0, m * 8));
  CK(cudaMalloc(&d_out, 6 * m * 8));
  uint64_t x = seed * 7 + 1;
  for (uint32_t a = 0; a < A; ++a) {
    uint64_t const nw = (sizes[a] + 31) / 32;
    std::vector<uint32_t> words(nw);
    for (uint64_t w = 0; w < nw; ++w)
      words[w] = a % 4 == 3 ? (init ? 0xFFFFFFFFu : 0u) : word_of(a, w, seed);
    std::fwrite(words.data(), 4, nw, f);
    std::vector<uint64_t> pos(m), k1(m), k0(m);
    for (uint64_t i = 0; i < m; ++i) {
      x = mix(x);
      pos[i] = x % (sizes[a] + 1);
      k1[i] = mix(x + 1) % (sizes[a] + 2);  // includes 0 and past the end
      k0[i] = mix(x + 2) % (sizes[a] + 2);
    }
    pos[0] = 0;
    pos[1] = sizes[a];
    CK(cudaMemcpy(d_pos, pos.data(), m * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_k1, k1.data(), m * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_k0, k0.data(), m * 8, cudaMemcpyHostToDevice));
    query_kernel<<<(m + 127) / 128, 128>>>(rs, a, d_pos, d_k1, d_k0, m, d_out);
    CK(cudaGetLastError());
    std::vector<uint64_t> out(6 * m);
    CK(cudaMemcpy(out.data(), d_out, 6 * m * 8, cudaMemcpyDeviceToHost));
    std::fwrite(pos.data(), 8, m, f);
    std::fwrite(k1.data(), 8, m, f);
    std::fwrite(k0.data(), 8, m, f);
    std::fwrite(out.data(), 8, 6 * m, f);
  }
  std::fclose(f);
  cudaFree(d_pos);
  cudaFree(d_k1);
  cudaFree(d_k0);
  cudaFree(d_out);
  // the shortened codes the library builds with, as createMinimalCodes
  auto const codes = ecl::WaveletTree<uint8_t>::createMinimalCodes(
      std::vector<uint8_t>(75));
  std::printf("arrays %u, bounds %zu / %zu bytes, codes(75) %zu\n", A,
              need_ba, need_rs, codes.size());
  return 0;
}
