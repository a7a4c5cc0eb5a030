// Cooperative RankSelect::rank<NumThreads, ...> / select<Value, NumThreads>
// against the single-lane answers, the way the reference's rank/select
// tests sweep NumThreads over 32, 16, 8, 4, 2, 1 (test_rank_select.cu of
// mfranzreb/ECL_wavelet).  Two structures:
//   - a WaveletTree<uint8_t> over an LCG text (its levels' RankSelect, with
//     rank blocks and dense select samples), and
//   - a standalone RankSelect over BitArray(sizes) arrays filled by a user
//     kernel with dense, sparse (one set bit in ~20000, so that select's
//     sample brackets span many L1 blocks), all-ones and all-zero words
//     (rank blocks and the reference-format samples).
// Every group of NumThreads lanes answers one query; lane 0 of the group
// writes it.  Exit status 5 and a message on any difference.
//
//   coop_rank_select <seed>
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

__device__ inline uint32_t word_of(uint32_t a, uint64_t w, uint64_t seed) {
  uint64_t const h = mix(seed ^ (uint64_t(a) << 40) ^ w);
  switch (a % 4) {
    case 0: return static_cast<uint32_t>(h);                        // dense
    case 1: return (h % 625) == 0 ? 1u << (h >> 59) : 0u;          // sparse
    case 2: return ~0u;                                             // ones
    default: return 0u;                                             // zeros
  }
}

__global__ void fill_kernel(ecl::BitArray ba, uint32_t a, uint64_t nwords,
                            uint64_t seed) {
  uint64_t const stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t w = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
       w < nwords; w += stride)
    ba.writeWord(a, w, word_of(a, w, seed));
}

// Query q of array arr[q]: rank1 at pos, rank0 + bit at pos, select1 of k1,
// select0 of k0.
template <int NT>
__global__ void coop_kernel(ecl::RankSelect rs, uint32_t const* arr,
                            uint64_t const* pos, uint64_t const* k1,
                            uint64_t const* k0, uint64_t m, uint64_t* out) {
  uint64_t const g = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) / NT;
  if (g >= m) return;  // whole groups leave together: m groups of NT lanes
  uint8_t const a = static_cast<uint8_t>(arr[g]);
  size_t const off = rs.bit_array_.getOffset(a);
  uint64_t const r1 = rs.rank<NT, false, 1>(a, pos[g], off);
  auto const r0 = rs.rank<NT, true, 0>(a, pos[g], off);
  uint64_t const s1 = rs.select<1, NT>(a, k1[g], off);
  uint64_t const s0 = rs.select<0, NT>(a, k0[g], off);
  if (threadIdx.x % NT == 0) {
    out[5 * g + 0] = r1;
    out[5 * g + 1] = r0.rank;
    out[5 * g + 2] = r0.bit;
    out[5 * g + 3] = s1;
    out[5 * g + 4] = s0;
  }
}

#define CK(x)                                                      \
  do {                                                             \
    cudaError_t e = (x);                                           \
    if (e != cudaSuccess) {                                        \
      std::fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e)); \
      return 2;                                                    \
    }                                                              \
  } while (0)

template <int NT>
int run(ecl::RankSelect const& rs, uint32_t const* d_arr, uint64_t const* d_pos,
        uint64_t const* d_k1, uint64_t const* d_k0, uint64_t m,
        uint64_t* d_out, std::vector<uint64_t>& host) {
  CK(cudaMemset(d_out, 0xFF, 5 * m * 8));
  uint64_t const threads = m * NT;
  coop_kernel<NT><<<static_cast<unsigned>((threads + 255) / 256), 256>>>(
      rs, d_arr, d_pos, d_k1, d_k0, m, d_out);
  CK(cudaGetLastError());
  host.resize(5 * m);
  CK(cudaMemcpy(host.data(), d_out, 5 * m * 8, cudaMemcpyDeviceToHost));
  return 0;
}

// All NumThreads against NumThreads = 1 on one structure; arrays a < A with
// sizes[a] bits and totals ones[a].
int check(char const* name, ecl::RankSelect const& rs,
          std::vector<uint64_t> const& sizes, std::vector<uint64_t> const& ones,
          uint64_t seed) {
  uint64_t const A = sizes.size(), m = 1 << 14;
  std::vector<uint32_t> arr(m);
  std::vector<uint64_t> pos(m), k1(m), k0(m);
  uint64_t x = seed;
  for (uint64_t q = 0; q < m; ++q) {
    x = mix(x);
    uint32_t const a = static_cast<uint32_t>(x % A);
    arr[q] = a;
    pos[q] = mix(x + 1) % (sizes[a] + 1);
    k1[q] = mix(x + 2) % (ones[a] + 2);  // 0 and past the end included
    k0[q] = mix(x + 3) % (sizes[a] - ones[a] + 2);
  }
  pos[0] = 0;
  pos[1] = sizes[arr[1]];
  uint32_t* d_arr;
  uint64_t *d_pos, *d_k1, *d_k0, *d_out;
  CK(cudaMalloc(&d_arr, m * 4));
  CK(cudaMalloc(&d_pos, m * 8));
  CK(cudaMalloc(&d_k1, m * 8));
  CK(cudaMalloc(&d_k0, m * 8));
  CK(cudaMalloc(&d_out, 5 * m * 8));
  CK(cudaMemcpy(d_arr, arr.data(), m * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_pos, pos.data(), m * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_k1, k1.data(), m * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_k0, k0.data(), m * 8, cudaMemcpyHostToDevice));
  std::vector<uint64_t> ref, got;
  int st = run<1>(rs, d_arr, d_pos, d_k1, d_k0, m, d_out, ref);
  int const nts[5] = {2, 4, 8, 16, 32};
  uint64_t bad = 0;
  for (int ni = 0; ni < 5 && st == 0; ++ni) {
    switch (nts[ni]) {
      case 2: st = run<2>(rs, d_arr, d_pos, d_k1, d_k0, m, d_out, got); break;
      case 4: st = run<4>(rs, d_arr, d_pos, d_k1, d_k0, m, d_out, got); break;
      case 8: st = run<8>(rs, d_arr, d_pos, d_k1, d_k0, m, d_out, got); break;
      case 16: st = run<16>(rs, d_arr, d_pos, d_k1, d_k0, m, d_out, got); break;
      default: st = run<32>(rs, d_arr, d_pos, d_k1, d_k0, m, d_out, got); break;
    }
    for (uint64_t i = 0; i < 5 * m && st == 0; ++i) {
      if (got[i] != ref[i]) {
        if (bad < 5)
          std::fprintf(stderr, "%s NumThreads %d query %llu field %llu: %llu vs %llu\n",
                       name, nts[ni], (unsigned long long)(i / 5),
                       (unsigned long long)(i % 5), (unsigned long long)got[i],
                       (unsigned long long)ref[i]);
        ++bad;
      }
    }
  }
  // the single-lane answers themselves: select past the end gives the size
  for (uint64_t q = 0; q < m && st == 0; ++q) {
    uint32_t const a = arr[q];
    if ((k1[q] == 0 || k1[q] > ones[a]) && ref[5 * q + 3] != sizes[a]) ++bad;
    if (pos[q] == sizes[a] && ref[5 * q + 0] != ones[a]) ++bad;
  }
  cudaFree(d_arr);
  cudaFree(d_pos);
  cudaFree(d_k1);
  cudaFree(d_k0);
  cudaFree(d_out);
  if (st) return st;
  std::printf("%s: %llu arrays, %llu queries x 5 NumThreads, %llu differences\n",
              name, (unsigned long long)A, (unsigned long long)m,
              (unsigned long long)bad);
  return bad ? 5 : 0;
}

__global__ void totals_kernel(ecl::RankSelect rs, uint32_t A, uint64_t* out) {
  for (uint32_t a = threadIdx.x; a < A; a += blockDim.x)
    out[a] = rs.getTotalNumVals<1>(a);
}

// Ones of every array, read on the device.
int totals(ecl::RankSelect const& rs, uint32_t A, std::vector<uint64_t>& ones) {
  uint64_t* d;
  CK(cudaMalloc(&d, 8 * A));
  totals_kernel<<<1, 32>>>(rs, A, d);
  CK(cudaGetLastError());
  ones.resize(A);
  CK(cudaMemcpy(ones.data(), d, 8 * A, cudaMemcpyDeviceToHost));
  cudaFree(d);
  return 0;
}

int main(int argc, char** argv) {
  if (argc != 2) return 1;
  uint64_t const seed = std::strtoull(argv[1], nullptr, 10);
  try {
    // the tree's levels: rank blocks and dense select samples
    size_t const n = 3000017;
    std::vector<uint8_t> text(n);
    uint64_t x = seed;
    for (auto& c : text) {
      x = x * 6364136223846793005ull + 1442695040888963407ull;
      c = static_cast<uint8_t>(x >> 56);
    }
    ecl::WaveletTree<uint8_t> wt(text.data(), n, std::vector<uint8_t>(), 0);
    uint32_t const L = wt.getNumLevels();
    std::vector<uint64_t> sizes(L, n), ones;
    int st = totals(wt.rank_select_, L, ones);
    if (st == 0) st = check("tree levels", wt.rank_select_, sizes, ones, seed + 1);
    if (st) return st;
    // standalone arrays: rank blocks and reference-format samples
    std::vector<size_t> const bsizes = {50000000, 50000017, 1 << 20, 300001,
                                        8000003,  65536 * 3 + 5, 4097, 33};
    uint32_t const A = static_cast<uint32_t>(bsizes.size());
    ecl::BitArray ba(bsizes, false);
    for (uint32_t a = 0; a < A; ++a) {
      fill_kernel<<<512, 256>>>(ba, a, (bsizes[a] + 31) / 32, seed);
      CK(cudaGetLastError());
    }
    ecl::RankSelect rs(std::move(ba), 0);
    std::vector<uint64_t> bs(bsizes.begin(), bsizes.end()), bo;
    st = totals(rs, A, bo);
    if (st == 0) st = check("standalone arrays", rs, bs, bo, seed + 2);
    return st;
  } catch (std::runtime_error const& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 3;
  }
}
