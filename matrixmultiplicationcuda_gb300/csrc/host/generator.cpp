// Seeded synthetic inputs.
//
// 1. mg::generate_matrix: the reference's generator (matrix_generator.cpp:28-140)
//    with the same patterns, the same std::mt19937 stream and the same draw
//    order, so a given (pattern, sparsity, blocksize, seed) yields the same
//    matrix bit for bit. This is how the 1024 x 1024 blockrandom workload
//    (16x16 blocks, 10% of blocks kept) is produced.
// 2. spmm_gen_structure / spmm_gen_values / spmm_gen_dense: generators for the
//    larger workloads the reference has no code for (diagonal band, 256 x 256
//    block-diagonal tiles, log-normal row counts, N(0,1) x 10^U[-3,3] block
//    magnitudes). They build BCSR directly (no dense intermediate) from a
//    counter-based hash RNG, so any part can be regenerated independently.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>
#include "../../../include/bcsr_spmm.hpp"
#include "host_internal.h"

namespace mg {

namespace {
template <typename T>
struct Filler {
  Matrix<T>& mat;
  std::mt19937& rng;
  int rows, cols;
  // generate_dense_block + copy, for the rectangle at (r0, c0) clipped to the matrix
  void rect(int r0, int c0, int h, int w) {
    const int r1 = std::min(r0 + h, rows), c1 = std::min(c0 + w, cols);
    if (r1 <= r0 || c1 <= c0) return;
    std::uniform_real_distribution<double> dist(-1.0, 1.0);
    for (int i = r0; i < r1; ++i)
      for (int j = c0; j < c1; ++j) mat[i][j] = static_cast<T>(dist(rng));
  }
};
}  // namespace

template <typename T>
Matrix<T> generate_matrix(int num_rows, int num_cols, double sparsity, const std::string& pattern,
                          int blocksize, unsigned int seed) {
  Matrix<T> mat(num_rows, std::vector<T>(num_cols));
  std::mt19937 rng(seed);
  Filler<T> f{mat, rng, num_rows, num_cols};
  auto nblk = [&](int n, int b) { return (n + b - 1) / b; };
  if (pattern == "random") {
    std::bernoulli_distribution keep(1.0 - sparsity);
    for (int i = 0; i < num_rows; ++i)
      for (int j = 0; j < num_cols; ++j)
        if (keep(rng)) {
          std::uniform_real_distribution<double> d(-1.0, 1.0);
          mat[i][j] = static_cast<T>(d(rng));
        }
  } else if (pattern == "checkerboard") {
    for (int i = 0; i < nblk(num_rows, blocksize); ++i)
      for (int j = 0; j < nblk(num_cols, blocksize); ++j)
        if (((i % 2) ^ (j % 2)) == 0) f.rect(i * blocksize, j * blocksize, blocksize, blocksize);
  } else if (pattern == "diagonal") {
    for (int i = 0; i < std::min(num_rows, num_cols); ++i) f.rect(i, i, 1, 1);
  } else if (pattern == "blockdiagonal") {
    const int n = std::min(num_rows, num_cols) / blocksize + 1;
    for (int i = 0; i < n; ++i) f.rect(i * blocksize, i * blocksize, blocksize, blocksize);
  } else if (pattern == "blockrandom") {
    std::bernoulli_distribution keep(1.0 - sparsity);
    for (int i = 0; i < nblk(num_rows, blocksize); ++i)
      for (int j = 0; j < nblk(num_cols, blocksize); ++j)
        if (keep(rng)) f.rect(i * blocksize, j * blocksize, blocksize, blocksize);
  } else if (pattern == "pattern64by16" || pattern == "pattern32by16") {
    const int brow = pattern == "pattern64by16" ? 64 : 32;
    std::bernoulli_distribution keep(1.0 - sparsity);
    for (int bi = 0; bi < nblk(num_rows, brow); ++bi)
      for (int bj = 0; bj < nblk(num_cols, 16); ++bj)
        if (keep(rng)) f.rect(bi * brow, bj * 16, brow, 16);
  } else {
    throw std::invalid_argument("Unknown pattern: " + pattern);
  }
  return mat;
}

template Matrix<float> generate_matrix<float>(int, int, double, const std::string&, int, unsigned int);
template Matrix<double> generate_matrix<double>(int, int, double, const std::string&, int, unsigned int);

}  // namespace mg

namespace {

// SplitMix64 finaliser as a stateless hash (counter-based stream).
inline uint64_t mix64(uint64_t x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}
inline uint64_t h2(uint64_t seed, uint64_t stream, uint64_t i) {
  return mix64(mix64(seed * 0x2545f4914f6cdd1dull + stream) ^ i);
}
inline double u01(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }
inline double normal(uint64_t seed, uint64_t stream, uint64_t i) {  // Box-Muller
  double a = u01(h2(seed, stream, 2 * i)), b = u01(h2(seed, stream, 2 * i + 1));
  if (a < 1e-300) a = 1e-300;
  return std::sqrt(-2.0 * std::log(a)) * std::cos(6.283185307179586 * b);
}

enum Pattern { P_RANDOM = 0, P_BAND = 1, P_BLOCKDIAG = 2, P_LOGNORMAL = 3 };
enum Dist { D_UNIFORM = 0, D_SCALED_NORMAL = 1, D_NORMAL = 2 };

template <typename F>
void parallel_for(long long n, F f) {
  unsigned nt = std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()), 32u);
  if (n < 4096 || nt == 1) {
    f(0, n);
    return;
  }
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; ++t) {
    long long a = n * t / nt, b = n * (t + 1) / nt;
    if (a < b) th.emplace_back([=] { f(a, b); });
  }
  for (auto& x : th) x.join();
}

}  // namespace

extern "C" {

// mg::generate_matrix<float> into a flat row-major buffer; -1 on unknown pattern.
int spmm_generate_matrix(int rows, int cols, double sparsity, const char* pattern, int blocksize,
                         unsigned seed, float* out) {
  try {
    auto m = mg::generate_matrix<float>(rows, cols, sparsity, std::string(pattern), blocksize, seed);
    for (int i = 0; i < rows; ++i) std::memcpy(out + (size_t)i * cols, m[i].data(), sizeof(float) * cols);
    return 0;
  } catch (const std::exception& e) {
    spmm::host_fail(SPMM_ERR_INVALID_ARG, e.what());
    return -1;
  }
}

// Block structure of an M x K matrix with bR x 16 blocks.
//   pattern 0 random:    each block kept with probability `density`.
//   pattern 1 band:      blocks within `param` block columns of the diagonal
//                        (block row i spans block columns [i*bR/16, ((i+1)*bR-1)/16]),
//                        each kept with probability min(1, density*KB / band length).
//   pattern 2 blockdiag: square diagonal tiles of `param` x `param` elements, fully dense.
//   pattern 3 lognormal: per-row block counts ~ LogNormal with mean density*KB and
//                        coefficient of variation `param`, clipped to [0, KB], columns
//                        uniform without replacement.
// col_idx must hold MB*KB entries; returns nnzb (or -1).
long long spmm_gen_structure(int M, int K, int bR, int pattern, double density, double param,
                             unsigned long long seed, int* row_ptr, int* col_idx) {
  if (bR <= 0 || M % bR || K % 16) {
    spmm::host_fail(SPMM_ERR_INVALID_ARG, "bad sizes");
    return -1;
  }
  const int MB = M / bR, KB = K / 16;
  std::vector<int> cols;
  long long k = 0;
  row_ptr[0] = 0;
  const double sigma2 = std::log(1.0 + param * param);
  for (int i = 0; i < MB; ++i) {
    cols.clear();
    if (pattern == P_RANDOM) {
      for (int j = 0; j < KB; ++j)
        if (u01(h2(seed, 1, (uint64_t)i * KB + j)) < density) cols.push_back(j);
    } else if (pattern == P_BAND) {
      const int w = (int)param;
      const int lo = std::max(0, (int)((long long)i * bR / 16) - w);
      const int hi = std::min(KB - 1, (int)(((long long)(i + 1) * bR - 1) / 16) + w);
      const double avg_len = 2.0 * w + (double)bR / 16.0;
      const double q = std::min(1.0, density * KB / avg_len);
      for (int j = lo; j <= hi; ++j)
        if (q >= 1.0 || u01(h2(seed, 2, (uint64_t)i * KB + j)) < q) cols.push_back(j);
    } else if (pattern == P_BLOCKDIAG) {
      const long long T = (long long)param;
      for (int j = 0; j < KB; ++j)
        if (((long long)i * bR) / T == ((long long)j * 16) / T) cols.push_back(j);
    } else if (pattern == P_LOGNORMAL) {
      const double mean = density * KB;
      const double mu = std::log(std::max(mean, 1e-9)) - 0.5 * sigma2;
      const double z = normal(seed, 3, (uint64_t)i);
      long long cnt = std::llround(std::exp(mu + std::sqrt(sigma2) * z));
      cnt = std::max(0LL, std::min<long long>(cnt, KB));
      // Floyd's sampling of cnt distinct columns
      std::vector<char> used(KB, 0);
      uint64_t ctr = 0;
      for (long long j = KB - cnt; j < KB; ++j) {
        const long long t = (long long)(u01(h2(seed, 4, ((uint64_t)i << 32) + ctr++)) * (double)(j + 1));
        const int pick = used[t] ? (int)j : (int)t;
        used[pick] = 1;
      }
      for (int j = 0; j < KB; ++j)
        if (used[j]) cols.push_back(j);
    } else {
      spmm::host_fail(SPMM_ERR_INVALID_ARG, "unknown pattern");
      return -1;
    }
    for (int c : cols) col_idx[k++] = c;
    row_ptr[i + 1] = (int)k;
  }
  return k;
}

// Block values (fp32, nnzb blocks of bR*bC).
//   dist 0: uniform[-1, 1]; dist 1: N(0,1) x 10^u per block, u ~ uniform[-3, 3];
//   dist 2: N(0,1).
void spmm_gen_values(long long nnzb, int bR, int bC, int dist, unsigned long long seed, float* out) {
  const long long per = (long long)bR * bC;
  parallel_for(nnzb, [&](long long a, long long b) {
    for (long long blk = a; blk < b; ++blk) {
      float* o = out + blk * per;
      if (dist == D_UNIFORM) {
        for (long long e = 0; e < per; ++e)
          o[e] = (float)(2.0 * u01(h2(seed, 5, (uint64_t)(blk * per + e))) - 1.0);
      } else {
        const double mag = dist == D_SCALED_NORMAL ? std::pow(10.0, 6.0 * u01(h2(seed, 6, (uint64_t)blk)) - 3.0) : 1.0;
        for (long long e = 0; e < per; ++e) o[e] = (float)(normal(seed, 7, (uint64_t)(blk * per + e)) * mag);
      }
    }
  });
}

// Dense values (fp32): dist 0 uniform[-1, 1], dist 2 N(0,1).
void spmm_gen_dense(long long count, int dist, unsigned long long seed, float* out) {
  parallel_for(count, [&](long long a, long long b) {
    for (long long i = a; i < b; ++i)
      out[i] = dist == D_UNIFORM ? (float)(2.0 * u01(h2(seed, 8, (uint64_t)i)) - 1.0)
                                 : (float)normal(seed, 9, (uint64_t)i);
  });
}

}  // extern "C"
