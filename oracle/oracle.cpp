// CPU oracle for the BCSR SpMM path.
//
// This file is test infrastructure. It restates, on the host and in plain
// C++, the reference algorithms the GPU library must reproduce, so that the
// tests can check the library against it. Nothing in the shipped library links
// or calls it; only the tests, the smoke check and the CPU-baseline leg of the
// benchmark load it.
//
// Pinning: the generator and BCSR restatements below are checked against the
// reference's own sources built from its tree (oracle/Makefile, `make ref`),
// and against committed fixtures made from that build (tests/golden/).
//
// Reference citations are paths inside hosseinal/MatrixMultiplicationCUDA.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <thread>
#include <vector>
#include <algorithm>

namespace {

// ---------------------------------------------------------------------------
// IEEE binary16 <-> binary32, round-to-nearest-even (the semantics of the
// reference's __float2half / __half2float on the host, Matrix.cu:27-28,
// nvbench_main.cu:67-75). Written from the IEEE 754 definition.
// ---------------------------------------------------------------------------
inline uint32_t f2u(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float u2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

inline uint16_t f32_to_f16_rne(float f) {
  uint32_t x = f2u(f);
  uint32_t sign = (x >> 16) & 0x8000u;
  uint32_t absx = x & 0x7fffffffu;
  if (absx >= 0x7f800000u) {                 // inf or nan
    if (absx > 0x7f800000u) return (uint16_t)(sign | 0x7e00u | ((absx >> 13) & 0x3ffu));
    return (uint16_t)(sign | 0x7c00u);
  }
  int32_t e = (int32_t)(absx >> 23) - 127;   // unbiased exponent
  uint32_t mant = absx & 0x7fffffu;
  if (e > 15) return (uint16_t)(sign | 0x7c00u);  // overflow -> inf (RNE of huge)
  if (e >= -14) {                            // normal half range
    uint32_t m = mant | 0x800000u;           // 24-bit significand
    // keep 11 bits, shift out 13
    uint32_t keep = m >> 13, rem = m & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (keep & 1u))) keep++;
    uint32_t he = (uint32_t)(e + 15);
    if (keep == 0x800u) { keep = 0x400u; he++; }    // significand rounded up to 2.0
    if (he >= 31) return (uint16_t)(sign | 0x7c00u);
    return (uint16_t)(sign | (he << 10) | (keep & 0x3ffu));
  }
  // subnormal half: value = m * 2^(e-23); half subnormal unit = 2^-24
  if (absx == 0) return (uint16_t)sign;
  uint32_t m = (e == -127) ? (mant << 1) : (mant | 0x800000u); // float subnormal handled as tiny
  if (e == -127) e = -126;
  int shift = (-14 - e) + 13;                // bits to drop to reach 2^-24 units
  if (shift > 24) return (uint16_t)sign;     // rounds to zero (below half of 2^-24)
  uint32_t keep = m >> shift;
  uint32_t rem = m & ((1u << shift) - 1u);
  uint32_t half = 1u << (shift - 1);
  if (rem > half || (rem == half && (keep & 1u))) keep++;
  return (uint16_t)(sign | keep);            // keep may reach 0x400 -> smallest normal, still correct
}

inline float f16_to_f32(uint16_t h) {
  uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
  uint32_t e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
  if (e == 0) {
    if (m == 0) return u2f(sign);
    float v = std::ldexp((float)m, -24);
    return sign ? -v : v;
  }
  if (e == 31) return u2f(sign | 0x7f800000u | (m << 13));
  return u2f(sign | ((e + 112u) << 23) | (m << 13));
}

// ---------------------------------------------------------------------------
// Synthetic generator: restates mg::generate_dense_block / mg::generate_matrix
// for T = float (matrix_generator.cpp:10-140). The RNG stream is the one the
// reference consumes: std::mt19937(seed), std::uniform_real_distribution<double>
// and std::bernoulli_distribution, drawn in the same order.
// ---------------------------------------------------------------------------
struct Gen {
  int R, Cc, bs;
  std::mt19937 rng;
  float* out;  // row-major R x Cc, pre-zeroed
  // matrix_generator.cpp:10-26 (float branch) + the fill_block lambda :35-43
  void fill_rect(int r0, int c0, int h, int w) {
    int r1 = std::min(r0 + h, R), c1 = std::min(c0 + w, Cc);
    int rows = r1 - r0, cols = c1 - c0;
    if (rows <= 0 || cols <= 0) {
      // generate_dense_block with a non-positive extent draws nothing
      return;
    }
    std::uniform_real_distribution<double> dist(-1.0, 1.0);
    for (int i = 0; i < rows; ++i)
      for (int j = 0; j < cols; ++j)
        out[(size_t)(r0 + i) * Cc + (c0 + j)] = (float)dist(rng);
  }
};

}  // namespace

extern "C" {

int oracle_abi_version() { return 1; }

void oracle_f32_to_f16(const float* in, uint16_t* out, size_t n) {
  for (size_t i = 0; i < n; ++i) out[i] = f32_to_f16_rne(in[i]);
}
void oracle_f16_to_f32(const uint16_t* in, float* out, size_t n) {
  for (size_t i = 0; i < n; ++i) out[i] = f16_to_f32(in[i]);
}

// Restates mg::generate_matrix<float> (matrix_generator.cpp:28-140).
// out: rows*cols floats (written fully). Returns 0, or -1 for an unknown
// pattern (the reference throws std::invalid_argument, :136).
int oracle_generate_matrix(int num_rows, int num_cols, double sparsity,
                           const char* pattern, int blocksize, unsigned seed,
                           float* out) {
  std::memset(out, 0, sizeof(float) * (size_t)num_rows * num_cols);
  Gen g{num_rows, num_cols, blocksize, std::mt19937(seed), out};
  std::string p(pattern);
  if (p == "random") {                                   // :49-66
    std::bernoulli_distribution keep(1.0 - sparsity);
    for (int i = 0; i < num_rows; ++i)
      for (int j = 0; j < num_cols; ++j) {
        if (keep(g.rng)) {
          std::uniform_real_distribution<double> d(-1.0, 1.0);
          out[(size_t)i * num_cols + j] = (float)d(g.rng);
        }
      }
  } else if (p == "checkerboard") {                       // :68-74
    int nbi = (num_rows + blocksize - 1) / blocksize;
    int nbj = (num_cols + blocksize - 1) / blocksize;
    for (int i = 0; i < nbi; ++i)
      for (int j = 0; j < nbj; ++j)
        if (((i % 2) ^ (j % 2)) == 0) g.fill_rect(i * blocksize, j * blocksize, blocksize, blocksize);
  } else if (p == "diagonal") {                           // :76-81
    int minrc = std::min(num_rows, num_cols);
    for (int i = 0; i < minrc; ++i) g.fill_rect(i, i, 1, 1);
  } else if (p == "blockdiagonal") {                      // :83-85
    int n = std::min(num_rows, num_cols) / blocksize + 1;
    for (int i = 0; i < n; ++i) g.fill_rect(i * blocksize, i * blocksize, blocksize, blocksize);
  } else if (p == "blockrandom") {                        // :87-93
    int nbi = (num_rows + blocksize - 1) / blocksize;
    int nbj = (num_cols + blocksize - 1) / blocksize;
    std::bernoulli_distribution keep(1.0 - sparsity);
    for (int i = 0; i < nbi; ++i)
      for (int j = 0; j < nbj; ++j)
        if (keep(g.rng)) g.fill_rect(i * blocksize, j * blocksize, blocksize, blocksize);
  } else if (p == "pattern64by16" || p == "pattern32by16") {  // :95-134
    const int brow = (p == "pattern64by16") ? 64 : 32, bcol = 16;
    int nbi = (num_rows + brow - 1) / brow;
    int nbj = (num_cols + bcol - 1) / bcol;
    std::bernoulli_distribution keep(1.0 - sparsity);
    for (int bi = 0; bi < nbi; ++bi)
      for (int bj = 0; bj < nbj; ++bj) {
        if (!keep(g.rng)) continue;
        g.fill_rect(bi * brow, bj * bcol, brow, bcol);
      }
  } else {
    return -1;
  }
  return 0;
}

// blockDensity(...) > 0 test of miscutil.cpp:76-87: an element counts when its
// half value converts to a float that compares != 0 (so -0 is zero, NaN is not).
static inline bool half_nonzero(uint16_t h) { return f16_to_f32(h) != 0.0f; }

// Pass 1 of the BCSRMatrix constructor (formats/BCSRMatrix.cu:36-49):
// hdr[MB+1] prefix count of nonzero blocks per block row. Returns nnzb, or -1
// for block sizes the constructor rejects (:24-34).
long long oracle_bcsr_count(const uint16_t* A, int rows, int cols, int bR, int bC, int* hdr) {
  if (bR < 16 || bC < 16 || bR % 16 || bC % 16) return -1;
  int MB = rows / bR, KB = cols / bC;
  hdr[0] = 0;
  for (int br = 0; br < MB; ++br) {
    hdr[br + 1] = hdr[br];
    for (int bc = 0; bc < KB; ++bc) {
      bool nz = false;
      for (int x = 0; x < bR && !nz; ++x)
        for (int y = 0; y < bC; ++y)
          if (half_nonzero(A[(size_t)(br * bR + x) * cols + bc * bC + y])) { nz = true; break; }
      if (nz) hdr[br + 1]++;
    }
  }
  return hdr[MB];
}

// Pass 2 (formats/BCSRMatrix.cu:55-71): idx = block column, data = the block's
// bR x bC values row-major, blocks in row-major block order.
void oracle_bcsr_fill(const uint16_t* A, int rows, int cols, int bR, int bC,
                      int* idx, uint16_t* data) {
  int MB = rows / bR, KB = cols / bC;
  long long k = 0;
  for (int br = 0; br < MB; ++br)
    for (int bc = 0; bc < KB; ++bc) {
      bool nz = false;
      for (int x = 0; x < bR && !nz; ++x)
        for (int y = 0; y < bC; ++y)
          if (half_nonzero(A[(size_t)(br * bR + x) * cols + bc * bC + y])) { nz = true; break; }
      if (!nz) continue;
      idx[k] = bc;
      for (int x = 0; x < bR; ++x)
        for (int y = 0; y < bC; ++y)
          data[(size_t)k * bR * bC + x * bC + y] = A[(size_t)(br * bR + x) * cols + bc * bC + y];
      ++k;
    }
}

// cpu_matmul_ref (nvbench_main.cu:78-91): dense i-k-j, FP32 accumulation,
// half -> float per element, zeros multiplied too. Rows [row0, row1) only, so a
// caller can time or check a bounded sample. Compiled with -ffp-contract=off so
// the product and the add round separately, as on the x86 hosts the reference ran on.
void oracle_cpu_matmul_ref_rows(const uint16_t* A, const uint16_t* B, int M, int K, int N,
                                int row0, int row1, float* C) {
  (void)M;
  std::vector<float> brow((size_t)N);
  for (int i = row0; i < row1; ++i) {
    float* c = C + (size_t)(i - row0) * N;
    for (int j = 0; j < N; ++j) c[j] = 0.0f;
    for (int k = 0; k < K; ++k) {
      float a = f16_to_f32(A[(size_t)i * K + k]);
      const uint16_t* b = B + (size_t)k * N;
      for (int j = 0; j < N; ++j) c[j] += a * f16_to_f32(b[j]);
    }
  }
}

// Same computation over [row0,row1) split across nthreads host threads, each
// thread running the reference loop on its own rows (the loop order inside a
// row is unchanged, so results are identical to the single-thread version).
void oracle_cpu_matmul_ref_rows_mt(const uint16_t* A, const uint16_t* B, int M, int K, int N,
                                   int row0, int row1, float* C, int nthreads) {
  if (nthreads <= 1) { oracle_cpu_matmul_ref_rows(A, B, M, K, N, row0, row1, C); return; }
  std::vector<std::thread> th;
  int rows = row1 - row0;
  for (int t = 0; t < nthreads; ++t) {
    int a = row0 + (int)((long long)rows * t / nthreads);
    int b = row0 + (int)((long long)rows * (t + 1) / nthreads);
    if (a >= b) continue;
    th.emplace_back([=] { oracle_cpu_matmul_ref_rows(A, B, M, K, N, a, b, C + (size_t)(a - row0) * N); });
  }
  for (auto& x : th) x.join();
}

// Block-sparse host multiply, a CPU baseline only (not a reference algorithm):
// C = A (BCSR, fp16 bits) x B (fp32, K x N), fp32 accumulation, over block rows
// [br0, br1), split across nthreads threads by block row. Each stored block
// adds a * B[k][:] into its rows, so only the stored blocks' MACs are done.
// C holds (br1 - br0) * bR rows of N.
void oracle_bcsr_matmul_f32_mt(const int* row_ptr, const int* col_idx, const uint16_t* vals, int bR,
                               const float* B, int K, int N, int br0, int br1, float* C, int nthreads) {
  (void)K;
  auto rows = [&](int a0, int a1) {
    for (int br = a0; br < a1; ++br) {
      float* c = C + (size_t)(br - br0) * bR * N;
      std::fill(c, c + (size_t)bR * N, 0.0f);
      for (int k = row_ptr[br]; k < row_ptr[br + 1]; ++k) {
        const uint16_t* a = vals + (size_t)k * bR * 16;
        const float* b = B + (size_t)col_idx[k] * 16 * N;
        for (int x = 0; x < bR; ++x) {
          float* crow = c + (size_t)x * N;
          for (int y = 0; y < 16; ++y) {
            const float av = f16_to_f32(a[x * 16 + y]);
            if (av == 0.0f) continue;
            const float* brow = b + (size_t)y * N;
            for (int j = 0; j < N; ++j) crow[j] += av * brow[j];
          }
        }
      }
    }
  };
  if (nthreads <= 1) {
    rows(br0, br1);
    return;
  }
  std::vector<std::thread> th;
  const int n = br1 - br0;
  for (int t = 0; t < nthreads; ++t) {
    const int a = br0 + (int)((long long)n * t / nthreads), b = br0 + (int)((long long)n * (t + 1) / nthreads);
    if (a < b) th.emplace_back(rows, a, b);
  }
  for (auto& x : th) x.join();
}

// FP64 BCSR x dense product, the error reference for every precision.
// A is given by its BCSR structure and block values in double (the exact
// values before any storage rounding), B as double, row-major ld = N.
// Writes C (M x N double) for block rows [br0, br1).
void oracle_bcsr_matmul_f64(const int* row_ptr, const int* col_idx, const double* vals,
                            int bR, int bC, const double* B, int N, int br0, int br1,
                            double* C) {
  for (int br = br0; br < br1; ++br) {
    double* c = C + (size_t)(br - br0) * bR * N;
    std::fill(c, c + (size_t)bR * N, 0.0);
    for (int k = row_ptr[br]; k < row_ptr[br + 1]; ++k) {
      const double* a = vals + (size_t)k * bR * bC;
      const double* b = B + (size_t)col_idx[k] * bC * N;
      for (int x = 0; x < bR; ++x)
        for (int y = 0; y < bC; ++y) {
          double av = a[x * bC + y];
          if (av == 0.0) continue;
          const double* brow = b + (size_t)y * N;
          double* crow = c + (size_t)x * N;
          for (int j = 0; j < N; ++j) crow[j] += av * brow[j];
        }
    }
  }
}

// The same product split by block rows over nthreads host threads (each block
// row's arithmetic is unchanged, so the result equals the one-thread call).
void oracle_bcsr_matmul_f64_mt(const int* row_ptr, const int* col_idx, const double* vals,
                               int bR, int bC, const double* B, int N, int br0, int br1,
                               double* C, int nthreads) {
  if (nthreads <= 1) {
    oracle_bcsr_matmul_f64(row_ptr, col_idx, vals, bR, bC, B, N, br0, br1, C);
    return;
  }
  std::vector<std::thread> th;
  const int n = br1 - br0;
  for (int t = 0; t < nthreads; ++t) {
    const int a = br0 + (int)((long long)n * t / nthreads), b = br0 + (int)((long long)n * (t + 1) / nthreads);
    if (a < b)
      th.emplace_back([=] {
        oracle_bcsr_matmul_f64(row_ptr, col_idx, vals, bR, bC, B, N, a, b, C + (size_t)(a - br0) * bR * N);
      });
  }
  for (auto& x : th) x.join();
}

// ---------------------------------------------------------------------------
// The synthetic workloads' generators, restated so that a run of the
// reference's host multiply can build its inputs without the library. The
// library's definition (bcsr_spmm_host.h, spmm_gen_structure / _values /
// _dense): every random number is a stateless hash of (seed, stream, index)
// -- the SplitMix64 finaliser applied twice -- so any block or element can be
// drawn on its own. Uniform draws take the hash's top 53 bits; normal draws
// are Box-Muller over two uniform draws 2i and 2i + 1. The tests check these
// bit for bit against the library's host generators.
// ---------------------------------------------------------------------------
namespace {
uint64_t splitmix_final(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
double draw_u01(uint64_t seed, uint64_t stream, uint64_t index) {
  const uint64_t key = splitmix_final(seed * 0x2545f4914f6cdd1dull + stream);
  return (double)(splitmix_final(key ^ index) >> 11) / 9007199254740992.0;
}
double draw_normal(uint64_t seed, uint64_t stream, uint64_t index) {
  const double u1 = std::max(draw_u01(seed, stream, 2 * index), 1e-300);
  const double u2 = draw_u01(seed, stream, 2 * index + 1);
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}
}  // namespace

// Block structure (row_ptr[M/bR + 1], col_idx up to (M/bR)*(K/16) entries).
// pattern 0: each block independently kept with probability `density`;
// 1: a band of `param` block columns either side of the block row's diagonal
//    span, each kept with probability min(1, density*KB / (2*param + bR/16));
// 2: dense square diagonal tiles of `param` elements;
// 3: per-row counts round(exp(mu + sigma z)) (log-normal with mean density*KB
//    and coefficient of variation `param`, clipped to [0, KB]) of distinct
//    columns drawn by Floyd's method.
// Returns nnzb, or -1 for bad sizes or an unknown pattern.
long long oracle_gen_structure(int M, int K, int bR, int pattern, double density, double param,
                               unsigned long long seed, int* row_ptr, int* col_idx) {
  if (bR <= 0 || M % bR != 0 || K % 16 != 0 || pattern < 0 || pattern > 3) return -1;
  const int rows = M / bR, kb = K / 16;
  long long nnz = 0;
  row_ptr[0] = 0;
  std::vector<char> taken;
  for (int r = 0; r < rows; ++r) {
    switch (pattern) {
      case 0:
        for (int c = 0; c < kb; ++c)
          if (draw_u01(seed, 1, (uint64_t)r * kb + c) < density) col_idx[nnz++] = c;
        break;
      case 1: {
        const int half = (int)param;
        const int first = std::max(0, (int)((long long)r * bR / 16) - half);
        const int last = std::min(kb - 1, (int)(((long long)r * bR + bR - 1) / 16) + half);
        const double keep = std::min(1.0, density * kb / (2.0 * half + bR / 16.0));
        for (int c = first; c <= last; ++c)
          if (keep >= 1.0 || draw_u01(seed, 2, (uint64_t)r * kb + c) < keep) col_idx[nnz++] = c;
        break;
      }
      case 2: {
        const long long tile = (long long)param;
        const long long t = (long long)r * bR / tile;
        for (int c = 0; c < kb; ++c)
          if ((long long)c * 16 / tile == t) col_idx[nnz++] = c;
        break;
      }
      default: {
        const double s2 = std::log(1.0 + param * param);
        const double mu = std::log(std::max(density * kb, 1e-9)) - 0.5 * s2;
        long long count = std::llround(std::exp(mu + std::sqrt(s2) * draw_normal(seed, 3, (uint64_t)r)));
        count = std::min<long long>(std::max(count, 0LL), kb);
        taken.assign(kb, 0);
        uint64_t n = 0;
        for (long long top = kb - count; top < kb; ++top) {
          const long long pick = (long long)(draw_u01(seed, 4, ((uint64_t)r << 32) + n++) * (double)(top + 1));
          taken[taken[pick] ? top : pick] = 1;
        }
        for (int c = 0; c < kb; ++c)
          if (taken[c]) col_idx[nnz++] = c;
      }
    }
    row_ptr[r + 1] = (int)nnz;
  }
  return nnz;
}

// Block values, nnzb blocks of bR*bC fp32. dist 0: uniform[-1, 1] (stream 5);
// dist 1: N(0,1) (stream 7) times 10^(6u - 3) per block (u from stream 6);
// dist 2: N(0,1).
void oracle_gen_values(long long nnzb, int bR, int bC, int dist, unsigned long long seed, float* out) {
  const long long per = (long long)bR * bC;
  for (long long b = 0; b < nnzb; ++b) {
    const double scale = dist == 1 ? std::pow(10.0, 6.0 * draw_u01(seed, 6, (uint64_t)b) - 3.0) : 1.0;
    for (long long e = 0; e < per; ++e) {
      const uint64_t i = (uint64_t)(b * per + e);
      out[b * per + e] = dist == 0 ? (float)(2.0 * draw_u01(seed, 5, i) - 1.0)
                                   : (float)(draw_normal(seed, 7, i) * scale);
    }
  }
}

// Dense values: dist 0 uniform[-1, 1] (stream 8), otherwise N(0,1) (stream 9).
void oracle_gen_dense(long long count, int dist, unsigned long long seed, float* out) {
  for (long long i = 0; i < count; ++i)
    out[i] = dist == 0 ? (float)(2.0 * draw_u01(seed, 8, (uint64_t)i) - 1.0) : (float)draw_normal(seed, 9, (uint64_t)i);
}

// maxdiff / avgrelerr / rmse of miscutil.cpp:35-74, generalised from n x n to a
// flat array of `count` entries (A = result under test, B = reference).
float oracle_maxdiff(const float* A, const float* B, size_t count) {
  float m = 0.0f;
  for (size_t i = 0; i < count; ++i) m = std::max(m, std::fabs(A[i] - B[i]));
  return m;
}
float oracle_avgrelerr(const float* A, const float* B, size_t count) {
  double s = 0.0;
  for (size_t i = 0; i < count; ++i) {
    double den = std::fabs((double)B[i]), num = std::fabs((double)A[i] - (double)B[i]);
    s += den > 1e-12 ? num / den : num;
  }
  return (float)(s / (double)count);
}
double oracle_rmse(const float* A, const float* B, size_t count) {
  double s = 0.0;
  for (size_t i = 0; i < count; ++i) { double d = (double)A[i] - (double)B[i]; s += d * d; }
  return std::sqrt(s / (double)count);
}
// Normwise errors against an FP64 reference: out[0] = max|A-R| / max|R|,
// out[1] = ||A-R||_F / ||R||_F.
void oracle_rel_errors(const float* A, const double* R, size_t count, double* out) {
  double md = 0, mr = 0, sd = 0, sr = 0;
  for (size_t i = 0; i < count; ++i) {
    double d = std::fabs((double)A[i] - R[i]);
    md = std::max(md, d); mr = std::max(mr, std::fabs(R[i]));
    sd += d * d; sr += R[i] * R[i];
  }
  out[0] = mr > 0 ? md / mr : md;
  out[1] = sr > 0 ? std::sqrt(sd / sr) : std::sqrt(sd);
}

}  // extern "C"
