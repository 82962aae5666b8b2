// Seeded synthetic inputs generated on the GPU.
//
// The same counter-based streams as the host generators (csrc/host/generator.cpp:
// a SplitMix64 hash of (seed, stream, index)), evaluated in parallel:
//   * structures: random, band and block-diagonal are bit-identical to
//     spmm_gen_structure (hashes and exactly rounded double arithmetic only);
//     log-normal draws its row counts through log / exp / cos, whose device
//     implementations may differ from the host's in the last bit, so a count
//     can differ by one where it rounds at .5 -- same distribution, not the
//     same bits;
//   * values: uniform values are bit-identical to spmm_gen_values /
//     spmm_gen_dense, normal ones follow the same Box-Muller transform;
//   * dense matrices in the reference generator's patterns
//     (matrix_generator.cpp:28-140: random, checkerboard, diagonal,
//     blockdiagonal, blockrandom, pattern64by16, pattern32by16) with the
//     counter-based stream instead of the reference's sequential mt19937: the
//     same shapes and distributions, not the reference's bits (the host
//     mg::generate_matrix is the bit-identical one).
#include <cuda_fp16.h>
#include <cstring>
#include <string>
#include "internal.h"

namespace spmm {
namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}
__device__ __forceinline__ uint64_t h2(uint64_t seed, uint64_t stream, uint64_t i) {
  return mix64(mix64(seed * 0x2545f4914f6cdd1dull + stream) ^ i);
}
__device__ __forceinline__ double u01(uint64_t h) { return __dmul_rn((double)(h >> 11), 1.0 / 9007199254740992.0); }
__device__ __forceinline__ double normal(uint64_t seed, uint64_t stream, uint64_t i) {   // Box-Muller
  double a = u01(h2(seed, stream, 2 * i)), b = u01(h2(seed, stream, 2 * i + 1));
  if (a < 1e-300) a = 1e-300;
  return sqrt(-2.0 * log(a)) * cos(6.283185307179586 * b);
}

constexpr int kRowsPerCta = 8;           // one warp per block row
constexpr int kMaxKB = 16384;            // log-normal rows keep a bitmap of KB bits in shared memory (<= 16 KB per CTA)

// Whether block (i, j) is part of the structure (random, band, blockdiag).
__device__ __forceinline__ bool keep(int pattern, int i, int j, int KB, int bR, double density, double param,
                                     uint64_t seed) {
  if (pattern == 0) return u01(h2(seed, 1, (uint64_t)i * KB + j)) < density;
  if (pattern == 1) {
    const int w = (int)param;
    const int lo = max(0, (int)((long long)i * bR / 16) - w);
    const int hi = min(KB - 1, (int)(((long long)(i + 1) * bR - 1) / 16) + w);
    if (j < lo || j > hi) return false;
    const double avg_len = __dadd_rn(2.0 * w, (double)bR / 16.0);
    const double q = fmin(1.0, __ddiv_rn(__dmul_rn(density, (double)KB), avg_len));
    return q >= 1.0 || u01(h2(seed, 2, (uint64_t)i * KB + j)) < q;
  }
  const long long T = (long long)param;
  return ((long long)i * bR) / T == ((long long)j * 16) / T;
}

// Log-normal rows: the row's count, then Floyd's sampling into a bitmap (lane 0).
__device__ int lognormal_row(int i, int KB, double density, double param, uint64_t seed, uint32_t* bits, int lane) {
  for (int w = lane; w < (KB + 31) / 32; w += 32) bits[w] = 0;
  __syncwarp();
  int cnt = 0;
  if (lane == 0) {
    const double sigma2 = log(1.0 + param * param);
    const double mean = density * KB;
    const double mu = log(fmax(mean, 1e-9)) - 0.5 * sigma2;
    long long c = llround(exp(mu + sqrt(sigma2) * normal(seed, 3, (uint64_t)i)));
    c = max(0LL, min(c, (long long)KB));
    uint64_t ctr = 0;
    for (long long j = KB - c; j < KB; ++j) {
      const long long t = (long long)__dmul_rn(u01(h2(seed, 4, ((uint64_t)i << 32) + ctr++)), (double)(j + 1));
      const int pick = ((bits[t >> 5] >> (t & 31)) & 1u) ? (int)j : (int)t;
      bits[pick >> 5] |= 1u << (pick & 31);
    }
    cnt = (int)c;
  }
  __syncwarp();
  return __shfl_sync(0xffffffffu, cnt, 0);
}

// FILL = false: counts[i] = blocks in block row i. FILL = true: col_idx from row_ptr[i].
template <bool FILL>
__global__ void k_gen_structure(int MB, int KB, int bR, int pattern, double density, double param, uint64_t seed,
                                int* counts, const int* row_ptr, int* col_idx) {
  extern __shared__ uint32_t bitmaps[];   // log-normal only: kRowsPerCta x ceil(KB / 32)
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * kRowsPerCta + warp;
  if (i >= MB) return;
  const int words = (KB + 31) / 32;
  if (pattern == 3) {
    uint32_t* bits = bitmaps + warp * words;
    const int cnt = lognormal_row(i, KB, density, param, seed, bits, lane);
    if (!FILL) {
      if (lane == 0) counts[i] = cnt;
      return;
    }
    int pos = row_ptr[i];
    for (int w0 = 0; w0 < words; w0 += 32) {
      const uint32_t word = (w0 + lane < words) ? bits[w0 + lane] : 0u;
      int n = __popc(word), incl = n;
      for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
      }
      int p = pos + incl - n;
      for (uint32_t b = word; b; b &= b - 1) col_idx[p++] = (w0 + lane) * 32 + __ffs(b) - 1;
      pos += __shfl_sync(0xffffffffu, incl, 31);
    }
    return;
  }
  int pos = FILL ? row_ptr[i] : 0;
  for (int j0 = 0; j0 < KB; j0 += 32) {
    const int j = j0 + lane;
    const bool k = j < KB && keep(pattern, i, j, KB, bR, density, param, seed);
    const uint32_t bal = __ballot_sync(0xffffffffu, k);
    if (FILL && k) col_idx[pos + __popc(bal & ((1u << lane) - 1u))] = j;
    pos += __popc(bal);
  }
  if (!FILL && lane == 0) counts[i] = pos;
}

__global__ void k_gen_values(long long nnzb, int per, int dist, uint64_t seed, float* out) {
  const long long n = nnzb * per;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    if (dist == 0) {
      out[e] = (float)(2.0 * u01(h2(seed, 5, (uint64_t)e)) - 1.0);
    } else {
      const long long blk = e / per;
      const double mag = dist == 1 ? pow(10.0, 6.0 * u01(h2(seed, 6, (uint64_t)blk)) - 3.0) : 1.0;
      out[e] = (float)(normal(seed, 7, (uint64_t)e) * mag);
    }
  }
}

__global__ void k_gen_dense(long long count, int dist, uint64_t seed, float* out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = dist == 0 ? (float)(2.0 * u01(h2(seed, 8, (uint64_t)i)) - 1.0) : (float)normal(seed, 9, (uint64_t)i);
}

// The reference generator's patterns (dense, fp16). Every element decides
// from hashes of its block and itself, so any order of evaluation gives the
// same matrix.
__global__ void k_gen_matrix(int rows, int cols, double sparsity, int pat, int bs, uint64_t seed, __half* out) {
  const long long n = (long long)rows * cols;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e / cols), c = (int)(e % cols);
    bool on = false;
    switch (pat) {
      case 0: on = u01(h2(seed, 20, (uint64_t)e)) < 1.0 - sparsity; break;                          // random
      case 1: on = (((r / bs) % 2) ^ ((c / bs) % 2)) == 0; break;                                     // checkerboard
      case 2: on = r == c; break;                                                                    // diagonal
      case 3: on = r / bs == c / bs; break;                                                          // blockdiagonal
      case 4: {                                                                                      // blockrandom
        const long long nbj = (cols + bs - 1) / bs;
        on = u01(h2(seed, 21, (uint64_t)((r / bs) * nbj + c / bs))) < 1.0 - sparsity;
        break;
      }
      default: {                                                                                     // 64x16 / 32x16
        const int brow = pat == 5 ? 64 : 32;
        const long long nbj = (cols + 15) / 16;
        on = u01(h2(seed, 22, (uint64_t)((r / brow) * nbj + c / 16))) < 1.0 - sparsity;
      }
    }
    out[e] = __float2half(on ? (float)(2.0 * u01(h2(seed, 23, (uint64_t)e)) - 1.0) : 0.f);
  }
}

unsigned gen_grid(long long n) {
  long long g = (n + 255) / 256;
  const long long cap = (long long)sm_count() * 16;
  return (unsigned)(g < 1 ? 1 : g > cap ? cap : g);
}

}  // namespace
}  // namespace spmm

using namespace spmm;

extern "C" {

spmm_status spmm_gpu_gen_structure(int M, int K, int bR, int pattern, double density, double param,
                                   unsigned long long seed, int* row_ptr, int* col_idx, long long capacity,
                                   long long* nnzb_out, void* stream) {
  if (!row_ptr || !nnzb_out || bR <= 0 || M < 0 || K < 0 || M % bR || K % 16 || pattern < 0 || pattern > 3 ||
      (pattern == 2 && param < 1) || (pattern == 1 && param < 0))
    return fail(SPMM_ERR_INVALID_ARG, "bad structure arguments");
  const int MB = M / bR, KB = K / 16;
  if (pattern == 3 && KB > kMaxKB) return fail(SPMM_ERR_UNSUPPORTED, "log-normal rows need K <= 262144");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int* counts = nullptr;
  SPMM_CUDA_TRY(cudaMallocAsync(&counts, sizeof(int) * (MB + 1), s));
  const size_t sm = pattern == 3 ? (size_t)kRowsPerCta * ((KB + 31) / 32) * 4 : 0;
  const unsigned g = (unsigned)((MB + kRowsPerCta - 1) / kRowsPerCta);
  if (MB > 0) k_gen_structure<false><<<g, 32 * kRowsPerCta, sm, s>>>(MB, KB, bR, pattern, density, param, seed, counts,
                                                                   nullptr, nullptr);
  SPMM_CUDA_TRY(cudaGetLastError());
  spmm_status st = scan_counts(counts, row_ptr, MB, s);
  if (st != SPMM_OK) {
    cudaFreeAsync(counts, s);
    return st;
  }
  int total = 0;
  SPMM_CUDA_TRY(cudaMemcpyAsync(&total, row_ptr + MB, sizeof(int), cudaMemcpyDeviceToHost, s));
  SPMM_CUDA_TRY(cudaStreamSynchronize(s));
  *nnzb_out = total;
  if (col_idx && capacity >= total && MB > 0) {
    k_gen_structure<true><<<g, 32 * kRowsPerCta, sm, s>>>(MB, KB, bR, pattern, density, param, seed, nullptr, row_ptr,
                                                         col_idx);
    SPMM_CUDA_TRY(cudaGetLastError());
  }
  SPMM_CUDA_TRY(cudaFreeAsync(counts, s));
  return SPMM_OK;
}

spmm_status spmm_gpu_gen_values(long long nnzb, int bR, int bC, int dist, unsigned long long seed, float* out,
                                void* stream) {
  if (nnzb < 0 || bR <= 0 || bC <= 0 || dist < 0 || dist > 2 || (nnzb && !out))
    return fail(SPMM_ERR_INVALID_ARG, "bad value arguments");
  if (!nnzb) return SPMM_OK;
  const long long n = nnzb * bR * bC;
  k_gen_values<<<gen_grid(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(nnzb, bR * bC, dist, seed, out);
  SPMM_CUDA_TRY(cudaGetLastError());
  return SPMM_OK;
}

spmm_status spmm_gpu_gen_dense(long long count, int dist, unsigned long long seed, float* out, void* stream) {
  if (count < 0 || (dist != 0 && dist != 2) || (count && !out)) return fail(SPMM_ERR_INVALID_ARG, "bad arguments");
  if (!count) return SPMM_OK;
  k_gen_dense<<<gen_grid(count), 256, 0, static_cast<cudaStream_t>(stream)>>>(count, dist, seed, out);
  SPMM_CUDA_TRY(cudaGetLastError());
  return SPMM_OK;
}

spmm_status spmm_gpu_generate_matrix(int rows, int cols, double sparsity, const char* pattern, int blocksize,
                                     unsigned long long seed, void* out_half, void* stream) {
  static const char* names[] = {"random", "checkerboard", "diagonal", "blockdiagonal", "blockrandom",
                                "pattern64by16", "pattern32by16"};
  int pat = -1;
  for (int k = 0; k < 7; ++k)
    if (pattern && std::strcmp(pattern, names[k]) == 0) pat = k;
  if (pat < 0) return fail(SPMM_ERR_INVALID_ARG, std::string("Unknown pattern: ") + (pattern ? pattern : "(null)"));
  if (rows < 0 || cols < 0 || blocksize <= 0 || (rows && cols && !out_half))
    return fail(SPMM_ERR_INVALID_ARG, "bad arguments");
  const long long n = (long long)rows * cols;
  if (!n) return SPMM_OK;
  k_gen_matrix<<<gen_grid(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(rows, cols, sparsity, pat, blocksize, seed,
                                                                          static_cast<__half*>(out_half));
  SPMM_CUDA_TRY(cudaGetLastError());
  return SPMM_OK;
}

}  // extern "C"
