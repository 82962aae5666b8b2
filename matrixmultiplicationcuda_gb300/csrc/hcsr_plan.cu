// The planned hybrid product: the CSR part of an HCSR matrix packed once into
// "gather blocks", which the tcgen05 pipeline runs on the tensor cores.
//
// A gather block holds up to 16 CSR entries of one 16-row block row, in the
// CSR's order. Entry c (0..15) with row r and value v becomes column c of a
// 16 x 16 fp16 block whose only nonzero in that column is v at row r, and the
// block's B panel row c is B's row k (the entry's column). So
//     block x panel = sum over the 16 entries of v * B[k][:] in row r,
// exactly the CSR terms, in one UMMA per 128 output columns. The panel rows
// are fetched with TMA tile::gather4 (four B rows per copy); unused slots of a
// block row's last gather block have value 0 and row index K, which lies past
// the end of B and reads zeros, so they add exact zeros.
//
// The packed matrix is one BCSR matrix with 16 x 16 blocks: per block row, its
// stored blocks (copied from the BCSR part) followed by its gather blocks,
// marked by col_idx = -(g + 1) for the g-th gather block overall; the B-row
// indices sit in gather_rows[16 g .. 16 g + 15].
//
// The reference computes the same product with three launches and a second C
// (main.cu:567-590: the scalar CSR kernel, the BCSR WMMA kernel, addMatrices).
#include <cuda_fp16.h>
#include <cstring>
#include <string>
#include "internal.h"

struct spmm_hcsr_plan {
  int M = 0, K = 0;
  long long blocks = 0;          // stored + gather blocks
  long long gather_blocks = 0;
  int* row_ptr = nullptr;        // M / 16 + 1
  int* col_idx = nullptr;        // blocks
  __half* vals = nullptr;        // blocks x 256
  int* gather_rows = nullptr;    // gather_blocks x 16
  int* counts = nullptr;         // scratch: 2 x (M / 16)
  int* gptr = nullptr;           // M / 16 + 1: gather blocks before each block row
};

namespace spmm {
namespace {

constexpr int kFillThreads = 128;

// Per block row: blocks of the packed matrix (stored + gather) and gather blocks.
__global__ void k_hcsr_count(const int* __restrict__ brow_ptr, const int* __restrict__ crow_ptr, int MB,
                             int* __restrict__ total, int* __restrict__ gathers) {
  const int br = blockIdx.x * blockDim.x + threadIdx.x;
  if (br >= MB) return;
  const int entries = __ldg(crow_ptr + 16 * br + 16) - __ldg(crow_ptr + 16 * br);
  const int g = (entries + 15) / 16;
  gathers[br] = g;
  total[br] = __ldg(brow_ptr + br + 1) - __ldg(brow_ptr + br) + g;
}

// One CTA per block row: copies its stored blocks, then builds its gather blocks.
__global__ void __launch_bounds__(kFillThreads)
    k_hcsr_fill(const int* __restrict__ brow_ptr, const int* __restrict__ bcol_idx, const uint4* __restrict__ bvals,
                const int* __restrict__ crow_ptr, const int* __restrict__ ccol_idx, const __half* __restrict__ cvals,
                const int* __restrict__ row_ptr, const int* __restrict__ gptr, int K, int* __restrict__ col_idx,
                uint4* __restrict__ vals, int* __restrict__ gather_rows) {
  __shared__ int bnd[17];   // CSR row bounds of the block row's 16 rows
  const int br = blockIdx.x, t = threadIdx.x;
  if (t < 17) bnd[t] = __ldg(crow_ptr + 16 * br + t);
  __syncthreads();
  const long long base = __ldg(row_ptr + br);
  const int b0 = __ldg(brow_ptr + br), nb = __ldg(brow_ptr + br + 1) - b0;
  // stored blocks: 32 x 16 bytes each
  for (int i = t; i < nb * 32; i += kFillThreads) {
    const int j = i >> 5, w = i & 31;
    vals[(base + j) * 32 + w] = __ldg(bvals + (long long)(b0 + j) * 32 + w);
    if (w == 0) col_idx[base + j] = __ldg(bcol_idx + b0 + j);
  }
  // gather blocks: thread (gi, r) writes row r of block gi and its B-row index r
  const long long g0 = __ldg(gptr + br);
  const int ng = __ldg(gptr + br + 1) - (int)g0;
  const int E0 = bnd[0], E1 = bnd[16];
  for (int i = t; i < ng * 16; i += kFillThreads) {
    const int gi = i >> 4, r = i & 15;
    const long long g = g0 + gi, pos = base + nb + gi;
    const int eb = E0 + 16 * gi;
    gather_rows[16 * g + r] = eb + r < E1 ? __ldg(ccol_idx + eb + r) : K;
    if (r == 0) col_idx[pos] = (int)(-g - 1);
    __align__(16) __half row[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      const int e = eb + c;
      __half v = __float2half(0.f);
      if (e < E1) {
        int rr = 0;   // the entry's row: bnd[rr] <= e < bnd[rr + 1]
#pragma unroll
        for (int q = 1; q < 16; ++q) rr += bnd[q] <= e ? 1 : 0;
        if (rr == r) v = cvals[e];
      }
      row[c] = v;
    }
    uint4* dst = vals + pos * 32 + r * 2;
    dst[0] = reinterpret_cast<const uint4*>(row)[0];
    dst[1] = reinterpret_cast<const uint4*>(row)[1];
  }
}

void plan_free(spmm_hcsr_plan* p) {
  if (!p) return;
  cudaFree(p->row_ptr);
  cudaFree(p->col_idx);
  cudaFree(p->vals);
  cudaFree(p->gather_rows);
  cudaFree(p->counts);
  cudaFree(p->gptr);
  delete p;
}

bool aligned16(const void* q) { return (reinterpret_cast<uintptr_t>(q) & 15u) == 0; }

}  // namespace
}  // namespace spmm

using namespace spmm;

extern "C" spmm_status spmm_hcsr_plan_create(const spmm_bcsr_desc* A, const spmm_csr_desc* R, void* stream,
                                             spmm_hcsr_plan** out) {
  if (!out) return fail(SPMM_ERR_INVALID_ARG, "null output");
  *out = nullptr;
  if (!A || !R) return fail(SPMM_ERR_INVALID_ARG, "null descriptor");
  if (A->dtype != SPMM_F16) return fail(SPMM_ERR_UNSUPPORTED, "the hybrid product is fp16");
  if (A->bR != 16 || A->bC != 16) return fail(SPMM_ERR_UNSUPPORTED, "the hybrid product has 16x16 blocks");
  if (A->M < 0 || A->K < 0) return fail(SPMM_ERR_INVALID_ARG, "negative size");
  if (A->M % 16 || A->K % 16) return fail(SPMM_ERR_INVALID_ARG, "M / K not multiples of 16");
  if (R->M != A->M || R->K != A->K) return fail(SPMM_ERR_INVALID_ARG, "the two parts must have the same shape");
  if (A->M > 0 && (!A->row_ptr || !R->row_ptr)) return fail(SPMM_ERR_INVALID_ARG, "null row_ptr");
  if (A->vals && !aligned16(A->vals)) return fail(SPMM_ERR_MISALIGNED, "A values must be 16-byte aligned");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  spmm_hcsr_plan* p = new spmm_hcsr_plan;
  p->M = A->M;
  p->K = A->K;
  const int MB = A->M / 16;
  auto bail = [&](spmm_status st) {
    plan_free(p);
    return st;
  };
  if (cudaMalloc(&p->row_ptr, sizeof(int) * (MB + 1)) != cudaSuccess ||
      cudaMalloc(&p->gptr, sizeof(int) * (MB + 1)) != cudaSuccess ||
      cudaMalloc(&p->counts, sizeof(int) * 2 * (MB > 0 ? MB : 1)) != cudaSuccess)
    return bail(fail(SPMM_ERR_CUDA, "plan allocation failed"));
  if (MB == 0) {
    if (cudaMemsetAsync(p->row_ptr, 0, sizeof(int), s) != cudaSuccess ||
        cudaMemsetAsync(p->gptr, 0, sizeof(int), s) != cudaSuccess)
      return bail(fail(SPMM_ERR_CUDA, "plan set-up failed"));
    *out = p;
    return SPMM_OK;
  }
  k_hcsr_count<<<(MB + 255) / 256, 256, 0, s>>>(A->row_ptr, R->row_ptr, MB, p->counts, p->counts + MB);
  spmm_status st = scan_counts(p->counts, p->row_ptr, MB, s);
  if (st == SPMM_OK) st = scan_counts(p->counts + MB, p->gptr, MB, s);
  if (st != SPMM_OK) return bail(st);
  int tot[2] = {0, 0};
  if (cudaMemcpyAsync(&tot[0], p->row_ptr + MB, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(&tot[1], p->gptr + MB, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return bail(fail(SPMM_ERR_CUDA, std::string("plan count pass: ") + cudaGetErrorString(cudaGetLastError())));
  p->blocks = tot[0];
  p->gather_blocks = tot[1];
  if (p->blocks < 0 || p->gather_blocks < 0 || p->gather_blocks * 16 >= (1ll << 31))
    return bail(fail(SPMM_ERR_UNSUPPORTED, "hybrid matrix too large"));
  const size_t nb = (size_t)(p->blocks > 0 ? p->blocks : 1), ng = (size_t)(p->gather_blocks > 0 ? p->gather_blocks : 1);
  if (cudaMalloc(&p->col_idx, sizeof(int) * nb) != cudaSuccess ||
      cudaMalloc(&p->vals, sizeof(__half) * 256 * nb) != cudaSuccess ||
      cudaMalloc(&p->gather_rows, sizeof(int) * 16 * ng) != cudaSuccess)
    return bail(fail(SPMM_ERR_CUDA, "plan allocation failed"));
  k_hcsr_fill<<<MB, kFillThreads, 0, s>>>(A->row_ptr, A->col_idx, static_cast<const uint4*>(A->vals), R->row_ptr,
                                          R->col_idx, static_cast<const __half*>(R->vals), p->row_ptr, p->gptr,
                                          A->K, p->col_idx, reinterpret_cast<uint4*>(p->vals), p->gather_rows);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return bail(fail(SPMM_ERR_CUDA, std::string("plan fill: ") + cudaGetErrorString(e)));
  *out = p;
  return SPMM_OK;
}

extern "C" spmm_status spmm_hcsr_plan_info(const spmm_hcsr_plan* p, long long* blocks, long long* gather_blocks) {
  if (!p) return fail(SPMM_ERR_INVALID_ARG, "null plan");
  if (blocks) *blocks = p->blocks;
  if (gather_blocks) *gather_blocks = p->gather_blocks;
  return SPMM_OK;
}

extern "C" spmm_status spmm_hcsr_plan_run(const spmm_hcsr_plan* p, const spmm_dense_desc* B, int N, float* C,
                                          int ldc, const spmm_config* cfg, void* stream) {
  if (!p || !B) return fail(SPMM_ERR_INVALID_ARG, "null plan or descriptor");
  spmm_config c;
  std::memset(&c, 0, sizeof(c));
  if (cfg) c = *cfg;
  if (c.kernel != 0 && c.kernel != 2) return fail(SPMM_ERR_UNSUPPORTED, "the planned hybrid product runs on kernel 2");
  c.kernel = 2;
  if (N < 0) return fail(SPMM_ERR_INVALID_ARG, "negative size");
  if (p->M == 0 || N == 0) return SPMM_OK;
  if (!C || !B->data) return fail(SPMM_ERR_INVALID_ARG, "null pointer");
  if (N % 8) return fail(SPMM_ERR_UNSUPPORTED, "N must be a multiple of 8");
  if (B->ldb < N || B->ldb % 8) return fail(SPMM_ERR_MISALIGNED, "ldb must be >= N and a multiple of 8");
  if (ldc < N || ldc % 4) return fail(SPMM_ERR_MISALIGNED, "ldc must be >= N and a multiple of 4");
  if (!aligned16(B->data) || !aligned16(C)) return fail(SPMM_ERR_MISALIGNED, "B and C must be 16-byte aligned");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (p->K == 0) {
    SPMM_CUDA_TRY(cudaMemset2DAsync(C, (size_t)ldc * 4, 0, (size_t)N * 4, p->M, s));
    return SPMM_OK;
  }
  spmm_bcsr_desc a;
  std::memset(&a, 0, sizeof(a));
  a.M = p->M;
  a.K = p->K;
  a.bR = 16;
  a.bC = 16;
  a.row_ptr = p->row_ptr;
  a.col_idx = p->col_idx;
  a.vals = p->vals;
  a.dtype = SPMM_F16;
  LaunchRequest r;
  r.A = &a;
  r.B = B;
  r.N = N;
  r.C = C;
  r.ldc = ldc;
  r.cfg = c;
  r.stream = s;
  r.gather_rows = p->gather_rows;
  r.total_blocks = p->blocks;
  return launch_tc(r);
}

extern "C" spmm_status spmm_hcsr_plan_destroy(spmm_hcsr_plan* p) {
  plan_free(p);
  return SPMM_OK;
}
