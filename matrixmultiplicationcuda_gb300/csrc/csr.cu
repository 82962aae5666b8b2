// CSR x dense product (fp16 A and B, fp32 C): the comparator beside the BCSR
// path, replacing the reference's scalar CSR kernel (one thread per output
// element walking its row, src/cuda_kernels.cu:271-299).
//
// One warp per (row, 256-column slice), through the row-slice routine of
// csr.cuh: every lane owns 8 consecutive output columns, B rows are read as
// 512-byte warp loads with 4 entries in flight, and the row's results leave as
// two 16-byte streaming stores per lane.
#include <cuda_fp16.h>
#include "csr.cuh"
#include "internal.h"

namespace spmm {
namespace {

constexpr int kCsrWarps = 8;

__global__ void __launch_bounds__(32 * kCsrWarps)
    k_csr_mm(const int* __restrict__ row_ptr, const int* __restrict__ col_idx, const __half* __restrict__ vals,
             const __half* __restrict__ B, long long ldb, float* __restrict__ C, long long ldc, int M, int N) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row = blockIdx.x * kCsrWarps + warp;
  if (row >= M) return;
  const int n = blockIdx.y * 256 + lane * 8;
  const bool valid = n < N;   // N is a multiple of 8
  float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  csr_row_slice<4>(col_idx, vals, B, ldb, __ldg(row_ptr + row), __ldg(row_ptr + row + 1), n, valid, acc);
  if (valid) {
    float* c = C + (long long)row * ldc + n;
    __stcs(reinterpret_cast<float4*>(c), make_float4(acc[0], acc[1], acc[2], acc[3]));
    __stcs(reinterpret_cast<float4*>(c + 4), make_float4(acc[4], acc[5], acc[6], acc[7]));
  }
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace
}  // namespace spmm

using namespace spmm;

extern "C" spmm_status spmm_csr_mm(const spmm_csr_desc* A, const spmm_dense_desc* B, int N, float* C, int ldc,
                                   void* stream) {
  if (!A || !B) return fail(SPMM_ERR_INVALID_ARG, "null descriptor");
  if (A->M < 0 || A->K < 0 || N < 0) return fail(SPMM_ERR_INVALID_ARG, "negative size");
  if (A->M == 0 || N == 0) return SPMM_OK;
  if (!A->row_ptr || !B->data || !C) return fail(SPMM_ERR_INVALID_ARG, "null pointer");
  if (N % 8) return fail(SPMM_ERR_UNSUPPORTED, "N must be a multiple of 8");
  if (B->ldb < N || B->ldb % 8 || ldc < N || ldc % 4 || !aligned16(B->data) || !aligned16(C))
    return fail(SPMM_ERR_MISALIGNED, "B / C must be 16-byte aligned with ldb % 8 == 0 and ldc % 4 == 0");
  const dim3 grid((unsigned)((A->M + kCsrWarps - 1) / kCsrWarps), (unsigned)((N + 255) / 256));
  if (grid.y > 65535) return fail(SPMM_ERR_UNSUPPORTED, "N too large");
  k_csr_mm<<<grid, 32 * kCsrWarps, 0, static_cast<cudaStream_t>(stream)>>>(
      A->row_ptr, A->col_idx, static_cast<const __half*>(A->vals), static_cast<const __half*>(B->data), B->ldb, C,
      ldc, A->M, N);
  SPMM_CUDA_TRY(cudaGetLastError());
  return SPMM_OK;
}
