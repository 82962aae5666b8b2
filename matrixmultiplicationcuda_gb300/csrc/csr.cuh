// CSR x dense row slices (fp16 A and B, fp32 accumulation), shared by the CSR
// product kernel and the CSR pass of the hybrid product.
//
// A warp computes one row of A times a 256-column slice of B: every lane owns 8
// consecutive columns. For each entry the warp reads that B row's slice as one
// 512-byte load (16 bytes per lane), with several entries' loads in flight
// before their FMAs.
#pragma once
#include <cuda_fp16.h>
#include <cstdint>

namespace spmm {

__device__ __forceinline__ void fma8(float (&acc)[8], float a, uint4 b) {
  const __half2* h = reinterpret_cast<const __half2*>(&b);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float2 f = __half22float2(h[k]);
    acc[2 * k] = fmaf(a, f.x, acc[2 * k]);
    acc[2 * k + 1] = fmaf(a, f.y, acc[2 * k + 1]);
  }
}

// acc[0..7] += sum over entries e in [e0, e1) of vals[e] * B[col_idx[e]][n..n+7],
// U entries' B loads in flight. Warp-uniform e0 / e1 (every lane reads the same
// entry, one broadcast load); `valid` (this lane's columns lie inside B) may
// differ per lane.
template <int U>
__device__ __forceinline__ void csr_row_slice(const int* __restrict__ col_idx, const __half* __restrict__ vals,
                                              const __half* __restrict__ B, long long ldb, int e0, int e1, int n,
                                              bool valid, float (&acc)[8]) {
  int e = e0;
  for (; e + U <= e1; e += U) {
    int k[U];
    float a[U];
    uint4 b[U];
#pragma unroll
    for (int t = 0; t < U; ++t) {
      k[t] = __ldg(col_idx + e + t);
      a[t] = __half2float(vals[e + t]);
    }
#pragma unroll
    for (int t = 0; t < U; ++t)
      b[t] = valid ? __ldg(reinterpret_cast<const uint4*>(B + (long long)k[t] * ldb + n)) : make_uint4(0, 0, 0, 0);
#pragma unroll
    for (int t = 0; t < U; ++t) fma8(acc, a[t], b[t]);
  }
  for (; e < e1; ++e) {
    const int k = __ldg(col_idx + e);
    const float a = __half2float(vals[e]);
    if (valid) fma8(acc, a, __ldg(reinterpret_cast<const uint4*>(B + (long long)k * ldb + n)));
  }
}

// The CSR part of one output tile of the hybrid product: rows [row0, row0 + rows)
// and columns [n0, n1) of C (n1 - n0 a multiple of 8) gain A_csr x B in place.
// Called by the four epilogue warps of a CTA (`wq` = 0..3) after their stores of
// the tile are ordered by a barrier; each warp takes every fourth row.
__device__ __forceinline__ void csr_tile_pass(const int* __restrict__ row_ptr, const int* __restrict__ col_idx,
                                              const __half* __restrict__ vals, const __half* __restrict__ B,
                                              long long ldb, float* C, long long ldc, long long row0, int rows,
                                              int n0, int n1, int wq, int lane) {
  for (int r = wq; r < rows; r += 4) {
    const long long row = row0 + r;
    const int e0 = __ldg(row_ptr + row), e1 = __ldg(row_ptr + row + 1);
    if (e0 >= e1) continue;
    for (int nb = n0; nb < n1; nb += 256) {
      const int n = nb + lane * 8;
      const bool valid = n < n1;
      float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      csr_row_slice<8>(col_idx, vals, B, ldb, e0, e1, n, valid, acc);
      if (valid) {
        float4* c = reinterpret_cast<float4*>(C + row * ldc + n);
        float4 x = __ldcg(c), y = __ldcg(c + 1);
        x.x += acc[0];
        x.y += acc[1];
        x.z += acc[2];
        x.w += acc[3];
        y.x += acc[4];
        y.y += acc[5];
        y.z += acc[6];
        y.w += acc[7];
        c[0] = x;
        c[1] = y;
      }
    }
  }
}

}  // namespace spmm
