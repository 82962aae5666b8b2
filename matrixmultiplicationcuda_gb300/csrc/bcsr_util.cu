// Dense -> BCSR conversion, structure validation, precision conversion and the
// bounded-wait diagnostic. All device work; the host functions are C ABI.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>
#include <cstring>
#include "internal.h"
#include "ptx.cuh"

namespace spmm {
namespace {

constexpr int kConvThreads = 256;

// An fp16 element is "nonzero" for the reference's blockDensity test
// (miscutil.cpp:76-87, `if (matrix.data[...])`) when its float value compares
// != 0: every encoding except +0 and -0, NaN included.
__device__ __forceinline__ bool any_nonzero_h8(uint4 v) {
  auto nz = [](uint32_t w) { return ((w & 0x7fffu) != 0u) || ((w & 0x7fff0000u) != 0u); };
  return nz(v.x) || nz(v.y) || nz(v.z) || nz(v.w);
}

// One CTA per block row. A warp covers 32 lanes x 16 bytes of a row of A, i.e.
// 256 / bC whole blocks (bC / 8 lanes each), and walks the bR rows of the block
// row, so every load is a coalesced 512-byte row segment.
// Pass 1 (FILL = false) writes the block count of the row to counts[br].
// Pass 2 (FILL = true) writes col_idx and copies the kept blocks, in ascending
// block-column order, starting at row_ptr[br] (formats/BCSRMatrix.cu:55-71).
template <bool FILL>
__global__ void __launch_bounds__(kConvThreads)
    k_dense_to_bcsr(const uint16_t* __restrict__ A, long long lda, int bR, int bC, int KB,
                    int* __restrict__ counts, const int* __restrict__ row_ptr,
                    int* __restrict__ col_idx, uint16_t* __restrict__ vals) {
  extern __shared__ uint32_t sm[];  // masks[ngroups], offsets[ngroups]
  const int br = blockIdx.x;
  const int lpb = bC / 8;                 // lanes per block
  const int gblk = 32 / lpb;              // blocks per warp pass
  const int ngroups = (KB + gblk - 1) / gblk;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  uint32_t* masks = sm;
  uint32_t* offs = sm + ngroups;
  __shared__ int row_total;
  if (threadIdx.x == 0) row_total = 0;
  __syncthreads();

  const uint16_t* arow = A + (long long)br * bR * lda;
  int local = 0;
  for (int gi = warp; gi < ngroups; gi += nwarps) {
    const int j = gi * gblk + lane / lpb;   // block column of this lane
    const int sub = lane % lpb;
    bool nz = false;
    if (j < KB) {
      // eight rows per step, all loads in flight before the test (a test per
      // row would serialise the loads of an all-zero block)
      const uint16_t* p = arow + (long long)j * bC + sub * 8;
      for (int x0 = 0; x0 < bR && !nz; x0 += 8) {
        uint4 v[8];
#pragma unroll
        for (int x = 0; x < 8; ++x) v[x] = __ldg(reinterpret_cast<const uint4*>(p + (long long)(x0 + x) * lda));
#pragma unroll
        for (int x = 0; x < 8; ++x) nz = nz || any_nonzero_h8(v[x]);
      }
    }
    const uint32_t bal = __ballot_sync(0xffffffffu, nz);
    uint32_t mask = 0;
    const uint32_t lm = (lpb >= 32) ? 0xffffffffu : ((1u << lpb) - 1u);
    for (int b = 0; b < gblk; ++b)
      if ((bal >> (b * lpb)) & lm) mask |= 1u << b;
    if (lane == 0) {
      masks[gi] = mask;
      local += __popc(mask);
    }
  }
  if (!FILL) {
    if (lane == 0 && local) atomicAdd(&row_total, local);
    __syncthreads();
    if (threadIdx.x == 0) counts[br] = row_total;
    return;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t run = 0;
    for (int gi = 0; gi < ngroups; ++gi) {
      offs[gi] = run;
      run += __popc(masks[gi]);
    }
  }
  __syncthreads();
  const int base = row_ptr[br];
  const int chunks = bR * lpb;              // 16-byte chunks per block
  for (int gi = warp; gi < ngroups; gi += nwarps) {
    uint32_t mask = masks[gi];
    int pos = base + (int)offs[gi];
    while (mask) {
      const int b = __ffs(mask) - 1;
      mask &= mask - 1;
      const int j = gi * gblk + b;
      if (lane == 0) col_idx[pos] = j;
      uint4* dst = reinterpret_cast<uint4*>(vals + (long long)pos * bR * bC);
      const uint16_t* src = arow + (long long)j * bC;
      for (int c = lane; c < chunks; c += 32) {
        const int x = c / lpb, y = c % lpb;
        dst[c] = __ldg(reinterpret_cast<const uint4*>(src + (long long)x * lda + y * 8));
      }
      ++pos;
    }
  }
}

// Exclusive scan of counts[0..n) into row_ptr[0..n] (row_ptr[0] = 0); one CTA.
__global__ void __launch_bounds__(1024) k_scan_counts(const int* counts, int* row_ptr, int n) {
  __shared__ long long warp_sums[32];
  const int t = threadIdx.x, T = blockDim.x;
  const long long per = (n + T - 1) / T;
  const long long lo = min((long long)n, t * per), hi = min((long long)n, lo + per);
  long long s = 0;
  for (long long i = lo; i < hi; ++i) s += counts[i];
  // block-wide exclusive scan of s
  long long v = s;
  for (int o = 1; o < 32; o <<= 1) {
    long long u = __shfl_up_sync(0xffffffffu, v, o);
    if ((t & 31) >= o) v += u;
  }
  if ((t & 31) == 31) warp_sums[t >> 5] = v;
  __syncthreads();
  if (t < 32) {
    long long w = (t < (T >> 5)) ? warp_sums[t] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      long long u = __shfl_up_sync(0xffffffffu, w, o);
      if (t >= o) w += u;
    }
    warp_sums[t] = w;
  }
  __syncthreads();
  long long run = v - s + ((t >> 5) ? warp_sums[(t >> 5) - 1] : 0);
  if (t == 0) row_ptr[0] = 0;
  for (long long i = lo; i < hi; ++i) {
    run += counts[i];
    row_ptr[i + 1] = (int)run;
  }
}

// Structure checks. bad[0] |= 1: row_ptr[0] != 0 or not monotone or
// row_ptr[MB] != nnzb; bad[0] |= 2: a col_idx out of range or not ascending.
__global__ void k_validate_rows(const int* row_ptr, int MB, long long nnzb, unsigned* bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0 && (row_ptr[0] != 0 || row_ptr[MB] != nnzb)) atomicOr(bad, 1u);
  if (i < MB && row_ptr[i] > row_ptr[i + 1]) atomicOr(bad, 1u);
}
__global__ void k_validate_cols(const int* row_ptr, const int* col_idx, int MB, int KB,
                                unsigned* bad) {
  const int br = blockIdx.x * blockDim.x + threadIdx.x;
  if (br >= MB) return;
  int prev = -1;
  for (int k = row_ptr[br]; k < row_ptr[br + 1]; ++k) {
    const int c = col_idx[k];
    if (c < 0 || c >= KB || c <= prev) {
      atomicOr(bad, 2u);
      return;
    }
    prev = c;
  }
}

// ---- precision conversion -------------------------------------------------------
// Conversions read 16 bytes (four values) per thread per step when every
// pointer allows it (vec != 0), then finish the last n % 4 values one by one.
__device__ __forceinline__ uint32_t h2_bits(__half2 h) { return *reinterpret_cast<uint32_t*>(&h); }

__global__ void k_to_f16(const float* src, size_t n, __half* dst, __half* lo, int vec) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t n4 = vec ? n / 4 : 0;
  for (size_t q = t; q < n4; q += stride) {
    const float4 x = __ldg(reinterpret_cast<const float4*>(src) + q);
    const __half2 a = __floats2half2_rn(x.x, x.y), b = __floats2half2_rn(x.z, x.w);
    reinterpret_cast<uint2*>(dst)[q] = make_uint2(h2_bits(a), h2_bits(b));
    if (lo) {
      const float2 fa = __half22float2(a), fb = __half22float2(b);
      const __half2 la = __floats2half2_rn(x.x - fa.x, x.y - fa.y), lb = __floats2half2_rn(x.z - fb.x, x.w - fb.y);
      reinterpret_cast<uint2*>(lo)[q] = make_uint2(h2_bits(la), h2_bits(lb));
    }
  }
  for (size_t i = n4 * 4 + t; i < n; i += stride) {
    const float x = src[i];
    const __half h = __float2half_rn(x);
    dst[i] = h;
    if (lo) lo[i] = __float2half_rn(x - __half2float(h));
  }
}
__global__ void k_to_bf16(const float* src, size_t n, __nv_bfloat16* dst, int vec) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t n4 = vec ? n / 4 : 0;
  for (size_t q = t; q < n4; q += stride) {
    const float4 x = __ldg(reinterpret_cast<const float4*>(src) + q);
    __nv_bfloat162 a = __floats2bfloat162_rn(x.x, x.y), b = __floats2bfloat162_rn(x.z, x.w);
    reinterpret_cast<uint2*>(dst)[q] =
        make_uint2(*reinterpret_cast<uint32_t*>(&a), *reinterpret_cast<uint32_t*>(&b));
  }
  for (size_t i = n4 * 4 + t; i < n; i += stride) dst[i] = __float2bfloat16_rn(src[i]);
}
// Absolute maximum of large scale blocks: CTA (x, y) reduces chunk x of scale
// block y and merges it with one atomicMax (ordered uint bits; scales zeroed first).
constexpr int kAbsChunk = 256 * 16;
__global__ void k_absmax(const float* src, size_t n, int block_elems, unsigned* smax) {
  __shared__ float red[32];
  const size_t blo = (size_t)blockIdx.y * block_elems;
  const size_t lo = blo + (size_t)blockIdx.x * kAbsChunk;
  const size_t hi = min(min(lo + (size_t)kAbsChunk, blo + (size_t)block_elems), n);
  float m = 0.f;
  for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) m = fmaxf(m, fabsf(src[i]));
  for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
    for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0 && m > 0.f) atomicMax(smax + blockIdx.y, __float_as_uint(m));
  }
}
// One warp per scale block when blocks are small (<= 8192 elements): 16-byte
// loads when the block starts 16-byte aligned (vec), a shuffle reduction.
__global__ void k_absmax_small(const float* src, size_t n, int block_elems, float* scales, size_t nblocks,
                               int vec) {
  const size_t b = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (b >= nblocks) return;
  const size_t lo = b * (size_t)block_elems;
  const size_t hi = min(lo + (size_t)block_elems, n);
  float m = 0.f;
  if (vec && hi - lo == (size_t)block_elems) {
    const float4* p = reinterpret_cast<const float4*>(src + lo);
    for (int q = lane; q < block_elems / 4; q += 32) {
      const float4 x = __ldg(p + q);
      m = fmaxf(m, fmaxf(fmaxf(fabsf(x.x), fabsf(x.y)), fmaxf(fabsf(x.z), fabsf(x.w))));
    }
  } else {
    for (size_t i = lo + lane; i < hi; i += 32) m = fmaxf(m, fabsf(src[i]));
  }
  for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) scales[b] = m;
}
// max -> scale: the smallest power of two >= max / 448 (448 is the largest
// finite e4m3), 1 for an all-zero block, kept within the normal fp32 range.
// A power of two is exact as a UE8M0 scale factor (the tcgen05 e4m3 kernels
// apply it inside the MMA), and dividing by it is exact; the block's largest
// value lands in (224, 448], where e4m3 keeps its full 4 significant bits.
__global__ void k_finish_scales(float* scales, size_t nblocks) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nblocks;
       i += (size_t)gridDim.x * blockDim.x) {
    const float m = scales[i];
    float sc = 1.0f;
    if (m > 0.f) {
      int e = 0;
      const float f = frexpf(m / 448.0f, &e);   // m / 448 = f * 2^e, f in [0.5, 1)
      sc = ldexpf(1.0f, f == 0.5f ? e - 1 : e);
      sc = fminf(fmaxf(sc, 0x1p-126f), 0x1p127f);
    }
    scales[i] = sc;
  }
}
__global__ void k_to_e4m3(const float* src, size_t n, int block_elems, const float* scales,
                          __nv_fp8_storage_t* dst, int vec) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t n4 = vec ? n / 4 : 0;
  // vec is set only when block_elems % 4 == 0: the four values share a scale
  for (size_t q = t; q < n4; q += stride) {
    const float4 x = __ldg(reinterpret_cast<const float4*>(src) + q);
    const float sc = scales[(q * 4) / (size_t)block_elems];
    const uint32_t packed = (uint32_t)__nv_cvt_float_to_fp8(x.x / sc, __NV_SATFINITE, __NV_E4M3) |
                            (uint32_t)__nv_cvt_float_to_fp8(x.y / sc, __NV_SATFINITE, __NV_E4M3) << 8 |
                            (uint32_t)__nv_cvt_float_to_fp8(x.z / sc, __NV_SATFINITE, __NV_E4M3) << 16 |
                            (uint32_t)__nv_cvt_float_to_fp8(x.w / sc, __NV_SATFINITE, __NV_E4M3) << 24;
    reinterpret_cast<uint32_t*>(dst)[q] = packed;
  }
  for (size_t i = n4 * 4 + t; i < n; i += stride)
    dst[i] = __nv_cvt_float_to_fp8(src[i] / scales[i / block_elems], __NV_SATFINITE, __NV_E4M3);
}

// Bounded-wait diagnostic: waits on a barrier that no one arrives on.
__global__ void k_wait_diag(unsigned long long limit_ns, unsigned* out) {
  __shared__ uint64_t bar;
  const uint32_t b = smem_u32(&bar);
  if (threadIdx.x == 0) {
    mbar_init(b, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) out[0] = mbar_wait(b, 0, limit_ns) ? 0u : 1u;
}

unsigned grid_for(size_t n) {
  size_t g = (n + 255) / 256;
  const size_t cap = (size_t)sm_count() * 8;
  if (g > cap) g = cap;
  return (unsigned)(g ? g : 1);
}

}  // namespace

spmm_status scan_counts(const int* counts, int* row_ptr, int n, cudaStream_t s) {
  k_scan_counts<<<1, 1024, 0, s>>>(counts, row_ptr, n);
  SPMM_CUDA_TRY(cudaGetLastError());
  return SPMM_OK;
}

}  // namespace spmm

using namespace spmm;

extern "C" {

static spmm_status conv_checks(const void* A, int M, int K, int lda, int bR, int bC) {
  if (bR < 16 || bC < 16 || bR % 16 || bC % 16)
    return fail(SPMM_ERR_INVALID_ARG,
                "Block sizes must be at least 16x16 and multiples of 16 (got " +
                    std::to_string(bR) + "x" + std::to_string(bC) + ")");
  if (bC > 256) return fail(SPMM_ERR_UNSUPPORTED, "block width above 256");
  if (M < 0 || K < 0 || lda < K) return fail(SPMM_ERR_INVALID_ARG, "bad size or lda");
  if (lda % 8 || (reinterpret_cast<uintptr_t>(A) & 15))
    return fail(SPMM_ERR_MISALIGNED, "A must be 16-byte aligned with lda a multiple of 8");
  const int KB = K / bC, gblk = 32 / (bC / 8);
  const int ngroups = (KB + gblk - 1) / gblk;
  if ((size_t)ngroups * 8 > 48 * 1024) return fail(SPMM_ERR_UNSUPPORTED, "K too large");
  return SPMM_OK;
}

spmm_status spmm_dense_to_bcsr_count(const void* A, int M, int K, int lda, int bR, int bC,
                                     int* row_ptr, long long* nnzb_out, void* stream) {
  spmm_status st = conv_checks(A, M, K, lda, bR, bC);
  if (st != SPMM_OK) return st;
  if (!row_ptr || !nnzb_out) return fail(SPMM_ERR_INVALID_ARG, "null pointer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int MB = M / bR, KB = K / bC;
  const int gblk = 32 / (bC / 8), ngroups = (KB + gblk - 1) / gblk;
  // counts go to row_ptr[1..MB] first, then the scan rewrites row_ptr in place
  // from a copy held in the tail of the same launch sequence.
  int* counts = row_ptr + 1;
  if (MB > 0 && KB > 0) {
    k_dense_to_bcsr<false><<<MB, kConvThreads, (size_t)ngroups * 8, s>>>(
        static_cast<const uint16_t*>(A), lda, bR, bC, KB, counts, nullptr, nullptr, nullptr);
    SPMM_CUDA_TRY(cudaGetLastError());
  } else if (MB > 0) {
    SPMM_CUDA_TRY(cudaMemsetAsync(counts, 0, sizeof(int) * MB, s));
  }
  // in-place scan: counts live in row_ptr[1..MB]; k_scan_counts reads all
  // counts of a thread's chunk before writing, and chunks are disjoint and
  // shifted by one, so read counts[i] then write row_ptr[i+1] = counts[i]'s slot.
  k_scan_counts<<<1, 1024, 0, s>>>(counts, row_ptr, MB);
  SPMM_CUDA_TRY(cudaGetLastError());
  int total = 0;
  SPMM_CUDA_TRY(cudaMemcpyAsync(&total, row_ptr + MB, sizeof(int), cudaMemcpyDeviceToHost, s));
  SPMM_CUDA_TRY(cudaStreamSynchronize(s));
  *nnzb_out = total;
  return SPMM_OK;
}

spmm_status spmm_dense_to_bcsr_fill(const void* A, int M, int K, int lda, int bR, int bC,
                                    const int* row_ptr, int* col_idx, void* vals, void* stream) {
  spmm_status st = conv_checks(A, M, K, lda, bR, bC);
  if (st != SPMM_OK) return st;
  const int MB = M / bR, KB = K / bC;
  if (MB == 0 || KB == 0) return SPMM_OK;
  if (!row_ptr || !col_idx || !vals) return fail(SPMM_ERR_INVALID_ARG, "null pointer");
  if (reinterpret_cast<uintptr_t>(vals) & 15) return fail(SPMM_ERR_MISALIGNED, "vals must be 16-byte aligned");
  const int gblk = 32 / (bC / 8), ngroups = (KB + gblk - 1) / gblk;
  k_dense_to_bcsr<true><<<MB, kConvThreads, (size_t)ngroups * 8, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const uint16_t*>(A), lda, bR, bC, KB, nullptr, row_ptr, col_idx,
      static_cast<uint16_t*>(vals));
  SPMM_CUDA_TRY(cudaGetLastError());
  return SPMM_OK;
}

spmm_status spmm_bcsr_validate(const int* row_ptr, const int* col_idx, int M, int K, int bR,
                               long long nnzb, void* stream) {
  if (bR <= 0 || M < 0 || K < 0 || M % bR || K % 16 || nnzb < 0)
    return fail(SPMM_ERR_INVALID_ARG, "bad sizes");
  const int MB = M / bR, KB = K / 16;
  if (!row_ptr || (nnzb > 0 && !col_idx)) return fail(SPMM_ERR_INVALID_ARG, "null pointer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned* w = device_error_word();
  if (!w) return fail(SPMM_ERR_CUDA, "no device word");
  unsigned* bad = w + 1;
  SPMM_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(unsigned), s));
  k_validate_rows<<<(MB + 256) / 256, 256, 0, s>>>(row_ptr, MB, nnzb, bad);
  SPMM_CUDA_TRY(cudaGetLastError());
  unsigned v = 0;
  SPMM_CUDA_TRY(cudaMemcpyAsync(&v, bad, sizeof(v), cudaMemcpyDeviceToHost, s));
  SPMM_CUDA_TRY(cudaStreamSynchronize(s));
  if (v) return fail(SPMM_ERR_BAD_STRUCTURE, "row_ptr is not a monotone prefix from 0 to nnzb");
  if (MB > 0 && nnzb > 0) {
    k_validate_cols<<<(MB + 255) / 256, 256, 0, s>>>(row_ptr, col_idx, MB, KB, bad);
    SPMM_CUDA_TRY(cudaGetLastError());
    SPMM_CUDA_TRY(cudaMemcpyAsync(&v, bad, sizeof(v), cudaMemcpyDeviceToHost, s));
    SPMM_CUDA_TRY(cudaStreamSynchronize(s));
    if (v) return fail(SPMM_ERR_BAD_STRUCTURE, "col_idx out of range or not ascending in a row");
  }
  return SPMM_OK;
}

spmm_status spmm_quantize(const float* src, size_t count, spmm_dtype dtype, int block_elems,
                          void* dst, void* dst_lo, float* scales, void* stream) {
  if (count == 0) return SPMM_OK;
  if (!src || !dst) return fail(SPMM_ERR_INVALID_ARG, "null pointer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const unsigned g = grid_for((count + 3) / 4);
  auto al = [](const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; };
  const int vec2 = al(src, 16) && al(dst, 8) && (!dst_lo || al(dst_lo, 8)) ? 1 : 0;
  switch (dtype) {
    case SPMM_F16:
      k_to_f16<<<g, 256, 0, s>>>(src, count, static_cast<__half*>(dst), nullptr, vec2);
      break;
    case SPMM_F16_SPLIT:
      if (!dst_lo) return fail(SPMM_ERR_INVALID_ARG, "F16_SPLIT needs dst_lo");
      k_to_f16<<<g, 256, 0, s>>>(src, count, static_cast<__half*>(dst), static_cast<__half*>(dst_lo), vec2);
      break;
    case SPMM_BF16:
      k_to_bf16<<<g, 256, 0, s>>>(src, count, static_cast<__nv_bfloat16*>(dst), vec2);
      break;
    case SPMM_E4M3: {
      if (!scales || block_elems <= 0) return fail(SPMM_ERR_INVALID_ARG, "E4M3 needs scales and block_elems");
      const size_t nblocks = (count + block_elems - 1) / block_elems;
      if (block_elems <= 8192) {
        const int vec = al(src, 16) && block_elems % 4 == 0 ? 1 : 0;
        k_absmax_small<<<(unsigned)((nblocks + 7) / 8), 256, 0, s>>>(src, count, block_elems, scales, nblocks, vec);
      } else {
        SPMM_CUDA_TRY(cudaMemsetAsync(scales, 0, nblocks * sizeof(float), s));
        if (nblocks > 65535) return fail(SPMM_ERR_UNSUPPORTED, "too many large scale blocks");
        const dim3 ag((unsigned)((block_elems + kAbsChunk - 1) / kAbsChunk), (unsigned)nblocks);
        k_absmax<<<ag, 256, 0, s>>>(src, count, block_elems, reinterpret_cast<unsigned*>(scales));
      }
      SPMM_CUDA_TRY(cudaGetLastError());
      k_finish_scales<<<grid_for(nblocks), 256, 0, s>>>(scales, nblocks);
      SPMM_CUDA_TRY(cudaGetLastError());
      k_to_e4m3<<<g, 256, 0, s>>>(src, count, block_elems, scales, static_cast<__nv_fp8_storage_t*>(dst),
                                  al(src, 16) && al(dst, 4) && block_elems % 4 == 0 ? 1 : 0);
      break;
    }
    default:
      return fail(SPMM_ERR_INVALID_ARG, "unknown dtype");
  }
  SPMM_CUDA_TRY(cudaGetLastError());
  return SPMM_OK;
}

spmm_status spmm_debug_wait_timeout(unsigned long long timeout_ns, void* stream) {
  unsigned* w = device_error_word();
  if (!w) return fail(SPMM_ERR_CUDA, "no device word");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_wait_diag<<<1, 32, 0, s>>>(timeout_ns, w + 2);
  SPMM_CUDA_TRY(cudaGetLastError());
  unsigned v = 0;
  SPMM_CUDA_TRY(cudaMemcpyAsync(&v, w + 2, sizeof(v), cudaMemcpyDeviceToHost, s));
  SPMM_CUDA_TRY(cudaStreamSynchronize(s));
  if (v) return fail(SPMM_ERR_TIMEOUT, "bounded wait gave up as intended");
  return SPMM_OK;
}

}  // extern "C"
