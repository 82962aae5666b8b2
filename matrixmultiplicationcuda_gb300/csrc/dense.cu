// Dense x dense product on the tcgen05 tensor cores (fp16 or bf16 A and B,
// fp32 C): the native dense comparator beside the BCSR path. It replaces the
// reference's denseMatrixMulTensor (src/cuda_kernels.cu:246-270: one WMMA warp
// per 16 x 16 tile, operands read straight from global memory) and its scalar
// dense kernels (:86-244).
//
// C tile 128 x 256 per item, K in steps of 64, a persistent grid of one CTA per SM:
//   * warp 0 (one thread) copies each step's A tile (128 x 64, K-major) and B
//     tile (64 x 256, four 64 x 64 boxes, MN-major), both 128-byte swizzled,
//     into a 4-deep ring with TMA;
//   * warp 1 (one thread) issues four tcgen05.mma (M = 128, N = 256, K = 16)
//     per step into one of two 256-column TMEM accumulators and commits each
//     ring slot back to the producer;
//   * warp 2 allocates and frees TMEM;
//   * warps 4-7 drain an accumulator (TMEM lane = row, column = column) into C
//     while the other one fills.
// Tiles are ordered along N first, so CTAs working at the same time share A's
// rows in L2. Ragged edges: TMA reads zeros past M, N and K; the epilogue
// stores only inside C. Every wait is bounded.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cstdio>
#include <cstdlib>
#include "internal.h"
#include "ptx.cuh"
#include "tcgen05.cuh"

namespace spmm {
namespace {

constexpr int kBM = 128, kBN = 256, kBK = 64, kStages = 4;
constexpr int kABytes = kBM * kBK * 2;        // 16 KB
constexpr int kBBox = kBK * 128;              // 64 rows x 64 columns: 8 KB
constexpr int kBBytes = (kBN / 64) * kBBox;   // 32 KB
constexpr int kStage = kABytes + kBBytes;
constexpr size_t kSmem = 1024 + (size_t)kStages * kStage + 1024;
constexpr int kThreads = 256;

struct DenseParams {
  float* C;
  long long ldc;
  int M, N, K;
  int tiles_n, tiles;
  unsigned long long timeout_ns;
  unsigned* err;
};

template <bool BF16>
__global__ void __launch_bounds__(kThreads, 1)
    k_dense_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, const DenseParams p) {
  // kind::f16: D f32, A K-major, B MN-major, N = 256, M = 128
  constexpr uint32_t kIdesc = (1u << 4) | ((BF16 ? 1u : 0u) << 7) | ((BF16 ? 1u : 0u) << 10) | (0u << 15) |
                              (1u << 16) | ((uint32_t)(kBN >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)kStages * kStage);
  const uint32_t full0 = smem_u32(bars), empty0 = full0 + 8 * kStages;
  const uint32_t tfull0 = empty0 + 8 * kStages, tempty0 = tfull0 + 16, done_bar = tempty0 + 16;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kStages + 5);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = (p.K + kBK - 1) / kBK;

  if (threadIdx.x == 32) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(tfull0 + 8 * b, 1);
      mbar_init(tempty0 + 8 * b, 4);
    }
    mbar_init(done_bar, 1);
    fence_mbar_init();
  }
  if (warp == 2) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  grid_dep_launch_dependents();
  grid_dep_wait();

  if (warp == 0) {
    // ------------------------------ producer ---------------------------------------
    if (lane == 0) {
      tma_prefetch_desc(&tmA);
      tma_prefetch_desc(&tmB);
      const uint64_t pol = l2_policy_evict_last();
      uint32_t gs = 0;
      bool failed = false;
      for (int t = blockIdx.x; t < p.tiles && !failed; t += gridDim.x) {
        const int tm = t / p.tiles_n, tn = t % p.tiles_n;
        for (int kb = 0; kb < nk; ++kb, ++gs) {
          const int s = (int)(gs % kStages);
          if (gs >= (uint32_t)kStages && !mbar_wait(empty0 + 8 * s, ((gs / kStages) + 1) & 1, p.timeout_ns)) {
            atomicOr(p.err, 4u);
            failed = true;
            break;
          }
          const uint32_t fb = full0 + 8 * s;
          mbar_arrive_expect_tx(fb, (uint32_t)kStage);
          uint8_t* a_dst = smem + (size_t)s * kStage;
          tma_tile_2d_g2s(smem_u32(a_dst), &tmA, kb * kBK, tm * kBM, fb, pol);
#pragma unroll
          for (int bx = 0; bx < kBN / 64; ++bx)
            tma_tile_2d_g2s(smem_u32(a_dst + kABytes + bx * kBBox), &tmB, tn * kBN + bx * 64, kb * kBK, fb, pol);
        }
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    // ------------------------------ MMA issuer -------------------------------------
    if (lane == 0) {
      uint32_t gs = 0, it = 0;
      bool failed = false;
      for (int t = blockIdx.x; t < p.tiles && !failed; t += gridDim.x, ++it) {
        const uint32_t acc = it & 1;
        if (it >= 2 && !mbar_wait(tempty0 + 8 * acc, ((it >> 1) + 1) & 1, p.timeout_ns)) {
          atomicOr(p.err, 8u);
          break;
        }
        tc_fence_after();
        const uint32_t d = tmem + acc * kBN;
        for (int kb = 0; kb < nk; ++kb, ++gs) {
          const int s = (int)(gs % kStages);
          if (!mbar_wait(full0 + 8 * s, (gs / kStages) & 1, p.timeout_ns)) {
            atomicOr(p.err, 8u);
            failed = true;
            break;
          }
          tc_fence_after();
          const uint32_t a_addr = smem_u32(smem + (size_t)s * kStage);
          const uint32_t b_addr = a_addr + kABytes;
#pragma unroll
          for (int kk = 0; kk < kBK / 16; ++kk) {
            // A: 128 rows of 128 bytes (64 k), the K = 16 slice 32 bytes in; B:
            // rows 16kk .. 16kk + 15 of the four 64-column boxes (8 KB apart)
            const uint64_t ad = smem_desc(a_addr + kk * 32, 16, 1024, kLayoutSW128);
            const uint64_t bd = smem_desc(b_addr + kk * 2048, kBBox, 1024, kLayoutSW128);
            umma_f16(d, ad, bd, kIdesc, (kb > 0 || kk > 0) ? 1u : 0u);
          }
          umma_commit(empty0 + 8 * s);
        }
        if (failed) break;
        umma_commit(tfull0 + 8 * acc);
      }
      umma_commit(done_bar);
      if (!mbar_wait(done_bar, 0, p.timeout_ns)) atomicOr(p.err, 8u);
    }
    __syncwarp();
  } else if (warp >= 4) {
    // ------------------------------ epilogue (warps 4-7) ---------------------------
    // Warp q reads TMEM lanes 32q .. 32q + 31, rows 32q .. 32q + 31 of the tile;
    // each lane writes its row, 16 columns (four 16-byte stores) per TMEM load.
    const int q4 = warp & 3;
    uint32_t it = 0;
    for (int t = blockIdx.x; t < p.tiles; t += gridDim.x, ++it) {
      const uint32_t acc = it & 1;
      if (!mbar_wait(tfull0 + 8 * acc, (it >> 1) & 1, p.timeout_ns)) {
        if (lane == 0) atomicOr(p.err, 16u);
        break;
      }
      tc_fence_after();
      const int tm = t / p.tiles_n, tn = t % p.tiles_n;
      const int row = tm * kBM + q4 * 32 + lane;
      float* crow = p.C + (long long)row * p.ldc;
      const uint32_t taddr = tmem + ((uint32_t)(q4 * 32) << 16) + acc * kBN;
#pragma unroll 1
      for (int c = 0; c < kBN; c += 16) {
        const int n0 = tn * kBN + c;
        if (n0 >= p.N) break;   // warp-uniform
        float v[16];
        tmem_ld16(taddr + c, v);
        if (row < p.M) {
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int n = n0 + 4 * i;
            if (n + 4 <= p.N)
              __stcs(reinterpret_cast<float4*>(crow + n), make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]));
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(tempty0 + 8 * acc);
    }
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 2) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
  }
}

bool aligned16(const void* q) { return (reinterpret_cast<uintptr_t>(q) & 15u) == 0; }

}  // namespace
}  // namespace spmm

using namespace spmm;

extern "C" spmm_status spmm_dense_mm(const void* A, int lda, const spmm_dense_desc* B, int M, int K, int N,
                                     spmm_dtype dtype, float* C, int ldc, void* stream) {
  if (!B) return fail(SPMM_ERR_INVALID_ARG, "null descriptor");
  if (dtype != SPMM_F16 && dtype != SPMM_BF16) return fail(SPMM_ERR_UNSUPPORTED, "the dense product is fp16 or bf16");
  if (M < 0 || K < 0 || N < 0) return fail(SPMM_ERR_INVALID_ARG, "negative size");
  if (M == 0 || N == 0) return SPMM_OK;
  if (!C || (K > 0 && (!A || !B->data))) return fail(SPMM_ERR_INVALID_ARG, "null pointer");
  if (N % 8) return fail(SPMM_ERR_UNSUPPORTED, "N must be a multiple of 8");
  if (lda < K || lda % 8 || B->ldb < N || B->ldb % 8 || ldc < N || ldc % 4)
    return fail(SPMM_ERR_MISALIGNED, "lda >= K and ldb >= N multiples of 8, ldc >= N a multiple of 4");
  if ((K > 0 && (!aligned16(A) || !aligned16(B->data))) || !aligned16(C))
    return fail(SPMM_ERR_MISALIGNED, "A, B and C must be 16-byte aligned");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (K == 0) {
    SPMM_CUDA_TRY(cudaMemset2DAsync(C, (size_t)ldc * 4, 0, (size_t)N * 4, M, s));
    return SPMM_OK;
  }
  CUtensorMap tmA, tmB;
  spmm_status st = encode_tile_map_2d(&tmA, CU_TENSOR_MAP_DATA_TYPE_UINT16, A, (uint64_t)K, (uint64_t)M,
                                      (uint64_t)lda * 2, kBK, kBM, CU_TENSOR_MAP_SWIZZLE_128B);
  if (st != SPMM_OK) return st;
  st = encode_tile_map_2d(&tmB, CU_TENSOR_MAP_DATA_TYPE_UINT16, B->data, (uint64_t)N, (uint64_t)K,
                          (uint64_t)B->ldb * 2, 64, kBK, CU_TENSOR_MAP_SWIZZLE_128B);
  if (st != SPMM_OK) return st;
  DenseParams p;
  p.C = C;
  p.ldc = ldc;
  p.M = M;
  p.N = N;
  p.K = K;
  p.tiles_n = (N + kBN - 1) / kBN;
  const long long tiles = (long long)((M + kBM - 1) / kBM) * p.tiles_n;
  if (tiles >= (1ll << 31)) return fail(SPMM_ERR_UNSUPPORTED, "too many tiles");
  p.tiles = (int)tiles;
  p.timeout_ns = wait_limit_ns();
  p.err = device_error_word();
  if (!p.err) return fail(SPMM_ERR_CUDA, "could not set up the device error word");
  const void* fn = dtype == SPMM_BF16 ? reinterpret_cast<const void*>(&k_dense_tc<true>)
                                      : reinterpret_cast<const void*>(&k_dense_tc<false>);
  SPMM_CUDA_TRY(ensure_smem_attr(fn, (int)kSmem));
  long long grid = sm_count();
  if (grid > p.tiles) grid = p.tiles;
  if (dtype == SPMM_BF16)
    SPMM_CUDA_TRY(launch_kernel(&k_dense_tc<true>, dim3((unsigned)grid), dim3(kThreads), kSmem, s, tmA, tmB, p));
  else
    SPMM_CUDA_TRY(launch_kernel(&k_dense_tc<false>, dim3((unsigned)grid), dim3(kThreads), kSmem, s, tmA, tmB, p));
  return SPMM_OK;
}
