// BCSR x dense product on the 5th-generation tensor cores (tcgen05 + TMEM).
//
// The MMA runs transposed: for one stored block A_blk (bR x 16) at block
// column c and a 128-column slice of the output,
//     D (128 x bR, fp32, TMEM) += B[16c : 16c+16, n0 : n0+128]^T  x  A_blk^T
// so the MMA's M dimension (128) walks output columns and its N dimension is
// the block height (16, 32 or 64). A 64-row block is one M=128, N=64, K=16
// UMMA; D's TMEM lane i holds output column n0 + i and TMEM column j holds
// output row j of the block row, so the epilogue writes whole 128-byte row
// segments of C.
//
// Operands come from shared memory through TMA:
//   * the B row-panel (16 rows x NT columns) as 64-column boxes with 128-byte
//     swizzle -- the MMA's A operand in the MN-major canonical layout
//     (atoms of 64 columns x 8 rows; 8-row groups 1024 B apart, 64-column
//     atoms 2048 B apart);
//   * the A block (bR rows x 16) as one box with 32-byte swizzle -- the MMA's
//     B operand in the K-major canonical layout (8-row groups 256 B apart).
//
// Warp roles (256 threads, two CTAs per SM): warp 0 streams TMA copies into a
// STAGES-deep mbarrier ring (one copy for the A block and, when N % 64 == 0,
// one 3-D copy for the whole B panel: a TMA instruction holds its issuing thread
// for tens of cycles, so copies per block bound the block rate); warp 1 (one
// thread) issues the UMMAs, releases each ring slot with tcgen05.commit and
// hands finished accumulators to the epilogue; warp 2 owns the TMEM
// allocation; warps 4-7 drain TMEM (double-buffered, so the next item's MMAs
// overlap) with tcgen05.ld and store C with streaming stores. The grid is persistent over
// items = (block row, NT-column tile). Every mbarrier wait is bounded; a wait
// that gives up sets the device error word, all roles leave their loops, and
// the allocating warp frees TMEM after the MMA thread has drained its commits.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include "internal.h"
#include "ptx.cuh"
#include "spmm_mma.cuh"

namespace spmm {
namespace {

struct TcParams {
  const int* row_ptr;
  const int* col_idx;
  float* C;
  long long ldc;
  int N;
  int ntiles;
  int n_items;
  unsigned long long timeout_ns;
  unsigned* err;
  int panel3d;      // B panel loaded by one 3-D copy (N % 64 == 0)
};

template <int BR, int NT, int STAGES, int MODE>
struct TcCfg {
  static constexpr bool kSplit = MODE == MODE_SPLIT;
  static constexpr int kParts = kSplit ? 2 : 1;
  static constexpr int kJ = NT / 128;                 // 128-column MMA slices per item
  static constexpr int kBoxBytes = 16 * 128;          // 16 rows x 64 fp16 columns
  static constexpr int kPanelBytes = (NT / 64) * kBoxBytes;
  static constexpr int kABytes = BR * 32;             // bR rows x 16 fp16
  static constexpr int kABytesPad = kABytes < 1024 ? 1024 : kABytes;
  static constexpr int kStageB = kPanelBytes * kParts;
  static constexpr int kStageA = kABytesPad * kParts;
  static constexpr int kTx = kPanelBytes * kParts + kABytes * kParts;
  static constexpr int kAccCols = kJ * BR;            // TMEM columns of one accumulator
  static constexpr int kTmemCols = (2 * kAccCols) < 32 ? 32 : 2 * kAccCols;
  static constexpr size_t kSmem = 1024 + (size_t)STAGES * (kStageB + kStageA) + 512;
  static_assert((kTmemCols & (kTmemCols - 1)) == 0 && kTmemCols <= 512, "TMEM columns");
  static_assert(NT % 128 == 0, "NT");
  // kind::f16 instruction descriptor: D f32, A/B f16 or bf16, A MN-major, B K-major,
  // N = BR, M = 128.
  static constexpr uint32_t kIdesc = (1u << 4) | ((MODE == MODE_BF16 ? 1u : 0u) << 7) |
                                     ((MODE == MODE_BF16 ? 1u : 0u) << 10) | (1u << 15) |
                                     ((uint32_t)(BR >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
};

// Shared-memory matrix descriptor (tcgen05): start, leading / stride byte
// offsets (16-byte units), version 1, swizzle mode.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo,
                                              uint32_t layout) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46) | ((uint64_t)layout << 61);
}
constexpr uint32_t kLayoutSW128 = 2, kLayoutSW32 = 6;

__device__ __forceinline__ void umma_f16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// 16 consecutive TMEM columns of this thread's lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

template <int BR, int NT, int STAGES, int MODE>
__global__ void __launch_bounds__(256, 2)
    k_bcsr_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmAlo,
              const __grid_constant__ CUtensorMap tmB, const __grid_constant__ CUtensorMap tmBlo,
              const TcParams p) {
  using Cfg = TcCfg<BR, NT, STAGES, MODE>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  uint8_t* sB = smem;
  uint8_t* sA = smem + (size_t)STAGES * Cfg::kStageB;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sA + (size_t)STAGES * Cfg::kStageA);
  // bars: full[STAGES], empty[STAGES], tfull[2], tempty[2], done; then the TMEM
  // address and the producer's column-index staging buffer
  const uint32_t full0 = smem_u32(bars), empty0 = full0 + 8 * STAGES;
  const uint32_t tfull0 = empty0 + 8 * STAGES, tempty0 = tfull0 + 16, done_bar = tempty0 + 16;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 5);
  int* s_cols = reinterpret_cast<int*>(tmem_slot + 1);    // 32 entries

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 32) {
    for (int s = 0; s < STAGES; ++s) {
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
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(Cfg::kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ------------------------------ TMA producer ---------------------------------
    // Lane 0 issues every copy; the other lanes fetch column indices 32 at a time
    // into s_cols and prefetch the next item's row range, so the issuing lane
    // never waits on a global load or a shuffle between two blocks.
    if (lane == 0) {
      tma_prefetch_desc(&tmA);
      tma_prefetch_desc(&tmB);
    }
    const uint64_t pol_b = l2_policy_evict_last();
    const uint64_t pol_a = l2_policy_evict_first();
    uint32_t g = 0;
    int failed = 0;
    int item = blockIdx.x;
    int br = item / p.ntiles;
    int start = item < p.n_items ? __ldg(p.row_ptr + br) : 0;
    int end = item < p.n_items ? __ldg(p.row_ptr + br + 1) : 0;
    int mycol = (item < p.n_items && lane < end - start) ? __ldg(p.col_idx + start + lane) : 0;
    for (; item < p.n_items && !failed; item += gridDim.x) {
      const int nt = item - br * p.ntiles;
      // next item's row range, loaded now and used after this item's copies
      const int nitem = item + gridDim.x;
      const int nbr = nitem / p.ntiles;
      const int nstart = nitem < p.n_items ? __ldg(p.row_ptr + nbr) : 0;
      const int nend = nitem < p.n_items ? __ldg(p.row_ptr + nbr + 1) : 0;
      for (int base = start; base < end && !failed; base += 32) {
        const int cnt = min(32, end - base);
        s_cols[lane] = mycol;
        __syncwarp();
        // column indices of the next chunk (this item's, else the next item's first)
        const bool more = base + 32 < end;
        const int nb = more ? base + 32 : nstart;
        const int nn = more ? end : nend;
        mycol = (lane < nn - nb && (more || nitem < p.n_items)) ? __ldg(p.col_idx + nb + lane) : 0;
        if (lane == 0) {
          for (int i = 0; i < cnt; ++i, ++g) {
            const int s = (int)(g % STAGES);
            if (g >= (uint32_t)STAGES && !mbar_wait(empty0 + 8 * s, ((g / STAGES) + 1) & 1, p.timeout_ns)) {
              atomicOr(p.err, 4u);
              failed = 1;
              break;
            }
            const int col = s_cols[i];
            const uint32_t fb = full0 + 8 * s;
            mbar_arrive_expect_tx(fb, Cfg::kTx);
            uint8_t* a_dst = sA + (size_t)s * Cfg::kStageA;
            tma_tile_2d_g2s(smem_u32(a_dst), &tmA, 0, (base + i) * BR, fb, pol_a);
            if (Cfg::kSplit)
              tma_tile_2d_g2s(smem_u32(a_dst + Cfg::kABytesPad), &tmAlo, 0, (base + i) * BR, fb, pol_a);
            uint8_t* b_dst = sB + (size_t)s * Cfg::kStageB;
            if (p.panel3d) {
              tma_tile_3d_g2s(smem_u32(b_dst), &tmB, 0, col * 16, nt * (NT / 64), fb, pol_b);
              if (Cfg::kSplit)
                tma_tile_3d_g2s(smem_u32(b_dst + Cfg::kPanelBytes), &tmBlo, 0, col * 16, nt * (NT / 64), fb, pol_b);
            } else {
#pragma unroll
              for (int b = 0; b < NT / 64; ++b) {
                tma_tile_2d_g2s(smem_u32(b_dst + b * Cfg::kBoxBytes), &tmB, nt * NT + b * 64, col * 16, fb, pol_b);
                if (Cfg::kSplit)
                  tma_tile_2d_g2s(smem_u32(b_dst + Cfg::kPanelBytes + b * Cfg::kBoxBytes), &tmBlo,
                                  nt * NT + b * 64, col * 16, fb, pol_b);
              }
            }
          }
        }
        failed = __shfl_sync(0xffffffffu, failed, 0);
        __syncwarp();
      }
      if (start >= end) {
        // empty row: the prefetch above did not run; fetch the next item's first chunk
        mycol = (nitem < p.n_items && lane < nend - nstart) ? __ldg(p.col_idx + nstart + lane) : 0;
      }
      br = nbr;
      start = nstart;
      end = nend;
    }
  } else if (warp == 1) {
    // ------------------------------ MMA issuer -----------------------------------
    if (lane == 0) {
      uint32_t g = 0, it = 0;
      bool failed = false;
      int item = blockIdx.x;
      int start = item < p.n_items ? __ldg(p.row_ptr + item / p.ntiles) : 0;
      int end = item < p.n_items ? __ldg(p.row_ptr + item / p.ntiles + 1) : 0;
      for (; item < p.n_items && !failed; item += gridDim.x, ++it) {
        const int nitem = item + gridDim.x;
        const int nstart = nitem < p.n_items ? __ldg(p.row_ptr + nitem / p.ntiles) : 0;
        const int nend = nitem < p.n_items ? __ldg(p.row_ptr + nitem / p.ntiles + 1) : 0;
        const uint32_t acc = it & 1;
        if (it >= 2 && !mbar_wait(tempty0 + 8 * acc, ((it >> 1) + 1) & 1, p.timeout_ns)) {
          atomicOr(p.err, 8u);
          break;
        }
        tc_fence_after();
        const uint32_t d0 = tmem + acc * Cfg::kAccCols;
        for (int k = start; k < end; ++k, ++g) {
          const int s = (int)(g % STAGES);
          if (!mbar_wait(full0 + 8 * s, (g / STAGES) & 1, p.timeout_ns)) {
            atomicOr(p.err, 8u);
            failed = true;
            break;
          }
          tc_fence_after();
          const uint32_t a_addr = smem_u32(sA + (size_t)s * Cfg::kStageA);
          const uint32_t b_addr = smem_u32(sB + (size_t)s * Cfg::kStageB);
          const uint64_t blk_hi = smem_desc(a_addr, 16, 256, kLayoutSW32);
          const uint32_t accum = (k != start) ? 1u : 0u;
#pragma unroll
          for (int j = 0; j < Cfg::kJ; ++j) {
            const uint64_t pan_hi = smem_desc(b_addr + j * 2 * Cfg::kBoxBytes, 2048, 1024, kLayoutSW128);
            umma_f16(d0 + j * BR, pan_hi, blk_hi, Cfg::kIdesc, accum);
            if constexpr (Cfg::kSplit) {
              const uint64_t pan_lo =
                  smem_desc(b_addr + Cfg::kPanelBytes + j * 2 * Cfg::kBoxBytes, 2048, 1024, kLayoutSW128);
              const uint64_t blk_lo = smem_desc(a_addr + Cfg::kABytesPad, 16, 256, kLayoutSW32);
              umma_f16(d0 + j * BR, pan_lo, blk_hi, Cfg::kIdesc, 1u);
              umma_f16(d0 + j * BR, pan_hi, blk_lo, Cfg::kIdesc, 1u);
            }
          }
          umma_commit(empty0 + 8 * s);   // frees the ring slot once these MMAs have read it
        }
        if (failed) break;
        umma_commit(tfull0 + 8 * acc);   // accumulator ready (immediately, for an empty row)
        start = nstart;
        end = nend;
      }
      // every MMA this thread issued has completed before TMEM is released
      umma_commit(done_bar);
      if (!mbar_wait(done_bar, 0, p.timeout_ns)) atomicOr(p.err, 8u);
    }
    __syncwarp();
  } else if (warp >= 4) {
    // ------------------------------ epilogue (warps 4-7) ---------------------------
    const int q = warp & 3;                 // TMEM lane quarter this warp may access
    uint32_t it = 0;
    for (int item = blockIdx.x; item < p.n_items; item += gridDim.x, ++it) {
      const int br = item / p.ntiles, nt = item - br * p.ntiles;
      const bool empty = __ldg(p.row_ptr + br) == __ldg(p.row_ptr + br + 1);
      const uint32_t acc = it & 1;
      if (!mbar_wait(tfull0 + 8 * acc, (it >> 1) & 1, p.timeout_ns)) {
        if (lane == 0) atomicOr(p.err, 16u);
        break;
      }
      tc_fence_after();
      const long long row0 = (long long)br * BR;
#pragma unroll 1
      for (int j = 0; j < Cfg::kJ; ++j) {
        const int n = nt * NT + j * 128 + q * 32 + lane;
        float* cptr = p.C + row0 * p.ldc + n;
        const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + acc * Cfg::kAccCols + j * BR;
#pragma unroll
        for (int c0 = 0; c0 < BR; c0 += 16) {
          float v[16];
          if (!empty) {
            tmem_ld16(taddr + c0, v);
          } else {
#pragma unroll
            for (int i = 0; i < 16; ++i) v[i] = 0.f;
          }
          if (n < p.N) {
#pragma unroll
            for (int i = 0; i < 16; ++i) __stcs(cptr + (long long)(c0 + i) * p.ldc, v[i]);
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
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Cfg::kTmemCols)
                 : "memory");
  }
}

using TcFn = void (*)(const CUtensorMap, const CUtensorMap, const CUtensorMap, const CUtensorMap,
                      const TcParams);
struct TcEntry {
  int br, mode, nt, stages;
  TcFn fn;
  size_t smem;
  int tmem_cols;
};
#define SPMM_TC_ENTRY(BR, NT, ST, MODE) \
  TcEntry{BR, MODE, NT, ST, &k_bcsr_tc<BR, NT, ST, MODE>, TcCfg<BR, NT, ST, MODE>::kSmem, TcCfg<BR, NT, ST, MODE>::kTmemCols}

const TcEntry kTcEntries[] = {
    SPMM_TC_ENTRY(64, 128, 8, MODE_F16),   SPMM_TC_ENTRY(64, 256, 6, MODE_F16),
    SPMM_TC_ENTRY(64, 512, 6, MODE_F16),   SPMM_TC_ENTRY(32, 256, 8, MODE_F16),
    SPMM_TC_ENTRY(64, 128, 16, MODE_F16),  SPMM_TC_ENTRY(64, 256, 10, MODE_F16),
    SPMM_TC_ENTRY(64, 256, 4, MODE_F16),   SPMM_TC_ENTRY(64, 512, 10, MODE_F16),
    SPMM_TC_ENTRY(16, 256, 8, MODE_F16),   SPMM_TC_ENTRY(64, 128, 8, MODE_BF16),
    SPMM_TC_ENTRY(64, 256, 6, MODE_BF16),  SPMM_TC_ENTRY(64, 512, 6, MODE_BF16),
    SPMM_TC_ENTRY(32, 256, 8, MODE_BF16),  SPMM_TC_ENTRY(16, 256, 8, MODE_BF16),
    SPMM_TC_ENTRY(64, 256, 4, MODE_SPLIT), SPMM_TC_ENTRY(64, 128, 6, MODE_SPLIT),
};

}  // namespace

spmm_status launch_tc(const LaunchRequest& r) {
  const spmm_bcsr_desc& A = *r.A;
  const spmm_dense_desc& B = *r.B;
  int mode = A.dtype == SPMM_F16 ? MODE_F16 : A.dtype == SPMM_BF16 ? MODE_BF16
                                               : A.dtype == SPMM_F16_SPLIT ? MODE_SPLIT : -1;
  if (mode < 0) return fail(SPMM_ERR_UNSUPPORTED, "tcgen05 pipeline: fp16, bf16 and split fp16 only");
  int nt = r.cfg.n_tile;
  if (nt <= 0) nt = r.N >= 512 && A.bR == 64 && mode != MODE_SPLIT ? 256 : (r.N >= 256 ? 256 : 128);
  const TcEntry* e = nullptr;
  for (const TcEntry& c : kTcEntries)
    if (c.br == A.bR && c.mode == mode && c.nt == nt && (r.cfg.stages <= 0 || c.stages == r.cfg.stages)) {
      e = &c;
      break;
    }
  if (!e)
    return fail(SPMM_ERR_UNSUPPORTED, "no tcgen05 kernel for bR=" + std::to_string(A.bR) +
                                          " n_tile=" + std::to_string(nt));
  // A's values viewed as a [rows x 16] fp16 tensor; rows bounded by the densest
  // possible matrix (only coordinates of stored blocks are ever requested).
  const unsigned long long rows_bound = (unsigned long long)(A.M / A.bR) * (A.K / 16) * A.bR;
  if (rows_bound >= (1ull << 31)) return fail(SPMM_ERR_UNSUPPORTED, "A too large for the tcgen05 pipeline");
  CUtensorMap tmA, tmAlo, tmB, tmBlo;
  const void* vals = A.vals ? A.vals : B.data;   // no stored blocks: never dereferenced
  spmm_status st = encode_tile_map_2d(&tmA, CU_TENSOR_MAP_DATA_TYPE_UINT16, vals, 16, rows_bound, 32,
                                      16, (uint32_t)A.bR, CU_TENSOR_MAP_SWIZZLE_32B);
  if (st != SPMM_OK) return st;
  // B panels: one 3-D copy per panel when N is a multiple of 64, else one 2-D
  // copy per 64-column box.
  int panel3d = (r.N % 64 == 0 && r.cfg.kernel != 3) ? 1 : 0;
  if (panel3d && encode_panel_map_3d(&tmB, B.data, (uint64_t)r.N, (uint64_t)A.K, (uint64_t)B.ldb * 2,
                                     (uint32_t)(nt / 64)) != SPMM_OK)
    panel3d = 0;
  if (!panel3d) {
    st = encode_tile_map_2d(&tmB, CU_TENSOR_MAP_DATA_TYPE_UINT16, B.data, (uint64_t)r.N, (uint64_t)A.K,
                            (uint64_t)B.ldb * 2, 64, 16, CU_TENSOR_MAP_SWIZZLE_128B);
    if (st != SPMM_OK) return st;
  }
  tmAlo = tmA;
  tmBlo = tmB;
  if (mode == MODE_SPLIT) {
    const void* lo = A.vals_lo ? A.vals_lo : B.data_lo;
    st = encode_tile_map_2d(&tmAlo, CU_TENSOR_MAP_DATA_TYPE_UINT16, lo, 16, rows_bound, 32, 16,
                            (uint32_t)A.bR, CU_TENSOR_MAP_SWIZZLE_32B);
    if (st != SPMM_OK) return st;
    st = panel3d ? encode_panel_map_3d(&tmBlo, B.data_lo, (uint64_t)r.N, (uint64_t)A.K, (uint64_t)B.ldb * 2,
                                       (uint32_t)(nt / 64))
                 : encode_tile_map_2d(&tmBlo, CU_TENSOR_MAP_DATA_TYPE_UINT16, B.data_lo, (uint64_t)r.N,
                                      (uint64_t)A.K, (uint64_t)B.ldb * 2, 64, 16, CU_TENSOR_MAP_SWIZZLE_128B);
    if (st != SPMM_OK) return st;
  }
  TcParams p;
  p.row_ptr = A.row_ptr;
  p.col_idx = A.col_idx;
  p.C = r.C;
  p.ldc = r.ldc;
  p.N = r.N;
  p.ntiles = (r.N + nt - 1) / nt;
  p.n_items = (A.M / A.bR) * p.ntiles;
  p.timeout_ns = wait_limit_ns();
  p.err = device_error_word();
  p.panel3d = panel3d;
  if (!p.err) return fail(SPMM_ERR_CUDA, "could not set up the device error word");
  if (p.n_items == 0) return SPMM_OK;
  SPMM_CUDA_TRY(cudaFuncSetAttribute(reinterpret_cast<const void*>(e->fn),
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->smem));
  // CTAs per SM from the real limits: TMEM columns (512 per SM), shared memory
  // per SM, and the two CTAs the launch bounds budget registers for. (The
  // runtime's occupancy query reports one CTA per SM for this kernel, while two
  // run side by side.)
  int dev = 0, smem_sm = 0;
  SPMM_CUDA_TRY(cudaGetDevice(&dev));
  SPMM_CUDA_TRY(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
  const int tmem_fit = 512 / e->tmem_cols;
  const int smem_fit = smem_sm / (int)(e->smem + 1024);
  int per_sm = std::min(2, std::min(tmem_fit, smem_fit));
  if (r.cfg.ctas_per_sm > 0 && r.cfg.ctas_per_sm < per_sm) per_sm = r.cfg.ctas_per_sm;
  if (per_sm < 1) per_sm = 1;
  long long grid = (long long)sm_count() * per_sm;
  if (grid > p.n_items) grid = p.n_items;
  if (std::getenv("SPMM_DEBUG"))
    std::fprintf(stderr, "[spmm] tcgen05 bR=%d nt=%d stages=%d smem=%zu tmem=%d per_sm=%d grid=%lld items=%d panel3d=%d\n",
                 A.bR, nt, e->stages, e->smem, e->tmem_cols, per_sm, grid, p.n_items, panel3d);
  e->fn<<<(unsigned)grid, 256, e->smem, r.stream>>>(tmA, tmAlo, tmB, tmBlo, p);
  SPMM_CUDA_TRY(cudaGetLastError());
  return SPMM_OK;
}

}  // namespace spmm
