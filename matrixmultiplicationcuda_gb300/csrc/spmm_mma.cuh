// BCSR x dense product on the legacy tensor path (mma.sync m16n8k16), for any
// block height (16, 32, 64) and every storage type.
//
// Schedule: a persistent grid walks "items" = (block row, column tile of NT
// output columns). Within a CTA one producer warp streams, for every stored
// block of the item's block row, the A block (one untiled TMA bulk copy of its
// contiguous bR x 16 values) and the matching B row-panel (the 16 rows of B
// selected by col_idx, NT columns, as 128-byte-swizzled TMA tiles) into a
// STAGES-deep mbarrier ring. WM x WN consumer warps read fragments with
// ldmatrix and accumulate in fp32 registers, then write their part of C with
// streaming stores. The producer runs ahead across item boundaries, so one
// item's epilogue overlaps the next item's loads.
//
// This replaces the reference kernels' one-warp-per-tile loop that loads A and
// B fragments straight from global memory each k step
// (src/cuda_kernels.cu:301-328, :618-695, :699-762).
#pragma once
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cstdint>
#include "ptx.cuh"

namespace spmm {

enum Mode : int { MODE_F16 = 0, MODE_BF16 = 1, MODE_SPLIT = 2, MODE_E4M3 = 3 };

struct MmaParams {
  const int* row_ptr;
  const int* col_idx;
  const uint8_t* vals;
  const uint8_t* vals_lo;
  const float* scales;
  float* C;
  long long ldc;
  int MB;          // block rows
  int N;           // output columns
  int ntiles;      // ceil(N / NT)
  int n_items;     // MB * ntiles
  float b_scale;   // E4M3: scale of B
  unsigned long long timeout_ns;
  unsigned* err;   // device error word (bit 0: consumer wait timed out, bit 1: producer)
  int panel3d;     // 16-bit B panel loaded by one 3-D copy (N % 64 == 0)
};

template <int BR, int NT, int WM, int WN, int STAGES, int MODE>
struct MmaCfg {
  static constexpr int kConsumerWarps = WM * WN;
  static constexpr int kThreads = (kConsumerWarps + 1) * 32;
  static constexpr int kEsz = (MODE == MODE_E4M3) ? 1 : 2;
  static constexpr bool kSplit = (MODE == MODE_SPLIT);
  // B panel: TMA boxes of 16 rows x 128 bytes (64 fp16 or 128 e4m3 columns).
  static constexpr int kBoxCols = 128 / kEsz;
  static constexpr int kNBox = NT / kBoxCols;
  static constexpr int kBoxBytes = 16 * 128;
  static constexpr int kPanelBytes = kNBox * kBoxBytes;
  static constexpr int kABytes = BR * 16 * kEsz;
  static constexpr int kParts = kSplit ? 2 : 1;            // hi (+ lo)
  static constexpr int kStageB = kPanelBytes * kParts;      // multiple of 1024
  static constexpr int kStageA = kABytes * kParts;
  static constexpr int kTxBytes = kStageB + kStageA;
  static constexpr int kWTM = BR / WM;                      // warp tile rows
  static constexpr int kWTN = NT / WN;                      // warp tile cols
  static constexpr int kMT = kWTM / 16;
  static constexpr int kNT8 = kWTN / 8;
  static constexpr size_t kSmem = 1024 /*align slack*/ + (size_t)STAGES * (kStageB + kStageA) +
                                  (size_t)STAGES * 16 /*barriers*/ + 128 /*column staging*/;
  static_assert(BR % (16 * WM) == 0, "warp rows");
  static_assert(NT % (WN * (MODE == MODE_E4M3 ? 32 : 16)) == 0, "warp cols");
  static_assert(NT % kBoxCols == 0, "box cols");
  static_assert(kABytes % 16 == 0, "bulk copy granularity");
};

template <int BR, int NT, int WM, int WN, int STAGES, int MODE>
__global__ void __launch_bounds__(MmaCfg<BR, NT, WM, WN, STAGES, MODE>::kThreads, 1)
    k_bcsr_mma(const __grid_constant__ CUtensorMap tmB, const __grid_constant__ CUtensorMap tmBlo,
               const MmaParams p) {
  using Cfg = MmaCfg<BR, NT, WM, WN, STAGES, MODE>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  uint8_t* sB = smem;                                         // STAGES x kStageB
  uint8_t* sA = smem + (size_t)STAGES * Cfg::kStageB;         // STAGES x kStageA
  uint64_t* bars = reinterpret_cast<uint64_t*>(sA + (size_t)STAGES * Cfg::kStageA);
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + STAGES);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, Cfg::kConsumerWarps);
    }
    fence_mbar_init();
  }
  __syncthreads();
  grid_dep_launch_dependents();
  grid_dep_wait();

  if (warp == Cfg::kConsumerWarps) {
    // ------------------------------ producer warp ------------------------------
    // Lane 0 issues every copy; the other lanes stage column indices 32 at a time
    // in shared memory and prefetch the next item's row range, so the issuing
    // lane never waits on a global load or a shuffle between two blocks.
    int* s_cols = reinterpret_cast<int*>(bars + 2 * STAGES);
    if (lane == 0) {
      tma_prefetch_desc(&tmB);
      if (Cfg::kSplit) tma_prefetch_desc(&tmBlo);
    }
    const uint64_t pol_b = l2_policy_evict_last();    // B panels are re-read by other rows
    const uint64_t pol_a = l2_policy_evict_first();   // A blocks are read once per column tile
    uint32_t g = 0;
    int failed = 0;
    int item = blockIdx.x;
    int br = item / p.ntiles;
    int start = item < p.n_items ? __ldg(p.row_ptr + br) : 0;
    int end = item < p.n_items ? __ldg(p.row_ptr + br + 1) : 0;
    int mycol = (item < p.n_items && lane < end - start) ? __ldg(p.col_idx + start + lane) : 0;
    for (; item < p.n_items && !failed; item += gridDim.x) {
      const int nt = item - br * p.ntiles;
      const int nitem = item + gridDim.x;
      const int nbr = nitem / p.ntiles;
      const int nstart = nitem < p.n_items ? __ldg(p.row_ptr + nbr) : 0;
      const int nend = nitem < p.n_items ? __ldg(p.row_ptr + nbr + 1) : 0;
      for (int base = start; base < end && !failed; base += 32) {
        const int cnt = min(32, end - base);
        s_cols[lane] = mycol;
        __syncwarp();
        const bool more = base + 32 < end;
        const int nb = more ? base + 32 : nstart;
        const int nn = more ? end : nend;
        mycol = (lane < nn - nb && (more || nitem < p.n_items)) ? __ldg(p.col_idx + nb + lane) : 0;
        if (lane == 0) {
          for (int i = 0; i < cnt; ++i, ++g) {
            const int s = (int)(g % STAGES);
            if (g >= (uint32_t)STAGES &&
                !mbar_wait(empty0 + 8 * s, ((g / STAGES) + 1) & 1, p.timeout_ns)) {
              atomicOr(p.err, 2u);
              failed = 1;
              break;
            }
            const int col = s_cols[i];
            const uint32_t fb = full0 + 8 * s;
            mbar_arrive_expect_tx(fb, Cfg::kTxBytes);
            const size_t aoff = (size_t)(base + i) * Cfg::kABytes;
            uint8_t* a_dst = sA + (size_t)s * Cfg::kStageA;
            tma_bulk_g2s(smem_u32(a_dst), p.vals + aoff, Cfg::kABytes, fb, pol_a);
            if (Cfg::kSplit)
              tma_bulk_g2s(smem_u32(a_dst + Cfg::kABytes), p.vals_lo + aoff, Cfg::kABytes, fb, pol_a);
            uint8_t* b_dst = sB + (size_t)s * Cfg::kStageB;
            if (MODE != MODE_E4M3 && p.panel3d) {
              tma_tile_3d_g2s(smem_u32(b_dst), &tmB, 0, col * 16, nt * Cfg::kNBox, fb, pol_b);
              if (Cfg::kSplit)
                tma_tile_3d_g2s(smem_u32(b_dst + Cfg::kPanelBytes), &tmBlo, 0, col * 16, nt * Cfg::kNBox, fb, pol_b);
            } else {
#pragma unroll
              for (int b = 0; b < Cfg::kNBox; ++b) {
                tma_tile_2d_g2s(smem_u32(b_dst + b * Cfg::kBoxBytes), &tmB,
                                nt * NT + b * Cfg::kBoxCols, col * 16, fb, pol_b);
                if (Cfg::kSplit)
                  tma_tile_2d_g2s(smem_u32(b_dst + Cfg::kPanelBytes + b * Cfg::kBoxBytes), &tmBlo,
                                  nt * NT + b * Cfg::kBoxCols, col * 16, fb, pol_b);
              }
            }
          }
        }
        failed = __shfl_sync(0xffffffffu, failed, 0);
        __syncwarp();
      }
      if (start >= end)
        mycol = (nitem < p.n_items && lane < nend - nstart) ? __ldg(p.col_idx + nstart + lane) : 0;
      br = nbr;
      start = nstart;
      end = nend;
    }
    return;
  }

  // ------------------------------ consumer warps ---------------------------------
  const int wm = warp / WN, wn = warp - (warp / WN) * WN;
  const int gq = lane >> 2, tq = lane & 3;
  uint32_t g = 0;
  for (int item = blockIdx.x; item < p.n_items; item += gridDim.x) {
    const int br = item / p.ntiles, nt = item - br * p.ntiles;
    const int start = __ldg(p.row_ptr + br), end = __ldg(p.row_ptr + br + 1);
    float acc[Cfg::kMT][Cfg::kNT8][4];
#pragma unroll
    for (int i = 0; i < Cfg::kMT; ++i)
#pragma unroll
      for (int j = 0; j < Cfg::kNT8; ++j)
#pragma unroll
        for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;

    for (int k = start; k < end; ++k, ++g) {
      const int s = (int)(g % STAGES);
      if (!mbar_wait(full0 + 8 * s, (g / STAGES) & 1, p.timeout_ns)) {
        if (lane == 0) atomicOr(p.err, 1u);
        return;
      }
      const uint32_t a_base = smem_u32(sA + (size_t)s * Cfg::kStageA);
      const uint32_t b_base = smem_u32(sB + (size_t)s * Cfg::kStageB);
      if constexpr (MODE != MODE_E4M3) {
        // A fragments: rows wm*WTM + mt*16 .. +15, the block's 32-byte rows.
        uint32_t af[Cfg::kParts][Cfg::kMT][4];
#pragma unroll
        for (int part = 0; part < Cfg::kParts; ++part)
#pragma unroll
          for (int mt = 0; mt < Cfg::kMT; ++mt) {
            const int row = wm * Cfg::kWTM + mt * 16 + (lane & 7) + ((lane >> 3) & 1) * 8;
            ldsm_x4(a_base + part * Cfg::kABytes + row * 32 + (lane >> 4) * 16, af[part][mt][0],
                    af[part][mt][1], af[part][mt][2], af[part][mt][3]);
          }
#pragma unroll
        for (int np = 0; np < Cfg::kNT8 / 2; ++np) {
          const int n0 = wn * Cfg::kWTN + np * 16;       // first column of this 16-col pair
          const int kr = (lane & 7) + ((lane >> 3) & 1) * 8;
          const int chunk = ((n0 & 63) >> 3) + (lane >> 4);
          const uint32_t boff = (n0 >> 6) * Cfg::kBoxBytes + kr * 128 + ((chunk ^ (kr & 7)) << 4);
          uint32_t bh[4];
          ldsm_x4_t(b_base + boff, bh[0], bh[1], bh[2], bh[3]);
#pragma unroll
          for (int mt = 0; mt < Cfg::kMT; ++mt) {
            mma_16816<MODE == MODE_BF16>(acc[mt][2 * np], af[0][mt], bh[0], bh[1]);
            mma_16816<MODE == MODE_BF16>(acc[mt][2 * np + 1], af[0][mt], bh[2], bh[3]);
          }
          if constexpr (Cfg::kSplit) {
            uint32_t bl[4];
            ldsm_x4_t(b_base + Cfg::kPanelBytes + boff, bl[0], bl[1], bl[2], bl[3]);
#pragma unroll
            for (int mt = 0; mt < Cfg::kMT; ++mt) {
              mma_16816<false>(acc[mt][2 * np], af[0][mt], bl[0], bl[1]);       // hi * lo
              mma_16816<false>(acc[mt][2 * np + 1], af[0][mt], bl[2], bl[3]);
              mma_16816<false>(acc[mt][2 * np], af[1][mt], bh[0], bh[1]);       // lo * hi
              mma_16816<false>(acc[mt][2 * np + 1], af[1][mt], bh[2], bh[3]);
            }
          }
        }
      } else {
        // e4m3: A fragment from 16-byte rows, dequantised with the block scale
        // into fp16; B from the 128-byte swizzled e4m3 panel, split into even and
        // odd columns (see the store below for the column order).
        const float sc = __ldg(p.scales + k);
        uint32_t af[Cfg::kMT][4];
#pragma unroll
        for (int mt = 0; mt < Cfg::kMT; ++mt) {
          const int r0 = wm * Cfg::kWTM + mt * 16 + gq;
          const uint8_t* a8 = sA + (size_t)s * Cfg::kStageA;
          const uint32_t v[4] = {*reinterpret_cast<const uint16_t*>(a8 + r0 * 16 + 2 * tq),
                                 *reinterpret_cast<const uint16_t*>(a8 + (r0 + 8) * 16 + 2 * tq),
                                 *reinterpret_cast<const uint16_t*>(a8 + r0 * 16 + 2 * tq + 8),
                                 *reinterpret_cast<const uint16_t*>(a8 + (r0 + 8) * 16 + 2 * tq + 8)};
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            uint32_t h = e4m3x2_to_f16x2(v[r]);
            float2 f = __half22float2(*reinterpret_cast<__half2*>(&h));
            __half2 q = __floats2half2_rn(f.x * sc, f.y * sc);
            af[mt][r] = *reinterpret_cast<uint32_t*>(&q);
          }
        }
#pragma unroll
        for (int nq = 0; nq < Cfg::kWTN / 32; ++nq) {
          const int n0 = wn * Cfg::kWTN + nq * 32;        // 32 e4m3 columns = 2 chunks
          const int kr = (lane & 7) + ((lane >> 3) & 1) * 8;
          const int chunk = ((n0 & 127) >> 4) + (lane >> 4);
          const uint32_t boff = (n0 >> 7) * Cfg::kBoxBytes + kr * 128 + ((chunk ^ (kr & 7)) << 4);
          uint32_t r[4];
          ldsm_x4_t(b_base + boff, r[0], r[1], r[2], r[3]);
          // r[0]/r[1]: k 0-7 / 8-15 of columns n0..n0+15; r[2]/r[3]: n0+16..n0+31.
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const uint32_t e0 = e4m3x2_to_f16x2(byte_perm(r[2 * h], 0, 0x0020));
            const uint32_t e1 = e4m3x2_to_f16x2(byte_perm(r[2 * h + 1], 0, 0x0020));
            const uint32_t o0 = e4m3x2_to_f16x2(byte_perm(r[2 * h], 0, 0x0031));
            const uint32_t o1 = e4m3x2_to_f16x2(byte_perm(r[2 * h + 1], 0, 0x0031));
#pragma unroll
            for (int mt = 0; mt < Cfg::kMT; ++mt) {
              mma_16816<false>(acc[mt][nq * 4 + 2 * h], af[mt], e0, e1);
              mma_16816<false>(acc[mt][nq * 4 + 2 * h + 1], af[mt], o0, o1);
            }
          }
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(empty0 + 8 * s);
    }

    // ---------------------------- epilogue: C tile -------------------------------
    const long long row_base = (long long)br * BR + wm * Cfg::kWTM;
    const int col_base = nt * NT + wn * Cfg::kWTN;
    if constexpr (MODE != MODE_E4M3) {
#pragma unroll
      for (int mt = 0; mt < Cfg::kMT; ++mt)
#pragma unroll
        for (int j = 0; j < Cfg::kNT8; ++j) {
          const int col = col_base + j * 8 + 2 * tq;
          if (col < p.N) {
            float* c0 = p.C + (row_base + mt * 16 + gq) * p.ldc + col;
            __stcs(reinterpret_cast<float2*>(c0), make_float2(acc[mt][j][0], acc[mt][j][1]));
            __stcs(reinterpret_cast<float2*>(c0 + 8 * p.ldc), make_float2(acc[mt][j][2], acc[mt][j][3]));
          }
        }
    } else {
      // Tile 2h+0 holds columns 16q + 4t + {0, 2}, tile 2h+1 columns 16q + 4t + {1, 3}.
      const float bs = p.b_scale;
#pragma unroll
      for (int mt = 0; mt < Cfg::kMT; ++mt)
#pragma unroll
        for (int q = 0; q < Cfg::kNT8 / 2; ++q) {
          const int col = col_base + q * 16 + 4 * tq;
          if (col < p.N) {
            const float* e = acc[mt][2 * q];
            const float* o = acc[mt][2 * q + 1];
            float* c0 = p.C + (row_base + mt * 16 + gq) * p.ldc + col;
            __stcs(reinterpret_cast<float4*>(c0), make_float4(e[0] * bs, o[0] * bs, e[1] * bs, o[1] * bs));
            __stcs(reinterpret_cast<float4*>(c0 + 8 * p.ldc),
                   make_float4(e[2] * bs, o[2] * bs, e[3] * bs, o[3] * bs));
          }
        }
    }
  }
}

}  // namespace spmm
