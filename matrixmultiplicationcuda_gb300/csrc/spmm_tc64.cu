// BCSR x dense product for 64-row blocks on the tcgen05 tensor cores, one
// UMMA per block and 256 output columns.
//
// For a stored block A_blk (64 x 16) at block column c and output columns
// [n, n + 256):
//     D (64 x 256, fp32, TMEM) += A_blk (64 x 16, K-major) x B[16c : 16c+16, n : n+256]
// with tcgen05.mma.cta_group::1.kind::f16, M = 64, N = 256, K = 16. Row r of
// the block row lands in TMEM lane 32 * (r / 16) + r % 16 (lanes 0-15 of each
// 32-lane quarter) and output column n + j in TMEM column j. So epilogue warp
// q (4-7) reads rows 16q .. 16q + 15 with its lanes 0-15. Each of those threads
// holds 16 consecutive columns of one row per TMEM load and writes them as
// four 16-byte stores.
//
// Against the 128-column transposed form (spmm_tc.cu), a 64-row block costs
// half the UMMA instructions, and an M = 64, N = 256 instruction keeps the
// tensor pipe at full rate where M = 128, N = 64 runs at about half. The
// kernel runs one CTA per SM, so that CTA gets the SM's whole shared memory
// (a 5-deep ring of 4-block groups: 20 blocks in flight), all 512 TMEM
// columns (two 256-column accumulators) and the SM's L2 bandwidth.
//
// The roles and the ring protocol are those of the 128-column pipeline:
//   * warp 0 takes items and copies A groups;
//   * warps 2, 3, 8, 9 copy B panels;
//   * warp 1 issues the UMMAs;
//   * warps 4-7 run the epilogue.
// Every wait is bounded.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include "internal.h"
#include "ptx.cuh"
#include "spmm_mma.cuh"
#include "tcgen05.cuh"

namespace spmm {
namespace {

struct Tc64Params {
  const int* row_ptr;
  const int* col_idx;
  float* C;
  long long ldc;
  int N;
  int ntiles;
  int n_items;
  unsigned long long timeout_ns;
  unsigned* err;
  int panel3d;
  unsigned* queue;
};

// NT: output columns per item (256 or 512); STAGES: ring depth in groups;
// ACC: TMEM accumulators (ACC * NT = 512); G: blocks per group (one A copy).
template <int NT, int STAGES, int MODE, int ACC, int G>
struct Tc64Cfg {
  static constexpr int BR = 64;
  static constexpr bool kSplit = MODE == MODE_SPLIT;
  static constexpr int kParts = kSplit ? 2 : 1;
  static constexpr int kJ = NT / 256;                 // UMMAs per block (per part)
  static constexpr int kBoxBytes = 16 * 128;          // 16 rows x 64 fp16 columns
  static constexpr int kPanelBytes = (NT / 64) * kBoxBytes;
  static constexpr int kABytes = BR * 32;
  static constexpr int kAPart = G * kABytes;
  static constexpr int kAStage = ((kAPart * kParts + 1023) / 1024) * 1024;
  static constexpr int kStage = kAStage + G * kPanelBytes * kParts;
  static constexpr int kTmemCols = ACC * NT;
  // epilogue staging: per epilogue warp 16 rows x 64 columns fp32, rows padded
  // to 68 floats so the row-per-lane writes spread over the banks
  static constexpr int kStageRow = 68;
  static constexpr int kEpiBytes = 4 * 16 * kStageRow * 4;
  static constexpr size_t kSmem = 1024 + (size_t)STAGES * kStage + kEpiBytes + 1024;
  static_assert(kTmemCols == 512 || kTmemCols == 256, "TMEM columns");
  static_assert(G * BR <= 256 && 32 % G == 0, "a group is one TMA box and never straddles an index chunk");
  static_assert(kSmem <= 232448, "shared memory");
  // kind::f16: D f32, A K-major (the block), B MN-major (the panel), N = 256, M = 64
  static constexpr uint32_t kIdesc = (1u << 4) | ((MODE == MODE_BF16 ? 1u : 0u) << 7) |
                                     ((MODE == MODE_BF16 ? 1u : 0u) << 10) | (0u << 15) | (1u << 16) |
                                     ((uint32_t)(256 >> 3) << 17) | ((uint32_t)(64 >> 4) << 24);
};

constexpr int kTc64Threads = 320;

template <int NT, int STAGES, int MODE, int ACC, int G>
__global__ void __launch_bounds__(kTc64Threads, 1)
    k_bcsr_tc64(const __grid_constant__ CUtensorMap tmA1, const __grid_constant__ CUtensorMap tmAg,
                const __grid_constant__ CUtensorMap tmAlo1, const __grid_constant__ CUtensorMap tmAlog,
                const __grid_constant__ CUtensorMap tmB, const __grid_constant__ CUtensorMap tmBlo,
                const Tc64Params p) {
  using Cfg = Tc64Cfg<NT, STAGES, MODE, ACC, G>;
  constexpr int BR = Cfg::BR;
  constexpr int kQ = 4;
  constexpr int kBIssuers = 4;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  float* s_epi = reinterpret_cast<float*>(smem + (size_t)STAGES * Cfg::kStage);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)STAGES * Cfg::kStage + Cfg::kEpiBytes);
  const uint32_t full0 = smem_u32(bars), empty0 = full0 + 8 * STAGES;
  const uint32_t tfull0 = empty0 + 8 * STAGES, tempty0 = tfull0 + 16, done_bar = tempty0 + 16;
  const uint32_t qfull0 = done_bar + 8, qempty0 = qfull0 + 8 * kQ;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 5 + 2 * kQ);
  int* s_item = reinterpret_cast<int*>(tmem_slot + 1);      // kQ x {item, start, end}

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
    for (int q = 0; q < kQ; ++q) {
      mbar_init(qfull0 + 8 * q, 1);
      mbar_init(qempty0 + 8 * q, 1 + kBIssuers + 4);
    }
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
  grid_dep_launch_dependents();
  grid_dep_wait();

  auto read_item = [&](uint32_t it, int* item, int* start, int* end, unsigned code) -> bool {
    const uint32_t q = it % kQ;
    if (!mbar_wait(qfull0 + 8 * q, (it / kQ) & 1, p.timeout_ns)) {
      atomicOr(p.err, code);
      return false;
    }
    *item = s_item[3 * q];
    *start = s_item[3 * q + 1];
    *end = s_item[3 * q + 2];
    mbar_arrive(qempty0 + 8 * q);
    return true;
  };
  const int bidx = warp == 2 ? 0 : warp == 3 ? 1 : warp == 8 ? 2 : warp == 9 ? 3 : -1;

  if (warp == 0) {
    // ------------------------------ lead producer ----------------------------------
    if (lane == 0) {
      tma_prefetch_desc(&tmAg);
      tma_prefetch_desc(&tmA1);
      const uint64_t pol_a = l2_policy_evict_first();
      auto next_item = [&](int cur) -> int {
        int v = p.queue ? (int)atomicAdd(p.queue, 1u) : (cur < 0 ? (int)blockIdx.x : cur + (int)gridDim.x);
        return v < p.n_items ? v : -1;
      };
      // block range of an item: its block row's range
      auto range = [&](int v, int* s0, int* s1) {
        if (v < 0) {
          *s0 = *s1 = 0;
          return;
        }
        const int row = v / p.ntiles;
        *s0 = __ldg(p.row_ptr + row);
        *s1 = __ldg(p.row_ptr + row + 1);
      };
      uint32_t gs = 0, it = 0;
      bool failed = false;
      int item = next_item(-1);
      int start = 0, end = 0;
      range(item, &start, &end);
      for (;; ++it) {
        const uint32_t q = it % kQ;
        if (it >= (uint32_t)kQ && !mbar_wait(qempty0 + 8 * q, ((it / kQ) + 1) & 1, p.timeout_ns)) {
          atomicOr(p.err, 4u);
          failed = true;
        }
        s_item[3 * q] = failed ? -1 : item;
        s_item[3 * q + 1] = start;
        s_item[3 * q + 2] = end;
        mbar_arrive(qfull0 + 8 * q);
        if (item < 0 || failed) break;
        const int nitem = next_item(item);
        int nstart = 0, nend = 0;
        range(nitem, &nstart, &nend);
        for (int j0 = start; j0 < end; j0 += G, ++gs) {
          const int n = min(G, end - j0);
          const int s = (int)(gs % STAGES);
          if (gs >= (uint32_t)STAGES && !mbar_wait(empty0 + 8 * s, ((gs / STAGES) + 1) & 1, p.timeout_ns)) {
            atomicOr(p.err, 4u);
            failed = true;
            break;
          }
          const uint32_t fb = full0 + 8 * s;
          mbar_arrive_expect_tx(fb, (uint32_t)(n * (Cfg::kABytes + Cfg::kPanelBytes) * Cfg::kParts));
          uint8_t* a_dst = smem + (size_t)s * Cfg::kStage;
          const int y0 = j0 * BR;
          if (n == G) {
            tma_tile_2d_g2s(smem_u32(a_dst), &tmAg, 0, y0, fb, pol_a);
            if (Cfg::kSplit) tma_tile_2d_g2s(smem_u32(a_dst + Cfg::kAPart), &tmAlog, 0, y0, fb, pol_a);
          } else {
            for (int b = 0; b < n; ++b) {
              tma_tile_2d_g2s(smem_u32(a_dst + b * Cfg::kABytes), &tmA1, 0, y0 + b * BR, fb, pol_a);
              if (Cfg::kSplit)
                tma_tile_2d_g2s(smem_u32(a_dst + Cfg::kAPart + b * Cfg::kABytes), &tmAlo1, 0, y0 + b * BR,
                                fb, pol_a);
            }
          }
        }
        if (failed) break;
        item = nitem;
        start = nstart;
        end = nend;
      }
      if (p.queue) {
        __threadfence();
        if (atomicAdd(p.queue + 1, 1u) == gridDim.x - 1) {
          p.queue[0] = 0;
          p.queue[1] = 0;
          __threadfence();
        }
      }
    }
    __syncwarp();
  } else if (bidx >= 0) {
    // ------------------------------ B-panel issuers ----------------------------------
    if (lane == 0) tma_prefetch_desc(&tmB);
    const uint64_t pol_b = l2_policy_evict_last();
    uint32_t gs = 0;
    int failed = 0;
    for (uint32_t it = 0; !failed; ++it) {
      int item = -1, start = 0, end = 0, ok = 1;
      if (lane == 0) ok = read_item(it, &item, &start, &end, 4u) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      item = __shfl_sync(0xffffffffu, item, 0);
      start = __shfl_sync(0xffffffffu, start, 0);
      end = __shfl_sync(0xffffffffu, end, 0);
      if (!ok || item < 0) break;
      const int nt = item % p.ntiles;
      int mycol = lane < end - start ? __ldg(p.col_idx + start + lane) : 0;
      for (int base = start; base < end && !failed; base += 32) {
        const int cnt = min(32, end - base);
        const int cur = mycol;
        if (base + 32 < end) mycol = lane < end - base - 32 ? __ldg(p.col_idx + base + 32 + lane) : 0;
        for (int i0 = 0; i0 < cnt; i0 += G, ++gs) {
          const int n = min(G, cnt - i0);
          const int s = (int)(gs % STAGES);
          // wait only in groups this issuer copies into (such a group cannot
          // release its slot without these bytes: at most one phase behind)
          int bad = 0;
          if (lane == 0 && bidx < n && gs >= (uint32_t)STAGES &&
              !mbar_wait(empty0 + 8 * s, ((gs / STAGES) + 1) & 1, p.timeout_ns)) {
            atomicOr(p.err, 4u);
            bad = 1;
          }
          failed = __shfl_sync(0xffffffffu, bad, 0);
          if (failed) break;
          uint8_t* b_dst0 = smem + (size_t)s * Cfg::kStage + Cfg::kAStage;
          for (int b = bidx; b < n; b += kBIssuers) {
            const int col = __shfl_sync(0xffffffffu, cur, i0 + b);
            if (lane == 0) {
              const uint32_t fb = full0 + 8 * s;
              uint8_t* b_dst = b_dst0 + (size_t)b * Cfg::kPanelBytes * Cfg::kParts;
              if (p.panel3d) {
                tma_tile_3d_g2s(smem_u32(b_dst), &tmB, 0, col * 16, nt * (NT / 64), fb, pol_b);
                if (Cfg::kSplit)
                  tma_tile_3d_g2s(smem_u32(b_dst + Cfg::kPanelBytes), &tmBlo, 0, col * 16, nt * (NT / 64), fb, pol_b);
              } else {
#pragma unroll
                for (int bx = 0; bx < NT / 64; ++bx) {
                  tma_tile_2d_g2s(smem_u32(b_dst + bx * Cfg::kBoxBytes), &tmB, nt * NT + bx * 64, col * 16, fb, pol_b);
                  if (Cfg::kSplit)
                    tma_tile_2d_g2s(smem_u32(b_dst + Cfg::kPanelBytes + bx * Cfg::kBoxBytes), &tmBlo,
                                    nt * NT + bx * 64, col * 16, fb, pol_b);
                }
              }
            }
          }
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------ MMA issuer -----------------------------------
    if (lane == 0) {
      uint32_t gs = 0, it = 0;
      bool failed = false;
      for (;; ++it) {
        int item, start, end;
        if (!read_item(it, &item, &start, &end, 8u) || item < 0) break;
        const uint32_t acc = it % ACC;
        if (it >= (uint32_t)ACC && !mbar_wait(tempty0 + 8 * acc, ((it / ACC) + 1) & 1, p.timeout_ns)) {
          atomicOr(p.err, 8u);
          break;
        }
        tc_fence_after();
        const uint32_t d0 = tmem + acc * NT;
        for (int j0 = start; j0 < end; j0 += G, ++gs) {
          const int n = min(G, end - j0);
          const int s = (int)(gs % STAGES);
          if (!mbar_wait(full0 + 8 * s, (gs / STAGES) & 1, p.timeout_ns)) {
            atomicOr(p.err, 8u);
            failed = true;
            break;
          }
          tc_fence_after();
          const uint32_t a_slot = smem_u32(smem + (size_t)s * Cfg::kStage);
          const uint32_t b_slot = a_slot + Cfg::kAStage;
          for (int b = 0; b < n; ++b) {
            const uint32_t b_addr = b_slot + b * Cfg::kPanelBytes * Cfg::kParts;
            const uint64_t blk_hi = smem_desc(a_slot + b * Cfg::kABytes, 16, 256, kLayoutSW32);
            const uint32_t accum = (j0 + b != start) ? 1u : 0u;
#pragma unroll
            for (int j = 0; j < Cfg::kJ; ++j) {
              const uint64_t pan_hi = smem_desc(b_addr + j * 4 * Cfg::kBoxBytes, 2048, 1024, kLayoutSW128);
              umma_f16(d0 + j * 256, blk_hi, pan_hi, Cfg::kIdesc, accum);
              if constexpr (Cfg::kSplit) {
                const uint64_t pan_lo =
                    smem_desc(b_addr + Cfg::kPanelBytes + j * 4 * Cfg::kBoxBytes, 2048, 1024, kLayoutSW128);
                const uint64_t blk_lo = smem_desc(a_slot + Cfg::kAPart + b * Cfg::kABytes, 16, 256, kLayoutSW32);
                umma_f16(d0 + j * 256, blk_hi, pan_lo, Cfg::kIdesc, 1u);
                umma_f16(d0 + j * 256, blk_lo, pan_hi, Cfg::kIdesc, 1u);
              }
            }
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
  } else if (warp >= 4 && warp < 8) {
    // ------------------------------ epilogue (warps 4-7) ---------------------------
    // Warp q reads TMEM lanes 32q .. 32q + 31, of which lanes 0-15 hold rows
    // 16q .. 16q + 15. Per 64 columns: four TMEM loads (16 columns each) into
    // the warp's staging rows, then 256-byte row segments out to C (lanes
    // 0-15 one row, lanes 16-31 the next, a float4 each).
    const int q4 = warp & 3;
    float* stg = s_epi + q4 * 16 * Cfg::kStageRow;
    for (uint32_t it = 0;; ++it) {
      int item = -1, start = 0, end = 0, ok = 1;
      if (lane == 0) ok = read_item(it, &item, &start, &end, 16u) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      item = __shfl_sync(0xffffffffu, item, 0);
      const bool empty = __shfl_sync(0xffffffffu, start == end ? 1 : 0, 0) != 0;
      if (!ok || item < 0) break;
      const int br = item / p.ntiles, nt = item % p.ntiles;
      const uint32_t acc = it % ACC;
      if (!mbar_wait(tfull0 + 8 * acc, (it / ACC) & 1, p.timeout_ns)) {
        if (lane == 0) atomicOr(p.err, 16u);
        break;
      }
      tc_fence_after();
      float* cblk = p.C + ((long long)br * BR + 16 * q4) * p.ldc;
      const uint32_t taddr = tmem + ((uint32_t)(q4 * 32) << 16) + acc * NT;
#pragma unroll 1
      for (int c64 = 0; c64 < NT; c64 += 64) {
        const int n0 = nt * NT + c64;
        if (n0 >= p.N) break;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          float v[16];
          if (!empty) {
            tmem_ld16(taddr + c64 + 16 * k, v);
          } else {
#pragma unroll
            for (int i = 0; i < 16; ++i) v[i] = 0.f;
          }
          if (lane < 16) {
            float4* dst = reinterpret_cast<float4*>(stg + lane * Cfg::kStageRow + 16 * k);
#pragma unroll
            for (int i = 0; i < 4; ++i) dst[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
          }
        }
        __syncwarp();
        const int c4 = lane & 15;
        const int n = n0 + 4 * c4;
#pragma unroll
        for (int r0 = 0; r0 < 16; r0 += 2) {
          const int r = r0 + (lane >> 4);
          const float4 x = *reinterpret_cast<const float4*>(stg + r * Cfg::kStageRow + 4 * c4);
          float* dstp = cblk + (long long)r * p.ldc + n;
          if (n + 4 <= p.N) {
            __stcs(reinterpret_cast<float4*>(dstp), x);
          } else if (n < p.N) {
            const float xs[4] = {x.x, x.y, x.z, x.w};
            for (int i = 0; i < 4 && n + i < p.N; ++i) __stcs(dstp + i, xs[i]);
          }
        }
        __syncwarp();
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

using Tc64Fn = void (*)(const CUtensorMap, const CUtensorMap, const CUtensorMap, const CUtensorMap,
                        const CUtensorMap, const CUtensorMap, const Tc64Params);
struct Tc64Entry {
  int mode, nt, stages, acc, group;
  Tc64Fn fn;
  size_t smem;
};
#define SPMM_TC64_ENTRY(NT, ST, MODE, ACC, G) \
  Tc64Entry{MODE, NT, ST, ACC, G, &k_bcsr_tc64<NT, ST, MODE, ACC, G>, Tc64Cfg<NT, ST, MODE, ACC, G>::kSmem}
// (column tile, ring depth in groups, accumulators, group size); the first
// entry of a (type, column tile) is its default
const Tc64Entry kTc64Entries[] = {
    SPMM_TC64_ENTRY(256, 5, MODE_F16, 2, 4),   SPMM_TC64_ENTRY(256, 8, MODE_F16, 2, 2),
    SPMM_TC64_ENTRY(512, 5, MODE_F16, 1, 2),   SPMM_TC64_ENTRY(512, 4, MODE_F16, 1, 2),
    SPMM_TC64_ENTRY(256, 5, MODE_BF16, 2, 4),  SPMM_TC64_ENTRY(256, 8, MODE_BF16, 2, 2),
    SPMM_TC64_ENTRY(512, 5, MODE_BF16, 1, 2),  SPMM_TC64_ENTRY(512, 4, MODE_BF16, 1, 2),
    SPMM_TC64_ENTRY(256, 5, MODE_SPLIT, 2, 2), SPMM_TC64_ENTRY(512, 2, MODE_SPLIT, 1, 2),
};

int tc64_mode(spmm_dtype d) {
  return d == SPMM_F16 ? MODE_F16 : d == SPMM_BF16 ? MODE_BF16 : d == SPMM_F16_SPLIT ? MODE_SPLIT : -1;
}

const Tc64Entry* find_tc64(int mode, int N, const spmm_config& cfg, int* nt_out) {
  int nt = cfg.n_tile > 0 ? cfg.n_tile : (N <= 256 ? 256 : 512);
  *nt_out = nt;
  for (const Tc64Entry& c : kTc64Entries) {
    if (c.mode != mode || c.nt != nt) continue;
    if (cfg.stages > 0 && c.stages != cfg.stages) continue;
    if (cfg.acc_buffers > 0 && c.acc != cfg.acc_buffers) continue;
    return &c;
  }
  return nullptr;
}

}  // namespace

bool tc64_supported(int bR, spmm_dtype dtype, int N, const spmm_config& cfg) {
  const int mode = tc64_mode(dtype);
  int nt = 0;
  // no split-K: lanes map to rows here, so partial sums would be added with
  // one uncoalesced atomic per element
  return bR == 64 && mode >= 0 && cfg.split_k <= 1 && find_tc64(mode, N, cfg, &nt) != nullptr;
}

spmm_status launch_tc64(const LaunchRequest& r) {
  const spmm_bcsr_desc& A = *r.A;
  const spmm_dense_desc& B = *r.B;
  const int mode = tc64_mode(A.dtype);
  if (A.bR != 64 || mode < 0)
    return fail(SPMM_ERR_UNSUPPORTED, "64-row tcgen05 pipeline: 64-row blocks, fp16 / bf16 / split fp16");
  int nt = 0;
  const Tc64Entry* e = find_tc64(mode, r.N, r.cfg, &nt);
  if (!e) return fail(SPMM_ERR_UNSUPPORTED, "no 64-row tcgen05 kernel for n_tile=" + std::to_string(nt));
  const unsigned long long rows_bound =
      std::max<unsigned long long>((unsigned long long)(A.M / 64) * (A.K / 16) * 64, 256ull);
  if (rows_bound >= (1ull << 31)) return fail(SPMM_ERR_UNSUPPORTED, "A too large for the tcgen05 pipeline");
  CUtensorMap tmA1, tmAg, tmAlo1, tmAlog, tmB, tmBlo;
  const void* vals = A.vals ? A.vals : B.data;   // no stored blocks: never dereferenced
  spmm_status st = encode_tile_map_2d(&tmA1, CU_TENSOR_MAP_DATA_TYPE_UINT16, vals, 16, rows_bound, 32, 16, 64,
                                      CU_TENSOR_MAP_SWIZZLE_32B);
  if (st != SPMM_OK) return st;
  st = encode_tile_map_2d(&tmAg, CU_TENSOR_MAP_DATA_TYPE_UINT16, vals, 16, rows_bound, 32, 16,
                          (uint32_t)(e->group * 64), CU_TENSOR_MAP_SWIZZLE_32B);
  if (st != SPMM_OK) return st;
  int panel3d = (r.N % 64 == 0) ? 1 : 0;
  if (panel3d && encode_panel_map_3d(&tmB, B.data, (uint64_t)r.N, (uint64_t)A.K, (uint64_t)B.ldb * 2,
                                     (uint32_t)(nt / 64)) != SPMM_OK)
    panel3d = 0;
  if (!panel3d) {
    st = encode_tile_map_2d(&tmB, CU_TENSOR_MAP_DATA_TYPE_UINT16, B.data, (uint64_t)r.N, (uint64_t)A.K,
                            (uint64_t)B.ldb * 2, 64, 16, CU_TENSOR_MAP_SWIZZLE_128B);
    if (st != SPMM_OK) return st;
  }
  tmAlo1 = tmA1;
  tmAlog = tmAg;
  tmBlo = tmB;
  if (mode == MODE_SPLIT) {
    const void* lo = A.vals_lo ? A.vals_lo : B.data_lo;
    st = encode_tile_map_2d(&tmAlo1, CU_TENSOR_MAP_DATA_TYPE_UINT16, lo, 16, rows_bound, 32, 16, 64,
                            CU_TENSOR_MAP_SWIZZLE_32B);
    if (st != SPMM_OK) return st;
    st = encode_tile_map_2d(&tmAlog, CU_TENSOR_MAP_DATA_TYPE_UINT16, lo, 16, rows_bound, 32, 16,
                            (uint32_t)(e->group * 64), CU_TENSOR_MAP_SWIZZLE_32B);
    if (st != SPMM_OK) return st;
    st = panel3d ? encode_panel_map_3d(&tmBlo, B.data_lo, (uint64_t)r.N, (uint64_t)A.K, (uint64_t)B.ldb * 2,
                                       (uint32_t)(nt / 64))
                 : encode_tile_map_2d(&tmBlo, CU_TENSOR_MAP_DATA_TYPE_UINT16, B.data_lo, (uint64_t)r.N,
                                      (uint64_t)A.K, (uint64_t)B.ldb * 2, 64, 16, CU_TENSOR_MAP_SWIZZLE_128B);
    if (st != SPMM_OK) return st;
  }
  Tc64Params p;
  p.row_ptr = A.row_ptr;
  p.col_idx = A.col_idx;
  p.C = r.C;
  p.ldc = r.ldc;
  p.N = r.N;
  p.ntiles = (r.N + nt - 1) / nt;
  if (r.cfg.split_k > 1) return fail(SPMM_ERR_UNSUPPORTED, "the 64-row pipeline has no split-K");
  const long long n_items = (long long)(A.M / 64) * p.ntiles;
  if (n_items >= (1ll << 30)) return fail(SPMM_ERR_UNSUPPORTED, "too many work items");
  p.n_items = (int)n_items;
  p.timeout_ns = wait_limit_ns();
  p.err = r.err_word ? r.err_word : device_error_word();
  p.panel3d = panel3d;
  p.queue = r.queue ? r.queue : (r.cfg.schedule == 1 ? work_queue_slot() : nullptr);
  if (!p.err) return fail(SPMM_ERR_CUDA, "could not set up the device error word");
  if (p.n_items == 0) return SPMM_OK;
  SPMM_CUDA_TRY(ensure_smem_attr(reinterpret_cast<const void*>(e->fn), (int)e->smem));
  long long grid = sm_count();
  if (grid > p.n_items) grid = p.n_items;
  if (std::getenv("SPMM_DEBUG"))
    std::fprintf(stderr, "[spmm] tcgen05-64 nt=%d stages=%d acc=%d group=%d smem=%zu grid=%lld items=%d queue=%d\n",
                 nt, e->stages, e->acc, e->group, e->smem, grid, p.n_items, p.queue != nullptr);
  SPMM_CUDA_TRY(launch_kernel(e->fn, dim3((unsigned)grid), dim3(kTc64Threads), e->smem, r.stream, tmA1, tmAg, tmAlo1,
                              tmAlog, tmB, tmBlo, p));
  return SPMM_OK;
}

}  // namespace spmm
